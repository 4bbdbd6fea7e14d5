// propagate.cu — the delta kick (tddft_excite.f90), the dipole (tddft_plot.f90),
// the RK4 step with stage-wise rebuild (rk4.f90, tddft_prop.f90) and the
// TDDFT time loop (tddft.f90:67-91), plus the C ABI of the rebuild chain.
//
// Precision modes:
//   OPAW_PREC_FP64  : everything complex128 / double.
//   OPAW_PREC_MIXED : S^-1/2 H S^-1/2, the S^-1/2 of the rebuild, the density
//                     and box sums on complex64 orbitals; psi, the RK4
//                     accumulation p = p + dt/6 sum_k, the norms, rho_ij,
//                     potentials, D_ij, S^-1/2 coefficients and the dipole in
//                     double.
#include <cmath>

#include "fft.cuh"

namespace opaw {

template <typename R> int rebuild_from(opaw_ctx *c, int set, const typename Tr<R>::C *psibar, int norb);
template <typename R> int rhoij_density_from(opaw_ctx *c, int set, const typename Tr<R>::C *psit, int norb, int what);
int nhat_step(opaw_ctx *c, int set);
int vks_step(opaw_ctx *c, int set, int fp32_hartree);
int dij_step(opaw_ctx *c, int set);

__device__ __forceinline__ double bsum256(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) r += sh[i];
  return r;
}

// --------------------------------------------------------------- kick --
// pp = p * exp(-i gamma r_ipol), r = (i - n/2) d   (tddft_excite.f90:11-12)
__global__ void k_excite(const double2 *__restrict__ p, double2 *__restrict__ pp, int64_t nn, int norb, int nx,
                         int ny, int nz, int ipol, double gamma, double dx, double dy, double dz) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= nn) return;
  const int x = (int)(g % nx), y = (int)((g / nx) % ny), z = (int)(g / ((int64_t)nx * ny));
  double r;
  if (ipol == 1) r = (double)(x - nx / 2) * dx;
  else if (ipol == 2) r = (double)(y - ny / 2) * dy;
  else r = (double)(z - nz / 2) * dz;
  double sn, cs;
  sincos(-gamma * r, &sn, &cs);
  for (int o = 0; o < norb; o++) {
    const double2 v = p[(int64_t)o * nn + g];
    pp[(int64_t)o * nn + g] = make_double2(v.x * cs - v.y * sn, v.x * sn + v.y * cs);
  }
}

// ------------------------------------------------------------- dipole --
// partial sums of dv * r * rho for both sets, rho = 2 sum |psi|^2
// (tddft_plot.f90:40-55, 116-147)
constexpr int kDipBlocks = 512;
__global__ void k_dipole_part(const double2 *__restrict__ p0, const double2 *__restrict__ p1, int norb, int64_t nn,
                              int nx, int ny, int nz, double dx, double dy, double dz, double dv,
                              double *__restrict__ part) {
  __shared__ double sh[8];
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nn; g += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(g % nx), y = (int)((g / nx) % ny), z = (int)(g / ((int64_t)nx * ny));
    const double r[3] = {(double)(x - nx / 2) * dx, (double)(y - ny / 2) * dy, (double)(z - nz / 2) * dz};
    double rho0 = 0, rho1 = 0;
    for (int o = 0; o < norb; o++) {
      const double2 a = p0[(int64_t)o * nn + g], b = p1[(int64_t)o * nn + g];
      rho0 += a.x * a.x + a.y * a.y;
      rho1 += b.x * b.x + b.y * b.y;
    }
    rho0 *= 2.0;
    rho1 *= 2.0;
    for (int k = 0; k < 3; k++) {
      acc[k] += dv * r[k] * rho0;
      acc[3 + k] += dv * r[k] * rho1;
    }
  }
  for (int k = 0; k < 6; k++) {
    const double s = bsum256(acc[k], sh);
    if (threadIdx.x == 0) part[6 * blockIdx.x + k] = s;
  }
}

// out[0..2] dip, [3..5] dip_pert, [6..8] d_dip = (dip_pert - dip)/gamma
__global__ void k_dipole_final(const double *__restrict__ part, int nb, double gamma, double *__restrict__ out) {
  __shared__ double sh[8];
  double s[6];
  for (int k = 0; k < 6; k++) s[k] = block_sum_seq(part + k, nb, 6, sh);
  if (threadIdx.x != 0) return;
  for (int k = 0; k < 6; k++) out[k] = s[k];
  for (int k = 0; k < 3; k++) out[6 + k] = (s[3 + k] - s[k]) / gamma;  // tddft_plot.f90:57
}

// ----------------------------------------------------------- RK4 pieces --
constexpr int kNormBlocks = 64;
template <typename C>
__global__ void k_norm_part(const C *__restrict__ p, int64_t nn, double *__restrict__ part) {
  __shared__ double sh[8];
  const int o = blockIdx.y;
  const C *q = p + (int64_t)o * nn;
  double acc = 0;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nn; g += (int64_t)gridDim.x * blockDim.x) {
    const C z = q[g];
    const double x = z.x, y = z.y;
    acc += x * x + y * y;
  }
  acc = bsum256(acc, sh);
  if (threadIdx.x == 0) part[(int64_t)o * gridDim.x + blockIdx.x] = acc;
}

// nrm[o] = sqrt(dv * sum |p_o|^2)   (rk4.f90:87, :98)
__global__ void k_norm_final(const double *__restrict__ part, int nb, int norb, double dv, double *__restrict__ nrm) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= norb) return;
  double s = 0;
  for (int b = 0; b < nb; b++) s += part[(int64_t)o * nb + b];
  nrm[o] = sqrt(dv * s);
}

template <typename C> static int norms(opaw_ctx *c, const C *p, int norb, double *part, double *nrm) {
  dim3 g(kNormBlocks, norb);
  k_norm_part<C><<<g, 256, 0, c->stream>>>(p, c->nn, part);
  k_norm_final<<<grid1(norb, 128), 128, 0, c->stream>>>(part, kNormBlocks, norb, c->dv, nrm);
  c->launches += 2;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

// stage update (rk4.f90:44-48): k = -i * shs(pin); ksum (+)= w k; y = p + dts k.
// Arithmetic in the precision of the stage vectors: FP64 for the FP64 path,
// FP32 for the mixed path (p is read as FP64 and rounded once).
template <typename R>
__global__ void k_rk4_stage(const typename Tr<R>::C *__restrict__ kraw, const double2 *__restrict__ p,
                            typename Tr<R>::C *__restrict__ ksum, typename Tr<R>::C *__restrict__ y, int64_t n,
                            R w, int first, R dts, int write_y) {
  typedef typename Tr<R>::C C;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const C kr = kraw[i];
  const R kx = kr.y, ky = -kr.x;  // -i*(a + ib) = b - ia
  C s;
  if (first) {
    s.x = w * kx;
    s.y = w * ky;
  } else {
    s = ksum[i];
    s.x += w * kx;
    s.y += w * ky;
  }
  ksum[i] = s;
  if (write_y) {
    const double2 pv = p[i];
    C yv;
    yv.x = (R)pv.x + dts * kx;
    yv.y = (R)pv.y + dts * ky;
    y[i] = yv;
  }
}

// p = p + dt/6 ksum  (rk4.f90:22)
template <typename CS>
__global__ void k_rk4_final(double2 *__restrict__ p, const CS *__restrict__ ksum, int64_t n, double h6) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const CS s = ksum[i];
  double2 v = p[i];
  v.x += h6 * (double)s.x;
  v.y += h6 * (double)s.y;
  p[i] = v;
}

// f[o] = nrm0[o] / nrm1[o], then p_o *= f[o]  (rk4.f90:99)
__global__ void k_rescale_factor(const double *__restrict__ nrm0, double *__restrict__ nrm1, int norb) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o < norb) nrm1[o] = nrm0[o] / nrm1[o];
}
__global__ void k_rescale(double2 *__restrict__ p, int64_t nn, const double *__restrict__ f) {
  const int o = blockIdx.y;
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= nn) return;
  const double s = f[o];
  double2 v = p[(int64_t)o * nn + g];
  v.x *= s;
  v.y *= s;
  p[(int64_t)o * nn + g] = v;
}

__global__ void k_down(const double2 *__restrict__ a, float2 *__restrict__ b, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    const double2 v = a[i];
    b[i] = make_float2(d2f(v.x), d2f(v.y));
  }
}

static int scratch_red(opaw_ctx *c, double **part, double **nrm0, double **nrm1, double **dip, int norb) {
  // norm partials, nrm0, nrm1, dipole partials
  OPAW_CHECK(ensure(c->work[10], sizeof(double) * ((size_t)norb * kNormBlocks + 2 * (size_t)norb + 6 * kDipBlocks + 16)));
  double *w = (double *)c->work[10].p;
  *part = w;
  *nrm0 = w + (size_t)norb * kNormBlocks;
  *nrm1 = *nrm0 + norb;
  *dip = *nrm1 + norb;
  return OPAW_OK;
}

// one rk4_prop_shs pass over one set (rk4.f90:15-33), FP64.  Each stage's
// shs starts from S^-1/2 y and <p~|S^-1/2 y>, which the rebuild that precedes
// it (the loop-top rebuild for stage 1, rk4.f90:53-55 for the others) has
// just computed from the same y: the identical values are reused.
static int rk4_set64(opaw_ctx *c, int set, double dt) {
  typedef double2 C;
  const int norb = c->norb[set];
  const int64_t tot = c->nn * (int64_t)norb;
  double2 *p = c->d_psi[set];
  OPAW_CHECK(ensure(c->work[7], sizeof(C) * tot));
  OPAW_CHECK(ensure(c->work[8], sizeof(C) * tot));
  OPAW_CHECK(ensure(c->work[9], sizeof(C) * tot));
  C *k = (C *)c->work[7].p, *y = (C *)c->work[8].p, *ks = (C *)c->work[9].p;
  double *part, *nrm0, *nrm1, *dipw;
  OPAW_CHECK(scratch_red(c, &part, &nrm0, &nrm1, &dipw, norb));
  OPAW_CHECK(norms<double2>(c, p, norb, part, nrm0));  // norm0 (rk4.f90:16)
  const double wts[4] = {1.0, 2.0, 2.0, 1.0};
  const double dts[4] = {dt / 2.0, dt / 2.0, dt, dt};
  for (int st = 0; st < 4; st++) {
    // shs (shs.f90:19-22) from the rebuild's S^-1/2 y (work[4]) and projections (coef[0])
    OPAW_CHECK(h_apply_ex<double>(c, c->d_vks[set], c->d_dij[set], (const C *)c->work[4].p, k, norb,
                                  (const double2 *)c->coef[0].p, nullptr, nullptr, nullptr, nullptr));
    OPAW_CHECK(sn_apply<double>(c, -0.5, k, k, norb));
    k_rk4_stage<double><<<grid1(tot, 256), 256, 0, c->stream>>>(k, p, ks, y, tot, wts[st], st == 0, dts[st], st < 3);
    c->launches++;
    OPAW_CUDA(cudaGetLastError());
    if (st < 3) OPAW_CHECK(rebuild_from<double>(c, set, y, norb));  // rk4.f90:53-55
  }
  k_rk4_final<C><<<grid1(tot, 256), 256, 0, c->stream>>>(p, ks, tot, dt / 6.0);
  c->launches++;
  OPAW_CHECK(norms<double2>(c, p, norb, part, nrm1));  // norm1 (rk4.f90:98)
  k_rescale_factor<<<grid1(norb, 128), 128, 0, c->stream>>>(nrm0, nrm1, norb);
  dim3 g(grid1(c->nn, 256), norb);
  k_rescale<<<g, 256, 0, c->stream>>>(p, c->nn, nrm1);
  c->launches += 2;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

// rebuild from the resident orbitals of `set` in the given precision
static int rebuild_resident(opaw_ctx *c, int set, int prec) {
  const int norb = c->norb[set];
  if (prec == OPAW_PREC_FP64) return rebuild_from<double>(c, set, c->d_psi[set], norb);
  const int64_t tot = c->nn * (int64_t)norb;
  OPAW_CHECK(ensure(c->work[8], sizeof(float2) * tot));
  float2 *y = (float2 *)c->work[8].p;
  k_down<<<grid1(tot, 256), 256, 0, c->stream>>>(c->d_psi[set], y, tot);
  c->launches++;
  return rebuild_from<float>(c, set, y, norb);
}

static int dipole_dev(opaw_ctx *c, double gamma, double *out_dev) {
  double *part, *n0, *n1, *dipw;
  OPAW_CHECK(scratch_red(c, &part, &n0, &n1, &dipw, c->norb[0]));
  k_dipole_part<<<kDipBlocks, 256, 0, c->stream>>>(c->d_psi[0], c->d_psi[1], c->norb[0], c->nn, c->nx, c->ny, c->nz,
                                                   c->dx, c->dy, c->dz, c->dv, dipw);
  k_dipole_final<<<1, 256, 0, c->stream>>>(dipw, kDipBlocks, gamma, out_dev);
  c->launches += 2;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

static int need_psi(opaw_ctx *c, int set) {
  if (!c || c->norb[set] == 0) {
    set_error("no orbitals uploaded for this set");
    return OPAW_ERR_STATE;
  }
  return OPAW_OK;
}

// Points the set-1 pointers of the context at kicked set k (the FP64 path
// runs each kicked set through the set-1 routines); unbind restores them.
struct KickBind {
  double2 *psi;
  double *vks, *dij, *rhoij, *dens, *nhat, *vh, *vxc;
  float *vksf;
};
static KickBind bind_kick(opaw_ctx *c, int k) {
  KickBind b{c->d_psi[1], c->d_vks[1], c->d_dij[1], c->d_rhoij[1], c->d_dens[1], c->d_nhat[1], c->d_vh[1],
             c->d_vxc[1], c->d_vks_f[1]};
  const size_t nn = (size_t)c->nn, nd = (size_t)c->nd;
  c->d_psi[1] += (size_t)k * c->norb[1] * nn;
  c->d_vks[1] += k * nn;
  c->d_vks_f[1] += k * nn;
  c->d_dij[1] += k * nd;
  c->d_rhoij[1] += k * nd;
  c->d_dens[1] += k * nn;
  c->d_nhat[1] += k * nn;
  c->d_vh[1] += k * nn;
  c->d_vxc[1] += k * nn;
  return b;
}
static void unbind_kick(opaw_ctx *c, const KickBind &b) {
  c->d_psi[1] = b.psi;
  c->d_vks[1] = b.vks;
  c->d_vks_f[1] = b.vksf;
  c->d_dij[1] = b.dij;
  c->d_rhoij[1] = b.rhoij;
  c->d_dens[1] = b.dens;
  c->d_nhat[1] = b.nhat;
  c->d_vh[1] = b.vh;
  c->d_vxc[1] = b.vxc;
}

// nsteps steps of the unperturbed set and every kicked set; per step
// 3 + 6 nkick doubles into dd (device): dip, then dip'_k, d_dip_k per kick.
// tmp: 9 nkick device doubles of scratch (FP64 path).
// the fewest steps of a call that replay a captured graph (instantiating it
// costs about as much as a few steps of plain launches)
constexpr int kGraphMinSteps = 8;

// tmp: max(9 nkick, 2 (3 + 6 nkick)) device doubles of scratch
static int steps_dev(opaw_ctx *c, int nsteps, double dt, int prec, double *dd, double *tmp) {
  const size_t per = 3 + 6 * (size_t)c->nkick;
  if (prec == OPAW_PREC_MIXED) {
    // a block of steps replays a captured two-step graph (one context of the
    // ensemble path); with per-launch kernel timing on, or for a few steps,
    // the launches are issued one by one
    if (!c->ktime_on && nsteps >= kGraphMinSteps) {
      opaw_ctx *cs[1] = {c};
      double *ddv[1] = {dd}, *fx[1] = {tmp};
      return ensemble_steps(cs, 1, nsteps, dt, ddv, fx);
    }
    return mixed_steps(c, nsteps, dt, c->d_kgamma, dd);
  }
  for (int it = 0; it < nsteps; it++) {
    // ncpaw_make_hamiltonian_tddft (tddft.f90:75) and propdt (:80), one set
    // after the other: the sets never interact, so this equals the
    // reference's order (both rebuilds, then both propagations)
    OPAW_CHECK(rebuild_resident(c, 0, prec));
    OPAW_CHECK(rk4_set64(c, 0, dt));
    double *o = dd + per * (size_t)it;
    for (int k = 0; k < c->nkick; k++) {
      const KickBind b = bind_kick(c, k);
      int st = rebuild_resident(c, 1, prec);
      if (st == OPAW_OK) st = rk4_set64(c, 1, dt);
      // plot_dip (tddft.f90:84): [dip, dip'_k, d_dip_k] of this kick
      if (st == OPAW_OK) st = dipole_dev(c, c->h_kgamma[k], tmp + 9 * k);
      unbind_kick(c, b);
      OPAW_CHECK(st);
    }
    // dip (the same for every kick) once, then dip'_k, d_dip_k per kick
    OPAW_CUDA(cudaMemcpyAsync(o, tmp, sizeof(double) * 3, cudaMemcpyDeviceToDevice, c->stream));
    for (int k = 0; k < c->nkick; k++)
      OPAW_CUDA(cudaMemcpyAsync(o + 3 + 6 * k, tmp + 9 * k + 3, sizeof(double) * 6, cudaMemcpyDeviceToDevice,
                                c->stream));
  }
  return OPAW_OK;
}

int tddft_steps(opaw_ctx *c, int nsteps, double dt, double gamma, int prec, double *d_dip_out, double *dip_out,
                double *dip_pert_out) {
  OPAW_CHECK(need_psi(c, 0));
  OPAW_CHECK(need_psi(c, 1));
  OPAW_ARG(c->norb[0] == c->norb[1], "both sets must hold the same number of orbitals");
  OPAW_ARG(prec == OPAW_PREC_FP64 || prec == OPAW_PREC_MIXED, "precision must be OPAW_PREC_FP64 or OPAW_PREC_MIXED");
  OPAW_ARG(nsteps >= 0, "nsteps must be >= 0");
  if (c->nkick != 1) {
    set_error("the context holds several kicked sets: use opaw_tddft_steps_kicks");
    return OPAW_ERR_STATE;
  }
  c->h_kgamma.assign(1, gamma);
  OPAW_CHECK(upload_kgamma(c));
  const size_t nout = 9 * (size_t)(nsteps > 0 ? nsteps : 1);
  OPAW_CHECK(ensure(c->work[11], sizeof(double) * (nout + 18 + 16)));
  double *dd = (double *)c->work[11].p;  // 9 values per step: dip, dip_pert, d_dip
  OPAW_CHECK(steps_dev(c, nsteps, dt, prec, dd, dd + nout));
  if ((d_dip_out || dip_out || dip_pert_out) && nsteps > 0) {
    std::vector<double> h(9 * (size_t)nsteps);
    OPAW_CUDA(cudaMemcpyAsync(h.data(), dd, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    OPAW_CUDA(cudaStreamSynchronize(c->stream));
    for (int it = 0; it < nsteps; it++)
      for (int k = 0; k < 3; k++) {
        if (dip_out) dip_out[3 * it + k] = h[9 * (size_t)it + k];
        if (dip_pert_out) dip_pert_out[3 * it + k] = h[9 * (size_t)it + 3 + k];
        if (d_dip_out) d_dip_out[3 * it + k] = h[9 * (size_t)it + 6 + k];
      }
  }
  return OPAW_OK;
}

// the same for every kicked set of the context: dip [nsteps][3],
// dip_pert and d_dip [nsteps][nkick][3] (any may be NULL)
static int tddft_steps_kicks(opaw_ctx *c, int nsteps, double dt, int prec, double *dip_out, double *dip_pert_out,
                             double *d_dip_out) {
  OPAW_CHECK(need_psi(c, 0));
  OPAW_CHECK(need_psi(c, 1));
  OPAW_ARG(c->norb[0] == c->norb[1], "every set must hold the same number of orbitals");
  OPAW_ARG(prec == OPAW_PREC_FP64 || prec == OPAW_PREC_MIXED, "precision must be OPAW_PREC_FP64 or OPAW_PREC_MIXED");
  OPAW_ARG(nsteps >= 0, "nsteps must be >= 0");
  OPAW_ARG((int)c->h_kgamma.size() == c->nkick, "kick strengths missing: excite with opaw_excite_kicks");
  OPAW_CHECK(upload_kgamma(c));
  const size_t per = 3 + 6 * (size_t)c->nkick;
  const size_t nout = per * (size_t)(nsteps > 0 ? nsteps : 1);
  OPAW_CHECK(ensure(c->work[11], sizeof(double) * (nout + 12 * (size_t)c->nkick + 6 + 16)));
  double *dd = (double *)c->work[11].p;
  OPAW_CHECK(steps_dev(c, nsteps, dt, prec, dd, dd + nout));
  if ((d_dip_out || dip_out || dip_pert_out) && nsteps > 0) {
    std::vector<double> h(per * (size_t)nsteps);
    OPAW_CUDA(cudaMemcpyAsync(h.data(), dd, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    OPAW_CUDA(cudaStreamSynchronize(c->stream));
    const int K = c->nkick;
    for (int it = 0; it < nsteps; it++) {
      const double *q = h.data() + per * (size_t)it;
      for (int j = 0; j < 3; j++) {
        if (dip_out) dip_out[3 * it + j] = q[j];
        for (int k = 0; k < K; k++) {
          if (dip_pert_out) dip_pert_out[3 * ((size_t)it * K + k) + j] = q[3 + 6 * k + j];
          if (d_dip_out) d_dip_out[3 * ((size_t)it * K + k) + j] = q[6 + 6 * k + j];
        }
      }
    }
  }
  return OPAW_OK;
}

// excite_psi_bar_pert for nkick kicks at once (tddft_excite.f90:1-16):
// kicked set k = set 0 * exp(-i gamma_k r_{ipol_k})
static int excite_kicks(opaw_ctx *c, int nkick, const int *ipol, const double *gamma) {
  OPAW_CHECK(need_psi(c, 0));
  OPAW_ARG(nkick >= 1 && ipol && gamma, "nkick must be >= 1 with ipol and gamma arrays");
  for (int k = 0; k < nkick; k++) {
    OPAW_ARG(ipol[k] >= 1 && ipol[k] <= 3, "ipol must be 1, 2 or 3");
    OPAW_ARG(std::isfinite(gamma[k]), "gamma must be finite");
  }
  const int norb = c->norb[0];
  OPAW_CHECK(kick_capacity(c, nkick));
  if (c->norb[1] != norb || c->nkick != nkick) {
    OPAW_CUDA(cudaStreamSynchronize(c->stream));
    cudaFree(c->d_psi[1]);
    c->d_psi[1] = nullptr;
    OPAW_CUDA(cudaMalloc(&c->d_psi[1], sizeof(double2) * (size_t)c->nn * norb * nkick));
    c->norb[1] = norb;
  }
  c->nkick = nkick;
  c->h_kgamma.assign(gamma, gamma + nkick);
  for (int k = 0; k < nkick; k++) {
    k_excite<<<grid1(c->nn, 256), 256, 0, c->stream>>>(c->d_psi[0], c->d_psi[1] + (size_t)k * norb * c->nn, c->nn,
                                                      norb, c->nx, c->ny, c->nz, ipol[k], gamma[k], c->dx, c->dy,
                                                      c->dz);
    c->launches++;
  }
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

}  // namespace opaw

using namespace opaw;

extern "C" {

static int check_cs(opaw_ctx *c, int set) {
  if (!c) {
    set_error("null context");
    return OPAW_ERR_ARG;
  }
  if (set != 0 && set != 1) {
    set_error("set must be 0 or 1");
    return OPAW_ERR_ARG;
  }
  return OPAW_OK;
}

static int finish(opaw_ctx *c) {
  OPAW_CUDA(cudaGetLastError());
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return tma_status(c);
}

int opaw_rhoij(opaw_ctx *c, int set, int precision) {
  OPAW_CHECK(check_cs(c, set));
  OPAW_CHECK(need_psi(c, set));
  if (precision == OPAW_PREC_FP64) OPAW_CHECK(rhoij_density_from<double>(c, set, c->d_psi[set], c->norb[set], 0));
  else {
    const int64_t tot = c->nn * (int64_t)c->norb[set];
    OPAW_CHECK(ensure(c->work[8], sizeof(float2) * tot));
    k_down<<<grid1(tot, 256), 256, 0, c->stream>>>(c->d_psi[set], (float2 *)c->work[8].p, tot);
    c->launches++;
    OPAW_CHECK(rhoij_density_from<float>(c, set, (float2 *)c->work[8].p, c->norb[set], 0));
  }
  return finish(c);
}

int opaw_density(opaw_ctx *c, int set, int precision) {
  OPAW_CHECK(check_cs(c, set));
  OPAW_CHECK(need_psi(c, set));
  if (precision == OPAW_PREC_FP64) OPAW_CHECK(rhoij_density_from<double>(c, set, c->d_psi[set], c->norb[set], 1));
  else {
    const int64_t tot = c->nn * (int64_t)c->norb[set];
    OPAW_CHECK(ensure(c->work[8], sizeof(float2) * tot));
    k_down<<<grid1(tot, 256), 256, 0, c->stream>>>(c->d_psi[set], (float2 *)c->work[8].p, tot);
    c->launches++;
    OPAW_CHECK(rhoij_density_from<float>(c, set, (float2 *)c->work[8].p, c->norb[set], 1));
  }
  return finish(c);
}

int opaw_nhat(opaw_ctx *c, int set) {
  OPAW_CHECK(check_cs(c, set));
  OPAW_CHECK(nhat_step(c, set));
  return finish(c);
}

int opaw_vks(opaw_ctx *c, int set) {
  OPAW_CHECK(check_cs(c, set));
  OPAW_CHECK(vks_step(c, set, 0));
  return finish(c);
}

int opaw_dij(opaw_ctx *c, int set) {
  OPAW_CHECK(check_cs(c, set));
  OPAW_CHECK(dij_step(c, set));
  return finish(c);
}

int opaw_rebuild(opaw_ctx *c, int set, int precision) {
  OPAW_CHECK(check_cs(c, set));
  OPAW_CHECK(need_psi(c, set));
  OPAW_ARG(precision == OPAW_PREC_FP64 || precision == OPAW_PREC_MIXED, "bad precision");
  OPAW_CHECK(rebuild_resident(c, set, precision));
  return finish(c);
}

int opaw_vh(opaw_ctx *c, const double *dens, double *vh) {
  if (!c) {
    set_error("null context");
    return OPAW_ERR_ARG;
  }
  OPAW_ARG(dens && vh, "null buffers");
  OPAW_CHECK(ensure(c->work[2], sizeof(double) * c->nn * 2));
  double *a = (double *)c->work[2].p, *b = a + c->nn;
  OPAW_CUDA(cudaMemcpyAsync(a, dens, sizeof(double) * c->nn, cudaMemcpyHostToDevice, c->stream));
  OPAW_CHECK(hartree(c, a, nullptr, b, nullptr));
  OPAW_CUDA(cudaMemcpyAsync(vh, b, sizeof(double) * c->nn, cudaMemcpyDeviceToHost, c->stream));
  return finish(c);
}

int opaw_vxc_lda(opaw_ctx *c, const double *dens, double *vxc, int64_t n) {
  if (!c) {
    set_error("null context");
    return OPAW_ERR_ARG;
  }
  OPAW_ARG(dens && vxc && n >= 0, "null buffers");
  if (n == 0) return OPAW_OK;
  OPAW_CHECK(ensure(c->work[2], sizeof(double) * (size_t)n * 2));
  double *a = (double *)c->work[2].p, *b = a + n;
  OPAW_CUDA(cudaMemcpyAsync(a, dens, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  OPAW_CHECK(vxc_points(c, a, b, n));
  OPAW_CUDA(cudaMemcpyAsync(vxc, b, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  return finish(c);
}

int opaw_rconv(int n0, int n1, int n2, const double *gin, const double *bk, double *gout) {
  OPAW_ARG(n0 > 0 && n1 > 0 && n2 > 0 && gin && bk && gout, "bad arguments");
  opaw_ctx *c = new opaw_ctx();
  int st = OPAW_OK;
  const int64_t n = (int64_t)n0 * n1 * n2;
  double2 *a = nullptr;
  double *kb = nullptr, *o = nullptr;
  do {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { st = OPAW_ERR_CUDA; break; }
    if ((st = fft3_init(c->fft, n0, n1, n2)) != OPAW_OK) break;
    if (cudaMalloc(&a, sizeof(double2) * n) != cudaSuccess || cudaMalloc(&kb, sizeof(double) * n) != cudaSuccess ||
        cudaMalloc(&o, sizeof(double) * n) != cudaSuccess) {
      set_error("device allocation failed");
      st = OPAW_ERR_NOMEM;
      break;
    }
    std::vector<double2> h(n);
    for (int64_t i = 0; i < n; i++) h[i] = make_double2(gin[i], 0.0);
    cudaMemcpy(a, h.data(), sizeof(double2) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(kb, bk, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (cudaDeviceSynchronize() != cudaSuccess) {
      set_error("rconv upload failed");
      st = OPAW_ERR_CUDA;
      break;
    }
    if ((st = rconv_device(c, a, kb, o, n0, n1, n2)) != OPAW_OK) break;
    if (cudaMemcpyAsync(gout, o, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
      set_error("rconv copy-out failed");
      st = OPAW_ERR_CUDA;
    }
  } while (0);
  cudaFree(a);
  cudaFree(kb);
  cudaFree(o);
  fft3_free(c->fft);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return st;
}

int opaw_excite(opaw_ctx *c, int ipol, double gamma) {
  OPAW_CHECK(check_cs(c, 0));
  OPAW_CHECK(excite_kicks(c, 1, &ipol, &gamma));
  return finish(c);
}

int opaw_excite_kicks(opaw_ctx *c, int nkick, const int *ipol, const double *gamma) {
  OPAW_CHECK(check_cs(c, 0));
  OPAW_CHECK(excite_kicks(c, nkick, ipol, gamma));
  return finish(c);
}

int opaw_kick_download(opaw_ctx *c, int kick, double *psi, int norb) {
  OPAW_CHECK(check_cs(c, 0));
  OPAW_CHECK(need_psi(c, 1));
  OPAW_ARG(psi, "psi must be non-null");
  OPAW_ARG(kick >= 0 && kick < c->nkick, "kick index out of range");
  OPAW_ARG(norb == c->norb[1], "norb differs from the kicked sets' count");
  OPAW_CUDA(cudaMemcpyAsync(psi, c->d_psi[1] + (size_t)kick * norb * c->nn, sizeof(double2) * (size_t)c->nn * norb,
                            cudaMemcpyDeviceToHost, c->stream));
  return finish(c);
}

int opaw_tddft_steps_kicks(opaw_ctx *c, int nsteps, double dt, int precision, double *dip_out, double *dip_pert_out,
                           double *d_dip_out) {
  OPAW_CHECK(check_cs(c, 0));
  OPAW_CHECK(tddft_steps_kicks(c, nsteps, dt, precision, dip_out, dip_pert_out, d_dip_out));
  return finish(c);
}

int opaw_dipole(opaw_ctx *c, double gamma, double *dip, double *dip_pert, double *d_dip) {
  OPAW_CHECK(check_cs(c, 0));
  OPAW_CHECK(need_psi(c, 0));
  OPAW_CHECK(need_psi(c, 1));
  OPAW_ARG(c->norb[0] == c->norb[1], "both sets must hold the same number of orbitals");
  OPAW_CHECK(ensure(c->work[11], sizeof(double) * 16));
  double *out = (double *)c->work[11].p;
  OPAW_CHECK(dipole_dev(c, gamma, out));
  double h[9];
  OPAW_CUDA(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  OPAW_CHECK(finish(c));
  for (int k = 0; k < 3; k++) {
    if (dip) dip[k] = h[k];
    if (dip_pert) dip_pert[k] = h[3 + k];
    if (d_dip) d_dip[k] = h[6 + k];
  }
  return OPAW_OK;
}

int opaw_tddft_steps(opaw_ctx *c, int nsteps, double dt, double gamma, int precision, double *d_dip_out) {
  OPAW_CHECK(check_cs(c, 0));
  OPAW_CHECK(tddft_steps(c, nsteps, dt, gamma, precision, d_dip_out, nullptr, nullptr));
  return finish(c);
}

int opaw_tddft_steps_dip(opaw_ctx *c, int nsteps, double dt, double gamma, int precision, double *dip_out,
                         double *dip_pert_out, double *d_dip_out) {
  OPAW_CHECK(check_cs(c, 0));
  OPAW_CHECK(tddft_steps(c, nsteps, dt, gamma, precision, d_dip_out, dip_out, dip_pert_out));
  return finish(c);
}

int opaw_tddft_steps_host(opaw_ctx *c, double *psi, double *psi_pert, int norb, int nsteps, double dt, double gamma,
                          int precision, double *d_dip_out) {
  OPAW_CHECK(check_cs(c, 0));
  OPAW_ARG(psi && psi_pert && norb > 0, "bad buffers");
  OPAW_CHECK(opaw_psi_upload(c, 0, psi, norb));
  OPAW_CHECK(opaw_psi_upload(c, 1, psi_pert, norb));
  OPAW_CHECK(tddft_steps(c, nsteps, dt, gamma, precision, d_dip_out, nullptr, nullptr));
  OPAW_CHECK(opaw_psi_download(c, 0, psi, norb));
  OPAW_CHECK(opaw_psi_download(c, 1, psi_pert, norb));
  return OPAW_OK;
}

}  // extern "C"

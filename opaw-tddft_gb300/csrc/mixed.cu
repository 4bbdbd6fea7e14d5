// mixed.cu — the mixed-precision TDDFT step (OPAW_PREC_MIXED).
//
// The reference propagates the unperturbed orbitals psi (phi_bar) and the
// kicked ones psi' (phi_bar_pert) independently (rk4.f90:15-33) and reports
// d_dip = (dip' - dip)/gamma (tddft_plot.f90:57).  With gamma ~ 1e-3 the signal
// lives in psi' - psi, so single-precision rounding of psi' alone would swamp
// it.  This step therefore carries the kicked set as the difference
// delta = psi' - psi and uses the exact splitting
//
//   S^-1/2 H' S^-1/2 (psi + delta) - S^-1/2 H S^-1/2 psi
//       = S^-1/2 [ H' t_delta + (v' - v) t_0 + sum_a p~ (D' - D) <p~|t_0> ],
//   t_0 = S^-1/2 psi,  t_delta = S^-1/2 delta,
//
// so every complex64 quantity of the kicked set is a difference and keeps its
// relative precision.  The rebuild forms the density, rho_ij, compensation
// charge and potential differences directly: Hartree is linear (the
// difference density gets its own complex64 transform), the LDA difference
// and the charge-renormalisation factors are taken in FP64.  psi, delta, the
// final RK4 combination, the norms and the dipole are FP64.
//
// Per stage the orbitals are touched by the three FFT passes of H (the last
// one fused with v_ks), one two-table gather of H's grid part, and one fused
// pass (RK4 accumulation, S^-1/2 of the next stage vector, its density); the
// projector algebra in between (S^-1/2, D_ij, overlaps) runs on [orbital][slot]
// coefficient vectors in FP64.
//
// In exact arithmetic this is the reference algorithm; OPAW_PREC_FP64 runs
// the reference's own form for comparison.
#include <cmath>

#include <type_traits>

#include "fft.cuh"

namespace opaw {

static __device__ __forceinline__ double bsum(double v, double *sh) {
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

// ---------------------------------------------------------------- kernels --


// difference of rho_ij: 2 sum_occ Re(conj(c0_i) cd_j + conj(cd_i) c0_j + conj(cd_i) cd_j);
// kicked set k = blockIdx.y (cd, drho and rho1 advance by one set per kick)
__global__ void k_mix_drhoij(const double2 *__restrict__ c0, const double2 *__restrict__ cd, int norb, int ns, int nd,
                             const int *__restrict__ dslot, const int64_t *__restrict__ soff,
                             const int64_t *__restrict__ doff, const int *__restrict__ ms,
                             const double *__restrict__ rho0, double *__restrict__ drho, double *__restrict__ rho1) {
  const int t = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);  // warp per entry
  const int lane = threadIdx.x & 31;
  if (t >= nd) return;
  cd += (int64_t)blockIdx.y * norb * ns;
  drho += (int64_t)blockIdx.y * nd;
  rho1 += (int64_t)blockIdx.y * nd;
  const int a = dslot[t];
  const int m = ms[a];
  const int loc = t - (int)doff[a];
  const int i = loc % m, j = loc / m;
  double acc = 0;
  for (int o = lane; o < norb; o += 32) {
    const double2 ai = c0[(int64_t)o * ns + soff[a] + i], aj = c0[(int64_t)o * ns + soff[a] + j];
    const double2 bi = cd[(int64_t)o * ns + soff[a] + i], bj = cd[(int64_t)o * ns + soff[a] + j];
    acc += 2.0 * (ai.x * bj.x + ai.y * bj.y + bi.x * aj.x + bi.y * aj.y + bi.x * bj.x + bi.y * bj.y);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);  // fixed order
  if (lane != 0) return;
  drho[t] = acc;
  rho1[t] = rho0[t] + acc;
}

// density difference 2 sum_occ (2 Re(conj(t0) td) + |td|^2), complex64 inputs,
// 16-orbital partial sums in FP32 added in FP64
// renormalisation factors (nhat.f90:32-37) of both sets from the raw sums:
// f0 = rnel / S0, f1 = rnel / (S0 + dS), df = f1 - f0 = -rnel dS / (S0 (S0 + dS))
// (block k: kicked set k, its partial sums at pd + 2 k nb, its factors at fac + 4 k)
__global__ void k_mix_factors(const double *__restrict__ p0, const double *__restrict__ pd, int nb, double dv,
                              double rnel, double *__restrict__ fac) {
  __shared__ double sh[8];
  pd += (int64_t)blockIdx.x * 2 * nb;
  fac += 4 * blockIdx.x;
  const double a = block_sum_seq(p0, nb, 2, sh);
  const double b = block_sum_seq(p0 + 1, nb, 2, sh);
  const double c = block_sum_seq(pd, nb, 2, sh);
  const double d = block_sum_seq(pd + 1, nb, 2, sh);
  if (threadIdx.x != 0) return;
  const double S0 = a * dv + b * dv, dS = c * dv + d * dv;
  fac[0] = rnel / S0;
  fac[1] = rnel / (S0 + dS);
  fac[2] = -rnel * dS / (S0 * (S0 + dS));
}

// apply the factors: renormalised n0, n^0, the differences and the sources
// of the packed Hartree solve (n0 + n^0, dn + dn^)
// (kicked set k = blockIdx.y: its arrays advance by n per kick, its factors by 4;
// the unperturbed set's outputs are written by k = 0)
__global__ void k_mix_renorm(const double *__restrict__ r0raw, const double *__restrict__ h0raw,
                             const double *__restrict__ drraw, const double *__restrict__ dhraw,
                             const double *__restrict__ fac, double *__restrict__ dens0, double *__restrict__ nhat0,
                             double *__restrict__ dens1, double *__restrict__ nhat1, double *__restrict__ src0,
                             double *__restrict__ srcd, double *__restrict__ ddens, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = blockIdx.y;
  const int64_t ko = (int64_t)k * n;
  drraw += ko;
  dhraw += ko;
  dens1 += ko;
  nhat1 += ko;
  srcd += ko;
  ddens += ko;
  fac += 4 * k;
  const double f0 = fac[0], f1 = fac[1], df = fac[2];
  const double r0 = f0 * r0raw[i], h0 = f0 * h0raw[i];
  const double dr = df * r0raw[i] + f1 * drraw[i];
  const double dh = df * h0raw[i] + f1 * dhraw[i];
  if (k == 0) {
    dens0[i] = r0;
    nhat0[i] = h0;
    src0[i] = r0 + h0;
  }
  dens1[i] = r0 + dr;
  nhat1[i] = h0 + dh;
  srcd[i] = dr + dh;
  ddens[i] = dr;
}

// Slater + PW92 LDA (the formula of vxc_point in rebuild.cu) in FP32, and the difference
// vxc(n0 + dn) - vxc(n0) from divided differences of every factor, so it
// keeps the relative precision of dn instead of losing it to the cancellation
// of two nearly equal potentials:
//   u = n^1/3:  du = dn / (u1^2 + u1 u0 + u0^2),  d rs = -(3/4pi)^1/3 du / (u1 u0)
//   d sqrt(rs) = d rs / (s1 + s0),  d(rs s) = d rs s1 + rs0 ds,  d(rs^2) = d rs (rs1 + rs0)
//   d log(1 + 1/Q) = log1p(-dQ / (Q1 (Q0 + 1)))
//   d(dQ/(Q(Q+1))) = (d(dQ) G0 - dQ0 dQ (Q1 + Q0 + 1)) / (G1 G0),  G = Q (Q + 1)
// and products by d(ab) = da b1 + a0 db.
struct LdaF {
  float u, rs, s, Q, dQ, lg;
};
constexpr float kPwA = 0.031091f, kPwA1 = 0.21370f, kPwB1 = 7.5957f, kPwB2 = 3.5876f, kPwB3 = 1.6382f,
                kPwB4 = 0.49294f;
constexpr float kCx = 0.98474502184269641f;   // (3/pi)^(1/3)
constexpr float kCrs = 0.62035049089940001f;  // (3/(4 pi))^(1/3)

__device__ __forceinline__ LdaF lda_parts(float n) {
  LdaF p;
  p.u = cbrtf(n);
  p.rs = kCrs / p.u;
  p.s = sqrtf(p.rs);
  p.Q = 2.f * kPwA * (kPwB1 * p.s + kPwB2 * p.rs + kPwB3 * p.rs * p.s + kPwB4 * p.rs * p.rs);
  p.dQ = 2.f * kPwA * (0.5f * kPwB1 / p.s + kPwB2 + 1.5f * kPwB3 * p.s + 2.f * kPwB4 * p.rs);
  p.lg = log1pf(1.f / p.Q);
  return p;
}

__device__ __forceinline__ float lda_dec(const LdaF &p) {
  return -2.f * kPwA * kPwA1 * p.lg + 2.f * kPwA * (1.f + kPwA1 * p.rs) * p.dQ / (p.Q * (p.Q + 1.f));
}

__device__ __forceinline__ float vxc_of_parts(const LdaF &p) {
  const float ec = -2.f * kPwA * (1.f + kPwA1 * p.rs) * p.lg;
  return -kCx * p.u + (ec - p.rs / 3.f * lda_dec(p));
}

__device__ __forceinline__ void vxc_pair_f(float n0, float dn, float &x0, float &dx) {
  const float n1 = n0 + dn;
  const bool ok0 = n0 > 1e-15f, ok1 = n1 > 1e-15f;
  if (!ok0 || !ok1) {  // below the cut-off of vxc_point one of the two is zero
    x0 = ok0 ? vxc_of_parts(lda_parts(n0)) : 0.f;
    dx = (ok1 ? vxc_of_parts(lda_parts(n1)) : 0.f) - x0;
    return;
  }
  const LdaF p0 = lda_parts(n0), p1 = lda_parts(n1);
  x0 = vxc_of_parts(p0);
  const float du = dn / (p1.u * p1.u + p1.u * p0.u + p0.u * p0.u);
  const float dvx = -kCx * du;
  const float drs = -kCrs * du / (p1.u * p0.u);
  const float ds = drs / (p1.s + p0.s);
  const float drss = drs * p1.s + p0.rs * ds;
  const float drs2 = drs * (p1.rs + p0.rs);
  const float dQ = 2.f * kPwA * (kPwB1 * ds + kPwB2 * drs + kPwB3 * drss + kPwB4 * drs2);
  const float ddQ = 2.f * kPwA * (-0.5f * kPwB1 * ds / (p1.s * p0.s) + 1.5f * kPwB3 * ds + 2.f * kPwB4 * drs);
  const float dlg = log1pf(-dQ / (p1.Q * (p0.Q + 1.f)));
  const float dec_ = -2.f * kPwA * (kPwA1 * drs * p1.lg + (1.f + kPwA1 * p0.rs) * dlg);
  const float G0 = p0.Q * (p0.Q + 1.f), G1 = p1.Q * (p1.Q + 1.f);
  const float F1 = p1.dQ / G1;
  const float dF = (ddQ * G0 - p0.dQ * dQ * (p1.Q + p0.Q + 1.f)) / (G1 * G0);
  const float ddec = -2.f * kPwA * kPwA1 * dlg + 2.f * kPwA * (kPwA1 * drs * F1 + (1.f + kPwA1 * p0.rs) * dF);
  dx = dvx + dec_ - (drs * lda_dec(p1) + p0.rs * ddec) / 3.f;
}

// potentials of both sets: v0 = vH0 + vxc(n0 + nc) + vloc, dv = dvH + vxc(n1 + nc) - vxc(n0 + nc),
// the LDA terms in FP32 (vxc_pair_f), the sums in FP64
// (kicked set k = blockIdx.y: its arrays advance by n per kick, its Hartree
// difference is dvh + k n with mean[1 + k]; the unperturbed set's outputs
// are written by k = 0)
__global__ void k_mix_pot(const double *__restrict__ dens0, const double *__restrict__ ddens,
                          const double *__restrict__ core, const double *__restrict__ vloc,
                          const double *__restrict__ vh0, const double *__restrict__ dvh, const double *__restrict__ mean,
                          double *__restrict__ vks0, double *__restrict__ vks1, float *__restrict__ vks0f,
                          float *__restrict__ vks1f, float *__restrict__ dvf, double *__restrict__ vxc0o,
                          double *__restrict__ vxc1o, double *__restrict__ vh1o, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = blockIdx.y;
  const int64_t ko = (int64_t)k * n;
  float x0f, dxf;
  vxc_pair_f(d2f(dens0[i] + core[i]), d2f(ddens[ko + i]), x0f, dxf);
  const double x0 = f2d(x0f), dxc = f2d(dxf);
  double h0 = vh0[i], dh = dvh[ko + i];
  if (mean) {
    h0 -= mean[0];
    dh -= mean[1 + k];
  }
  const double v0 = h0 + x0 + vloc[i];
  const double dv = dh + dxc;
  const double v1 = v0 + dv;
  if (k == 0) {
    vks0[i] = v0;
    vks0f[i] = (float)v0;
    vxc0o[i] = x0;
  }
  vks1[ko + i] = v1;
  vks1f[ko + i] = (float)v1;
  dvf[ko + i] = (float)dv;
  vxc1o[ko + i] = x0 + dxc;
  vh1o[ko + i] = h0 + dh;
}

// mean of each Hartree potential of the batch (block b: partial sums at part + 2 b nb)
__global__ void k_mix_mean(const double *__restrict__ part, int nb, int64_t n, double *__restrict__ mean) {
  __shared__ double sh[8];
  const double a = block_sum_seq(part + (int64_t)blockIdx.x * 2 * nb, nb, 2, sh);
  if (threadIdx.x != 0) return;
  mean[blockIdx.x] = a / (double)n;
}

// D' - D of every kicked set (kick k = blockIdx.y)
__global__ void k_mix_ddij(const double *__restrict__ d0, const double *__restrict__ d1, double *__restrict__ dd,
                           int nd) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t ko = (int64_t)blockIdx.y * nd;
  if (t < nd) dd[ko + t] = d1[ko + t] - d0[t];
}

// ------------------------------------------------------------ stage algebra --
// Every projection a stage needs follows from two gathers per set: S^-1/2 is
// x + P1 diag(sigma) <p~1|x> (snphi.f90:23-46) and the nonlocal part of H is
// P D <p~|t> (hphi.f90:31-64), so with the overlap blocks O_xy = <p_x|p_y>
//   u  = H t = u' + P cD,            u' = F^-1 ek F t + v t (+ dv t0),  cD = D <p~|t>
//   k  = S^-1/2 u = u' + P cD + P1 c2,   c2 = sigma (<p~1|u'> + O10 cD)
//   <p~1|k> = q1 + O11 c2,  <p~|k> = <p~|u'> + O00 cD + O01 c2,  q1 = <p~1|u'> + O10 cD
// and the next stage vector y = pf + dts (-i k) (rk4.f90:44-48) has
//   t' = S^-1/2 y = pf + dts (-i k) + P1 c3,   c3 = sigma (<p~1|pf> + dts (-i <p~1|k>))
//   <p~|t'> = <p~|pf> + dts (-i <p~|k>) + O01 c3.
// The coefficient algebra is FP64; arrays are [set][orbital][slot].
struct Ovl {
  const int *start, *atom;
  const int64_t *off;
  const double *O[4];  // <p~|p~>, <p~|p~1>, <p~1|p~>, <p~1|p~1>
  const int *ms, *slot_atom;
  const int64_t *soff;
};

static Ovl ovl_of(const opaw_ctx *c) {
  Ovl v;
  v.start = c->d_ovl_start;
  v.atom = c->d_ovl_atom;
  v.off = c->d_ovl_off;
  for (int k = 0; k < 4; k++) v.O[k] = c->d_ovl[k];
  v.ms = c->d_ms;
  v.slot_atom = c->d_slot_atom;
  v.soff = c->d_soff;
  return v;
}

// (O_k x)[a, i] for one orbital's slot vector x
__device__ __forceinline__ double2 ovl_mv(const Ovl &v, int k, int a, int i, const double2 *__restrict__ x) {
  double sx = 0, sy = 0;
  for (int q = v.start[a]; q < v.start[a + 1]; q++) {
    const int b = v.atom[q], mb = v.ms[b];
    const double *Ob = v.O[k] + v.off[q] + (int64_t)i * mb;
    const double2 *xb = x + v.soff[b];
    for (int j = 0; j < mb; j++) {
      sx += Ob[j] * xb[j].x;
      sy += Ob[j] * xb[j].y;
    }
  }
  return make_double2(sx, sy);
}

__device__ __forceinline__ double2 mi(double2 z) { return make_double2(z.y, -z.x); }  // -i z

// thread (slot t, orbital o, set X); grid (ceil(ns/128), norb, 1 + kicks):
// set 0 is the unperturbed set, set 1 + k the difference of kick k
#define MC_SLOT()                                                  \
  const int t = blockIdx.x * blockDim.x + threadIdx.x;             \
  if (t >= ns) return;                                             \
  const int o = blockIdx.y, X = blockIdx.z;                        \
  const int a = v.slot_atom[t];                                    \
  const int i = t - (int)v.soff[a];                                \
  const int64_t base = ((int64_t)X * norb + o) * ns;               \
  const int64_t g0 = ((int64_t)(2 * X) * norb + o) * ns;           \
  const int64_t g1 = ((int64_t)(2 * X + 1) * norb + o) * ns;       \
  (void)i; (void)g0; (void)g1

// q1 = <p~1|u'> + O10 cD, c2 = sigma q1
__global__ void k_mc_c2(Ovl v, const double2 *__restrict__ G, const double2 *__restrict__ cD,
                        const double *__restrict__ sigma, double2 *__restrict__ q1, double2 *__restrict__ c2, int norb,
                        int ns) {
  MC_SLOT();
  const double2 m = ovl_mv(v, 2, a, i, cD + base);
  const double2 q = make_double2(G[g1 + t].x + m.x, G[g1 + t].y + m.y);
  q1[base + t] = q;
  c2[base + t] = make_double2(sigma[t] * q.x, sigma[t] * q.y);
}

// <p~1|k>, <p~|k>; the packed box coefficients (-i cD, -i c2) of the fused
// pass; with write_t also c3 and <p~|pf> + dts (-i <p~|k>)
__global__ void k_mc_k(Ovl v, const double2 *__restrict__ G, const double2 *__restrict__ A,
                       const double2 *__restrict__ cD, const double2 *__restrict__ q1, const double2 *__restrict__ c2,
                       const double *__restrict__ sigma, double dts, int write_t, double2 *__restrict__ c3,
                       double2 *__restrict__ pre, float4 *__restrict__ cab, int norb, int ns) {
  MC_SLOT();
  const double2 d = cD[base + t], e = c2[base + t];
  const double2 al = mi(d), be = mi(e);
  cab[base + t] = make_float4(d2f(al.x), d2f(al.y), d2f(be.x), d2f(be.y));
  if (!write_t) return;
  const double2 m11 = ovl_mv(v, 3, a, i, c2 + base);
  const double2 m00 = ovl_mv(v, 0, a, i, cD + base);
  const double2 m01 = ovl_mv(v, 1, a, i, c2 + base);
  const double2 k1 = mi(make_double2(q1[base + t].x + m11.x, q1[base + t].y + m11.y));
  const double2 k0 = mi(make_double2(G[g0 + t].x + m00.x + m01.x, G[g0 + t].y + m00.y + m01.y));
  const double2 y1 = make_double2(A[g1 + t].x + dts * k1.x, A[g1 + t].y + dts * k1.y);
  c3[base + t] = make_double2(sigma[t] * y1.x, sigma[t] * y1.y);
  pre[base + t] = make_double2(A[g0 + t].x + dts * k0.x, A[g0 + t].y + dts * k0.y);
}

// start of a step: c3 = sigma <p~1|pf>, pre = <p~|pf>
__global__ void k_mc_start(Ovl v, const double2 *__restrict__ A, const double *__restrict__ sigma,
                           double2 *__restrict__ c3, double2 *__restrict__ pre, int norb, int ns) {
  MC_SLOT();
  const double2 p1 = A[g1 + t];
  c3[base + t] = make_double2(sigma[t] * p1.x, sigma[t] * p1.y);
  pre[base + t] = A[g0 + t];
}

// the gathers of the hi arrays restored like the arrays themselves:
// <p|psi> = f0 <p|x>, <p|delta_k> = df_k <p|x> + f1_k <p|y_k> (both tables,
// every kicked set k; factors [kick][orbital][3], f0 shared by the kicks)
__global__ void k_mc_scale_a(double2 *__restrict__ A, const double *__restrict__ fac, int norb, int ns, int nkick) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ns) return;
  const int o = blockIdx.y, tab = blockIdx.z;
  const int64_t sv = (int64_t)norb * ns;
  double2 *a0 = A + (int64_t)tab * sv + (int64_t)o * ns + t;  // set 0, table tab
  const double2 x = *a0;
  for (int k = 0; k < nkick; k++) {
    const double *f = fac + 3 * ((int64_t)k * norb + o);
    double2 *ad = A + (int64_t)(2 * (1 + k) + tab) * sv + (int64_t)o * ns + t;
    const double2 y = *ad;
    *ad = make_double2(f[2] * x.x + f[1] * y.x, f[2] * x.y + f[1] * y.y);
  }
  const double f0 = fac[3 * o];
  *a0 = make_double2(f0 * x.x, f0 * x.y);
}

// <p~|t'> = pre + O01 c3, and the box coefficient c3 of t'
__global__ void k_mc_t(Ovl v, const double2 *__restrict__ pre, const double2 *__restrict__ c3,
                       double2 *__restrict__ c0n, float2 *__restrict__ cg, int norb, int ns) {
  MC_SLOT();
  const double2 m = ovl_mv(v, 1, a, i, c3 + base);
  c0n[base + t] = make_double2(pre[base + t].x + m.x, pre[base + t].y + m.y);
  cg[base + t] = make_float2(d2f(c3[base + t].x), d2f(c3[base + t].y));
}
#undef MC_SLOT

// The fused grid pass of a stage, one thread per grid point over every
// orbital of both sets:
//   kf  = -i u' + P (-i cD) + P1 (-i c2)          (= -i S^-1/2 H t)
//   ks  = w kf  (first stage)  or  ks + w kf      (rk4.f90:44-48)
//   t'  = pf + dts kf + P1 c3                      (S^-1/2 of the next y)
// and the raw densities of t' (tddft_dens.f90:56-77): 2 sum |t0|^2 and the
// difference 2 sum (2 Re conj(t0) td + |td|^2), orbital partial sums of 16 in
// FP32 added with a compensated FP32 sum (DensAcc).  At the start of a step
// (stage = 0) it only forms t = pf + P1 c3 and the densities.  The box
// terms at the union points come precomputed from k_mix_boxcoef_t through
// the union index; two orbitals' loads are in flight per thread.  The last
// stage (no t', no densities) runs inside k_mix_final instead.
// Several kicks share the unperturbed set: the difference arrays (ud, pfd,
// ksd, td) hold [kick][orbital][point] and drraw [kick][point]; the thread of
// (point, kick k) forms the unperturbed values it needs itself and only k = 0
// stores them.
struct FusedArgs {
  const float2 *u0, *ud, *pf0, *pfd;  // pf: the hi arrays x, y of the state, restored on read
  const float *facf;                  // per kick and orbital f0, f1, df: psi = f0 x, delta = df x + f1 y
  float2 *ks0, *ksd, *t0, *td;
  double *r0raw, *drraw;
  int norb;
  int nkick;
  int64_t nn;
  float w, dts;
  int stage, first, write_t;
};

// Density accumulation without the FP64 pipe (1/64 of the FP32 rate here):
// FP32 sums of 16 orbitals, the group sums added with a compensated FP32
// two-sum (about 48 significant bits), converted to FP64 once per point.
__device__ __forceinline__ void two_sum_acc(float &s, float &c, float x) {
  const float t = s + x;
  const float bp = t - s;
  c += (s - (t - bp)) + (x - bp);
  s = t;
}

struct DensAcc {
  float h0 = 0.f, l0 = 0.f, hd = 0.f, ld = 0.f;  // compensated sums of the group sums
  float p0 = 0.f, pd = 0.f;                       // the current group of 16 orbitals
  int cnt = 0;
  __device__ __forceinline__ void add(float2 x, float2 y) {
    p0 += x.x * x.x + x.y * x.y;
    pd += 2.f * (x.x * y.x + x.y * y.y) + y.x * y.x + y.y * y.y;
    if (++cnt == 16) flush();
  }
  __device__ __forceinline__ void flush() {
    two_sum_acc(h0, l0, p0);
    two_sum_acc(hd, ld, pd);
    p0 = pd = 0.f;
    cnt = 0;
  }
  // 2 sum (occupation 2, tddft_dens.f90:73); scaling by 2 is exact in FP32
  __device__ __forceinline__ double total0() { return f2d(2.f * h0) + f2d(2.f * l0); }
  __device__ __forceinline__ double totald() { return f2d(2.f * hd) + f2d(2.f * ld); }
  __device__ __forceinline__ void store(const FusedArgs &f, int64_t g, int k) {
    flush();
    if (k == 0) f.r0raw[g] = total0();
    f.drraw[(int64_t)k * f.nn + g] = totald();
  }
};

// the restored complex64 psi and delta of orbital o (kick k) from the hi arrays
__device__ __forceinline__ void restore_pf(const FusedArgs &f, int k, int o, float2 x, float2 y, float2 &q0,
                                           float2 &qd) {
  const float *fk = f.facf + 3 * ((int64_t)k * f.norb + o);
  const float f0 = fk[0], f1 = fk[1], df = fk[2];
  q0 = make_float2(f0 * x.x, f0 * x.y);
  qd = make_float2(df * x.x + f1 * y.x, df * x.y + f1 * y.y);
}

// one orbital of both sets at one point, given the loaded values and the box
// terms; idx indexes the unperturbed arrays, idd the kick's difference arrays
__device__ __forceinline__ void fused_one(const FusedArgs &f, int k, int64_t idx, int64_t idd, float2 a0, float2 ad,
                                          float2 q0, float2 qd, float2 s0, float2 sd, const float2 *B,
                                          const float2 *Gt, DensAcc &acc) {
  float2 tv0, tvd;
  if (f.stage) {
    const float2 k0 = make_float2(a0.y + B[0].x, -a0.x + B[0].y);
    const float2 kd = make_float2(ad.y + B[1].x, -ad.x + B[1].y);
    float2 n0 = make_float2(f.w * k0.x, f.w * k0.y), nd = make_float2(f.w * kd.x, f.w * kd.y);
    if (!f.first) {
      n0.x += s0.x;
      n0.y += s0.y;
      nd.x += sd.x;
      nd.y += sd.y;
    }
    if (k == 0) f.ks0[idx] = n0;
    f.ksd[idd] = nd;
    if (!f.write_t) return;
    tv0 = make_float2(q0.x + f.dts * k0.x + Gt[0].x, q0.y + f.dts * k0.y + Gt[0].y);
    tvd = make_float2(qd.x + f.dts * kd.x + Gt[1].x, qd.y + f.dts * kd.y + Gt[1].y);
  } else {
    tv0 = make_float2(q0.x + Gt[0].x, q0.y + Gt[0].y);
    tvd = make_float2(qd.x + Gt[1].x, qd.y + Gt[1].y);
  }
  if (k == 0) f.t0[idx] = tv0;
  f.td[idd] = tvd;
  acc.add(tv0, tvd);
}

// every grid point; at the union points the box terms come from BG
// ([kind B, G][set][orbital][union point], sets 0 .. nkick, k_mix_boxcoef).
// Block b covers points (b / nkick) * 256 ... for kick b % nkick, so the
// blocks of all kicks of the same points run side by side and their reads of
// the unperturbed arrays are served by L2.
__global__ void __launch_bounds__(256)
    k_mix_dense(FusedArgs f, const int *__restrict__ uidx, const float2 *__restrict__ BG, int nunion) {
  const int k = blockIdx.x % f.nkick;
  const int64_t g = (blockIdx.x / f.nkick) * (int64_t)blockDim.x + threadIdx.x;
  if (g >= f.nn) return;
  const int u = uidx[g];
  const int64_t su = (int64_t)f.norb * nunion;  // between the (kind, set) blocks of BG
  const int64_t nset = 1 + f.nkick;
  const int64_t kd = (int64_t)k * f.norb * f.nn;  // this kick's difference arrays
  const float2 zero = make_float2(0.f, 0.f);
  DensAcc acc;
  for (int o = 0; o < f.norb; o += 2) {
    const int nj = (o + 1 < f.norb) ? 2 : 1;
    float2 a0[2], ad[2], q0[2], qd[2], s0[2], sd[2], B[2][2], G[2][2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
      a0[j] = ad[j] = q0[j] = qd[j] = s0[j] = sd[j] = zero;
      B[j][0] = B[j][1] = G[j][0] = G[j][1] = zero;
      if (j < nj) {
        const int64_t idx = (int64_t)(o + j) * f.nn + g;
        const int64_t bi = (int64_t)(o + j) * nunion + u;
        if (f.stage) {
          a0[j] = f.u0[idx];
          ad[j] = f.ud[kd + idx];
          if (!f.first) {
            if (k == 0) s0[j] = f.ks0[idx];
            sd[j] = f.ksd[kd + idx];
          }
          if (u >= 0) {
            B[j][0] = BG[bi];
            B[j][1] = BG[(1 + k) * su + bi];
          }
        }
        if (f.write_t) {
          q0[j] = f.pf0[idx];
          qd[j] = f.pfd[kd + idx];
          if (u >= 0) {
            G[j][0] = BG[nset * su + bi];
            G[j][1] = BG[(nset + 1 + k) * su + bi];
          }
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 2; j++)
      if (j < nj && f.write_t) restore_pf(f, k, o + j, q0[j], qd[j], q0[j], qd[j]);
#pragma unroll
    for (int j = 0; j < 2; j++)
      if (j < nj) {
        const int64_t idx = (int64_t)(o + j) * f.nn + g;
        fused_one(f, k, idx, kd + idx, a0[j], ad[j], q0[j], qd[j], s0[j], sd[j], B[j], G[j], acc);
      }
  }
  if (f.write_t) acc.store(f, g, k);
}

// The box terms of the fused pass at every union point u, orbital o and
// set X (thread per (u, o), set X = blockIdx.z of nset):
//   B = sum_entries sum_i  P~_i (-i cD_i) + P~1_i (-i c2_i)      (of -i S^-1/2 H t)
//   G = sum_entries sum_i  P~1_i c3_i                           (of S^-1/2 y)
// entries in atom order; projector values from the FP32 tables,
// coefficients packed by k_mc_k / k_mc_t.
__global__ void __launch_bounds__(128)
    k_mix_boxcoef(int nunion, int norb, int ns, const int *__restrict__ ustart, const int *__restrict__ uatom,
                  const int *__restrict__ ubox, const float *__restrict__ P0, const float *__restrict__ P1,
                  const int64_t *__restrict__ poff, const int *__restrict__ nrough, const int *__restrict__ ms,
                  const int64_t *__restrict__ soff, const float4 *__restrict__ cab, const float2 *__restrict__ cg,
                  int stage, int write_t, float2 *__restrict__ BG) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nunion) return;
  const int o = blockIdx.y, X = blockIdx.z, nset = gridDim.z;
  const int64_t kstride = (int64_t)norb * ns;
  float2 B = make_float2(0.f, 0.f), G = make_float2(0.f, 0.f);
  for (int e = ustart[u]; e < ustart[u + 1]; e++) {
    const int a = uatom[e], b = ubox[e];
    const int nbox = nrough[3 * a] * nrough[3 * a + 1] * nrough[3 * a + 2];
    const int m = ms[a];
    const int64_t s0 = X * kstride + (int64_t)o * ns + soff[a];
    for (int i = 0; i < m; i++) {
      const float p = P0[poff[a] + (int64_t)i * nbox + b], q = P1[poff[a] + (int64_t)i * nbox + b];
      if (stage) {
        const float4 c = cab[s0 + i];
        B.x += p * c.x + q * c.z;
        B.y += p * c.y + q * c.w;
      }
      if (write_t) {
        const float2 c = cg[s0 + i];
        G.x += q * c.x;
        G.y += q * c.y;
      }
    }
  }
  const int64_t su = (int64_t)norb * nunion, bi = (int64_t)o * nunion + u;
  if (stage) BG[X * su + bi] = B;
  if (write_t) BG[(nset + X) * su + bi] = G;
}

// The same terms by tiles of kUTile union points and OG orbitals, for the
// pair of sets X0 = 2 blockIdx.z and X1 = X0 + 1 (X1 absent when it reaches
// nset).  The CTA first copies the coefficients of its tile's atoms (utile)
// for its orbitals into shared memory, three float4 per (atom, orbital,
// projector): -i cD and -i c2 of set X0, of set X1, then c3 of both sets.  A
// thread then takes one union point: per entry (uent: table offset,
// tile-local atom, projector count, box size) it loads the projector values
// once and reads the coefficients as shared-memory broadcasts.  The sums of
// each set run in the order of the generic kernel above.  MODE bit 0: the B
// terms (stage), bit 1: the G terms (write_t).
template <int MODE, int MS, int OG>
__global__ void __launch_bounds__(kUTile, OG >= 8 ? 4 : 6)
    k_mix_boxcoef_t(int nunion, int norb, int ns, int amax, int nset, const int *__restrict__ ustart,
                    const int4 *__restrict__ uent, const int2 *__restrict__ utile, const int *__restrict__ utile_na,
                    const float *__restrict__ P0, const float *__restrict__ P1, const float4 *__restrict__ cab,
                    const float2 *__restrict__ cg, float2 *__restrict__ BG) {
  constexpr bool kB = (MODE & 1) != 0, kG = (MODE & 2) != 0;
  extern __shared__ float4 cs[];  // [tile atom][OG][MS][3]
  const int tile = blockIdx.x;
  const int o0 = blockIdx.y * OG;
  const int X0 = 2 * blockIdx.z, X1 = X0 + 1;
  const bool has1 = X1 < nset;
  const int64_t kstride = (int64_t)norb * ns;
  const int na = utile_na[tile];
  for (int t = threadIdx.x; t < na * OG * MS; t += kUTile) {
    const int la = t / (OG * MS), r = t - la * (OG * MS), j = r / MS, i = r - j * MS;
    const int2 at = utile[(int64_t)tile * amax + la];
    float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0, g = a0;
    if (i < at.y) {
      const int64_t k = (int64_t)min(o0 + j, norb - 1) * ns + at.x + i;
      if (kB) {
        a0 = cab[X0 * kstride + k];
        if (has1) a1 = cab[X1 * kstride + k];
      }
      if (kG) {
        const float2 g0 = cg[X0 * kstride + k];
        const float2 g1 = has1 ? cg[X1 * kstride + k] : make_float2(0.f, 0.f);
        g = make_float4(g0.x, g0.y, g1.x, g1.y);
      }
    }
    cs[3 * t] = a0;
    cs[3 * t + 1] = a1;
    cs[3 * t + 2] = g;
  }
  __syncthreads();
  const int u = tile * kUTile + threadIdx.x;
  if (u >= nunion) return;
  float2 B[OG][2], G[OG][2];
#pragma unroll
  for (int j = 0; j < OG; j++)
#pragma unroll
    for (int X = 0; X < 2; X++) B[j][X] = G[j][X] = make_float2(0.f, 0.f);
  const int e1 = ustart[u + 1];
  for (int e = ustart[u]; e < e1; e++) {
    const int4 E = uent[e];
    float p[MS], q[MS];
#pragma unroll
    for (int i = 0; i < MS; i++) {
      p[i] = q[i] = 0.f;
      if (i < E.z) {
        if (kB) p[i] = P0[E.x + i * E.w];
        q[i] = P1[E.x + i * E.w];
      }
    }
    const float4 *cb = cs + (int64_t)E.y * (OG * MS * 3);
#pragma unroll
    for (int j = 0; j < OG; j++) {
#pragma unroll
      for (int i = 0; i < MS; i++) {
        if (i < E.z) {
          const float4 *cc = cb + (j * MS + i) * 3;
          if (kB) {
            const float4 c0 = cc[0], c1 = cc[1];
            B[j][0].x += p[i] * c0.x + q[i] * c0.z;
            B[j][0].y += p[i] * c0.y + q[i] * c0.w;
            B[j][1].x += p[i] * c1.x + q[i] * c1.z;
            B[j][1].y += p[i] * c1.y + q[i] * c1.w;
          }
          if (kG) {
            const float4 c2 = cc[2];
            G[j][0].x += q[i] * c2.x;
            G[j][0].y += q[i] * c2.y;
            G[j][1].x += q[i] * c2.z;
            G[j][1].y += q[i] * c2.w;
          }
        }
      }
    }
  }
  const int64_t su = (int64_t)norb * nunion;
#pragma unroll
  for (int j = 0; j < OG; j++) {
    if (o0 + j < norb) {
      const int64_t bi = (int64_t)(o0 + j) * nunion + u;
      if (kB) {
        BG[X0 * su + bi] = B[j][0];
        if (has1) BG[X1 * su + bi] = B[j][1];
      }
      if (kG) {
        BG[(nset + X0) * su + bi] = G[j][0];
        if (has1) BG[(nset + X1) * su + bi] = G[j][1];
      }
    }
  }
}

// Tail of the step.  FP64 arithmetic only where psi and delta are updated;
// the norms and the dipole take FP32 products of the rounded values, summed
// in FP32 over chunks of 32 points and in FP64 across chunks (their relative
// rounding is ~1e-9, far below the FP32 work of the step).
constexpr int kMixNormBlocks = 64;
constexpr int kChunk = 32;

struct NormAcc {
  double A = 0, B = 0;
  float a = 0.f, b = 0.f;
  int n = 0;
  __device__ __forceinline__ void add(float2 x, float2 y) {
    a += x.x * x.x + x.y * x.y;
    b += 2.f * (x.x * y.x + x.y * y.y) + y.x * y.x + y.y * y.y;
    if (++n == kChunk) flush();
  }
  __device__ __forceinline__ void flush() {
    A += f2d(a);
    B += f2d(b);
    a = b = 0.f;
    n = 0;
  }
};

// ---- the state of a call in float-float ------------------------------------
// psi and delta live as unevaluated sums hi + lo of two FP32 arrays (about 48
// significant bits) while a call runs: FP64 arithmetic runs at 1/64 of the
// FP32 rate on this part, and the hi arrays are the complex64 copies every
// stage reads.  The error-free products and sums use rounding intrinsics so
// that no multiply-add contraction changes them.  The norm restore of
// rk4.f90:92-102 is kept as per-orbital factors (f0, f1, df) that the next
// update and every reader of the hi arrays apply: psi = f0 x,
// psi' - psi = df x + f1 y.
struct FF {
  float h, l;
};
__device__ __forceinline__ FF ff_of(double v) {
  const float h = d2f(v);
  return {h, d2f(v - f2d(h))};
}
__device__ __forceinline__ double ff_val(FF a) { return f2d(a.h) + f2d(a.l); }
__device__ __forceinline__ FF ff_norm(float p, float e) {
  const float h = __fadd_rn(p, e);
  return {h, __fsub_rn(e, __fsub_rn(h, p))};
}
// a x (the a.l x.l term, below 2^-46 relative, dropped)
__device__ __forceinline__ FF ff_mul(FF a, FF x) {
  const float p = __fmul_rn(a.h, x.h);
  float e = __fmaf_rn(a.h, x.h, -p);
  e = __fmaf_rn(a.h, x.l, e);
  e = __fmaf_rn(a.l, x.h, e);
  return ff_norm(p, e);
}
// a s for an FP32 s
__device__ __forceinline__ FF ff_mulf(FF a, float s) {
  const float p = __fmul_rn(a.h, s);
  float e = __fmaf_rn(a.h, s, -p);
  e = __fmaf_rn(a.l, s, e);
  return ff_norm(p, e);
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float t = __fadd_rn(a.h, b.h);
  const float bp = __fsub_rn(t, a.h);
  const float e = __fadd_rn(__fadd_rn(__fsub_rn(a.h, __fsub_rn(t, bp)), __fsub_rn(b.h, bp)), __fadd_rn(a.l, b.l));
  return ff_norm(t, e);
}

// start of a call: x = psi, y_k = psi'_k - psi in float-float, norm partials
// (the targets of every norm restore of the call, rk4.f90:16); kick k =
// blockIdx.z, its arrays (p1, yh, yl) advance by norb nn per kick, its
// partials are [kick][orbital][block][2]; x is written by k = 0
__global__ void k_mix_start(const double2 *__restrict__ p0, const double2 *__restrict__ p1,
                            float2 *__restrict__ xh, float2 *__restrict__ xl, float2 *__restrict__ yh,
                            float2 *__restrict__ yl, int64_t nn, double *__restrict__ part) {
  __shared__ double sh[8];
  const int o = blockIdx.y, k = blockIdx.z, norb = gridDim.y;
  const int64_t kd = (int64_t)k * norb * nn;
  NormAcc acc;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nn; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)o * nn + g;
    const double2 x = p0[i], y1 = p1[kd + i];
    const FF ax = ff_of(x.x), ay = ff_of(x.y), bx = ff_of(y1.x - x.x), by = ff_of(y1.y - x.y);
    if (k == 0) {
      xh[i] = make_float2(ax.h, ay.h);
      xl[i] = make_float2(ax.l, ay.l);
    }
    yh[kd + i] = make_float2(bx.h, by.h);
    yl[kd + i] = make_float2(bx.l, by.l);
    acc.add(make_float2(ax.h, ay.h), make_float2(bx.h, by.h));
  }
  acc.flush();
  const double A = bsum(acc.A, sh), B = bsum(acc.B, sh);
  if (threadIdx.x == 0) {
    const int64_t q = ((int64_t)(k * norb + o) * gridDim.x + blockIdx.x) * 2;
    part[q] = A;
    part[q + 1] = B;
  }
}

// pending factors of a fresh call: no restore yet (n = kicks x orbitals)
__global__ void k_mix_fac_init(double *__restrict__ fac, float *__restrict__ facf, int norb) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= norb) return;
  fac[3 * o] = facf[3 * o] = 1.f;
  fac[3 * o + 1] = facf[3 * o + 1] = 1.f;
  fac[3 * o + 2] = facf[3 * o + 2] = 0.f;
}

// final RK4 combination (rk4.f90:22) of both sets from the restored start
// values: x' = f0 x + h6 ks0, y' = df x + f1 y + h6 ksd (float-float), with
// the norm partials and the dipole partials (tddft_plot.f90:40-57) of x', y':
// per orbital sum r |x'|^2 and sum r (2 Re conj(x') y' + |y'|^2)
// With u0 non-null it also finishes the last RK4 stage first (the fused pass
// of that stage has no sum over orbitals): sum k = ks + k4, k4 = -i u' + B
// with the box terms B of both sets at the union points.
// Kicks: block x = chunk * nkick + k; the thread of kick k updates y_k in place
// and forms x' itself; x' goes to the other buffer (xh2, xl2), written by
// k = 0, so that every kick still reads the old x.  Partials are
// [kick][orbital][chunk][2 or 6] (the set-0 parts are the same in every kick).
__global__ void __launch_bounds__(256, 3) k_mix_final(const float2 *__restrict__ xh, const float2 *__restrict__ xl,
                            float2 *__restrict__ xh2, float2 *__restrict__ xl2, float2 *__restrict__ yh,
                            float2 *__restrict__ yl, const float2 *__restrict__ ks0, const float2 *__restrict__ ksd,
                            const double *__restrict__ fac, double h6, int64_t nn, int nx, int ny, int nz, float dx,
                            float dy, float dz, double *__restrict__ npart, double *__restrict__ dpart,
                            const float2 *__restrict__ u0, const float2 *__restrict__ ud, const int *__restrict__ uidx,
                            const float2 *__restrict__ BG, int nunion, int nkick) {
  __shared__ double sh[8];
  const int o = blockIdx.y, norb = gridDim.y;
  const int k = blockIdx.x % nkick, chunk = blockIdx.x / nkick, nchunk = gridDim.x / nkick;
  const int64_t kd = (int64_t)k * norb * nn;
  const double *fk = fac + 3 * ((int64_t)k * norb + o);
  const FF f0 = ff_of(fk[0]), f1 = ff_of(fk[1]), df = ff_of(fk[2]), hh = ff_of(h6);
  NormAcc acc;
  double D[6] = {0, 0, 0, 0, 0, 0};
  float Df[6] = {0, 0, 0, 0, 0, 0};
  int nd = 0;
  // grid coordinates carried along the grid-stride loop (no divisions per point)
  const int64_t g0 = chunk * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)nchunk * blockDim.x;
  int gx = (int)(g0 % nx), gy = (int)((g0 / nx) % ny), gz = (int)(g0 / ((int64_t)nx * ny));
  const int sx = (int)(stride % nx), sy = (int)((stride / nx) % ny), sz = (int)(stride / ((int64_t)nx * ny));
  // the six operands of the next point are loaded while this one is combined
  const int64_t ob = (int64_t)o * nn;
  float2 na = make_float2(0.f, 0.f), nal = na, nb = na, nbl = na, ns0 = na, nsd = na, np0 = na, npd = na;
  int nu = -1;
  if (g0 < nn) {
    na = xh[ob + g0], nal = xl[ob + g0], nb = yh[kd + ob + g0], nbl = yl[kd + ob + g0], ns0 = ks0[ob + g0],
    nsd = ksd[kd + ob + g0];
    if (u0) np0 = u0[ob + g0], npd = ud[kd + ob + g0], nu = uidx[g0];
  }
  const int64_t bo = (int64_t)o * nunion, su = (int64_t)norb * nunion;
  for (int64_t g = g0; g < nn; g += stride) {
    const int64_t i = ob + g;
    const float2 a = na, al = nal, b = nb, bl = nbl;
    float2 s0 = ns0, sd = nsd;
    const float2 p0 = np0, pd = npd;
    const int u = nu;
    float2 B0 = make_float2(0.f, 0.f), B1 = B0;
    if (u >= 0) {
      B0 = BG[bo + u];
      B1 = BG[(1 + k) * su + bo + u];
    }
    if (g + stride < nn) {
      const int64_t q = i + stride;
      na = xh[q], nal = xl[q], nb = yh[kd + q], nbl = yl[kd + q], ns0 = ks0[q], nsd = ksd[kd + q];
      if (u0) np0 = u0[q], npd = ud[kd + q], nu = uidx[g + stride];
    }
    if (u0) {  // k4 = -i u' + B, sum k = ks + 1 k4 (the w = 1 update of the stage pass)
      s0 = make_float2((p0.y + B0.x) + s0.x, (-p0.x + B0.y) + s0.y);
      sd = make_float2((pd.y + B1.x) + sd.x, (-pd.x + B1.y) + sd.y);
    }
    const FF Xx{a.x, al.x}, Xy{a.y, al.y}, Yx{b.x, bl.x}, Yy{b.y, bl.y};
    const FF nxx = ff_add(ff_mul(f0, Xx), ff_mulf(hh, s0.x));
    const FF nxy = ff_add(ff_mul(f0, Xy), ff_mulf(hh, s0.y));
    const FF nyx = ff_add(ff_add(ff_mul(df, Xx), ff_mul(f1, Yx)), ff_mulf(hh, sd.x));
    const FF nyy = ff_add(ff_add(ff_mul(df, Xy), ff_mul(f1, Yy)), ff_mulf(hh, sd.y));
    const float2 af = make_float2(nxx.h, nxy.h), bf = make_float2(nyx.h, nyy.h);
    if (k == 0) {
      xh2[i] = af;
      xl2[i] = make_float2(nxx.l, nxy.l);
    }
    yh[kd + i] = bf;
    yl[kd + i] = make_float2(nyx.l, nyy.l);
    acc.add(af, bf);
    const float rho = af.x * af.x + af.y * af.y;
    const float drho = 2.f * (af.x * bf.x + af.y * bf.y) + bf.x * bf.x + bf.y * bf.y;
    const float r[3] = {(float)(gx - nx / 2) * dx, (float)(gy - ny / 2) * dy, (float)(gz - nz / 2) * dz};
    gx += sx;
    if (gx >= nx) {
      gx -= nx;
      gy++;
    }
    gy += sy;
    if (gy >= ny) {
      gy -= ny;
      gz++;
    }
    gz += sz;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      Df[c] += r[c] * rho;
      Df[3 + c] += r[c] * drho;
    }
    if (++nd == kChunk) {
#pragma unroll
      for (int c = 0; c < 6; c++) {
        D[c] += f2d(Df[c]);
        Df[c] = 0.f;
      }
      nd = 0;
    }
  }
  acc.flush();
#pragma unroll
  for (int c = 0; c < 6; c++) D[c] += f2d(Df[c]);
  const double A = bsum(acc.A, sh), B = bsum(acc.B, sh);
  const int64_t pq = (int64_t)(k * norb + o) * nchunk + chunk;
  if (threadIdx.x == 0) {
    npart[pq * 2] = A;
    npart[pq * 2 + 1] = B;
  }
#pragma unroll
  for (int c = 0; c < 6; c++) {
    const double v = bsum(D[c], sh);
    if (threadIdx.x == 0) dpart[pq * 6 + c] = v;
  }
}

// per-orbital norm-restore factors (rk4.f90:92-102) of both sets against the
// norms at the start of the call: f0 = sqrt(A0/A1),
// f1 = sqrt((A0+B0)/(A1+B1)), df = f1 - f0 without cancellation
__global__ void k_mix_nfac(const double *__restrict__ part0, const double *__restrict__ part1, int nb, int norb,
                           double *__restrict__ fac, float *__restrict__ facf) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= norb) return;
  double A0 = 0, B0 = 0, A1 = 0, B1 = 0;
  for (int b = 0; b < nb; b++) {
    A0 += part0[((int64_t)o * nb + b) * 2];
    B0 += part0[((int64_t)o * nb + b) * 2 + 1];
    A1 += part1[((int64_t)o * nb + b) * 2];
    B1 += part1[((int64_t)o * nb + b) * 2 + 1];
  }
  const double f0 = sqrt(A0 / A1);
  const double a = B0 / A0, bb = B1 / A1;
  const double rm1 = (a - bb) / (1.0 + bb);  // r - 1, r = (1 + a) / (1 + b)
  const double sr = sqrt(1.0 + rm1);
  const double df = f0 * rm1 / (sr + 1.0);
  fac[3 * o] = f0;
  fac[3 * o + 1] = f0 + df;
  fac[3 * o + 2] = df;
  facf[3 * o] = d2f(f0);
  facf[3 * o + 1] = d2f(f0 + df);
  facf[3 * o + 2] = d2f(df);
}

// per-orbital dipole terms of the restored state: dip = f0^2 Sxx,
// dip' - dip = (f1^2 - f0^2) Sxx + f1^2 Sxy, f1^2 - f0^2 = df (2 f0 + df)
__global__ void k_mix_dip_orb(const double *__restrict__ dpart, const double *__restrict__ fac, int nb, int norb,
                              double *__restrict__ dorb) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= norb) return;
  double S[6] = {0, 0, 0, 0, 0, 0};
  for (int b = 0; b < nb; b++)
    for (int k = 0; k < 6; k++) S[k] += dpart[((int64_t)o * nb + b) * 6 + k];
  const double f0 = fac[3 * o], f1 = fac[3 * o + 1], df = fac[3 * o + 2];
  for (int k = 0; k < 3; k++) {
    dorb[6 * (int64_t)o + k] = f0 * f0 * S[k];
    dorb[6 * (int64_t)o + 3 + k] = df * (2.0 * f0 + df) * S[k] + f1 * f1 * S[3 + k];
  }
}

// dipoles from the per-orbital terms (block k: kick k, terms at part + 6 k
// nparts, strength gamma[k]): out[0..2] dip (written by k = 0), then per kick
// out[3 + 6k ..] dip'_k and out[6 + 6k ..] d_dip_k
__global__ void k_mix_dip_final(const double *__restrict__ part, int nparts, const double *__restrict__ gamma,
                                double dv, double *__restrict__ out) {
  __shared__ double sh[8];
  const int kk = blockIdx.x;
  part += (int64_t)kk * 6 * nparts;
  double s[6];
  for (int k = 0; k < 6; k++) s[k] = block_sum_seq(part + k, nparts, 6, sh);
  if (threadIdx.x != 0) return;
  for (int k = 0; k < 3; k++) {
    const double dip = 2.0 * dv * s[k], ddip = 2.0 * dv * s[3 + k];  // rho = 2 sum |psi|^2
    if (kk == 0) out[k] = dip;
    out[3 + 6 * kk + k] = dip + ddip;
    out[6 + 6 * kk + k] = ddip / gamma[kk];
  }
}

// end of a call: the restored psi = f0 x and psi'_k = f1_k (x + y_k) back to
// FP64 (kick k = blockIdx.z; psi written by k = 0)
__global__ void k_mix_end(double2 *__restrict__ p0, double2 *__restrict__ p1, const float2 *__restrict__ xh,
                          const float2 *__restrict__ xl, const float2 *__restrict__ yh, const float2 *__restrict__ yl,
                          const double *__restrict__ fac, int64_t nn) {
  const int o = blockIdx.y, k = blockIdx.z, norb = gridDim.y;
  const int64_t kd = (int64_t)k * norb * nn;
  const double *fk = fac + 3 * ((int64_t)k * norb + o);
  const FF f0 = ff_of(fk[0]), f1 = ff_of(fk[1]);
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nn; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)o * nn + g;
    const float2 a = xh[i], al = xl[i], b = yh[kd + i], bl = yl[kd + i];
    const FF Xx{a.x, al.x}, Xy{a.y, al.y}, Yx{b.x, bl.x}, Yy{b.y, bl.y};
    if (k == 0) p0[i] = make_double2(ff_val(ff_mul(f0, Xx)), ff_val(ff_mul(f0, Xy)));
    p1[kd + i] = make_double2(ff_val(ff_mul(f1, ff_add(Xx, Yx))), ff_val(ff_mul(f1, ff_add(Xy, Yy))));
  }
}

// ----------------------------------------------------------------- driver --
// Buffers of a call.  nset = 1 + nkick sets: the unperturbed set 0 and the
// differences of the nkick kicked sets, which all share set 0.  Per-point
// arrays of the unperturbed set are [orbital][point], those of the kicks
// [kick][orbital][point]; coefficient arrays are [set][orbital][slot].
struct Mix {
  int norb, nkick, nset;
  int64_t tot;         // norb nn
  float2 *u0, *ud, *ks0, *ksd, *t0, *td;
  float2 *pf0, *pfd;   // the hi arrays of the state x (psi), y (delta)
  float2 *xl, *yl;     // their lo arrays
  float2 *pf0b, *xlb;  // the other buffer of x: k_mix_final writes x' there
  double2 *c0, *cd;    // <p~|t> of set 0 and of the kicks (current buffer of the pair)
  double2 *cnext;      // the other buffer of the pair
  double2 *G, *A;      // [set][table][orbital][slot]: gathers of u' and of pf
  double2 *cD, *q1, *c2, *c3, *pre;  // [set][orbital][slot]
  float2 *bg;          // [kind B, G][set][orbital][union point]: box terms of the fused pass
  float4 *cab;         // [set][orbital][slot]: (-i cD, -i c2) in FP32
  float2 *cg;          // [set][orbital][slot]: c3 in FP32
  double *r0raw, *h0raw, *drraw, *dhraw, *src, *ddens, *vh;  // src, vh: [set][point]
  // the unperturbed set's Hartree source and potential at the first rebuild
  // of a mixed call since set 0 was last replaced from outside (FP64): later
  // rebuilds transform only the change in complex64
  double *src_ref, *vh_ref;
  bool ref_ready = false;
  float *dvf;          // [kick][point]
  double *drhoij, *ddij, *fac, *part0, *partd, *mean, *npart0, *npart1, *nfac, *dpart, *dorb;
  float *facf;         // FP32 copy of nfac
};

static int mix_bufs(opaw_ctx *c, int norb, int nkick, Mix &m) {
  m.norb = norb;
  m.nkick = nkick;
  m.nset = 1 + nkick;
  m.tot = c->nn * (int64_t)norb;
  const size_t cb = sizeof(float2) * (size_t)m.tot;
  const size_t K = (size_t)nkick;
  // unperturbed arrays (one set), difference arrays (nkick sets)
  float2 **c1[3] = {&m.u0, &m.ks0, &m.t0};
  for (int i = 0; i < 3; i++) {
    OPAW_CHECK(ensure(c->mix[i], cb));
    *c1[i] = (float2 *)c->mix[i].p;
  }
  float2 **ck[3] = {&m.ud, &m.ksd, &m.td};
  for (int i = 0; i < 3; i++) {
    OPAW_CHECK(ensure(c->mix[3 + i], cb * K));
    *ck[i] = (float2 *)c->mix[3 + i].p;
  }
  OPAW_CHECK(ensure(c->mix[6], 4 * cb));  // x hi/lo, twice
  m.pf0 = (float2 *)c->mix[6].p;
  m.xl = m.pf0 + m.tot;
  m.pf0b = m.xl + m.tot;
  m.xlb = m.pf0b + m.tot;
  OPAW_CHECK(ensure(c->mix[7], 2 * cb * K));  // y hi, lo
  m.pfd = (float2 *)c->mix[7].p;
  m.yl = m.pfd + m.tot * nkick;
  const size_t sv = (size_t)c->ns * norb;  // one slot vector per orbital
  const size_t S = (size_t)m.nset;
  // c pair x2, G (2 S sv), A (2 S sv), cD, q1, c2, c3, pre (S sv each)
  OPAW_CHECK(ensure(c->mix[11], sizeof(double2) * (sv * S * (2 + 2 + 2 + 5)) + 64));
  double2 *q = (double2 *)c->mix[11].p;
  m.c0 = q;
  m.cd = q + sv;
  m.cnext = q + S * sv;
  m.G = q + 2 * S * sv;
  m.A = q + 4 * S * sv;
  m.cD = q + 6 * S * sv;
  m.q1 = q + 7 * S * sv;
  m.c2 = q + 8 * S * sv;
  m.c3 = q + 9 * S * sv;
  m.pre = q + 10 * S * sv;
  OPAW_CHECK(ensure(c->mix[8], sizeof(float2) * 2 * S * (size_t)norb * c->nunion + 64));
  m.bg = (float2 *)c->mix[8].p;
  OPAW_CHECK(ensure(c->mix[14], sizeof(float4) * S * sv + 64));
  m.cab = (float4 *)c->mix[14].p;
  OPAW_CHECK(ensure(c->mix[15], sizeof(float2) * S * sv + 64));
  m.cg = (float2 *)c->mix[15].p;
  // per point: r0raw, h0raw, drraw (K), dhraw (K), src (S), ddens (K), vh (S), dvf (K floats)
  const size_t nn = (size_t)c->nn;
  OPAW_CHECK(ensure(c->mix[12], sizeof(double) * nn * (2 + 3 * K + 2 * S) + sizeof(float) * nn * K + 64));
  double *r = (double *)c->mix[12].p;
  m.r0raw = r;
  m.h0raw = r + nn;
  m.drraw = r + 2 * nn;
  m.dhraw = m.drraw + K * nn;
  m.src = m.dhraw + K * nn;
  m.ddens = m.src + S * nn;
  m.vh = m.ddens + K * nn;
  m.dvf = (float *)(m.vh + S * nn);
  const void *href_old = c->href.p;
  OPAW_CHECK(ensure(c->href, sizeof(double) * 2 * nn + 64));
  if (c->href.p != href_old) c->href_gen = -1;  // a new buffer holds no reference
  m.src_ref = (double *)c->href.p;
  m.vh_ref = m.src_ref + nn;
  m.ref_ready = c->href_gen == c->psi0_gen;  // a reference of this generation of set 0 exists
  const size_t nparts = K * (size_t)norb * kMixNormBlocks;
  const size_t small = 2 * K * (size_t)c->nd + 4 * K + 16 + 2 * kRedBlocks * (1 + K + S) + S + 16 +
                       4 * nparts + 3 * K * norb + 6 * nparts + 6 * K * norb + 2 * K * norb + 64;
  OPAW_CHECK(ensure(c->mix[13], sizeof(double) * small));
  double *qq = (double *)c->mix[13].p;
  m.drhoij = qq;                            // [K][nd]
  m.ddij = m.drhoij + K * c->nd;            // [K][nd]
  m.fac = m.ddij + K * c->nd;               // [K][4]
  m.part0 = m.fac + 4 * K + 16;             // [2 kRedBlocks], then per kick / source
  m.partd = m.part0 + 2 * kRedBlocks;       // [K][2 kRedBlocks]
  m.mean = m.partd + 2 * kRedBlocks * (K + S);  // [S]
  m.npart0 = m.mean + S + 16;               // [K][N][blocks][2]
  m.npart1 = m.npart0 + 2 * nparts;
  m.nfac = m.npart1 + 2 * nparts;           // [K][N][3]
  m.dpart = m.nfac + 3 * K * norb;          // [K][N][blocks][6]
  m.dorb = m.dpart + 6 * nparts;            // [K][N][6]
  m.facf = (float *)(m.dorb + 6 * K * norb);
  return OPAW_OK;
}

#define MIX_LAUNCHED()             \
  do {                             \
    c->launches++;                 \
    OPAW_CUDA(cudaGetLastError()); \
  } while (0)

// the <p~|t'> just formed become the current pair
static void mix_swap(Mix &m, size_t sv) {
  double2 *cur = m.c0;
  m.c0 = m.cnext;
  m.cd = m.cnext + sv;
  m.cnext = cur;
}

// the fused grid pass (start of a step: stage = 0)
static int mix_fused(opaw_ctx *c, Mix &m, int stage, int first, int write_t, float w, float dts,
                     bool box_only = false) {
  FusedArgs f;
  f.u0 = m.u0;
  f.ud = m.ud;
  f.pf0 = m.pf0;
  f.pfd = m.pfd;
  f.facf = m.facf;
  f.ks0 = m.ks0;
  f.ksd = m.ksd;
  f.t0 = m.t0;
  f.td = m.td;
  f.r0raw = m.r0raw;
  f.drraw = m.drraw;
  f.norb = m.norb;
  f.nkick = m.nkick;
  f.nn = c->nn;
  f.w = w;
  f.dts = dts;
  f.stage = stage;
  f.first = first;
  f.write_t = write_t;
  constexpr int MS = 8;
  const size_t bsmem = sizeof(float4) * 3 * 8 * MS * (size_t)c->uamax;  // at the largest orbital group
  if (c->nunion > 0 && c->ns > 0 && c->d_uent && c->msmax <= MS && bsmem <= 48 * 1024 && (stage || write_t)) {
    const int mode = (stage ? 1 : 0) | (write_t ? 2 : 0);
    // orbitals per CTA (tuned): every (union point, orbital) term is the same sum either way
    auto launch = [&](auto og) {
      constexpr int OG = decltype(og)::value;
      const dim3 nb((c->nunion + kUTile - 1) / kUTile, (m.norb + OG - 1) / OG, (m.nset + 1) / 2);
      const size_t sm = sizeof(float4) * 3 * OG * MS * (size_t)c->uamax;
      auto kern = mode == 1 ? k_mix_boxcoef_t<1, MS, OG>
                            : mode == 2 ? k_mix_boxcoef_t<2, MS, OG> : k_mix_boxcoef_t<3, MS, OG>;
      kern<<<nb, kUTile, sm, c->stream>>>(c->nunion, m.norb, c->ns, c->uamax, m.nset, c->d_ustart, c->d_uent,
                                          c->d_utile, c->d_utile_na, c->d_p3d_f, c->d_p3d1_f, m.cab, m.cg, m.bg);
    };
    static const std::vector<std::string> labels = {"4 orbitals per CTA", "2 orbitals per CTA",
                                                    "8 orbitals per CTA"};
    TuneSite *ts = nullptr;
    const int cand = tune_begin(c, "box terms mode " + std::to_string(mode) + " union " +
                                       std::to_string(c->nunion) + " orbitals " + std::to_string(m.norb) +
                                       " sets " + std::to_string(m.nset),
                                labels, 0, &ts);
    if (cand == 1) launch(std::integral_constant<int, 2>());
    else if (cand == 2) launch(std::integral_constant<int, 8>());
    else launch(std::integral_constant<int, 4>());
    MIX_LAUNCHED();
    OPAW_CHECK(tune_end(c, ts));
  } else if (c->nunion > 0 && c->ns > 0) {
    const dim3 nb(grid1(c->nunion, 128), m.norb, m.nset);
    k_mix_boxcoef<<<nb, 128, 0, c->stream>>>(c->nunion, m.norb, c->ns, c->d_ustart, c->d_uatom, c->d_ubox,
                                             c->d_p3d_f, c->d_p3d1_f, c->d_poff, c->d_nrough, c->d_ms, c->d_soff,
                                             m.cab, m.cg, stage, write_t, m.bg);
    MIX_LAUNCHED();
  }
  if (box_only) return OPAW_OK;  // the last stage's grid part runs inside k_mix_final
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  if (c->ktime_on) {  // live timing (opaw_ktime_begin): events from a reused pool
    while ((int)c->kev.size() < c->kev_used + 2) {
      cudaEvent_t e;
      OPAW_CUDA(cudaEventCreate(&e));
      c->kev.push_back(e);
    }
    ev0 = c->kev[c->kev_used];
    ev1 = c->kev[c->kev_used + 1];
    c->kev_used += 2;
    OPAW_CUDA(cudaEventRecord(ev0, c->stream));
  }
  // block size (tuned): a thread per grid point either way
  static const std::vector<std::string> dlabels = {"256 threads per CTA", "128 threads per CTA"};
  TuneSite *dts_site = nullptr;
  const int dcand = tune_begin(c, "dense pass points " + std::to_string(c->nn) + " orbitals " +
                                     std::to_string(m.norb) + " kicks " + std::to_string(m.nkick),
                              dlabels, 0, &dts_site);
  const int dthreads = dcand == 1 ? 128 : 256;
  k_mix_dense<<<grid1(c->nn, dthreads) * m.nkick, dthreads, 0, c->stream>>>(f, c->d_uidx, m.bg,
                                                                             c->ns > 0 ? c->nunion : 0);
  MIX_LAUNCHED();
  OPAW_CHECK(tune_end(c, dts_site));
  if (ev1) {
    OPAW_CUDA(cudaEventRecord(ev1, c->stream));
    // algorithmic bytes: the union index of every point; per point and
    // orbital the arrays this mode reads or writes once (complex64), of the
    // unperturbed set once and of every kick, the box terms at the union
    // points, the FP64 densities
    const double K = (double)m.nkick;
    double per = 0.0, perb = 0.0;  // bytes per (point, orbital)
    if (stage) per += (1.0 + K) * (8.0 + (first ? 0.0 : 8.0) + 8.0);  // u', ks read, ks write
    if (write_t) per += (1.0 + K) * 16.0;                             // pf read, t write
    if (stage) perb += (1.0 + K) * 8.0;
    if (write_t) perb += (1.0 + K) * 8.0;
    c->kbytes += 4.0 * (double)c->nn + (double)c->nn * (per * m.norb + (write_t ? 8.0 * (1.0 + K) : 0.0)) +
                 (double)c->nunion * perb * m.norb;
  }
  return OPAW_OK;
}

// t = S^-1/2 pf of every set at the start of a step, their <p~|t> and raw densities
static int mix_start_t(opaw_ctx *c, Mix &m) {
  const int norb = m.norb;
  const size_t sv = (size_t)c->ns * norb;
  if (c->ns > 0) {
    OPAW_CHECK(gather2<float>(c, m.pf0, norb, m.A, m.A + sv));
    for (int k = 0; k < m.nkick; k++) {
      double2 *a = m.A + 2 * (size_t)(1 + k) * sv;
      OPAW_CHECK(gather2<float>(c, m.pfd + (size_t)k * m.tot, norb, a, a + sv));
    }
    const Ovl v = ovl_of(c);
    k_mc_scale_a<<<dim3(grid1(c->ns, 128), norb, 2), 128, 0, c->stream>>>(m.A, m.nfac, norb, c->ns, m.nkick);
    MIX_LAUNCHED();
    const dim3 g(grid1(c->ns, 128), norb, m.nset);
    k_mc_start<<<g, 128, 0, c->stream>>>(v, m.A, c->d_sigma[1], m.c3, m.pre, norb, c->ns);
    MIX_LAUNCHED();
    k_mc_t<<<g, 128, 0, c->stream>>>(v, m.pre, m.c3, m.cnext, m.cg, norb, c->ns);
    MIX_LAUNCHED();
    mix_swap(m, sv);
  }
  return mix_fused(c, m, 0, 0, 1, 0.f, 0.f);
}

// one RK4 stage of every set from t, <p~|t> and the rebuilt potentials: the
// grid part of H, the two gathers, the FP64 algebra and the fused pass
static int mix_stage(opaw_ctx *c, Mix &m, int st, float w, double dts) {
  const int norb = m.norb;
  const size_t sv = (size_t)c->ns * norb;
  const int write_t = st < 3;
  int both;
  OPAW_CHECK(h_fftk<float>(c, c->d_vks_f[0], c->d_vks_f[1], m.t0, m.td, m.u0, m.ud, m.dvf, norb, m.nkick, &both));
  if (!both) {
    OPAW_CHECK(h_fft<float>(c, c->d_vks_f[0], m.t0, m.u0, norb, nullptr, nullptr));
    for (int k = 0; k < m.nkick; k++)
      OPAW_CHECK(h_fft<float>(c, c->d_vks_f[1] + (size_t)k * c->nn, m.td + (size_t)k * m.tot,
                              m.ud + (size_t)k * m.tot, norb, m.t0, m.dvf + (size_t)k * c->nn));
  }
  if (c->ns > 0) {
    OPAW_CHECK(gather2<float>(c, m.u0, norb, m.G, m.G + sv));
    for (int k = 0; k < m.nkick; k++) {
      double2 *gk = m.G + 2 * (size_t)(1 + k) * sv;
      OPAW_CHECK(gather2<float>(c, m.ud + (size_t)k * m.tot, norb, gk, gk + sv));
    }
    // cD = D <p~|t> (unperturbed), D'_k <p~|td_k> + (D'_k - D) <p~|t0> (differences)
    const dim3 gc(grid1(c->ns, 128), norb);
    k_coef_dij<<<gc, 128, 0, c->stream>>>(m.c0, m.cD, norb, c->ns, c->d_slot_atom, c->d_soff, c->d_doff, c->d_ms,
                                          c->d_dij[0]);
    MIX_LAUNCHED();
    for (int k = 0; k < m.nkick; k++) {
      k_coef_dij2<<<gc, 128, 0, c->stream>>>(m.cd + (size_t)k * sv, m.c0, m.cD + (size_t)(1 + k) * sv, norb, c->ns,
                                             c->d_slot_atom, c->d_soff, c->d_doff, c->d_ms,
                                             c->d_dij[1] + (size_t)k * c->nd, m.ddij + (size_t)k * c->nd);
      MIX_LAUNCHED();
    }
    const Ovl v = ovl_of(c);
    const dim3 g(grid1(c->ns, 128), norb, m.nset);
    k_mc_c2<<<g, 128, 0, c->stream>>>(v, m.G, m.cD, c->d_sigma[1], m.q1, m.c2, norb, c->ns);
    MIX_LAUNCHED();
    k_mc_k<<<g, 128, 0, c->stream>>>(v, m.G, m.A, m.cD, m.q1, m.c2, c->d_sigma[1], dts, write_t, m.c3, m.pre, m.cab,
                                     norb, c->ns);
    MIX_LAUNCHED();
    if (write_t) {
      k_mc_t<<<g, 128, 0, c->stream>>>(v, m.pre, m.c3, m.cnext, m.cg, norb, c->ns);
      MIX_LAUNCHED();
      mix_swap(m, sv);
    }
  }
  return mix_fused(c, m, 1, st == 0, write_t, w, (float)dts, st == 3);
}

// the rest of the rebuild (ncpaw_make_hamiltonian.f90:119-129) from <p~|t>
// and the raw densities of every set: rho_ij, n^, renormalisation, Hartree,
// v_ks, D_ij of set 0 and of every kick, and the kicks' differences
// x += a y over n points (FP64)
__global__ void k_mix_axpy(double *__restrict__ x, const double *__restrict__ y, double a, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) x[i] += a * y[i];
}

static int mix_potentials(opaw_ctx *c, Mix &m) {
  const int norb = m.norb, K = m.nkick;
  const int nb = grid1(c->nn, 256);
  const size_t sv = (size_t)c->ns * norb;
  OPAW_CHECK(rhoij_of(c, m.c0, norb, c->d_rhoij[0]));
  OPAW_CHECK(nhat_raw_of(c, c->d_rhoij[0], m.h0raw));
  if (c->nd > 0) {
    k_mix_drhoij<<<dim3(grid1((int64_t)c->nd * 32, 256), K), 256, 0, c->stream>>>(
        m.c0, m.cd, norb, c->ns, c->nd, c->d_dslot_atom, c->d_soff, c->d_doff, c->d_ms, c->d_rhoij[0], m.drhoij,
        c->d_rhoij[1]);
    MIX_LAUNCHED();
  }
  (void)sv;
  // the on-site XC term of every set depends on rho_ij alone: it runs on the
  // side stream while the compensation charges, the Hartree solves and v_ks
  // run here, and joins before D_ij
  double *dxc_sets = nullptr;
  if (c->oxc_on && c->nd > 0 && c->side) {
    OPAW_CHECK(ensure(c->oxc_sets, sizeof(double) * (size_t)(1 + K) * c->nd));
    dxc_sets = (double *)c->oxc_sets.p;
    OPAW_CUDA(cudaEventRecord(c->side_fork, c->stream));
    OPAW_CUDA(cudaStreamWaitEvent(c->side, c->side_fork, 0));
    OPAW_CHECK(onsite_xc_sets(c, c->d_rhoij[0], 1, dxc_sets, c->side));
    OPAW_CHECK(onsite_xc_sets(c, c->d_rhoij[1], K, dxc_sets + c->nd, c->side));
    OPAW_CUDA(cudaEventRecord(c->side_join, c->side));
  }
  for (int k = 0; k < K; k++)  // n^ is linear in rho_ij
    OPAW_CHECK(nhat_raw_of(c, m.drhoij + (size_t)k * c->nd, m.dhraw + (size_t)k * c->nn));
  // charge renormalisation of every set
  OPAW_CHECK(sums2(c, m.h0raw, m.r0raw, m.part0));
  for (int k = 0; k < K; k++)
    OPAW_CHECK(sums2(c, m.dhraw + (size_t)k * c->nn, m.drraw + (size_t)k * c->nn, m.partd + 2 * (size_t)k * kRedBlocks));
  k_mix_factors<<<K, 256, 0, c->stream>>>(m.part0, m.partd, kRedBlocks, c->dv, c->rnel, m.fac);
  MIX_LAUNCHED();
  k_mix_renorm<<<dim3(nb, K), 256, 0, c->stream>>>(m.r0raw, m.h0raw, m.drraw, m.dhraw, m.fac, c->d_dens[0],
                                                   c->d_nhat[0], c->d_dens[1], c->d_nhat[1], m.src, m.src + c->nn,
                                                   m.ddens, c->nn);
  MIX_LAUNCHED();
  // Hartree of n0 + n^0 and of every difference: one batch of complex64
  // transforms, so each difference keeps its own relative precision (packing
  // it with the ~1e3 times larger n0 into one transform would round it
  // relative to n0).  The unperturbed source itself goes in as its change
  // since a reference source (the first mixed rebuild after set 0 was last
  // replaced from outside), whose potential is solved once in FP64:
  // v_H[n0] = v_H[ref] + v_H[n0 - ref].  A complex64 solve of n0 rounds
  // relative to all of n0 (its low-k and k = 0 terms, amplified by the
  // Martyna-Tuckerman kernel, shift every orbital's potential), and that
  // error grows in the dipole step after step; the change since the
  // reference is orders of magnitude smaller than n0.
  if (!m.ref_ready) {
    OPAW_CUDA(cudaMemcpyAsync(m.src_ref, m.src, sizeof(double) * c->nn, cudaMemcpyDeviceToDevice, c->stream));
    OPAW_CHECK(hartree_batch_t<double>(c, m.src_ref, 1, m.vh_ref));
    m.ref_ready = true;
    c->href_gen = c->psi0_gen;
  }
  k_mix_axpy<<<nb, 256, 0, c->stream>>>(m.src, m.src_ref, -1.0, c->nn);
  MIX_LAUNCHED();
  OPAW_CHECK(hartree_batch_t<float>(c, m.src, m.nset, m.vh));
  k_mix_axpy<<<nb, 256, 0, c->stream>>>(m.vh, m.vh_ref, 1.0, c->nn);
  MIX_LAUNCHED();
  const double *mean = nullptr;
  if (c->periodic) {  // tddft_pot.f90:42-45
    for (int b = 0; b < m.nset; b++)
      OPAW_CHECK(sums2(c, m.vh + (size_t)b * c->nn, nullptr, m.partd + 2 * (size_t)(K + b) * kRedBlocks));
    k_mix_mean<<<m.nset, 256, 0, c->stream>>>(m.partd + 2 * (size_t)K * kRedBlocks, kRedBlocks, c->nn, m.mean);
    MIX_LAUNCHED();
    mean = m.mean;
  }
  k_mix_pot<<<dim3(nb, K), 256, 0, c->stream>>>(c->d_dens[0], m.ddens, c->d_ncoret, c->d_vloc, m.vh, m.vh + c->nn,
                                                mean, c->d_vks[0], c->d_vks[1], c->d_vks_f[0], c->d_vks_f[1], m.dvf,
                                                c->d_vxc[0], c->d_vxc[1], c->d_vh[1], c->nn);
  MIX_LAUNCHED();
  OPAW_CUDA(cudaMemcpyAsync(c->d_vh[0], m.vh, sizeof(double) * c->nn, cudaMemcpyDeviceToDevice, c->stream));
  // D_ij of every set (FP64) and the kicks' differences
  if (dxc_sets) OPAW_CUDA(cudaStreamWaitEvent(c->stream, c->side_join, 0));
  OPAW_CHECK(dij_of(c, c->d_rhoij[0], c->d_vks[0], c->d_vxc[0], c->d_dij[0], dxc_sets));
  for (int k = 0; k < K; k++)
    OPAW_CHECK(dij_of(c, c->d_rhoij[1] + (size_t)k * c->nd, c->d_vks[1] + (size_t)k * c->nn,
                      c->d_vxc[1] + (size_t)k * c->nn, c->d_dij[1] + (size_t)k * c->nd,
                      dxc_sets ? dxc_sets + (size_t)(1 + k) * c->nd : nullptr));
  if (c->nd > 0) {
    k_mix_ddij<<<dim3(grid1(c->nd, 128), K), 128, 0, c->stream>>>(c->d_dij[0], c->d_dij[1], m.ddij, c->nd);
    MIX_LAUNCHED();
  }
  return OPAW_OK;
}

// the call's first part: x, y_k in float-float and the norms to restore
// (rk4.f90:16), no pending factors yet
static int mix_begin(opaw_ctx *c, Mix &m) {
  const dim3 gn(kMixNormBlocks, m.norb, m.nkick);
  k_mix_start<<<gn, 256, 0, c->stream>>>(c->d_psi[0], c->d_psi[1], m.pf0, m.xl, m.pfd, m.yl, c->nn, m.npart0);
  MIX_LAUNCHED();
  const int nk = m.nkick * m.norb;
  k_mix_fac_init<<<grid1(nk, 128), 128, 0, c->stream>>>(m.nfac, m.facf, nk);
  MIX_LAUNCHED();
  return OPAW_OK;
}

// one TDDFT step of every set; 3 + 6 nkick doubles of dipoles into out
static int mix_step(opaw_ctx *c, Mix &m, double dt, const double *gamma_dev, double *out) {
  const float wts[4] = {1.f, 2.f, 2.f, 1.f};
  const double dts[4] = {dt / 2.0, dt / 2.0, dt, dt};
  const int norb = m.norb, nk = m.nkick * norb;
  // ncpaw_make_hamiltonian_tddft (tddft.f90:75)
  OPAW_CHECK(mix_start_t(c, m));
  OPAW_CHECK(mix_potentials(c, m));
  for (int st = 0; st < 4; st++) {
    OPAW_CHECK(mix_stage(c, m, st, wts[st], dts[st]));
    if (st < 3) OPAW_CHECK(mix_potentials(c, m));  // rk4.f90:53-55
  }
  // the last stage's grid part (k4 and the complete sum k) and the final combination
  const dim3 gf(kMixNormBlocks * m.nkick, norb);
  k_mix_final<<<gf, 256, 0, c->stream>>>(m.pf0, m.xl, m.pf0b, m.xlb, m.pfd, m.yl, m.ks0, m.ksd, m.nfac, dt / 6.0,
                                         c->nn, c->nx, c->ny, c->nz, (float)c->dx, (float)c->dy, (float)c->dz,
                                         m.npart1, m.dpart, m.u0, m.ud, c->d_uidx, m.bg, c->ns > 0 ? c->nunion : 0,
                                         m.nkick);
  MIX_LAUNCHED();
  std::swap(m.pf0, m.pf0b);
  std::swap(m.xl, m.xlb);
  k_mix_nfac<<<grid1(nk, 128), 128, 0, c->stream>>>(m.npart0, m.npart1, kMixNormBlocks, nk, m.nfac, m.facf);
  MIX_LAUNCHED();
  k_mix_dip_orb<<<grid1(nk, 128), 128, 0, c->stream>>>(m.dpart, m.nfac, kMixNormBlocks, nk, m.dorb);
  MIX_LAUNCHED();
  k_mix_dip_final<<<m.nkick, 256, 0, c->stream>>>(m.dorb, norb, gamma_dev, c->dv, out);
  MIX_LAUNCHED();
  return OPAW_OK;
}

// the call's last part: psi and every psi'_k back to complex128
static int mix_finish(opaw_ctx *c, Mix &m) {
  const dim3 gn(kMixNormBlocks, m.norb, m.nkick);
  k_mix_end<<<gn, 256, 0, c->stream>>>(c->d_psi[0], c->d_psi[1], m.pf0, m.xl, m.pfd, m.yl, m.nfac, c->nn);
  MIX_LAUNCHED();
  return OPAW_OK;
}

int mixed_steps(opaw_ctx *c, int nsteps, double dt, const double *gamma_dev, double *dd_dev) {
  Mix m;
  OPAW_CHECK(mix_bufs(c, c->norb[0], c->nkick, m));
  OPAW_CHECK(mix_begin(c, m));
  const size_t per = 3 + 6 * (size_t)c->nkick;
  for (int it = 0; it < nsteps; it++) OPAW_CHECK(mix_step(c, m, dt, gamma_dev, dd_dev + per * (size_t)it));
  return mix_finish(c, m);
}

// ------------------------------------------------------------- ensemble --
// Several contexts (molecules on their own grids, each with its kicked sets)
// stepped together.  The first step of each runs as plain launches (it also
// grows every scratch buffer to its final size); then two steps of every
// context are captured once into one CUDA graph, a branch per context on the
// context's own stream, and the graph is replayed: per replay one launch
// covers two steps of every molecule, and the molecules' kernels overlap on
// the GPU.  Two steps per graph return every double-buffered pointer of the
// step to where it started, so each replay is the same sequence of launches.
// A last odd step runs as plain launches.  dd[i]: device output of context i,
// (3 + 6 nkick) doubles per step; fixed[i]: 2 (3 + 6 nkick) device doubles the
// graph writes and the host copies out after each replay.
int ensemble_steps(opaw_ctx *const *cs, int n, int nsteps, double dt, double *const *dd, double *const *fixed) {
  std::vector<Mix> ms(n);
  std::vector<size_t> per(n);
  for (int i = 0; i < n; i++) {
    opaw_ctx *c = cs[i];
    OPAW_CHECK(mix_bufs(c, c->norb[0], c->nkick, ms[i]));
    OPAW_CHECK(mix_begin(c, ms[i]));
    per[i] = 3 + 6 * (size_t)c->nkick;
  }
  int it = 0;
  if (nsteps > 0) {
    for (int i = 0; i < n; i++) OPAW_CHECK(mix_step(cs[i], ms[i], dt, cs[i]->d_kgamma, dd[i]));
    it = 1;
  }
  const int npairs = (nsteps - it) / 2;
  if (npairs > 0) {
    cudaStream_t master = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaEvent_t> ev(n + 1, nullptr);
    std::vector<int64_t> dl(n, 0);
    int st = OPAW_OK;
    auto cuda_ok = [&](cudaError_t e, const char *what) {
      if (e != cudaSuccess && st == OPAW_OK) {
        set_error(std::string(what) + ": " + cudaGetErrorString(e));
        st = OPAW_ERR_CUDA;
      }
      return st == OPAW_OK;
    };
    bool capturing = false;
    do {
      if (!cuda_ok(cudaStreamCreateWithFlags(&master, cudaStreamNonBlocking), "ensemble stream")) break;
      for (auto &e : ev)
        if (!cuda_ok(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "ensemble event")) break;
      if (st != OPAW_OK) break;
      // the graph's first replay follows the plain first step of every context
      for (int i = 0; i < n; i++) {
        if (!cuda_ok(cudaEventRecord(ev[i], cs[i]->stream), "record")) break;
        if (!cuda_ok(cudaStreamWaitEvent(master, ev[i], 0), "wait")) break;
      }
      if (st != OPAW_OK) break;
      if (!cuda_ok(cudaStreamBeginCapture(master, cudaStreamCaptureModeRelaxed), "begin capture")) break;
      capturing = true;
      if (!cuda_ok(cudaEventRecord(ev[n], master), "fork")) break;
      for (int i = 0; i < n && st == OPAW_OK; i++) {
        opaw_ctx *c = cs[i];
        if (!cuda_ok(cudaStreamWaitEvent(c->stream, ev[n], 0), "fork wait")) break;
        const int64_t l0 = c->launches;
        for (int j = 0; j < 2 && st == OPAW_OK; j++) st = mix_step(c, ms[i], dt, c->d_kgamma, fixed[i] + per[i] * j);
        dl[i] = c->launches - l0;
        if (st != OPAW_OK) break;
        if (!cuda_ok(cudaEventRecord(ev[i], c->stream), "join")) break;
        if (!cuda_ok(cudaStreamWaitEvent(master, ev[i], 0), "join wait")) break;
      }
      cudaError_t ec = cudaStreamEndCapture(master, &graph);
      capturing = false;
      if (!cuda_ok(ec, "end capture")) break;
      if (!cuda_ok(cudaGraphInstantiate(&exec, graph, 0), "graph instantiate")) break;
      for (int p = 0; p < npairs && st == OPAW_OK; p++) {
        if (!cuda_ok(cudaGraphLaunch(exec, master), "graph launch")) break;
        for (int i = 0; i < n; i++)
          if (!cuda_ok(cudaMemcpyAsync(dd[i] + per[i] * (size_t)(it + 2 * p), fixed[i], sizeof(double) * 2 * per[i],
                                       cudaMemcpyDeviceToDevice, master),
                       "dipole copy"))
            break;
      }
      if (st != OPAW_OK) break;
      // the contexts' streams continue after the last replay
      if (!cuda_ok(cudaEventRecord(ev[n], master), "record")) break;
      for (int i = 0; i < n; i++) {
        if (!cuda_ok(cudaStreamWaitEvent(cs[i]->stream, ev[n], 0), "wait")) break;
        cs[i]->launches += dl[i] * (npairs - 1);  // captured once, run npairs times
      }
    } while (0);
    if (capturing) {  // a failure inside the capture: end it so the stream is usable again
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(master, &g);
      if (g) cudaGraphDestroy(g);
    }
    if (master) cudaStreamSynchronize(master);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
    if (master) cudaStreamDestroy(master);
    OPAW_CHECK(st);
    it += 2 * npairs;
  }
  for (; it < nsteps; it++)
    for (int i = 0; i < n; i++) OPAW_CHECK(mix_step(cs[i], ms[i], dt, cs[i]->d_kgamma, dd[i] + per[i] * it));
  for (int i = 0; i < n; i++) OPAW_CHECK(mix_finish(cs[i], ms[i]));
  return OPAW_OK;
}

}  // namespace opaw

using namespace opaw;

// opaw_ensemble_steps: see include/opaw_gb300.h
extern "C" int opaw_ensemble_steps(opaw_ctx *const *ctx, int nctx, int nsteps, double dt, double *const *dip_out,
                                   double *const *dip_pert_out, double *const *d_dip_out) {
  OPAW_ARG(ctx && nctx >= 1 && nsteps >= 0, "bad ensemble arguments");
  for (int i = 0; i < nctx; i++) {
    opaw_ctx *c = ctx[i];
    OPAW_ARG(c, "null context in the ensemble");
    for (int j = 0; j < i; j++) OPAW_ARG(ctx[j] != c, "a context appears twice in the ensemble");
    if (c->norb[0] == 0 || c->norb[1] == 0) {
      set_error("every context of the ensemble needs its orbitals and kicked sets (opaw_excite_kicks)");
      return OPAW_ERR_STATE;
    }
    OPAW_ARG(c->norb[0] == c->norb[1], "every set must hold the same number of orbitals");
    OPAW_ARG((int)c->h_kgamma.size() == c->nkick, "kick strengths missing: excite with opaw_excite_kicks");
    OPAW_ARG(!c->ktime_on, "kernel timing (opaw_ktime_begin) is not available in an ensemble run");
  }
  std::vector<double *> dd(nctx), fixed(nctx);
  std::vector<size_t> per(nctx);
  for (int i = 0; i < nctx; i++) {
    opaw_ctx *c = ctx[i];
    OPAW_CHECK(upload_kgamma(c));
    per[i] = 3 + 6 * (size_t)c->nkick;
    const size_t nout = per[i] * (size_t)(nsteps > 0 ? nsteps : 1);
    OPAW_CHECK(ensure(c->work[11], sizeof(double) * (nout + 2 * per[i] + 16)));
    dd[i] = (double *)c->work[11].p;
    fixed[i] = dd[i] + nout;
  }
  OPAW_CHECK(ensemble_steps(ctx, nctx, nsteps, dt, dd.data(), fixed.data()));
  for (int i = 0; i < nctx; i++) {
    opaw_ctx *c = ctx[i];
    const int K = c->nkick;
    std::vector<double> h(per[i] * (size_t)(nsteps > 0 ? nsteps : 0));
    if (!h.empty())
      OPAW_CUDA(cudaMemcpyAsync(h.data(), dd[i], sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    OPAW_CUDA(cudaStreamSynchronize(c->stream));
    for (int t = 0; t < nsteps; t++) {
      const double *q = h.data() + per[i] * (size_t)t;
      for (int j = 0; j < 3; j++) {
        if (dip_out && dip_out[i]) dip_out[i][3 * t + j] = q[j];
        for (int k = 0; k < K; k++) {
          if (dip_pert_out && dip_pert_out[i]) dip_pert_out[i][3 * ((size_t)t * K + k) + j] = q[3 + 6 * k + j];
          if (d_dip_out && d_dip_out[i]) d_dip_out[i][3 * ((size_t)t * K + k) + j] = q[6 + 6 * k + j];
        }
      }
    }
  }
  return OPAW_OK;
}

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
// and the charge-renormalisation factors are taken in FP64.  psi, delta, the RK4 accumulation, the norms and the dipole are FP64.
//
// In exact arithmetic this is the reference algorithm; OPAW_PREC_FP64 runs
// the reference's own form for comparison.
#include <cmath>

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


// difference of rho_ij: 2 sum_occ Re(conj(c0_i) cd_j + conj(cd_i) c0_j + conj(cd_i) cd_j)
__global__ void k_mix_drhoij(const double2 *__restrict__ c0, const double2 *__restrict__ cd, int norb, int ns, int nd,
                             const int *__restrict__ dslot, const int64_t *__restrict__ soff,
                             const int64_t *__restrict__ doff, const int *__restrict__ ms,
                             const double *__restrict__ rho0, double *__restrict__ drho, double *__restrict__ rho1) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nd) return;
  const int a = dslot[t];
  const int m = ms[a];
  const int loc = t - (int)doff[a];
  const int i = loc % m, j = loc / m;
  double acc = 0;
  for (int o = 0; o < norb; o++) {
    const double2 ai = c0[(int64_t)o * ns + soff[a] + i], aj = c0[(int64_t)o * ns + soff[a] + j];
    const double2 bi = cd[(int64_t)o * ns + soff[a] + i], bj = cd[(int64_t)o * ns + soff[a] + j];
    acc += 2.0 * (ai.x * bj.x + ai.y * bj.y + bi.x * aj.x + bi.y * aj.y + bi.x * bj.x + bi.y * bj.y);
  }
  drho[t] = acc;
  rho1[t] = rho0[t] + acc;
}

// density difference 2 sum_occ (2 Re(conj(t0) td) + |td|^2), complex64 inputs,
// 16-orbital partial sums in FP32 added in FP64
__global__ void k_mix_drho(const float2 *__restrict__ t0, const float2 *__restrict__ td, int norb, int64_t nn,
                           double *__restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nn) return;
  double acc = 0;
  for (int o0 = 0; o0 < norb; o0 += 16) {
    float part = 0.f;
    const int o1 = min(norb, o0 + 16);
    for (int o = o0; o < o1; o++) {
      const float2 a = t0[(int64_t)o * nn + i], b = td[(int64_t)o * nn + i];
      part += 2.f * (a.x * b.x + a.y * b.y) + b.x * b.x + b.y * b.y;
    }
    acc += (double)part;
  }
  out[i] = 2.0 * acc;
}

// renormalisation factors (nhat.f90:32-37) of both sets from the raw sums:
// f0 = rnel / S0, f1 = rnel / (S0 + dS), df = f1 - f0 = -rnel dS / (S0 (S0 + dS))
__global__ void k_mix_factors(const double *__restrict__ p0, const double *__restrict__ pd, int nb, double dv,
                              double rnel, double *__restrict__ fac) {
  __shared__ double sh[8];
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
__global__ void k_mix_renorm(const double *__restrict__ r0raw, const double *__restrict__ h0raw,
                             const double *__restrict__ drraw, const double *__restrict__ dhraw,
                             const double *__restrict__ fac, double *__restrict__ dens0, double *__restrict__ nhat0,
                             double *__restrict__ dens1, double *__restrict__ nhat1, double *__restrict__ src0,
                             double *__restrict__ srcd, double *__restrict__ ddens, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double f0 = fac[0], f1 = fac[1], df = fac[2];
  const double r0 = f0 * r0raw[i], h0 = f0 * h0raw[i];
  const double dr = df * r0raw[i] + f1 * drraw[i];
  const double dh = df * h0raw[i] + f1 * dhraw[i];
  dens0[i] = r0;
  nhat0[i] = h0;
  dens1[i] = r0 + dr;
  nhat1[i] = h0 + dh;
  src0[i] = r0 + h0;
  srcd[i] = dr + dh;
  ddens[i] = dr;
}

__device__ __forceinline__ double vxc_lda(double n) {
  if (!(n > 1e-15)) return 0.0;
  const double pi = 3.14159265358979323846;
  const double vx = -cbrt(3.0 * n / pi);
  const double A = 0.031091, a1 = 0.21370, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382, b4 = 0.49294;
  const double rs = cbrt(3.0 / (4.0 * pi * n));
  const double srs = sqrt(rs);
  const double Q = 2.0 * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  const double dQ = 2.0 * A * (0.5 * b1 / srs + b2 + 1.5 * b3 * srs + 2.0 * b4 * rs);
  const double lg = log(1.0 + 1.0 / Q);
  const double ec = -2.0 * A * (1.0 + a1 * rs) * lg;
  const double dec = -2.0 * A * a1 * lg + 2.0 * A * (1.0 + a1 * rs) * dQ / (Q * Q + Q);
  return vx + (ec - rs / 3.0 * dec);
}

// potentials of both sets: v0 = vH0 + vxc(n0 + nc) + vloc, dv = dvH + vxc(n1 + nc) - vxc(n0 + nc)
__global__ void k_mix_pot(const double *__restrict__ dens0, const double *__restrict__ ddens,
                          const double *__restrict__ core, const double *__restrict__ vloc,
                          const double *__restrict__ vh0, const double *__restrict__ dvh, const double *__restrict__ mean,
                          double *__restrict__ vks0, double *__restrict__ vks1, float *__restrict__ vks0f,
                          float *__restrict__ vks1f, float *__restrict__ dvf, double *__restrict__ vxc0o,
                          double *__restrict__ vxc1o, double *__restrict__ vh1o, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double n0 = dens0[i] + core[i];
  const double x0 = vxc_lda(n0);
  const double x1 = vxc_lda(n0 + ddens[i]);
  double h0 = vh0[i], dh = dvh[i];
  if (mean) {
    h0 -= mean[0];
    dh -= mean[1];
  }
  const double v0 = h0 + x0 + vloc[i];
  const double dv = dh + (x1 - x0);
  const double v1 = v0 + dv;
  vks0[i] = v0;
  vks1[i] = v1;
  vks0f[i] = (float)v0;
  vks1f[i] = (float)v1;
  dvf[i] = (float)dv;
  vxc0o[i] = x0;
  vxc1o[i] = x1;
  vh1o[i] = h0 + dh;
}

__global__ void k_mix_mean(const double *__restrict__ pa, const double *__restrict__ pb, int nb, int64_t n,
                           double *__restrict__ mean) {
  __shared__ double sh[8];
  const double a = block_sum_seq(pa, nb, 2, sh);
  const double b = block_sum_seq(pb, nb, 2, sh);
  if (threadIdx.x != 0) return;
  mean[0] = a / (double)n;
  mean[1] = b / (double)n;
}

__global__ void k_mix_ddij(const double *__restrict__ d0, const double *__restrict__ d1, double *__restrict__ dd,
                           int nd) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nd) dd[t] = d1[t] - d0[t];
}

// RK4 stage of both sets (rk4.f90:44-48): k = -i shs(y); ksum (+)= w k; y = p + dts k
__global__ void k_mix_stage(const float2 *__restrict__ k0r, const float2 *__restrict__ kdr,
                            const float2 *__restrict__ p0, const float2 *__restrict__ d,
                            float2 *__restrict__ ks0, float2 *__restrict__ ksd, float2 *__restrict__ y0,
                            float2 *__restrict__ yd, int64_t n, float w, int first, float dts, int write_y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 a = k0r[i], b = kdr[i];
  const float ax = a.y, ay = -a.x, bx = b.y, by = -b.x;
  float2 s0, sd;
  if (first) {
    s0 = make_float2(w * ax, w * ay);
    sd = make_float2(w * bx, w * by);
  } else {
    s0 = ks0[i];
    sd = ksd[i];
    s0.x += w * ax;
    s0.y += w * ay;
    sd.x += w * bx;
    sd.y += w * by;
  }
  ks0[i] = s0;
  ksd[i] = sd;
  if (write_y) {
    const float2 pv = p0[i], dvv = d[i];
    y0[i] = make_float2(pv.x + dts * ax, pv.y + dts * ay);
    yd[i] = make_float2(dvv.x + dts * bx, dvv.y + dts * by);
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

// start of a call: delta = psi' - psi, their complex64 copies, norm partials
__global__ void k_mix_start(const double2 *__restrict__ p0, const double2 *__restrict__ p1, double2 *__restrict__ d,
                            float2 *__restrict__ pf0, float2 *__restrict__ pfd, int64_t nn,
                            double *__restrict__ part) {
  __shared__ double sh[8];
  const int o = blockIdx.y;
  NormAcc acc;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nn; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)o * nn + g;
    const double2 x = p0[i], y1 = p1[i];
    const double2 y = make_double2(y1.x - x.x, y1.y - x.y);
    d[i] = y;
    const float2 xf = make_float2(d2f(x.x), d2f(x.y)), yf = make_float2(d2f(y.x), d2f(y.y));
    pf0[i] = xf;
    pfd[i] = yf;
    acc.add(xf, yf);
  }
  acc.flush();
  const double A = bsum(acc.A, sh), B = bsum(acc.B, sh);
  if (threadIdx.x == 0) {
    part[((int64_t)o * gridDim.x + blockIdx.x) * 2] = A;
    part[((int64_t)o * gridDim.x + blockIdx.x) * 2 + 1] = B;
  }
}

// final RK4 combination (rk4.f90:22) of both sets, in place, with the norm
// partials of the results
__global__ void k_mix_final(double2 *__restrict__ p0, double2 *__restrict__ d, const float2 *__restrict__ ks0,
                            const float2 *__restrict__ ksd, int64_t nn, double h6, double *__restrict__ part) {
  __shared__ double sh[8];
  const int o = blockIdx.y;
  NormAcc acc;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nn; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)o * nn + g;
    const float2 s0 = ks0[i], sd = ksd[i];
    double2 x = p0[i], y = d[i];
    x.x += h6 * f2d(s0.x);
    x.y += h6 * f2d(s0.y);
    y.x += h6 * f2d(sd.x);
    y.y += h6 * f2d(sd.y);
    p0[i] = x;
    d[i] = y;
    acc.add(make_float2(d2f(x.x), d2f(x.y)), make_float2(d2f(y.x), d2f(y.y)));
  }
  acc.flush();
  const double A = bsum(acc.A, sh), B = bsum(acc.B, sh);
  if (threadIdx.x == 0) {
    part[((int64_t)o * gridDim.x + blockIdx.x) * 2] = A;
    part[((int64_t)o * gridDim.x + blockIdx.x) * 2 + 1] = B;
  }
}

// per-orbital norm-restore factors (rk4.f90:92-102) of both sets:
// f0 = sqrt(A0/A1), f1 = sqrt((A0+B0)/(A1+B1)), df = f1 - f0 without cancellation
__global__ void k_mix_nfac(const double *__restrict__ part0, const double *__restrict__ part1, int nb, int norb,
                           double *__restrict__ fac) {
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
}

// norm restore p0 = f0 p0u, delta = df p0u + f1 du, fused with what the next
// step reads first: complex64 copies, norm partials, and the dipole partials
// of this step (tddft_plot.f90:40-57: dip = sum r rho0 dv, dip' - dip = sum r drho dv)
__global__ void k_mix_rescale(double2 *__restrict__ p0, double2 *__restrict__ d, float2 *__restrict__ pf0,
                              float2 *__restrict__ pfd, const double *__restrict__ fac, int64_t nn, int nx, int ny,
                              int nz, float dx, float dy, float dz, double *__restrict__ npart,
                              double *__restrict__ dpart) {
  __shared__ double sh[8];
  const int o = blockIdx.y;
  const double f0 = fac[3 * o], f1 = fac[3 * o + 1], df = fac[3 * o + 2];
  NormAcc acc;
  double D[6] = {0, 0, 0, 0, 0, 0};
  float Df[6] = {0, 0, 0, 0, 0, 0};
  int nd = 0;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nn; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)o * nn + g;
    const double2 x = p0[i], y = d[i];
    const double2 a = make_double2(f0 * x.x, f0 * x.y);
    const double2 b = make_double2(df * x.x + f1 * y.x, df * x.y + f1 * y.y);
    p0[i] = a;
    d[i] = b;
    const float2 af = make_float2(d2f(a.x), d2f(a.y)), bf = make_float2(d2f(b.x), d2f(b.y));
    pf0[i] = af;
    pfd[i] = bf;
    const float rho = af.x * af.x + af.y * af.y;
    const float drho = 2.f * (af.x * bf.x + af.y * bf.y) + bf.x * bf.x + bf.y * bf.y;
    acc.add(af, bf);
    const int gi = (int)g, gxy = gi / nx;
    const int gx = gi - gxy * nx, gz = gxy / ny, gy = gxy - gz * ny;
    const float r[3] = {(float)(gx - nx / 2) * dx, (float)(gy - ny / 2) * dy, (float)(gz - nz / 2) * dz};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      Df[k] += r[k] * rho;
      Df[3 + k] += r[k] * drho;
    }
    if (++nd == kChunk) {
#pragma unroll
      for (int k = 0; k < 6; k++) {
        D[k] += f2d(Df[k]);
        Df[k] = 0.f;
      }
      nd = 0;
    }
  }
  acc.flush();
#pragma unroll
  for (int k = 0; k < 6; k++) D[k] += f2d(Df[k]);
  const double A = bsum(acc.A, sh), B = bsum(acc.B, sh);
  if (threadIdx.x == 0) {
    npart[((int64_t)o * gridDim.x + blockIdx.x) * 2] = A;
    npart[((int64_t)o * gridDim.x + blockIdx.x) * 2 + 1] = B;
  }
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const double v = bsum(D[k], sh);
    if (threadIdx.x == 0) dpart[((int64_t)o * gridDim.x + blockIdx.x) * 6 + k] = v;
  }
}

// dipoles from the (orbital, block) partials: out[0..2] dip, [3..5] dip', [6..8] d_dip
__global__ void k_mix_dip_final(const double *__restrict__ part, int nparts, double gamma, double dv,
                                double *__restrict__ out) {
  __shared__ double sh[8];
  double s[6];
  for (int k = 0; k < 6; k++) s[k] = block_sum_seq(part + k, nparts, 6, sh);
  if (threadIdx.x != 0) return;
  for (int k = 0; k < 3; k++) {
    const double dip = 2.0 * dv * s[k], ddip = 2.0 * dv * s[3 + k];  // rho = 2 sum |psi|^2
    out[k] = dip;
    out[3 + k] = dip + ddip;
    out[6 + k] = ddip / gamma;
  }
}

// psi' = psi + delta (once at the end of a call)
__global__ void k_mix_p1(const double2 *__restrict__ p0, const double2 *__restrict__ d, double2 *__restrict__ p1,
                         int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) p1[i] = make_double2(p0[i].x + d[i].x, p0[i].y + d[i].y);
}

// ----------------------------------------------------------------- driver --
struct Mix {
  int norb;
  int64_t tot;
  float2 *y0, *yd, *k0, *kd, *ks0, *ksd, *t0, *td, *pf0, *pfd;
  double2 *d;
  double2 *c0, *cd;
  double *r0raw, *h0raw, *drraw, *dhraw, *src0, *srcd, *ddens, *vh0, *dvh;
  float *dvf;
  double *drhoij, *ddij, *fac, *part0, *partd, *mean, *npart0, *npart1, *nfac, *dpart;
};

static int mix_bufs(opaw_ctx *c, int norb, Mix &m) {
  m.norb = norb;
  m.tot = c->nn * (int64_t)norb;
  const size_t cb = sizeof(float2) * (size_t)m.tot;
  float2 **cs[10] = {&m.y0, &m.yd, &m.k0, &m.kd, &m.ks0, &m.ksd, &m.t0, &m.td, &m.pf0, &m.pfd};
  for (int i = 0; i < 10; i++) {
    OPAW_CHECK(ensure(c->mix[i], cb));
    *cs[i] = (float2 *)c->mix[i].p;
  }
  OPAW_CHECK(ensure(c->mix[10], sizeof(double2) * (size_t)m.tot));
  m.d = (double2 *)c->mix[10].p;
  OPAW_CHECK(ensure(c->mix[11], sizeof(double2) * (size_t)c->ns * norb * 2 + 32));
  m.c0 = (double2 *)c->mix[11].p;
  m.cd = m.c0 + (size_t)c->ns * norb;
  OPAW_CHECK(ensure(c->mix[12], sizeof(double) * (size_t)c->nn * 9 + sizeof(float) * (size_t)c->nn + 64));
  double *r = (double *)c->mix[12].p;
  double **rs[9] = {&m.r0raw, &m.h0raw, &m.drraw, &m.dhraw, &m.src0, &m.srcd, &m.ddens, &m.vh0, &m.dvh};
  for (int i = 0; i < 9; i++) *rs[i] = r + (size_t)i * c->nn;
  m.dvf = (float *)(r + (size_t)9 * c->nn);
  const size_t nparts = (size_t)norb * kMixNormBlocks;
  const size_t small = 2 * (size_t)c->nd + 16 + 4 * kRedBlocks + 16 + 4 * nparts + 3 * (size_t)norb + 6 * nparts + 64;
  OPAW_CHECK(ensure(c->mix[13], sizeof(double) * small));
  double *q = (double *)c->mix[13].p;
  m.drhoij = q;
  m.ddij = m.drhoij + c->nd;
  m.fac = m.ddij + c->nd;
  m.part0 = m.fac + 16;
  m.partd = m.part0 + 2 * kRedBlocks;
  m.mean = m.partd + 2 * kRedBlocks;
  m.npart0 = m.mean + 16;
  m.npart1 = m.npart0 + 2 * nparts;
  m.nfac = m.npart1 + 2 * nparts;
  m.dpart = m.nfac + 3 * (size_t)norb;
  return OPAW_OK;
}

#define MIX_LAUNCHED()             \
  do {                             \
    c->launches++;                 \
    OPAW_CUDA(cudaGetLastError()); \
  } while (0)

// rebuild of both sets from y0 and the difference yd: leaves t0 = S^-1/2 y0,
// td = S^-1/2 yd and their projections c0, cd for the following shs
static int mix_rebuild(opaw_ctx *c, Mix &m, const float2 *y0, const float2 *yd) {
  const int norb = m.norb;
  const int nb = grid1(c->nn, 256);
  // unperturbed set (ncpaw_make_hamiltonian.f90:119-129)
  OPAW_CHECK(sn_apply<float>(c, -0.5, y0, m.t0, norb));
  OPAW_CHECK(gather<float>(c, 0, m.t0, norb, m.c0));
  OPAW_CHECK(rhoij_of(c, m.c0, norb, c->d_rhoij[0]));
  OPAW_CHECK(density_raw<float>(c, m.t0, norb, m.r0raw));
  OPAW_CHECK(nhat_raw_of(c, c->d_rhoij[0], m.h0raw));
  // differences
  OPAW_CHECK(sn_apply<float>(c, -0.5, yd, m.td, norb));
  OPAW_CHECK(gather<float>(c, 0, m.td, norb, m.cd));
  if (c->nd > 0) {
    k_mix_drhoij<<<grid1(c->nd, 128), 128, 0, c->stream>>>(m.c0, m.cd, norb, c->ns, c->nd, c->d_dslot_atom,
                                                           c->d_soff, c->d_doff, c->d_ms, c->d_rhoij[0], m.drhoij,
                                                           c->d_rhoij[1]);
    MIX_LAUNCHED();
  }
  k_mix_drho<<<nb, 256, 0, c->stream>>>(m.t0, m.td, norb, c->nn, m.drraw);
  MIX_LAUNCHED();
  OPAW_CHECK(nhat_raw_of(c, m.drhoij, m.dhraw));  // n^ is linear in rho_ij
  // charge renormalisation of both sets
  OPAW_CHECK(sums2(c, m.h0raw, m.r0raw, m.part0));
  OPAW_CHECK(sums2(c, m.dhraw, m.drraw, m.partd));
  k_mix_factors<<<1, 256, 0, c->stream>>>(m.part0, m.partd, kRedBlocks, c->dv, c->rnel, m.fac);
  MIX_LAUNCHED();
  k_mix_renorm<<<nb, 256, 0, c->stream>>>(m.r0raw, m.h0raw, m.drraw, m.dhraw, m.fac, c->d_dens[0], c->d_nhat[0],
                                          c->d_dens[1], c->d_nhat[1], m.src0, m.srcd, m.ddens, c->nn);
  MIX_LAUNCHED();
  // Hartree of n0 + n^0 and of the difference: two complex64 transforms, so
  // the difference keeps its own relative precision (packing it with the
  // ~1e3 times larger n0 into one transform would round it relative to n0)
  OPAW_CHECK(hartree_t<float>(c, m.src0, nullptr, m.vh0, nullptr));
  OPAW_CHECK(hartree_t<float>(c, m.srcd, nullptr, m.dvh, nullptr));
  const double *mean = nullptr;
  if (c->periodic) {  // tddft_pot.f90:42-45
    OPAW_CHECK(sums2(c, m.vh0, nullptr, m.part0));
    OPAW_CHECK(sums2(c, m.dvh, nullptr, m.partd));
    k_mix_mean<<<1, 256, 0, c->stream>>>(m.part0, m.partd, kRedBlocks, c->nn, m.mean);
    MIX_LAUNCHED();
    mean = m.mean;
  }
  k_mix_pot<<<nb, 256, 0, c->stream>>>(c->d_dens[0], m.ddens, c->d_ncoret, c->d_vloc, m.vh0, m.dvh, mean,
                                       c->d_vks[0], c->d_vks[1], c->d_vks_f[0], c->d_vks_f[1], m.dvf, c->d_vxc[0],
                                       c->d_vxc[1], c->d_vh[1], c->nn);
  MIX_LAUNCHED();
  OPAW_CUDA(cudaMemcpyAsync(c->d_vh[0], m.vh0, sizeof(double) * c->nn, cudaMemcpyDeviceToDevice, c->stream));
  // D_ij of both sets (FP64) and their difference
  OPAW_CHECK(dij_of(c, c->d_rhoij[0], c->d_vks[0], c->d_dij[0]));
  OPAW_CHECK(dij_of(c, c->d_rhoij[1], c->d_vks[1], c->d_dij[1]));
  if (c->nd > 0) {
    k_mix_ddij<<<grid1(c->nd, 128), 128, 0, c->stream>>>(c->d_dij[0], c->d_dij[1], m.ddij, c->nd);
    MIX_LAUNCHED();
  }
  return OPAW_OK;
}

// S^-1/2 H S^-1/2 of both sets from t0, td and their projections
static int mix_shs(opaw_ctx *c, Mix &m) {
  const int norb = m.norb;
  OPAW_CHECK(h_apply_ex<float>(c, c->d_vks_f[0], c->d_dij[0], m.t0, m.k0, norb, m.c0, nullptr, nullptr, nullptr,
                               nullptr));
  OPAW_CHECK(sn_apply<float>(c, -0.5, m.k0, m.k0, norb));
  OPAW_CHECK(h_apply_ex<float>(c, c->d_vks_f[1], c->d_dij[1], m.td, m.kd, norb, m.cd, m.t0, m.dvf, m.c0, m.ddij));
  OPAW_CHECK(sn_apply<float>(c, -0.5, m.kd, m.kd, norb));
  return OPAW_OK;
}

int mixed_steps(opaw_ctx *c, int nsteps, double dt, double gamma, double *dd_dev) {
  const int norb = c->norb[0];
  Mix m;
  OPAW_CHECK(mix_bufs(c, norb, m));
  const int nb = grid1(m.tot, 256);
  double2 *p0 = c->d_psi[0], *p1 = c->d_psi[1];
  const dim3 gn(kMixNormBlocks, norb);
  // delta = psi' - psi, complex64 copies, norms of the step start (rk4.f90:16)
  k_mix_start<<<gn, 256, 0, c->stream>>>(p0, p1, m.d, m.pf0, m.pfd, c->nn, m.npart0);
  MIX_LAUNCHED();
  const float wts[4] = {1.f, 2.f, 2.f, 1.f};
  const double dts[4] = {dt / 2.0, dt / 2.0, dt, dt};
  for (int it = 0; it < nsteps; it++) {
    OPAW_CHECK(mix_rebuild(c, m, m.pf0, m.pfd));  // ncpaw_make_hamiltonian_tddft (tddft.f90:75)
    for (int st = 0; st < 4; st++) {
      OPAW_CHECK(mix_shs(c, m));
      k_mix_stage<<<nb, 256, 0, c->stream>>>(m.k0, m.kd, m.pf0, m.pfd, m.ks0, m.ksd, m.y0, m.yd, m.tot, wts[st],
                                             st == 0, (float)dts[st], st < 3);
      MIX_LAUNCHED();
      if (st < 3) OPAW_CHECK(mix_rebuild(c, m, m.y0, m.yd));  // rk4.f90:53-55
    }
    k_mix_final<<<gn, 256, 0, c->stream>>>(p0, m.d, m.ks0, m.ksd, c->nn, dt / 6.0, m.npart1);
    MIX_LAUNCHED();
    k_mix_nfac<<<grid1(norb, 128), 128, 0, c->stream>>>(m.npart0, m.npart1, kMixNormBlocks, norb, m.nfac);
    MIX_LAUNCHED();
    k_mix_rescale<<<gn, 256, 0, c->stream>>>(p0, m.d, m.pf0, m.pfd, m.nfac, c->nn, c->nx, c->ny, c->nz, (float)c->dx,
                                             (float)c->dy, (float)c->dz, m.npart0, m.dpart);
    MIX_LAUNCHED();
    k_mix_dip_final<<<1, 256, 0, c->stream>>>(m.dpart, norb * kMixNormBlocks, gamma, c->dv, dd_dev + 9 * (size_t)it);
    MIX_LAUNCHED();
  }
  k_mix_p1<<<nb, 256, 0, c->stream>>>(p0, m.d, p1, m.tot);  // psi' = psi + delta
  MIX_LAUNCHED();
  return OPAW_OK;
}

}  // namespace opaw

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
  const int t = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);  // warp per entry
  const int lane = threadIdx.x & 31;
  if (t >= nd) return;
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
__global__ void k_mix_pot(const double *__restrict__ dens0, const double *__restrict__ ddens,
                          const double *__restrict__ core, const double *__restrict__ vloc,
                          const double *__restrict__ vh0, const double *__restrict__ dvh, const double *__restrict__ mean,
                          double *__restrict__ vks0, double *__restrict__ vks1, float *__restrict__ vks0f,
                          float *__restrict__ vks1f, float *__restrict__ dvf, double *__restrict__ vxc0o,
                          double *__restrict__ vxc1o, double *__restrict__ vh1o, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x0f, dxf;
  vxc_pair_f(d2f(dens0[i] + core[i]), d2f(ddens[i]), x0f, dxf);
  const double x0 = f2d(x0f), dxc = f2d(dxf);
  double h0 = vh0[i], dh = dvh[i];
  if (mean) {
    h0 -= mean[0];
    dh -= mean[1];
  }
  const double v0 = h0 + x0 + vloc[i];
  const double dv = dh + dxc;
  const double v1 = v0 + dv;
  vks0[i] = v0;
  vks1[i] = v1;
  vks0f[i] = (float)v0;
  vks1f[i] = (float)v1;
  dvf[i] = (float)dv;
  vxc0o[i] = x0;
  vxc1o[i] = x0 + dxc;
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

// thread (slot t, orbital o, set X); grid (ceil(ns/128), norb, 2)
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
// <p|psi> = f0 <p|x>, <p|delta> = df <p|x> + f1 <p|y> (both tables)
__global__ void k_mc_scale_a(double2 *__restrict__ A, const double *__restrict__ fac, int norb, int ns) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ns) return;
  const int o = blockIdx.y, tab = blockIdx.z;
  const int64_t sv = (int64_t)norb * ns;
  const double f0 = fac[3 * o], f1 = fac[3 * o + 1], df = fac[3 * o + 2];
  double2 *a0 = A + (int64_t)tab * sv + (int64_t)o * ns + t;  // set 0, table tab
  double2 *ad = A + (int64_t)(2 + tab) * sv + (int64_t)o * ns + t;
  const double2 x = *a0, y = *ad;
  *ad = make_double2(df * x.x + f1 * y.x, df * x.y + f1 * y.y);
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
struct FusedArgs {
  const float2 *u0, *ud, *pf0, *pfd;  // pf: the hi arrays x, y of the state, restored on read
  const float *facf;                  // per orbital f0, f1, df: psi = f0 x, delta = df x + f1 y
  float2 *ks0, *ksd, *t0, *td;
  double *r0raw, *drraw;
  int norb;
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
  __device__ __forceinline__ void store(const FusedArgs &f, int64_t g) {
    flush();
    f.r0raw[g] = total0();
    f.drraw[g] = totald();
  }
};

// the restored complex64 psi and delta of orbital o from the hi arrays
__device__ __forceinline__ void restore_pf(const FusedArgs &f, int o, float2 x, float2 y, float2 &q0, float2 &qd) {
  const float f0 = f.facf[3 * o], f1 = f.facf[3 * o + 1], df = f.facf[3 * o + 2];
  q0 = make_float2(f0 * x.x, f0 * x.y);
  qd = make_float2(df * x.x + f1 * y.x, df * x.y + f1 * y.y);
}

// one orbital of both sets at one point, given the loaded values and the box terms
__device__ __forceinline__ void fused_one(const FusedArgs &f, int64_t idx, float2 a0, float2 ad, float2 q0, float2 qd,
                                          float2 s0, float2 sd, const float2 *B, const float2 *Gt, DensAcc &acc) {
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
    f.ks0[idx] = n0;
    f.ksd[idx] = nd;
    if (!f.write_t) return;
    tv0 = make_float2(q0.x + f.dts * k0.x + Gt[0].x, q0.y + f.dts * k0.y + Gt[0].y);
    tvd = make_float2(qd.x + f.dts * kd.x + Gt[1].x, qd.y + f.dts * kd.y + Gt[1].y);
  } else {
    tv0 = make_float2(q0.x + Gt[0].x, q0.y + Gt[0].y);
    tvd = make_float2(qd.x + Gt[1].x, qd.y + Gt[1].y);
  }
  f.t0[idx] = tv0;
  f.td[idx] = tvd;
  acc.add(tv0, tvd);
}

// every grid point; at the union points the box terms come from BG
// ([kind B, G][set][orbital][union point], k_mix_boxcoef)
__global__ void __launch_bounds__(256)
    k_mix_dense(FusedArgs f, const int *__restrict__ uidx, const float2 *__restrict__ BG, int nunion) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= f.nn) return;
  const int u = uidx[g];
  const int64_t su = (int64_t)f.norb * nunion;  // between the four (kind, set) blocks of BG
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
          ad[j] = f.ud[idx];
          if (!f.first) {
            s0[j] = f.ks0[idx];
            sd[j] = f.ksd[idx];
          }
          if (u >= 0) {
            B[j][0] = BG[bi];
            B[j][1] = BG[su + bi];
          }
        }
        if (f.write_t) {
          q0[j] = f.pf0[idx];
          qd[j] = f.pfd[idx];
          if (u >= 0) {
            G[j][0] = BG[2 * su + bi];
            G[j][1] = BG[3 * su + bi];
          }
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 2; j++)
      if (j < nj && f.write_t) restore_pf(f, o + j, q0[j], qd[j], q0[j], qd[j]);
#pragma unroll
    for (int j = 0; j < 2; j++)
      if (j < nj)
        fused_one(f, (int64_t)(o + j) * f.nn + g, a0[j], ad[j], q0[j], qd[j], s0[j], sd[j], B[j], G[j], acc);
  }
  if (f.write_t) acc.store(f, g);
}

// The box terms of the fused pass at every union point u, orbital o and
// set X (thread per (u, o)):
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
  const int o = blockIdx.y;
  const int64_t kstride = (int64_t)norb * ns;
  float2 B[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
  float2 G[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
  for (int e = ustart[u]; e < ustart[u + 1]; e++) {
    const int a = uatom[e], b = ubox[e];
    const int nbox = nrough[3 * a] * nrough[3 * a + 1] * nrough[3 * a + 2];
    const int m = ms[a];
    const int64_t s0 = (int64_t)o * ns + soff[a];
    for (int i = 0; i < m; i++) {
      const float p = P0[poff[a] + (int64_t)i * nbox + b], q = P1[poff[a] + (int64_t)i * nbox + b];
#pragma unroll
      for (int X = 0; X < 2; X++) {
        if (stage) {
          const float4 c = cab[X * kstride + s0 + i];
          B[X].x += p * c.x + q * c.z;
          B[X].y += p * c.y + q * c.w;
        }
        if (write_t) {
          const float2 c = cg[X * kstride + s0 + i];
          G[X].x += q * c.x;
          G[X].y += q * c.y;
        }
      }
    }
  }
  const int64_t su = (int64_t)norb * nunion, bi = (int64_t)o * nunion + u;
  if (stage) {
    BG[bi] = B[0];
    BG[su + bi] = B[1];
  }
  if (write_t) {
    BG[2 * su + bi] = G[0];
    BG[3 * su + bi] = G[1];
  }
}

// The same terms by tiles of kUTile union points and OG orbitals.  The CTA
// first copies the coefficients of its tile's atoms (utile) for its orbitals
// into shared memory, three float4 per (atom, orbital, projector):
// -i cD and -i c2 of set 0, of set 1, then c3 of both sets.  A thread then
// takes one union point: per entry (uent: table offset, tile-local atom,
// projector count, box size) it loads the projector values once and reads
// the coefficients as shared-memory broadcasts.  The sums run in the order
// of the generic kernel above.  MODE bit 0: the B terms (stage), bit 1: the
// G terms (write_t).
template <int MODE, int MS, int OG>
__global__ void __launch_bounds__(kUTile, 6)
    k_mix_boxcoef_t(int nunion, int norb, int ns, int amax, const int *__restrict__ ustart,
                    const int4 *__restrict__ uent, const int2 *__restrict__ utile, const int *__restrict__ utile_na,
                    const float *__restrict__ P0, const float *__restrict__ P1, const float4 *__restrict__ cab,
                    const float2 *__restrict__ cg, float2 *__restrict__ BG) {
  constexpr bool kB = (MODE & 1) != 0, kG = (MODE & 2) != 0;
  extern __shared__ float4 cs[];  // [tile atom][OG][MS][3]
  const int tile = blockIdx.x;
  const int o0 = blockIdx.y * OG;
  const int64_t kstride = (int64_t)norb * ns;
  const int na = utile_na[tile];
  for (int t = threadIdx.x; t < na * OG * MS; t += kUTile) {
    const int la = t / (OG * MS), r = t - la * (OG * MS), j = r / MS, i = r - j * MS;
    const int2 at = utile[(int64_t)tile * amax + la];
    float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0, g = a0;
    if (i < at.y) {
      const int64_t k = (int64_t)min(o0 + j, norb - 1) * ns + at.x + i;
      if (kB) {
        a0 = cab[k];
        a1 = cab[kstride + k];
      }
      if (kG) {
        const float2 g0 = cg[k], g1 = cg[kstride + k];
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
        BG[bi] = B[j][0];
        BG[su + bi] = B[j][1];
      }
      if (kG) {
        BG[2 * su + bi] = G[j][0];
        BG[3 * su + bi] = G[j][1];
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

// start of a call: x = psi, y = psi' - psi in float-float, norm partials (the
// targets of every norm restore of the call, rk4.f90:16)
__global__ void k_mix_start(const double2 *__restrict__ p0, const double2 *__restrict__ p1,
                            float2 *__restrict__ xh, float2 *__restrict__ xl, float2 *__restrict__ yh,
                            float2 *__restrict__ yl, int64_t nn, double *__restrict__ part) {
  __shared__ double sh[8];
  const int o = blockIdx.y;
  NormAcc acc;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nn; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)o * nn + g;
    const double2 x = p0[i], y1 = p1[i];
    const FF ax = ff_of(x.x), ay = ff_of(x.y), bx = ff_of(y1.x - x.x), by = ff_of(y1.y - x.y);
    xh[i] = make_float2(ax.h, ay.h);
    xl[i] = make_float2(ax.l, ay.l);
    yh[i] = make_float2(bx.h, by.h);
    yl[i] = make_float2(bx.l, by.l);
    acc.add(make_float2(ax.h, ay.h), make_float2(bx.h, by.h));
  }
  acc.flush();
  const double A = bsum(acc.A, sh), B = bsum(acc.B, sh);
  if (threadIdx.x == 0) {
    part[((int64_t)o * gridDim.x + blockIdx.x) * 2] = A;
    part[((int64_t)o * gridDim.x + blockIdx.x) * 2 + 1] = B;
  }
}

// pending factors of a fresh call: no restore yet
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
__global__ void __launch_bounds__(256, 3) k_mix_final(float2 *__restrict__ xh, float2 *__restrict__ xl, float2 *__restrict__ yh,
                            float2 *__restrict__ yl, const float2 *__restrict__ ks0, const float2 *__restrict__ ksd,
                            const double *__restrict__ fac, double h6, int64_t nn, int nx, int ny, int nz, float dx,
                            float dy, float dz, double *__restrict__ npart, double *__restrict__ dpart,
                            const float2 *__restrict__ u0, const float2 *__restrict__ ud, const int *__restrict__ uidx,
                            const float2 *__restrict__ BG, int nunion) {
  __shared__ double sh[8];
  const int o = blockIdx.y;
  const FF f0 = ff_of(fac[3 * o]), f1 = ff_of(fac[3 * o + 1]), df = ff_of(fac[3 * o + 2]), hh = ff_of(h6);
  NormAcc acc;
  double D[6] = {0, 0, 0, 0, 0, 0};
  float Df[6] = {0, 0, 0, 0, 0, 0};
  int nd = 0;
  // grid coordinates carried along the grid-stride loop (no divisions per point)
  const int64_t g0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  int gx = (int)(g0 % nx), gy = (int)((g0 / nx) % ny), gz = (int)(g0 / ((int64_t)nx * ny));
  const int sx = (int)(stride % nx), sy = (int)((stride / nx) % ny), sz = (int)(stride / ((int64_t)nx * ny));
  // the six operands of the next point are loaded while this one is combined
  const int64_t ob = (int64_t)o * nn;
  float2 na = make_float2(0.f, 0.f), nal = na, nb = na, nbl = na, ns0 = na, nsd = na, np0 = na, npd = na;
  int nu = -1;
  if (g0 < nn) {
    na = xh[ob + g0], nal = xl[ob + g0], nb = yh[ob + g0], nbl = yl[ob + g0], ns0 = ks0[ob + g0], nsd = ksd[ob + g0];
    if (u0) np0 = u0[ob + g0], npd = ud[ob + g0], nu = uidx[g0];
  }
  const int64_t bo = (int64_t)o * nunion, su = (int64_t)gridDim.y * nunion;
  for (int64_t g = g0; g < nn; g += stride) {
    const int64_t i = ob + g;
    const float2 a = na, al = nal, b = nb, bl = nbl;
    float2 s0 = ns0, sd = nsd;
    const float2 p0 = np0, pd = npd;
    const int u = nu;
    float2 B0 = make_float2(0.f, 0.f), B1 = B0;
    if (u >= 0) {
      B0 = BG[bo + u];
      B1 = BG[su + bo + u];
    }
    if (g + stride < nn) {
      const int64_t k = i + stride;
      na = xh[k], nal = xl[k], nb = yh[k], nbl = yl[k], ns0 = ks0[k], nsd = ksd[k];
      if (u0) np0 = u0[k], npd = ud[k], nu = uidx[g + stride];
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
    xh[i] = af;
    xl[i] = make_float2(nxx.l, nxy.l);
    yh[i] = bf;
    yl[i] = make_float2(nyx.l, nyy.l);
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

// dipoles from the per-orbital terms: out[0..2] dip, [3..5] dip', [6..8] d_dip
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

// end of a call: the restored psi = f0 x and psi' = f1 (x + y) back to FP64
__global__ void k_mix_end(double2 *__restrict__ p0, double2 *__restrict__ p1, const float2 *__restrict__ xh,
                          const float2 *__restrict__ xl, const float2 *__restrict__ yh, const float2 *__restrict__ yl,
                          const double *__restrict__ fac, int64_t nn) {
  const int o = blockIdx.y;
  const FF f0 = ff_of(fac[3 * o]), f1 = ff_of(fac[3 * o + 1]);
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nn; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)o * nn + g;
    const float2 a = xh[i], al = xl[i], b = yh[i], bl = yl[i];
    const FF Xx{a.x, al.x}, Xy{a.y, al.y}, Yx{b.x, bl.x}, Yy{b.y, bl.y};
    p0[i] = make_double2(ff_val(ff_mul(f0, Xx)), ff_val(ff_mul(f0, Xy)));
    p1[i] = make_double2(ff_val(ff_mul(f1, ff_add(Xx, Yx))), ff_val(ff_mul(f1, ff_add(Xy, Yy))));
  }
}

// ----------------------------------------------------------------- driver --
struct Mix {
  int norb;
  int64_t tot;
  float2 *u0, *ud, *ks0, *ksd, *t0, *td;
  float2 *pf0, *pfd;   // the hi arrays of the state x (psi), y (delta)
  float2 *xl, *yl;     // their lo arrays
  double2 *c0, *cd;    // <p~|t> of both sets (current buffer of the pair)
  double2 *cnext;      // the other buffer of the pair
  double2 *G, *A;      // [set][table][orbital][slot]: gathers of u' and of pf
  double2 *cD, *q1, *c2, *c3, *pre;  // [set][orbital][slot]
  float2 *bg;          // [kind B, G][set][orbital][union point]: box terms of the fused pass
  float4 *cab;         // [set][orbital][slot]: (-i cD, -i c2) in FP32
  float2 *cg;          // [set][orbital][slot]: c3 in FP32
  double *r0raw, *h0raw, *drraw, *dhraw, *src0, *srcd, *ddens, *vh0, *dvh;
  float *dvf;
  double *drhoij, *ddij, *fac, *part0, *partd, *mean, *npart0, *npart1, *nfac, *dpart, *dorb;
  float *facf;         // FP32 copy of nfac
};

static int mix_bufs(opaw_ctx *c, int norb, Mix &m) {
  m.norb = norb;
  m.tot = c->nn * (int64_t)norb;
  const size_t cb = sizeof(float2) * (size_t)m.tot;
  float2 **cs[8] = {&m.u0, &m.ud, &m.ks0, &m.ksd, &m.t0, &m.td, &m.pf0, &m.pfd};
  for (int i = 0; i < 8; i++) {
    OPAW_CHECK(ensure(c->mix[i], cb));
    *cs[i] = (float2 *)c->mix[i].p;
  }
  OPAW_CHECK(ensure(c->mix[10], 2 * sizeof(float2) * (size_t)m.tot));
  m.xl = (float2 *)c->mix[10].p;
  m.yl = m.xl + m.tot;
  const size_t sv = (size_t)c->ns * norb;  // one slot vector per orbital
  // c0/cd pair x2, G (4 sv), A (4 sv), cD, q1, c2, c3, pre (2 sv each)
  OPAW_CHECK(ensure(c->mix[11], sizeof(double2) * (sv * (4 + 4 + 4 + 10)) + 64));
  double2 *q = (double2 *)c->mix[11].p;
  m.c0 = q;
  m.cd = q + sv;
  m.cnext = q + 2 * sv;
  m.G = q + 4 * sv;
  m.A = q + 8 * sv;
  m.cD = q + 12 * sv;
  m.q1 = q + 14 * sv;
  m.c2 = q + 16 * sv;
  m.c3 = q + 18 * sv;
  m.pre = q + 20 * sv;
  OPAW_CHECK(ensure(c->mix[8], sizeof(float2) * 4 * (size_t)norb * c->nunion + 64));
  m.bg = (float2 *)c->mix[8].p;
  OPAW_CHECK(ensure(c->mix[14], sizeof(float4) * 2 * sv + 64));
  m.cab = (float4 *)c->mix[14].p;
  OPAW_CHECK(ensure(c->mix[15], sizeof(float2) * 2 * sv + 64));
  m.cg = (float2 *)c->mix[15].p;
  OPAW_CHECK(ensure(c->mix[12], sizeof(double) * (size_t)c->nn * 9 + sizeof(float) * (size_t)c->nn + 64));
  double *r = (double *)c->mix[12].p;
  double **rs[9] = {&m.r0raw, &m.h0raw, &m.drraw, &m.dhraw, &m.src0, &m.srcd, &m.ddens, &m.vh0, &m.dvh};
  for (int i = 0; i < 9; i++) *rs[i] = r + (size_t)i * c->nn;
  m.dvf = (float *)(r + (size_t)9 * c->nn);
  const size_t nparts = (size_t)norb * kMixNormBlocks;
  const size_t small = 2 * (size_t)c->nd + 16 + 4 * kRedBlocks + 16 + 4 * nparts + 3 * (size_t)norb + 6 * nparts +
                       6 * (size_t)norb + 2 * (size_t)norb + 64;
  OPAW_CHECK(ensure(c->mix[13], sizeof(double) * small));
  double *qq = (double *)c->mix[13].p;
  m.drhoij = qq;
  m.ddij = m.drhoij + c->nd;
  m.fac = m.ddij + c->nd;
  m.part0 = m.fac + 16;
  m.partd = m.part0 + 2 * kRedBlocks;
  m.mean = m.partd + 2 * kRedBlocks;
  m.npart0 = m.mean + 16;
  m.npart1 = m.npart0 + 2 * nparts;
  m.nfac = m.npart1 + 2 * nparts;
  m.dpart = m.nfac + 3 * (size_t)norb;
  m.dorb = m.dpart + 6 * nparts;
  m.facf = (float *)(m.dorb + 6 * (size_t)norb);
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
  f.nn = c->nn;
  f.w = w;
  f.dts = dts;
  f.stage = stage;
  f.first = first;
  f.write_t = write_t;
  constexpr int OG = 4, MS = 8;
  const size_t bsmem = sizeof(float4) * 3 * OG * MS * (size_t)c->uamax;
  if (c->nunion > 0 && c->ns > 0 && c->d_uent && c->msmax <= MS && bsmem <= 48 * 1024 && (stage || write_t)) {
    const dim3 nb((c->nunion + kUTile - 1) / kUTile, (m.norb + OG - 1) / OG);
    const int mode = (stage ? 1 : 0) | (write_t ? 2 : 0);
    auto kern = mode == 1 ? k_mix_boxcoef_t<1, MS, OG> : mode == 2 ? k_mix_boxcoef_t<2, MS, OG> : k_mix_boxcoef_t<3, MS, OG>;
    kern<<<nb, kUTile, bsmem, c->stream>>>(c->nunion, m.norb, c->ns, c->uamax, c->d_ustart, c->d_uent, c->d_utile,
                                          c->d_utile_na, c->d_p3d_f, c->d_p3d1_f, m.cab, m.cg, m.bg);
    MIX_LAUNCHED();
  } else if (c->nunion > 0 && c->ns > 0) {
    const dim3 nb(grid1(c->nunion, 128), m.norb);
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
  k_mix_dense<<<grid1(c->nn, 256), 256, 0, c->stream>>>(f, c->d_uidx, m.bg, c->ns > 0 ? c->nunion : 0);
  MIX_LAUNCHED();
  if (ev1) {
    OPAW_CUDA(cudaEventRecord(ev1, c->stream));
    // algorithmic bytes: the union index of every point; per point and
    // orbital of both sets the arrays this mode reads or writes once
    // (complex64), the box terms at the union points, the two FP64 densities
    double per = 0.0, perb = 0.0;  // bytes per (point, orbital), both sets
    if (stage) per += 16.0 + (first ? 0.0 : 16.0) + 16.0;  // u', ks read, ks write
    if (write_t) per += 32.0;                              // pf read, t write
    if (stage) perb += 16.0;
    if (write_t) perb += 16.0;
    c->kbytes += 4.0 * (double)c->nn + (double)c->nn * (per * m.norb + (write_t ? 16.0 : 0.0)) +
                 (double)c->nunion * perb * m.norb;
  }
  return OPAW_OK;
}

// t = S^-1/2 pf of both sets at the start of a step, their <p~|t> and raw densities
static int mix_start_t(opaw_ctx *c, Mix &m) {
  const int norb = m.norb;
  const size_t sv = (size_t)c->ns * norb;
  if (c->ns > 0) {
    OPAW_CHECK(gather2<float>(c, m.pf0, norb, m.A, m.A + sv));
    OPAW_CHECK(gather2<float>(c, m.pfd, norb, m.A + 2 * sv, m.A + 3 * sv));
    const Ovl v = ovl_of(c);
    const dim3 g(grid1(c->ns, 128), norb, 2);
    k_mc_scale_a<<<g, 128, 0, c->stream>>>(m.A, m.nfac, norb, c->ns);
    MIX_LAUNCHED();
    k_mc_start<<<g, 128, 0, c->stream>>>(v, m.A, c->d_sigma[1], m.c3, m.pre, norb, c->ns);
    MIX_LAUNCHED();
    k_mc_t<<<g, 128, 0, c->stream>>>(v, m.pre, m.c3, m.cnext, m.cg, norb, c->ns);
    MIX_LAUNCHED();
    mix_swap(m, sv);
  }
  return mix_fused(c, m, 0, 0, 1, 0.f, 0.f);
}

// one RK4 stage of both sets from t, <p~|t> and the rebuilt potentials: the
// grid part of H, the two gathers, the FP64 algebra and the fused pass
static int mix_stage(opaw_ctx *c, Mix &m, int st, float w, double dts) {
  const int norb = m.norb;
  const size_t sv = (size_t)c->ns * norb;
  const int write_t = st < 3;
  int both;
  OPAW_CHECK(h_fft2<float>(c, c->d_vks_f[0], c->d_vks_f[1], m.t0, m.td, m.u0, m.ud, m.dvf, norb, &both));
  if (!both) {
    OPAW_CHECK(h_fft<float>(c, c->d_vks_f[0], m.t0, m.u0, norb, nullptr, nullptr));
    OPAW_CHECK(h_fft<float>(c, c->d_vks_f[1], m.td, m.ud, norb, m.t0, m.dvf));
  }
  if (c->ns > 0) {
    OPAW_CHECK(gather2<float>(c, m.u0, norb, m.G, m.G + sv));
    OPAW_CHECK(gather2<float>(c, m.ud, norb, m.G + 2 * sv, m.G + 3 * sv));
    // cD = D <p~|t> (unperturbed), D' <p~|td> + (D' - D) <p~|t0> (difference)
    const dim3 gc(grid1(c->ns, 128), norb);
    k_coef_dij<<<gc, 128, 0, c->stream>>>(m.c0, m.cD, norb, c->ns, c->d_slot_atom, c->d_soff, c->d_doff, c->d_ms,
                                          c->d_dij[0]);
    MIX_LAUNCHED();
    k_coef_dij2<<<gc, 128, 0, c->stream>>>(m.cd, m.c0, m.cD + sv, norb, c->ns, c->d_slot_atom, c->d_soff, c->d_doff,
                                           c->d_ms, c->d_dij[1], m.ddij);
    MIX_LAUNCHED();
    const Ovl v = ovl_of(c);
    const dim3 g(grid1(c->ns, 128), norb, 2);
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
// and the raw densities of both sets: rho_ij, n^, renormalisation, Hartree,
// v_ks, D_ij of both sets and their differences
static int mix_potentials(opaw_ctx *c, Mix &m) {
  const int norb = m.norb;
  const int nb = grid1(c->nn, 256);
  OPAW_CHECK(rhoij_of(c, m.c0, norb, c->d_rhoij[0]));
  OPAW_CHECK(nhat_raw_of(c, c->d_rhoij[0], m.h0raw));
  if (c->nd > 0) {
    k_mix_drhoij<<<grid1((int64_t)c->nd * 32, 256), 256, 0, c->stream>>>(m.c0, m.cd, norb, c->ns, c->nd, c->d_dslot_atom,
                                                           c->d_soff, c->d_doff, c->d_ms, c->d_rhoij[0], m.drhoij,
                                                           c->d_rhoij[1]);
    MIX_LAUNCHED();
  }
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
  OPAW_CHECK(hartree_pair_t<float>(c, m.src0, m.srcd, m.vh0, m.dvh));
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

int mixed_steps(opaw_ctx *c, int nsteps, double dt, double gamma, double *dd_dev) {
  const int norb = c->norb[0];
  Mix m;
  OPAW_CHECK(mix_bufs(c, norb, m));
  double2 *p0 = c->d_psi[0], *p1 = c->d_psi[1];
  const dim3 gn(kMixNormBlocks, norb);
  // x = psi, y = psi' - psi in float-float, the norms to restore (rk4.f90:16)
  k_mix_start<<<gn, 256, 0, c->stream>>>(p0, p1, m.pf0, m.xl, m.pfd, m.yl, c->nn, m.npart0);
  MIX_LAUNCHED();
  k_mix_fac_init<<<grid1(norb, 128), 128, 0, c->stream>>>(m.nfac, m.facf, norb);
  MIX_LAUNCHED();
  const float wts[4] = {1.f, 2.f, 2.f, 1.f};
  const double dts[4] = {dt / 2.0, dt / 2.0, dt, dt};
  for (int it = 0; it < nsteps; it++) {
    // ncpaw_make_hamiltonian_tddft (tddft.f90:75)
    OPAW_CHECK(mix_start_t(c, m));
    OPAW_CHECK(mix_potentials(c, m));
    for (int st = 0; st < 4; st++) {
      OPAW_CHECK(mix_stage(c, m, st, wts[st], dts[st]));
      if (st < 3) OPAW_CHECK(mix_potentials(c, m));  // rk4.f90:53-55
    }
    // the last stage's grid part (k4 and the complete sum k) and the final combination
    k_mix_final<<<gn, 256, 0, c->stream>>>(m.pf0, m.xl, m.pfd, m.yl, m.ks0, m.ksd, m.nfac, dt / 6.0, c->nn, c->nx,
                                           c->ny, c->nz, (float)c->dx, (float)c->dy, (float)c->dz, m.npart1, m.dpart,
                                           m.u0, m.ud, c->d_uidx, m.bg, c->ns > 0 ? c->nunion : 0);
    MIX_LAUNCHED();
    k_mix_nfac<<<grid1(norb, 128), 128, 0, c->stream>>>(m.npart0, m.npart1, kMixNormBlocks, norb, m.nfac, m.facf);
    MIX_LAUNCHED();
    k_mix_dip_orb<<<grid1(norb, 128), 128, 0, c->stream>>>(m.dpart, m.nfac, kMixNormBlocks, norb, m.dorb);
    MIX_LAUNCHED();
    k_mix_dip_final<<<1, 256, 0, c->stream>>>(m.dorb, norb, gamma, c->dv, dd_dev + 9 * (size_t)it);
    MIX_LAUNCHED();
  }
  k_mix_end<<<gn, 256, 0, c->stream>>>(p0, p1, m.pf0, m.xl, m.pfd, m.yl, m.nfac, c->nn);
  MIX_LAUNCHED();
  return OPAW_OK;
}

}  // namespace opaw

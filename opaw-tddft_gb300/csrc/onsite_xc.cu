// onsite_xc.cu — the on-site exchange-correlation term of D_ij (part of A16).
//
// The reference gets D_ij from libpaw (get_dij.f90:17-29: pawdenpot, then
// pawdij).  With the libpaw_mod.f90 settings (LDA ixc = 7, nspden = 1,
// pawxcdev = xcdev = 1, usexcnhat = 0) the exchange-correlation part is
//
//   D_xc_ij = sum_L G^L_ij int_0^rpaw [ V_L(r) u_i u_j - V~_L(r) u~_i u~_j ] dr
//
// (4_m_pawdij.F90 pawdijxcm) with the one-centre densities of rho_ij in
// moments of the real spherical harmonics,
//
//   n_L(r) = sum_ij rho_ij u_i(r) u_j(r) / r^2 G^L_ij  (+ sqrt(4 pi) n_c(r) for L = 0)
//
// and the potential moments of the first-order development around the
// spherical density n_s = n_0 / sqrt(4 pi) (2_m_pawxc.F90 pawxcm):
//
//   V_0 = sqrt(4 pi) v(n_s) + (1/2) v''(n_s) sum_{L>0} n_L^2 / sqrt(4 pi),
//   V_L = v'(n_s) n_L   (L > 0),
//
// v the LDA potential (Slater + PW92), v' and v'' pawxcm's central finite
// differences with the relative step 1e-4 (evaluated from the potential's
// power series around n_s, oxc_vxc_series); the pseudo part V~ is the same
// with u~ and the pseudo core (the compensation charge is not in the
// XC density, usexcnhat = 0).  G^L_ij = int Y_L Y_i Y_j dOmega, real Y_lm in
// the ylm.f90 order.  Projectors with l <= 1 (s and p partial waves, those of
// the reference's datasets) are supported: L <= 2, 9 moments.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace opaw {

constexpr int kOxcL = 9;             // moments L = (l, m), l <= 2
constexpr double kOxcDelta = 1e-4;   // relative density step of the derivatives (pawxcm)
constexpr double kOxcRhoMin = 1e-14; // spin density below which the derivatives vanish (pawxcm rho_min)
constexpr double kOxcDenPos = 1e-14; // the spin density is kept above this (get_dij: xc_denpos)

// real spherical harmonics of l <= 2 at a unit vector, index l^2 + l + m:
// Y00; y, z, x (l = 1); xy, yz, 3z^2 - 1, xz, x^2 - y^2 (l = 2)
static void ylm2(double x, double y, double z, double *Y) {
  const double pi = 3.14159265358979323846;
  const double c0 = 0.5 / std::sqrt(pi), c1 = std::sqrt(3.0 / (4.0 * pi));
  const double c2 = 0.5 * std::sqrt(15.0 / pi), c20 = 0.25 * std::sqrt(5.0 / pi), c22 = 0.25 * std::sqrt(15.0 / pi);
  Y[0] = c0;
  Y[1] = c1 * y;
  Y[2] = c1 * z;
  Y[3] = c1 * x;
  Y[4] = c2 * x * y;
  Y[5] = c2 * y * z;
  Y[6] = c20 * (3.0 * z * z - 1.0);
  Y[7] = c2 * x * z;
  Y[8] = c22 * (x * x - y * y);
}

// Gauss-Legendre nodes and weights on [-1, 1] (Newton on P_n)
static void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
  const double pi = 3.14159265358979323846;
  x.resize(n);
  w.resize(n);
  for (int i = 0; i < n; i++) {
    double t = std::cos(pi * (i + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = t;
      for (int k = 2; k <= n; k++) {
        const double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (t * p1 - p0) / (t * t - 1.0);
      const double dt = p1 / dp;
      t -= dt;
      if (std::fabs(dt) < 1e-16) break;
    }
    x[i] = t;
    w[i] = 2.0 / ((1.0 - t * t) * dp * dp);
  }
}

// G[L][a][b] = int Y_L Y_a Y_b dOmega for L < 9 and a, b < 4 (l <= 1): exact
// for these degrees with 8 Gauss-Legendre nodes in cos(theta) x 16 in phi
static void gaunt_l1(double *G) {
  const double pi = 3.14159265358979323846;
  std::vector<double> ct, wt;
  gauss_legendre(8, ct, wt);
  for (int e = 0; e < kOxcL * 16; e++) G[e] = 0.0;
  const int nphi = 16;
  for (int it = 0; it < 8; it++) {
    const double st = std::sqrt(1.0 - ct[it] * ct[it]);
    for (int ip = 0; ip < nphi; ip++) {
      const double ph = 2.0 * pi * ip / nphi;
      double Y[kOxcL];
      ylm2(st * std::cos(ph), st * std::sin(ph), ct[it], Y);
      const double wq = wt[it] * 2.0 * pi / nphi;
      for (int L = 0; L < kOxcL; L++)
        for (int a = 0; a < 4; a++)
          for (int b = 0; b < 4; b++) G[(L * 4 + a) * 4 + b] += wq * Y[L] * Y[a] * Y[b];
    }
  }
  for (int e = 0; e < kOxcL * 16; e++)
    if (std::fabs(G[e]) < 1e-14) G[e] = 0.0;
}

constexpr double kPwA = 0.031091, kPwA1 = 0.21370, kPwB1 = 7.5957, kPwB2 = 3.5876, kPwB3 = 1.6382, kPwB4 = 0.49294;

// The same LDA potential as a truncated power series in the relative density
// change x = dn / n0, v(n0 (1 + x)) = sum_{k <= 4} v_k x^k (Taylor-mode
// arithmetic: rs, sqrt(rs) and n^(1/3) are binomial series of (1 + x)^p, Q a
// combination of them, log1p(1/Q) and the quotients by the recurrences of
// series division and logarithm).  pawxcm's central differences with the step
// h = t n0 are then, exactly up to the truncated order x^5 (t^4 = 1e-16),
//   (v(n0 + h) - v(n0 - h)) / 2h        = (v_1 + v_3 t^2) / n0,
//   (v(n0 + h) + v(n0 - h) - 2 v0) / h^2 = 2 (v_2 + v_4 t^2) / n0^2,
// from one cube root, one square root and one log1p per point instead of
// three evaluations of the potential, and without the rounding the
// differences amplify.
constexpr int kTs = 5;
struct Ts {
  double c[kTs];
};
__device__ __forceinline__ Ts ts_pow1p(double scale, double p) {  // scale (1 + x)^p
  Ts r;
  double b = scale;
#pragma unroll
  for (int k = 0; k < kTs; k++) {
    r.c[k] = b;
    b *= (p - k) / (k + 1);
  }
  return r;
}
__device__ __forceinline__ Ts ts_mul(const Ts &a, const Ts &b) {
  Ts r;
#pragma unroll
  for (int k = 0; k < kTs; k++) {
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j <= k; j++) acc += a.c[j] * b.c[k - j];
    r.c[k] = acc;
  }
  return r;
}
__device__ __forceinline__ Ts ts_recip(const Ts &a) {
  Ts r;
  const double i0 = 1.0 / a.c[0];
  r.c[0] = i0;
#pragma unroll
  for (int k = 1; k < kTs; k++) {
    double acc = 0.0;
#pragma unroll
    for (int j = 1; j <= k; j++) acc += a.c[j] * r.c[k - j];
    r.c[k] = -acc * i0;
  }
  return r;
}
// log(g) with log(g_0) given
__device__ __forceinline__ Ts ts_log(const Ts &g, double f0) {
  Ts f;
  f.c[0] = f0;
  const double i0 = 1.0 / g.c[0];
#pragma unroll
  for (int k = 1; k < kTs; k++) {
    double acc = 0.0;
#pragma unroll
    for (int j = 1; j < k; j++) acc += j * f.c[j] * g.c[k - j];
    f.c[k] = (g.c[k] - acc / k) * i0;
  }
  return f;
}
__device__ __forceinline__ Ts ts_axpy(double a, const Ts &x, const Ts &y) {  // a x + y
  Ts r;
#pragma unroll
  for (int k = 0; k < kTs; k++) r.c[k] = fma(a, x.c[k], y.c[k]);
  return r;
}

// v_0 .. v_4 of the LDA potential around n0 in x = dn / n0
__device__ __forceinline__ Ts oxc_vxc_series(double n0) {
  const double u0 = cbrt(n0);
  const double rs0 = 0.62035049089940001 / u0;  // (3/(4 pi))^(1/3) / n^(1/3)
  const double s0 = sqrt(rs0);
  const Ts u = ts_pow1p(u0, 1.0 / 3.0);
  const Ts rs = ts_pow1p(rs0, -1.0 / 3.0);
  const Ts sr = ts_pow1p(s0, -1.0 / 6.0);           // sqrt(rs)
  const Ts rss = ts_pow1p(rs0 * s0, -0.5);          // rs^(3/2)
  const Ts rs2 = ts_pow1p(rs0 * rs0, -2.0 / 3.0);   // rs^2
  const Ts isr = ts_pow1p(1.0 / s0, 1.0 / 6.0);     // rs^(-1/2)
  Ts Q, dQ;
#pragma unroll
  for (int k = 0; k < kTs; k++) {
    Q.c[k] = 2.0 * kPwA * (kPwB1 * sr.c[k] + kPwB2 * rs.c[k] + kPwB3 * rss.c[k] + kPwB4 * rs2.c[k]);
    dQ.c[k] = 2.0 * kPwA * (0.5 * kPwB1 * isr.c[k] + 1.5 * kPwB3 * sr.c[k] + 2.0 * kPwB4 * rs.c[k]);
  }
  dQ.c[0] += 2.0 * kPwA * kPwB2;
  // lg = log1p(1/Q) = log(1 + 1/Q)
  Ts T = ts_recip(Q);
  T.c[0] += 1.0;
  const Ts lg = ts_log(T, log1p(1.0 / Q.c[0]));
  Ts onea = rs;  // 1 + a1 rs
#pragma unroll
  for (int k = 0; k < kTs; k++) onea.c[k] *= kPwA1;
  onea.c[0] += 1.0;
  const Ts QQ = ts_mul(Q, ts_axpy(1.0, Q, Ts{{1.0, 0.0, 0.0, 0.0, 0.0}}));  // Q (Q + 1)
  const Ts F = ts_mul(dQ, ts_recip(QQ));
  const Ts ec = ts_mul(onea, lg);               // / (-2A)
  const Ts dec2 = ts_mul(onea, F);              // dec = -2A a1 lg + 2A dec2
  const Ts rsdec = ts_mul(rs, ts_axpy(-kPwA1, lg, dec2));  // rs dec / 2A
  Ts v;
#pragma unroll
  for (int k = 0; k < kTs; k++)
    v.c[k] = -0.98474502184269641 * u.c[k] - 2.0 * kPwA * ec.c[k] - 2.0 * kPwA * rsdec.c[k] / 3.0;
  return v;
}

constexpr int kOxcMaxW = 6;                          // partial waves per atom
constexpr int kOxcMaxP = kOxcMaxW * (kOxcMaxW + 1) / 2;  // unordered wave pairs
constexpr int kOxcChunk = 64;                        // radial points per CTA
constexpr int kOxcLiveMax = kOxcL * kOxcMaxP;        // (L, pair) entries of one atom

struct OxcTabs {
  const int *rad_n, *nphi;
  const int64_t *roff;     // per atom offset into r, w, core, tcore
  const double *r, *w, *core, *tcore;
  const int64_t *phioff;   // per atom offset into phi, tphi
  const double *phi, *tphi;
  const int *pwave;        // per slot: partial-wave index
  const double *gaunt;     // per atom [kOxcL][ms][ms]
  const int *ms;
  const int64_t *doff, *soff;
  const int *dslot;        // atom of every D_ij entry
  const short *live;       // per atom [kOxcLiveMax]: the (L, pair) entries L np + p with a
                           // non-zero Gaunt coefficient, ascending
  const int *nlive;        // per atom: their count
  int nchunk;              // radial chunks of the longest mesh
  int natom, nd;
};

// index of the unordered wave pair (a, b) among the nw (nw + 1) / 2
__device__ __forceinline__ int oxc_pair(int a, int b, int nw) {
  if (a > b) {
    const int t = a;
    a = b;
    b = t;
  }
  return a * nw - a * (a - 1) / 2 + (b - a);
}

// Partial integrals of the potential moments over one radial chunk of one
// part (all-electron s = 0, pseudo s = 1) of one atom, in wave pairs:
//
//   I^L_ab = sum_{k in chunk} w_k V_L(r_k) u_a(r_k) u_b(r_k),
//
// with n_L(r) = sum_ab C^L_ab u_a u_b / r^2 (+ sqrt(4 pi) n_c),
// C^L_ab = sum_{ij: {pw_i, pw_j} = {a, b}} rho_ij G^L_ij: the moments and the
// integrals run over wave pairs (at most 21) instead of projector pairs
// (64 for 8 projectors), the FP64 work is spread over (atom, part, chunk)
// CTAs, and every sum runs in a fixed order.  Only the (L, pair) entries
// whose Gaunt coefficients are not all zero are formed (33 of 90 for two s
// and two p waves: s s pairs have L = 0 only, s p pairs l = 1, p p pairs
// L = 0 and l = 2); the others are exact zeros, so D_xc is the same bit for
// bit with fewer FP64 operations.
__global__ void __launch_bounds__(kOxcChunk) k_oxc_radial(OxcTabs T, const double *__restrict__ rho,
                                                          double *__restrict__ part) {
  const int a = blockIdx.x, s = blockIdx.y & 1, set = blockIdx.y >> 1, ch = blockIdx.z, t = threadIdx.x;
  const int m = T.ms[a], nr = T.rad_n[a], nw = T.nphi[a], np = nw * (nw + 1) / 2;
  if (ch * kOxcChunk >= nr) return;
  __shared__ double C[kOxcL][kOxcMaxP];
  __shared__ double Vw[kOxcL][kOxcChunk];
  __shared__ double Us[kOxcMaxW][kOxcChunk];
  const double *R = rho + (int64_t)set * T.nd + T.doff[a];
  const double *G = T.gaunt + (int64_t)kOxcL * T.doff[a];
  const int *pw = T.pwave + T.soff[a];
  const short *lv = T.live + (int64_t)a * kOxcLiveMax;
  const int nl = T.nlive[a];
  for (int e = t; e < kOxcL * np; e += blockDim.x) C[e / np][e % np] = 0.0;
  __syncthreads();
  for (int q = t; q < nl; q += blockDim.x) {
    const int e = lv[q], L = e / np, p = e % np;
    double acc = 0.0;
    for (int j = 0; j < m; j++)
      for (int i = 0; i < m; i++)
        if (oxc_pair(pw[i], pw[j], nw) == p) acc += R[i + m * j] * G[(L * m + i) * m + j];
    C[L][p] = acc;
  }
  const int k = ch * kOxcChunk + t;
  const bool valid = k < nr;
  const double *U = (s ? T.tphi : T.phi) + T.phioff[a];
  for (int wv = 0; wv < nw; wv++) Us[wv][t] = valid ? U[(int64_t)wv * nr + k] : 0.0;
  __syncthreads();
  double V[kOxcL];
#pragma unroll
  for (int L = 0; L < kOxcL; L++) V[L] = 0.0;
  if (valid) {
    const double sq4pi = 3.5449077018110318;  // sqrt(4 pi)
    const double rk = T.r[T.roff[a] + k];
    const double inv_r2 = 1.0 / (rk * rk);
    double n[kOxcL];
#pragma unroll
    for (int L = 0; L < kOxcL; L++) n[L] = 0.0;
    for (int wa = 0; wa < nw; wa++)
      for (int wb = wa; wb < nw; wb++) {
        const double uu = Us[wa][t] * Us[wb][t] * inv_r2;
        const int p = oxc_pair(wa, wb, nw);
#pragma unroll
        for (int L = 0; L < kOxcL; L++) n[L] += C[L][p] * uu;
      }
    n[0] += sq4pi * (s ? T.tcore : T.core)[T.roff[a] + k];
    double up = 0.5 * n[0] / sq4pi;  // spin density of the spherical part
    if (up < kOxcDenPos) up = kOxcDenPos;
    const double ns = 2.0 * up;
    // the step is taken as the difference of two doubles, so that ns + h and
    // ns - h are exact and the divided differences see the steps they divide by
    const double h = (ns + kOxcDelta * ns) - ns;
    const Ts vs = oxc_vxc_series(ns);
    const double v0 = vs.c[0];
    double d1 = 0.0, d2 = 0.0;
    if (up > kOxcRhoMin) {  // pawxcm's central differences at the step h (series above)
      const double t = h / ns, t2 = t * t;
      d1 = fma(vs.c[3], t2, vs.c[1]) / ns;
      d2 = 2.0 * fma(vs.c[4], t2, vs.c[2]) / (ns * ns);
    }
    double v1sum = 0.0;
#pragma unroll
    for (int L = 1; L < kOxcL; L++) v1sum += n[L] * n[L];
    const double wk = T.w[T.roff[a] + k];
    V[0] = wk * (v0 * sq4pi + v1sum * d2 / (2.0 * sq4pi));
#pragma unroll
    for (int L = 1; L < kOxcL; L++) V[L] = wk * d1 * n[L];
  }
#pragma unroll
  for (int L = 0; L < kOxcL; L++) Vw[L][t] = V[L];
  __syncthreads();
  double *out = part + ((((int64_t)set * T.natom + a) * 2 + s) * T.nchunk + ch) * (kOxcL * kOxcMaxP);
  for (int e = t; e < kOxcL * np; e += blockDim.x) out[(e / np) * kOxcMaxP + e % np] = 0.0;
  __syncthreads();
  for (int li = t; li < nl; li += blockDim.x) {
    const int e = lv[li], L = e / np, p = e % np;
    int wa = 0, q = p;
    while (q >= nw - wa) {
      q -= nw - wa;
      wa++;
    }
    const int wb = wa + q;
    double acc = 0.0;
    for (int i = 0; i < kOxcChunk; i++) acc += Vw[L][i] * Us[wa][i] * Us[wb][i];
    out[L * kOxcMaxP + p] = acc;
  }
}

// D_xc_ij = sum_L G^L_ij sum_chunks (I^L_{pw_i pw_j} - I~^L_{pw_i pw_j}): a
// warp per entry, lanes over (L, chunk) in a fixed order (the same arithmetic
// for ij and ji, so every block is exactly symmetric)
__global__ void __launch_bounds__(256) k_oxc_assemble(OxcTabs T, const double *__restrict__ part, int nsets,
                                                      double *__restrict__ dxc) {
  const int64_t ea = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (ea >= (int64_t)nsets * T.nd) return;
  const int set = (int)(ea / T.nd), e = (int)(ea - (int64_t)set * T.nd);
  const int a = T.dslot[e];
  const int m = T.ms[a], nr = T.rad_n[a], nw = T.nphi[a];
  const int loc = e - (int)T.doff[a], i = loc % m, j = loc / m;
  const int nch = (nr + kOxcChunk - 1) / kOxcChunk;
  const double *G = T.gaunt + (int64_t)kOxcL * T.doff[a];
  const int *pw = T.pwave + T.soff[a];
  const int p = oxc_pair(pw[i], pw[j], nw);
  const double *ae = part + (((int64_t)set * T.natom + a) * 2) * T.nchunk * (kOxcL * kOxcMaxP);
  const double *ps = ae + (int64_t)T.nchunk * (kOxcL * kOxcMaxP);
  double acc = 0.0;
  for (int q = lane; q < kOxcL * nch; q += 32) {
    const int L = q / nch, c = q % nch;
    const int64_t o = (int64_t)c * (kOxcL * kOxcMaxP) + L * kOxcMaxP + p;
    acc += G[(L * m + i) * m + j] * (ae[o] - ps[o]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) dxc[ea] = acc;
}

// ---- set-up: validate and upload the radial tables (ctx.cu calls this)
int onsite_init(opaw_ctx *c, const opaw_system *s) {
  if (!s->rad_n) return OPAW_OK;  // term switched off
  OPAW_ARG(s->rad_r && s->rad_w && s->nphi && s->phi && s->tphi && s->coredens && s->tcoredens && s->proj_lmn,
           "on-site XC: every radial table is needed when rad_n is given");
  const int na = c->natom;
  std::vector<int64_t> roff(na + 1, 0), phioff(na + 1, 0);
  int nchunk = 1;
  std::vector<int> pwave(c->ns > 0 ? c->ns : 1);
  std::vector<double> gl(kOxcL * 16);
  gaunt_l1(gl.data());
  std::vector<double> gaunt((size_t)kOxcL * (c->nd > 0 ? c->nd : 1), 0.0);
  for (int a = 0; a < na; a++) {
    OPAW_ARG(s->rad_n[a] >= 3 && s->nphi[a] >= 1, "on-site XC: radial mesh or partial waves missing");
    OPAW_ARG(s->nphi[a] <= kOxcMaxW, "on-site XC: at most 6 partial waves per atom");
    nchunk = std::max(nchunk, (s->rad_n[a] + kOxcChunk - 1) / kOxcChunk);
    roff[a + 1] = roff[a] + s->rad_n[a];
    phioff[a + 1] = phioff[a] + (int64_t)s->nphi[a] * s->rad_n[a];
    const int m = c->h_ms[a];
    for (int i = 0; i < m; i++) {
      const int64_t q = c->h_soff[a] + i;
      const int l = s->proj_lmn[3 * q], mm = s->proj_lmn[3 * q + 1], pn = s->proj_lmn[3 * q + 2];
      OPAW_ARG(l >= 0 && l <= 1, "on-site XC: projectors with l <= 1 (s, p) are supported");
      OPAW_ARG(mm >= -l && mm <= l, "on-site XC: |m| > l in proj_lmn");
      OPAW_ARG(pn >= 0 && pn < s->nphi[a], "on-site XC: partial-wave index out of range");
      pwave[q] = pn;
    }
    for (int L = 0; L < kOxcL; L++)
      for (int j = 0; j < m; j++)
        for (int i = 0; i < m; i++) {
          const int64_t qi = c->h_soff[a] + i, qj = c->h_soff[a] + j;
          const int li = s->proj_lmn[3 * qi], lj = s->proj_lmn[3 * qj];
          const int ai = li * li + li + s->proj_lmn[3 * qi + 1];
          const int aj = lj * lj + lj + s->proj_lmn[3 * qj + 1];
          gaunt[(size_t)kOxcL * c->h_doff[a] + (L * m + i) * m + j] = gl[(L * 4 + ai) * 4 + aj];
        }
  }
  // the (L, pair) entries with a non-zero Gaunt coefficient, per atom
  std::vector<short> live((size_t)kOxcLiveMax * (na > 0 ? na : 1), 0);
  std::vector<int> nlive(na > 0 ? na : 1, 0);
  for (int a = 0; a < na; a++) {
    const int m = c->h_ms[a], nw = s->nphi[a], np = nw * (nw + 1) / 2;
    for (int L = 0; L < kOxcL; L++)
      for (int p = 0; p < np; p++) {
        bool any = false;
        for (int j = 0; j < m && !any; j++)
          for (int i = 0; i < m; i++) {
            int wa = pwave[c->h_soff[a] + i], wb = pwave[c->h_soff[a] + j];
            if (wa > wb) std::swap(wa, wb);
            const int pp = wa * nw - wa * (wa - 1) / 2 + (wb - wa);
            if (pp == p && gaunt[(size_t)kOxcL * c->h_doff[a] + (L * m + i) * m + j] != 0.0) {
              any = true;
              break;
            }
          }
        if (any) live[(size_t)kOxcLiveMax * a + nlive[a]++] = (short)(L * np + p);
      }
  }
  for (int64_t k = 0; k < roff[na]; k++) OPAW_ARG(s->rad_r[k] > 0.0, "on-site XC: radii must be > 0");
  auto up = [&](void **dst, const void *src, size_t bytes) -> int {
    OPAW_CUDA(cudaMalloc(dst, bytes > 0 ? bytes : 8));
    if (bytes && src) OPAW_CUDA(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
    else OPAW_CUDA(cudaMemset(*dst, 0, bytes > 0 ? bytes : 8));
    return OPAW_OK;
  };
  OPAW_CHECK(up((void **)&c->oxc_rad_n, s->rad_n, sizeof(int) * na));
  OPAW_CHECK(up((void **)&c->oxc_roff, roff.data(), sizeof(int64_t) * (na + 1)));
  OPAW_CHECK(up((void **)&c->oxc_r, s->rad_r, sizeof(double) * roff[na]));
  OPAW_CHECK(up((void **)&c->oxc_w, s->rad_w, sizeof(double) * roff[na]));
  OPAW_CHECK(up((void **)&c->oxc_core, s->coredens, sizeof(double) * roff[na]));
  OPAW_CHECK(up((void **)&c->oxc_tcore, s->tcoredens, sizeof(double) * roff[na]));
  OPAW_CHECK(up((void **)&c->oxc_phioff, phioff.data(), sizeof(int64_t) * (na + 1)));
  OPAW_CHECK(up((void **)&c->oxc_phi, s->phi, sizeof(double) * phioff[na]));
  OPAW_CHECK(up((void **)&c->oxc_tphi, s->tphi, sizeof(double) * phioff[na]));
  OPAW_CHECK(up((void **)&c->oxc_pwave, pwave.data(), sizeof(int) * pwave.size()));
  OPAW_CHECK(up((void **)&c->oxc_gaunt, gaunt.data(), sizeof(double) * gaunt.size()));
  OPAW_CHECK(up((void **)&c->oxc_nphi, s->nphi, sizeof(int) * na));
  OPAW_CHECK(up((void **)&c->oxc_live, live.data(), sizeof(short) * live.size()));
  OPAW_CHECK(up((void **)&c->oxc_nlive, nlive.data(), sizeof(int) * nlive.size()));
  c->oxc_nchunk = nchunk;
  c->oxc_on = 1;
  return OPAW_OK;
}

void onsite_free(opaw_ctx *c) {
  void *p[] = {c->oxc_rad_n, c->oxc_roff, c->oxc_r, c->oxc_w, c->oxc_core, c->oxc_tcore, c->oxc_phioff,
               c->oxc_phi, c->oxc_tphi, c->oxc_pwave, c->oxc_gaunt, c->oxc_nphi, c->oxc_part.p,
               c->oxc_live, c->oxc_nlive};
  for (void *q : p) cudaFree(q);
  c->oxc_part = DeviceBuf();
}

// D_xc of every atom for nsets consecutive rho_ij blocks (device [nsets][nd])
// into dxc (device [nsets][nd]), on stream st
int onsite_xc_sets(opaw_ctx *c, const double *rhoij, int nsets, double *dxc, cudaStream_t st) {
  if (!c->oxc_on || c->natom == 0 || nsets <= 0) return OPAW_OK;
  OPAW_CHECK(ensure(c->oxc_part,
                    sizeof(double) * (size_t)nsets * c->natom * 2 * c->oxc_nchunk * kOxcL * kOxcMaxP));
  OxcTabs T;
  T.rad_n = c->oxc_rad_n;
  T.nphi = c->oxc_nphi;
  T.nchunk = c->oxc_nchunk;
  T.natom = c->natom;
  T.nd = c->nd;
  T.roff = c->oxc_roff;
  T.r = c->oxc_r;
  T.w = c->oxc_w;
  T.core = c->oxc_core;
  T.tcore = c->oxc_tcore;
  T.phioff = c->oxc_phioff;
  T.phi = c->oxc_phi;
  T.tphi = c->oxc_tphi;
  T.pwave = c->oxc_pwave;
  T.gaunt = c->oxc_gaunt;
  T.ms = c->d_ms;
  T.doff = c->d_doff;
  T.soff = c->d_soff;
  T.dslot = c->d_dslot_atom;
  T.live = c->oxc_live;
  T.nlive = c->oxc_nlive;
  double *part = (double *)c->oxc_part.p;
  k_oxc_radial<<<dim3(c->natom, 2 * nsets, c->oxc_nchunk), kOxcChunk, 0, st>>>(T, rhoij, part);
  k_oxc_assemble<<<grid1((int64_t)nsets * c->nd * 32, 256), 256, 0, st>>>(T, part, nsets, dxc);
  c->launches += 2;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

// D_xc of every atom from rho_ij (device [nd]) into dxc (device [nd])
int onsite_xc_of(opaw_ctx *c, const double *rhoij, double *dxc) {
  return onsite_xc_sets(c, rhoij, 1, dxc, c->stream);
}

}  // namespace opaw

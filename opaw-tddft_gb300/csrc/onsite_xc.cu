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
// v the LDA potential (Slater + PW92), v' and v'' central finite differences
// with the relative step 1e-4 as pawxcm takes them (formed from
// cancellation-free potential differences, oxc_vdiff); the pseudo part V~ is
// the same with u~ and the pseudo core (the compensation charge is not in the
// XC density, usexcnhat = 0).  G^L_ij = int Y_L Y_i Y_j dOmega, real Y_lm in
// the ylm.f90 order.  Projectors with l <= 1 (s and p partial waves, those of
// the reference's datasets) are supported: L <= 2, 9 moments.
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

// LDA v_xc of the total density (Slater + PW92, the formula of vxc_point in
// rebuild.cu)
__device__ __forceinline__ double oxc_vxc(double n) {
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

// v(n + dn) - v(n) of the same LDA without the cancellation of two nearly
// equal potentials: divided differences of every factor of the formula (the
// FP64 form of vxc_pair_f in mixed.cu).  The finite-difference derivatives of
// pawxcm are formed from these differences, so their cancellation costs a
// factor 1/step instead of 1/step^2 of the rounding.
struct OxcParts {
  double u, rs, s, Q, dQ, lg;
};
constexpr double kPwA = 0.031091, kPwA1 = 0.21370, kPwB1 = 7.5957, kPwB2 = 3.5876, kPwB3 = 1.6382, kPwB4 = 0.49294;
__device__ __forceinline__ OxcParts oxc_parts(double n) {
  OxcParts p;
  p.u = cbrt(n);
  p.rs = 0.62035049089940001 / p.u;  // (3/(4 pi))^(1/3) / n^(1/3)
  p.s = sqrt(p.rs);
  p.Q = 2.0 * kPwA * (kPwB1 * p.s + kPwB2 * p.rs + kPwB3 * p.rs * p.s + kPwB4 * p.rs * p.rs);
  p.dQ = 2.0 * kPwA * (0.5 * kPwB1 / p.s + kPwB2 + 1.5 * kPwB3 * p.s + 2.0 * kPwB4 * p.rs);
  p.lg = log1p(1.0 / p.Q);
  return p;
}
__device__ __forceinline__ double oxc_dec(const OxcParts &p) {  // d eps_c / d rs
  return -2.0 * kPwA * kPwA1 * p.lg + 2.0 * kPwA * (1.0 + kPwA1 * p.rs) * p.dQ / (p.Q * (p.Q + 1.0));
}
__device__ double oxc_vdiff(double n0, double dn) {
  const double n1 = n0 + dn;
  if (!(n0 > 1e-15) || !(n1 > 1e-15)) return oxc_vxc(n1) - oxc_vxc(n0);
  const OxcParts p0 = oxc_parts(n0), p1 = oxc_parts(n1);
  const double du = dn / (p1.u * p1.u + p1.u * p0.u + p0.u * p0.u);
  const double dvx = -0.98474502184269641 * du;  // (3/pi)^(1/3)
  const double drs = -0.62035049089940001 * du / (p1.u * p0.u);
  const double ds = drs / (p1.s + p0.s);
  const double drss = drs * p1.s + p0.rs * ds;
  const double drs2 = drs * (p1.rs + p0.rs);
  const double dQ = 2.0 * kPwA * (kPwB1 * ds + kPwB2 * drs + kPwB3 * drss + kPwB4 * drs2);
  const double ddQ = 2.0 * kPwA * (-0.5 * kPwB1 * ds / (p1.s * p0.s) + 1.5 * kPwB3 * ds + 2.0 * kPwB4 * drs);
  const double dlg = log1p(-dQ / (p1.Q * (p0.Q + 1.0)));
  const double dec = -2.0 * kPwA * (kPwA1 * drs * p1.lg + (1.0 + kPwA1 * p0.rs) * dlg);
  const double G0 = p0.Q * (p0.Q + 1.0), G1 = p1.Q * (p1.Q + 1.0);
  const double F1 = p1.dQ / G1;
  const double dF = (ddQ * G0 - p0.dQ * dQ * (p1.Q + p0.Q + 1.0)) / (G1 * G0);
  const double ddec = -2.0 * kPwA * kPwA1 * dlg + 2.0 * kPwA * (kPwA1 * drs * F1 + (1.0 + kPwA1 * p0.rs) * dF);
  return dvx + dec - (drs * oxc_dec(p1) + p0.rs * ddec) / 3.0;
}

struct OxcTabs {
  const int *rad_n;
  const int64_t *roff;     // per atom offset into r, w, core, tcore, and of the scratch (x 2 kOxcL)
  const double *r, *w, *core, *tcore;
  const int64_t *phioff;   // per atom offset into phi, tphi
  const double *phi, *tphi;
  const int *pwave;        // per slot: partial-wave index
  const double *gaunt;     // per atom [kOxcL][ms][ms]
  const int *ms;
  const int64_t *doff, *soff;
};

__device__ __forceinline__ double oxc_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One CTA per atom.  Phase 1: the potential moments V_L(r_k) of the
// all-electron and pseudo one-centre densities into the scratch [2][L][k];
// phase 2: D_xc_ij, a warp per (i <= j), in a fixed order.
__global__ void __launch_bounds__(256) k_onsite_xc(OxcTabs T, const double *__restrict__ rho,
                                                   double *__restrict__ scratch, double *__restrict__ dxc) {
  const int a = blockIdx.x;
  const int m = T.ms[a], nr = T.rad_n[a];
  const double *R = rho + T.doff[a];
  const double *G = T.gaunt + (int64_t)kOxcL * T.doff[a];
  const double *r = T.r + T.roff[a], *w = T.w + T.roff[a];
  const int *pw = T.pwave + T.soff[a];
  double *V = scratch + 2 * kOxcL * T.roff[a];
  const double sq4pi = 3.5449077018110318;  // sqrt(4 pi)
  for (int k = threadIdx.x; k < nr; k += blockDim.x) {
    for (int s = 0; s < 2; s++) {
      const double *U = (s ? T.tphi : T.phi) + T.phioff[a];
      double n[kOxcL];
#pragma unroll
      for (int L = 0; L < kOxcL; L++) n[L] = 0.0;
      const double inv_r2 = 1.0 / (r[k] * r[k]);
      for (int j = 0; j < m; j++) {
        const double uj = U[(int64_t)pw[j] * nr + k];
        for (int i = 0; i < m; i++) {
          const double f = R[i + m * j] * U[(int64_t)pw[i] * nr + k] * uj * inv_r2;
#pragma unroll
          for (int L = 0; L < kOxcL; L++) n[L] += f * G[(L * m + i) * m + j];
        }
      }
      n[0] += sq4pi * (s ? T.tcore : T.core)[T.roff[a] + k];
      double up = 0.5 * n[0] / sq4pi;  // spin density of the spherical part
      if (up < kOxcDenPos) up = kOxcDenPos;
      const double ns = 2.0 * up;
      // the step is taken as the difference of two doubles, so that
      // ns + h and ns - h are exact and the divided differences see the
      // steps they divide by
      const double v0 = oxc_vxc(ns), h = (ns + kOxcDelta * ns) - ns;
      double d1 = 0.0, d2 = 0.0;
      if (up > kOxcRhoMin) {
        // (v+ - v-) / 2h and (v+ + v- - 2 v0) / h^2 of pawxcm from the
        // differences dp = v+ - v0, dm = v0 - v-
        const double dp = oxc_vdiff(ns, h), dm = -oxc_vdiff(ns, -h);
        d1 = (dp + dm) / (2.0 * h);
        d2 = (dp - dm) / (h * h);
      }
      double v1sum = 0.0;
#pragma unroll
      for (int L = 1; L < kOxcL; L++) v1sum += n[L] * n[L];
      double *Vs = V + (int64_t)s * kOxcL * nr;
      Vs[k] = v0 * sq4pi + v1sum * d2 / (2.0 * sq4pi);
#pragma unroll
      for (int L = 1; L < kOxcL; L++) Vs[(int64_t)L * nr + k] = d1 * n[L];
    }
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const double *U0 = T.phi + T.phioff[a], *U1 = T.tphi + T.phioff[a];
  for (int e = warp; e < m * m; e += nw) {
    const int i = e % m, j = e / m;
    if (i > j) continue;
    double acc = 0.0;
    for (int k = lane; k < nr; k += 32) {
      const double pp = U0[(int64_t)pw[i] * nr + k] * U0[(int64_t)pw[j] * nr + k];
      const double tt = U1[(int64_t)pw[i] * nr + k] * U1[(int64_t)pw[j] * nr + k];
      double s = 0.0;
#pragma unroll
      for (int L = 0; L < kOxcL; L++) {
        const double g = G[(L * m + i) * m + j];
        s += g * (V[(int64_t)L * nr + k] * pp - V[(int64_t)(kOxcL + L) * nr + k] * tt);
      }
      acc += w[k] * s;
    }
    acc = oxc_warp_sum(acc);
    if (lane == 0) {
      dxc[T.doff[a] + i + m * j] = acc;
      dxc[T.doff[a] + j + m * i] = acc;
    }
  }
}

// ---- set-up: validate and upload the radial tables (ctx.cu calls this)
int onsite_init(opaw_ctx *c, const opaw_system *s) {
  if (!s->rad_n) return OPAW_OK;  // term switched off
  OPAW_ARG(s->rad_r && s->rad_w && s->nphi && s->phi && s->tphi && s->coredens && s->tcoredens && s->proj_lmn,
           "on-site XC: every radial table is needed when rad_n is given");
  const int na = c->natom;
  std::vector<int64_t> roff(na + 1, 0), phioff(na + 1, 0);
  std::vector<int> pwave(c->ns > 0 ? c->ns : 1);
  std::vector<double> gl(kOxcL * 16);
  gaunt_l1(gl.data());
  std::vector<double> gaunt((size_t)kOxcL * (c->nd > 0 ? c->nd : 1), 0.0);
  for (int a = 0; a < na; a++) {
    OPAW_ARG(s->rad_n[a] >= 3 && s->nphi[a] >= 1, "on-site XC: radial mesh or partial waves missing");
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
  OPAW_CHECK(up((void **)&c->oxc_scratch, nullptr, sizeof(double) * 2 * kOxcL * roff[na]));
  c->oxc_on = 1;
  return OPAW_OK;
}

void onsite_free(opaw_ctx *c) {
  void *p[] = {c->oxc_rad_n, c->oxc_roff, c->oxc_r, c->oxc_w, c->oxc_core, c->oxc_tcore, c->oxc_phioff,
               c->oxc_phi, c->oxc_tphi, c->oxc_pwave, c->oxc_gaunt, c->oxc_scratch};
  for (void *q : p) cudaFree(q);
}

// D_xc of every atom from rho_ij (device [nd]) into dxc (device [nd])
int onsite_xc_of(opaw_ctx *c, const double *rhoij, double *dxc) {
  if (!c->oxc_on || c->natom == 0) return OPAW_OK;
  OxcTabs T;
  T.rad_n = c->oxc_rad_n;
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
  k_onsite_xc<<<c->natom, 256, 0, c->stream>>>(T, rhoij, c->oxc_scratch, dxc);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

}  // namespace opaw

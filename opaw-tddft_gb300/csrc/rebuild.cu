// rebuild.cu — the per-stage Hamiltonian rebuild of the TDDFT loop
// (ncpaw_make_hamiltonian.f90:213-281): psi~ = S^-1/2 psi_bar, rho_ij,
// density, compensation charge with the charge renormalisation, LDA v_xc,
// Martyna-Tuckerman Hartree on the 2x box, v_ks and D_ij; plus the one-time
// Martyna-Tuckerman kernel (vk_TuMa.f90, vk_scale.f90).
// All of it is FP64 (the small matrices and potentials); only psi~ and the
// box sums follow the orbital precision.
#include <cmath>
#include <type_traits>

#include "fft.cuh"

namespace opaw {

int refresh_vks_f(opaw_ctx *c, int set);  // ctx.cu

__device__ __forceinline__ double block_sum(double v, double *sh) {
  // fixed-order block reduction (blockDim.x == 256)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) r += sh[i];
  __syncthreads();
  return r;  // valid in thread 0
}

// ------------------------------------------------------ MT kernel (A14) --
struct BigBox {
  int nx, ny, nz;
  double dx, dy, dz;
};

__global__ void k_vk_real(double2 *cvk, BigBox b, double aa, double r0x, double r0y, double r0z, double dvb) {
  const int64_t n = (int64_t)b.nx * b.ny * b.nz;
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= n) return;
  const int x = (int)(g % b.nx), y = (int)((g / b.nx) % b.ny), z = (int)(g / ((int64_t)b.nx * b.ny));
  const double rx = r0x + x * b.dx, ry = r0y + y * b.dy, rz = r0z + z * b.dz;
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz));
  const double fl = (double)1e-26f;  // single-precision literal of vk_TuMa.f90:51
  const double rp = sqrt(r2 > fl ? r2 : fl);
  cvk[g] = make_double2(erf(aa * rp) / rp * dvb, 0.0);  // :52
}

__global__ void k_vk_finish(const double2 *cvk, double *vk, BigBox b, const double *kx, const double *ky,
                            const double *kz, double aa, double r0x, double r0y, double r0z, int periodic) {
  const int64_t n = (int64_t)b.nx * b.ny * b.nz;
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= n) return;
  const int x = (int)(g % b.nx), y = (int)((g / b.nx) % b.ny), z = (int)(g / ((int64_t)b.nx * b.ny));
  const double qx = kx[x], qy = ky[y], qz = kz[z];
  const double k2 = __dadd_rn(__dadd_rn(__dmul_rn(qx, qx), __dmul_rn(qy, qy)), __dmul_rn(qz, qz));
  const double pi = 3.14159265358979323846;
  double re = 0, ct;
  if (!periodic) {
    const double ph = __dadd_rn(__dadd_rn(__dmul_rn(r0x, qx), __dmul_rn(r0y, qy)), __dmul_rn(r0z, qz));
    double sn, cs;
    sincos(ph, &sn, &cs);
    const double2 v = cvk[g];
    re = v.x * cs - v.y * sn;  // real part of vk_TuMa.f90:77-78 (vk = real(cvk), :109)
    const double k2s = k2 / (4.0 * aa * aa);
    if (k2s > 1e-8) ct = 4.0 * pi / k2 * (1.0 - exp(-k2s));                      // :85
    else ct = 4.0 * pi / (4.0 * aa * aa) * (1.0 - 0.5 * k2s + k2s * k2s / 6.0);  // :88
  } else {
    ct = (k2 > 1e-8) ? 4.0 * pi / k2 : 0.0;  // :93-97
  }
  vk[g] = __ddiv_rn(__ddiv_rn(__ddiv_rn(re + ct, (double)b.nx), (double)b.ny), (double)b.nz);  // vk_scale.f90:46
}

__global__ void k_vk_to_float(const double *a, float *b, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

static double kcomp(int i, int n, double d) {
  const double pi = acos(-1.0);
  double dk = 2.0 * pi / ((double)n * d);
  double k = (double)i * dk;
  if (k > pi / d) k = k - 2.0 * pi / d;
  return k;
}

int vk_prep(opaw_ctx *c) {
  const int64_t nb = c->nnb;
  OPAW_CUDA(cudaMalloc(&c->d_vk, sizeof(double) * nb));
  OPAW_CHECK(ensure(c->work[0], sizeof(double2) * nb));
  double2 *cvk = (double2 *)c->work[0].p;
  BigBox b{c->nxb, c->nyb, c->nzb, c->dx, c->dy, c->dz};
  double lmin = std::min(std::min(c->nxb * c->dx, c->nyb * c->dy), c->nzb * c->dz);
  const double aa = 7.0 / lmin;  // vk_TuMa.f90:25
  const double r0x = -(c->nxb) / 2.0 * c->dx, r0y = -(c->nyb) / 2.0 * c->dy, r0z = -(c->nzb) / 2.0 * c->dz;
  if (!c->periodic) {
    k_vk_real<<<grid1(nb, 256), 256, 0, c->stream>>>(cvk, b, aa, r0x, r0y, r0z, c->dx * c->dy * c->dz);
    c->launches++;
    OPAW_CUDA(cudaGetLastError());
    OPAW_CHECK(fft3d<double>(c, c->fftb, cvk, 1, +1));  // fft3d_general(.,1)
  } else {
    OPAW_CUDA(cudaMemsetAsync(cvk, 0, sizeof(double2) * nb, c->stream));
  }
  std::vector<double> kt[3];
  const int nd[3] = {c->nxb, c->nyb, c->nzb};
  const double dd[3] = {c->dx, c->dy, c->dz};
  double *dk[3];
  for (int k = 0; k < 3; k++) {
    kt[k].resize(nd[k]);
    for (int i = 0; i < nd[k]; i++) kt[k][i] = kcomp(i, nd[k], dd[k]);
    OPAW_CUDA(cudaMalloc(&dk[k], sizeof(double) * nd[k]));
    OPAW_CUDA(cudaMemcpy(dk[k], kt[k].data(), sizeof(double) * nd[k], cudaMemcpyHostToDevice));
  }
  OPAW_CUDA(cudaDeviceSynchronize());
  k_vk_finish<<<grid1(nb, 256), 256, 0, c->stream>>>(cvk, c->d_vk, b, dk[0], dk[1], dk[2], aa, r0x, r0y, r0z,
                                                     c->periodic);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  OPAW_CUDA(cudaMalloc(&c->d_vk_f, sizeof(float) * nb));
  k_vk_to_float<<<grid1(nb, 256), 256, 0, c->stream>>>(c->d_vk, c->d_vk_f, nb);
  c->launches++;
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < 3; k++) cudaFree(dk[k]);
  return OPAW_OK;
}

// -------------------------------------------------- Hartree (A13) --
// big-box FFT pipeline: embed (x pass) .. times vk (z pass) .. crop (x pass).
// Two real densities ride in the real and imaginary parts of one complex
// transform; vk is real and even, so the two results separate exactly.
struct Embed {
  int nx, ny, nz, nxb, nyb, mx, my, mz;
  __device__ bool inner(int64_t g, int64_t &i) const {
    const int x = (int)(g % nxb), y = (int)((g / nxb) % nyb), z = (int)(g / ((int64_t)nxb * nyb));
    const int ix = x - mx, iy = y - my, iz = z - mz;
    if (ix < 0 || ix >= nx || iy < 0 || iy >= ny || iz < 0 || iz >= nz) return false;
    i = ix + (int64_t)nx * (iy + (int64_t)ny * iz);
    return true;
  }
};

template <typename R> struct OpEmbed {
  typedef typename Tr<R>::C C;
  Embed e;
  const double *d0, *d1;
  C *wb;
  int64_t bs = 0;  // batch stride of wb
  int pair = 0;    // 1: batch b transforms d0 (b = 0) or d1 (b = 1) alone; 2: d0 + b ss alone; 0: d0 + i d1
  int64_t ss = 0;  // source stride of pair mode 2
  static constexpr bool kMid = false;
  __device__ C load(int b, int64_t g) const {
    int64_t i;
    C v;
    v.x = 0;
    v.y = 0;
    if (!e.inner(g, i)) return v;
    if (pair) {
      v.x = (R)(pair == 2 ? d0 + b * ss : (b ? d1 : d0))[i];
      return v;
    }
    v.x = (R)d0[i];
    v.y = d1 ? (R)d1[i] : (R)0;
    return v;
  }
  __device__ void store(int b, int64_t g, C v) const { wb[b * bs + g] = v; }
  __device__ double line(int64_t) const { return 0.0; }
  __device__ C mid(int, int64_t, double, int, C v) const { return v; }
};

// in-place pass whose loads read zero outside [lo, hi) of one coordinate
// (axis 1: y, axis 2: z): the lines there were never written (the
// embedded source is zero there)
template <typename C> struct OpMasked {
  C *wb;
  int64_t div;  // nxb (y) or nxb*nyb (z)
  int nmod, lo, hi;
  int64_t bs = 0;  // batch stride of wb
  static constexpr bool kMid = false;
  __device__ C load(int b, int64_t g) const {
    const int q = (int)((g / div) % nmod);
    if (q < lo || q >= hi) {
      C z;
      z.x = 0;
      z.y = 0;
      return z;
    }
    return wb[b * bs + g];
  }
  __device__ void store(int b, int64_t g, C v) const { wb[b * bs + g] = v; }
  __device__ double line(int64_t) const { return 0.0; }
  __device__ C mid(int, int64_t, double, int, C v) const { return v; }
};

template <typename R> struct OpVk {
  static constexpr const char *kName = "hartree kernel";
  typedef typename Tr<R>::C C;
  C *wb;
  const R *vk;
  int64_t zdiv;  // nxb*nyb; loads outside z in [zlo, zhi) read zero
  int zlo, zhi;
  int64_t bs = 0;  // batch stride of wb
  static constexpr bool kMid = true;
  __device__ C load(int b, int64_t g) const {
    const int z = (int)(g / zdiv);
    if (z < zlo || z >= zhi) {
      C v;
      v.x = 0;
      v.y = 0;
      return v;
    }
    return wb[b * bs + g];
  }
  __device__ void store(int b, int64_t g, C v) const { wb[b * bs + g] = v; }
  __device__ double line(int64_t) const { return 0.0; }
  __device__ C mid(int, int64_t g, double, int, C v) const {
    const R k = vk[g];
    v.x *= k;
    v.y *= k;
    return v;
  }
};

template <typename R> struct OpCrop {
  typedef typename Tr<R>::C C;
  Embed e;
  const C *wb;
  double *v0, *v1;
  double cn, nbd;
  int64_t bs = 0;  // batch stride of wb
  int pair = 0;    // 1: batch b holds the potential of v0 (b = 0) or v1 (b = 1); 2: of v0 + b ss
  int64_t ss = 0;  // output stride of pair mode 2
  static constexpr bool kMid = false;
  __device__ C load(int b, int64_t g) const { return wb[b * bs + g]; }
  __device__ void store(int b, int64_t g, C v) const {
    int64_t i;
    if (!e.inner(g, i)) return;
    if (pair) {
      (pair == 2 ? v0 + b * ss : (b ? v1 : v0))[i] = ((double)v.x * cn) * nbd;
      return;
    }
    v0[i] = ((double)v.x * cn) * nbd;  // rconv :29, get_vcon :20
    if (v1) v1[i] = ((double)v.y * cn) * nbd;
  }
  __device__ double line(int64_t) const { return 0.0; }
  __device__ C mid(int, int64_t, double, int, C v) const { return v; }
};

template <typename R> struct VkOf;
template <> struct VkOf<double> {
  static const double *get(const opaw_ctx *c) { return c->d_vk; }
};
template <> struct VkOf<float> {
  static const float *get(const opaw_ctx *c) { return c->d_vk_f; }
};

template <typename R>
int hartree_t(opaw_ctx *c, const double *dens0, const double *dens1, double *vh0, double *vh1) {
  typedef typename Tr<R>::C C;
  OPAW_CHECK(ensure(c->work[3], sizeof(C) * c->nnb));
  C *wb = (C *)c->work[3].p;
  Embed e{c->nx, c->ny, c->nz, c->nxb, c->nyb, c->nxb / 2 - c->nx / 2, c->nyb / 2 - c->ny / 2, c->nzb / 2 - c->nz / 2};
  Dims3 d{c->nxb, c->nyb, c->nzb};
  const double nbd = (double)c->nxb * (double)c->nyb * (double)c->nzb;
  // The source fills only the inner nx x ny x nz block and only that block
  // is kept: x passes need the lines with y and z inside it, y passes the
  // planes with z inside it (3 of the 5 passes shrink to 1/4 or 1/2).  Lines
  // left unwritten are masked to zero where a later pass reads them.
  const LineSub xlines{e.my, c->ny, e.mz, c->nz}, ylines{0, c->nyb, e.mz, c->nz};
  OpEmbed<R> emb{e, dens0, dens1, wb};
  OpMasked<C> yfwd{wb, (int64_t)c->nxb, c->nyb, e.my, e.my + c->ny};
  OpCopy<C> inplace{wb, wb, c->nnb};
  OpVk<R> vkop{wb, VkOf<R>::get(c), (int64_t)c->nxb * c->nyb, e.mz, e.mz + c->nz};
  OpCrop<R> crop{e, wb, vh0, vh1, 1.0 / nbd, nbd};
  OPAW_CHECK((launch_axis<C, 0>(c, c->fftb.ax[0], d, 1, -1, emb, &xlines)));
  OPAW_CHECK((launch_axis<C, 1>(c, c->fftb.ax[1], d, 1, -1, yfwd, &ylines)));
  OPAW_CHECK((launch_axis<C, 2>(c, c->fftb.ax[2], d, 1, 0, vkop)));
  OPAW_CHECK((launch_axis<C, 1>(c, c->fftb.ax[1], d, 1, +1, inplace, &ylines)));
  OPAW_CHECK((launch_axis<C, 0>(c, c->fftb.ax[0], d, 1, +1, crop, &xlines)));
  return OPAW_OK;
}

// two independent real sources in one batch of two complex transforms (each
// keeps its own relative precision): vh0 from dens0, vh1 from dens1
template <typename R>
int hartree_pair_t(opaw_ctx *c, const double *dens0, const double *dens1, double *vh0, double *vh1) {
  typedef typename Tr<R>::C C;
  OPAW_CHECK(ensure(c->work[3], 2 * sizeof(C) * c->nnb));
  C *wb = (C *)c->work[3].p;
  Embed e{c->nx, c->ny, c->nz, c->nxb, c->nyb, c->nxb / 2 - c->nx / 2, c->nyb / 2 - c->ny / 2, c->nzb / 2 - c->nz / 2};
  Dims3 d{c->nxb, c->nyb, c->nzb};
  const double nbd = (double)c->nxb * (double)c->nyb * (double)c->nzb;
  const int64_t bs = c->nnb;
  const LineSub xlines{e.my, c->ny, e.mz, c->nz}, ylines{0, c->nyb, e.mz, c->nz};
  OpEmbed<R> emb{e, dens0, dens1, wb, bs, 1};
  OpMasked<C> yfwd{wb, (int64_t)c->nxb, c->nyb, e.my, e.my + c->ny, bs};
  OpCopy<C> inplace{wb, wb, bs};
  OpVk<R> vkop{wb, VkOf<R>::get(c), (int64_t)c->nxb * c->nyb, e.mz, e.mz + c->nz, bs};
  OpCrop<R> crop{e, wb, vh0, vh1, 1.0 / nbd, nbd, bs, 1};
  OPAW_CHECK((launch_axis<C, 0>(c, c->fftb.ax[0], d, 2, -1, emb, &xlines)));
  OPAW_CHECK((launch_axis<C, 1>(c, c->fftb.ax[1], d, 2, -1, yfwd, &ylines)));
  OPAW_CHECK((launch_axis<C, 2>(c, c->fftb.ax[2], d, 2, 0, vkop)));
  OPAW_CHECK((launch_axis<C, 1>(c, c->fftb.ax[1], d, 2, +1, inplace, &ylines)));
  OPAW_CHECK((launch_axis<C, 0>(c, c->fftb.ax[0], d, 2, +1, crop, &xlines)));
  return OPAW_OK;
}
template int hartree_pair_t<float>(opaw_ctx *, const double *, const double *, double *, double *);

// nsrc independent real sources (src + b nn) in one batch of complex
// transforms, each with its own relative precision: vh + b nn
template <typename R>
int hartree_batch_t(opaw_ctx *c, const double *src, int nsrc, double *vh) {
  typedef typename Tr<R>::C C;
  if (nsrc <= 0) return OPAW_OK;
  OPAW_CHECK(ensure(c->work[3], (size_t)nsrc * sizeof(C) * c->nnb));
  C *wb = (C *)c->work[3].p;
  Embed e{c->nx, c->ny, c->nz, c->nxb, c->nyb, c->nxb / 2 - c->nx / 2, c->nyb / 2 - c->ny / 2, c->nzb / 2 - c->nz / 2};
  Dims3 d{c->nxb, c->nyb, c->nzb};
  const double nbd = (double)c->nxb * (double)c->nyb * (double)c->nzb;
  const int64_t bs = c->nnb;
  const LineSub xlines{e.my, c->ny, e.mz, c->nz}, ylines{0, c->nyb, e.mz, c->nz};
  OpEmbed<R> emb{e, src, nullptr, wb, bs, 2, c->nn};
  OpMasked<C> yfwd{wb, (int64_t)c->nxb, c->nyb, e.my, e.my + c->ny, bs};
  OpCopy<C> inplace{wb, wb, bs};
  OpVk<R> vkop{wb, VkOf<R>::get(c), (int64_t)c->nxb * c->nyb, e.mz, e.mz + c->nz, bs};
  OpCrop<R> crop{e, wb, vh, nullptr, 1.0 / nbd, nbd, bs, 2, c->nn};
  OPAW_CHECK((launch_axis<C, 0>(c, c->fftb.ax[0], d, nsrc, -1, emb, &xlines)));
  OPAW_CHECK((launch_axis<C, 1>(c, c->fftb.ax[1], d, nsrc, -1, yfwd, &ylines)));
  OPAW_CHECK((launch_axis<C, 2>(c, c->fftb.ax[2], d, nsrc, 0, vkop)));
  OPAW_CHECK((launch_axis<C, 1>(c, c->fftb.ax[1], d, nsrc, +1, inplace, &ylines)));
  OPAW_CHECK((launch_axis<C, 0>(c, c->fftb.ax[0], d, nsrc, +1, crop, &xlines)));
  return OPAW_OK;
}
template int hartree_batch_t<float>(opaw_ctx *, const double *, int, double *);
template int hartree_batch_t<double>(opaw_ctx *, const double *, int, double *);
template int hartree_pair_t<double>(opaw_ctx *, const double *, const double *, double *, double *);

int hartree(opaw_ctx *c, const double *dens0, const double *dens1, double *vh0, double *vh1) {
  return hartree_t<double>(c, dens0, dens1, vh0, vh1);
}

// ------------------------------------------------------ LDA (A17) --
// Slater exchange + Perdew-Wang 1992 correlation (PRB 45, 13244, unpolarised
// parameters of Table I); zero below the density threshold.
__device__ __forceinline__ double vxc_point(double n) {
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

__global__ void k_vxc(const double *__restrict__ dens, const double *__restrict__ core, double *__restrict__ vxc,
                      int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) vxc[i] = vxc_point(core ? dens[i] + core[i] : dens[i]);
}

int vxc_points(opaw_ctx *c, const double *dens, double *vxc, int64_t n) {
  k_vxc<<<grid1(n, 256), 256, 0, c->stream>>>(dens, nullptr, vxc, n);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

// rconv on an arbitrary grid (library_vh_convolution_r8_r2c.f90:13-31): the
// r2c/c2r pair of the reference equals a complex transform of the real input
// whose inverse is real when bk(k) = bk(-k)
struct OpBk {
  double2 *a;
  const double *bk;
  static constexpr bool kMid = true;
  __device__ double2 load(int, int64_t g) const { return a[g]; }
  __device__ void store(int, int64_t g, double2 v) const { a[g] = v; }
  __device__ double line(int64_t) const { return 0.0; }
  __device__ double2 mid(int, int64_t g, double, int, double2 v) const {
    const double k = bk[g];
    return make_double2(v.x * k, v.y * k);
  }
};
struct OpReal {
  const double2 *a;
  double *out;
  double cn;
  static constexpr bool kMid = false;
  __device__ double2 load(int, int64_t g) const { return a[g]; }
  __device__ void store(int, int64_t g, double2 v) const { out[g] = v.x * cn; }
  __device__ double line(int64_t) const { return 0.0; }
  __device__ double2 mid(int, int64_t, double, int, double2 v) const { return v; }
};

int rconv_device(opaw_ctx *c, double2 *a, const double *bk, double *gout, int n0, int n1, int n2) {
  Dims3 d{n0, n1, n2};
  OpCopy<double2> inplace{a, a, (int64_t)n0 * n1 * n2};
  OpBk mid{a, bk};
  OpReal fin{a, gout, 1.0 / ((double)n0 * (double)n1 * (double)n2)};
  OPAW_CHECK((launch_axis<double2, 0>(c, c->fft.ax[0], d, 1, -1, inplace)));
  OPAW_CHECK((launch_axis<double2, 1>(c, c->fft.ax[1], d, 1, -1, inplace)));
  OPAW_CHECK((launch_axis<double2, 2>(c, c->fft.ax[2], d, 1, 0, mid)));
  OPAW_CHECK((launch_axis<double2, 1>(c, c->fft.ax[1], d, 1, +1, inplace)));
  OPAW_CHECK((launch_axis<double2, 0>(c, c->fft.ax[0], d, 1, +1, fin)));
  return OPAW_OK;
}

// v_ks = v_H + v_xc + v_loc (tddft_pot.f90:46-47), FP32 twin alongside
__global__ void k_vks(const double *__restrict__ vh, const double *__restrict__ vxc, const double *__restrict__ vloc,
                      const double *__restrict__ vhmean, double *__restrict__ vks, float *__restrict__ vksf, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double h = vh[i];
  if (vhmean) h -= *vhmean;
  const double v = h + vxc[i] + vloc[i];
  vks[i] = v;
  vksf[i] = (float)v;
}

// ------------------------------------------------ density (A10) --
template <typename C>
__global__ void k_density(const C *__restrict__ psi, int norb, int64_t nn, double *__restrict__ dens) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nn) return;
  typedef decltype(psi[0].x) RR;
  typedef typename std::remove_const<typename std::remove_reference<RR>::type>::type R;
  double acc = 0;
  // sums of up to 16 orbitals in the orbital precision, added in FP64
  for (int o0 = 0; o0 < norb; o0 += 16) {
    R part = 0;
    const int o1 = min(norb, o0 + 16);
    for (int o = o0; o < o1; o++) {
      const C z = psi[(int64_t)o * nn + i];
      part += z.x * z.x + z.y * z.y;
    }
    acc += (double)part;
  }
  dens[i] = 2.0 * acc;  // tddft_dens.f90:73
}

// ------------------------------------------------- rho_ij (A8) --
// one warp per entry (atom, i, j); lanes stride over the orbitals, a
// butterfly reduction in fixed order adds them (bit-reproducible)
__device__ __forceinline__ double warp_allsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void k_rhoij(const double2 *__restrict__ coef, int norb, int ns, int nd, const int *__restrict__ dslot,
                        const int64_t *__restrict__ soff, const int64_t *__restrict__ doff,
                        const int *__restrict__ ms, double *__restrict__ rho) {
  const int t = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (t >= nd) return;  // whole warps
  const int a = dslot[t];
  const int m = ms[a];
  const int loc = t - (int)doff[a];
  const int i = loc % m, j = loc / m;
  double acc = 0;
  for (int o = lane; o < norb; o += 32) {
    const double2 ci = coef[(int64_t)o * ns + soff[a] + i], cj = coef[(int64_t)o * ns + soff[a] + j];
    acc += 2.0 * (ci.x * cj.x + ci.y * cj.y);  // Re(conj(c_i) c_j) * 2, tddft_rhoij.f90:35
  }
  acc = warp_allsum(acc);
  if (lane == 0) rho[t] = acc;
}

// ---------------------------------------------------- nhat (A11) --
// w[a][lm] = sum_ij rho_a(i,j) Q_a(lm,i,j)
__global__ void k_nhat_w(const double *__restrict__ rho, const double *__restrict__ q, const int *__restrict__ ms,
                         const int *__restrict__ nlm, const int64_t *__restrict__ doff,
                         const int64_t *__restrict__ qoff, int natom, int nlmmax, double *__restrict__ w) {
  const int t = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);  // warp per (atom, lm)
  const int lane = threadIdx.x & 31;
  if (t >= natom * nlmmax) return;
  const int a = t / nlmmax, l = t % nlmmax;
  const int L = nlm[a], m = ms[a];
  if (l >= L) {
    if (lane == 0) w[t] = 0;
    return;
  }
  const double *R = rho + doff[a];
  const double *Q = q + qoff[a];
  double acc = 0;
  for (int e = lane; e < m * m; e += 32) acc += R[e] * Q[l + (int64_t)L * e];  // e = i + m j
  acc = warp_allsum(acc);
  if (lane == 0) w[t] = acc;
}

__global__ void k_nhat(const int *__restrict__ cpt, const int *__restrict__ cstart, const int *__restrict__ catom,
                       const int *__restrict__ cig, int ncu, const double *__restrict__ w, int nlmmax,
                       const int *__restrict__ ngrid, const int *__restrict__ nlm, const int64_t *__restrict__ g3off,
                       const double *__restrict__ g3d, double *__restrict__ nhat) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= ncu) return;
  double acc = 0;
  for (int e = cstart[u]; e < cstart[u + 1]; e++) {
    const int a = catom[e], ig = cig[e];
    const int L = nlm[a], ng = ngrid[a];
    const double *G = g3d + g3off[a];
    for (int l = 0; l < L; l++) acc += w[a * nlmmax + l] * G[ig + (int64_t)ng * l];
  }
  nhat[cpt[u]] = acc;
}

// fixed-grid partial sums of two arrays (for the renormalisation)
__global__ void k_sum2(const double *__restrict__ a, const double *__restrict__ b, int64_t n, double *__restrict__ part) {
  __shared__ double sh[8];
  double sa = 0, sb = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    sa += a[i];
    if (b) sb += b[i];
  }
  sa = block_sum(sa, sh);
  sb = block_sum(sb, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = sa;
    part[2 * blockIdx.x + 1] = sb;
  }
}

// factor = rnel / ((sum nhat + sum dens) * dv)  (nhat.f90:32-37); also the mean of a
__global__ void k_renorm_factor(const double *__restrict__ part, int nb, double dv, double rnel, int64_t n,
                                double *__restrict__ out) {
  __shared__ double sh[8];
  const double sa = block_sum_seq(part, nb, 2, sh);
  const double sb = block_sum_seq(part + 1, nb, 2, sh);
  if (threadIdx.x != 0) return;
  out[0] = rnel / (sa * dv + sb * dv);
  out[1] = sa / (double)n;
}

__global__ void k_scale2(double *__restrict__ a, double *__restrict__ b, int64_t n, const double *__restrict__ f) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double s = *f;
  a[i] *= s;
  b[i] *= s;
}

// --------------------------------------------------- D_ij (A16) --
// prod[a][lm] = dv sum_g (v_ks - v_xc)(r_g) g_lm(r_g): the potential of
// Dhat_ij without the XC part, as pawdij builds it when the compensation
// charge is not in the XC density (usexcnhat = 0, the value libpaw_mod.f90
// sets: libpaw/4_m_pawdij.F90:375-385 takes vtrial - vxc); vxc may be null
__global__ void k_dhat_prod(const double *__restrict__ vks, const double *__restrict__ vxc, const int *__restrict__ gpt,
                            const int64_t *__restrict__ goff, const int *__restrict__ ngrid,
                            const int *__restrict__ nlm, const int64_t *__restrict__ g3off,
                            const double *__restrict__ g3d, int nlmmax, double dv, double *__restrict__ prod) {
  __shared__ double sh[8];
  const int a = blockIdx.x;
  const int L = nlm[a], ng = ngrid[a];
  const double *G = g3d + g3off[a];
  const int *pts = gpt + goff[a];
  for (int l = 0; l < nlmmax; l++) {
    double acc = 0;
    if (l < L)
      for (int ig = threadIdx.x; ig < ng; ig += blockDim.x) {
        const int gp = pts[ig];
        acc += (vxc ? vks[gp] - vxc[gp] : vks[gp]) * G[ig + (int64_t)ng * l];
      }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) prod[a * nlmmax + l] = acc * dv;
  }
}

__global__ void k_dij(const double *__restrict__ prod, int nlmmax, const double *__restrict__ rho,
                      const double *__restrict__ q, const double *__restrict__ d0, const double *__restrict__ E,
                      const int *__restrict__ ms, const int *__restrict__ nlm, const int64_t *__restrict__ doff,
                      const int64_t *__restrict__ qoff, const int64_t *__restrict__ eoff,
                      const int *__restrict__ dslot, int nd, double dmax, const double *__restrict__ dxc,
                      double *__restrict__ dij) {
  const int t = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);  // warp per entry
  const int lane = threadIdx.x & 31;
  if (t >= nd) return;
  const int a = dslot[t];
  const int m = ms[a], L = nlm[a];
  const int loc = t - (int)doff[a];
  const int i = loc % m, j = loc / m;
  if (i < j) return;  // lower triangle computed, mirrored (get_dij.f90:140-146)
  const double *R = rho + doff[a];
  const double *Ea = E + eoff[a];
  const double *Q = q + qoff[a];
  double d = 0;
  for (int e = lane; e < m * m; e += 32)  // e = k + m l2: sum_kl E[i,j,k,l] rho_kl
    d += Ea[i + m * (j + (int64_t)m * e)] * R[e];
  for (int l = lane; l < L; l += 32) d += prod[a * nlmmax + l] * Q[l + L * (i + m * j)];
  d = warp_allsum(d);
  if (lane != 0) return;
  d += d0[doff[a] + i + m * j];
  if (dxc) d += dxc[doff[a] + i + m * j];  // on-site XC (pawdijxcm)
  if (dmax > 0 && fabs(d) > dmax) d = d / fabs(d) * dmax;  // get_dij.f90:144
  dij[doff[a] + i + m * j] = d;
  dij[doff[a] + j + m * i] = d;
}

// ------------------------------------------------------ the chain --
static int rhoij_from_coef(opaw_ctx *c, int set, const double2 *coef, int norb) {
  if (c->nd == 0) return OPAW_OK;
  k_rhoij<<<grid1((int64_t)c->nd * 32, 256), 256, 0, c->stream>>>(coef, norb, c->ns, c->nd, c->d_dslot_atom, c->d_soff, c->d_doff,
                                                    c->d_ms, c->d_rhoij[set]);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

template <typename R> static int density_of(opaw_ctx *c, int set, const typename Tr<R>::C *psit, int norb) {
  k_density<typename Tr<R>::C><<<grid1(c->nn, 256), 256, 0, c->stream>>>(psit, norb, c->nn, c->d_dens[set]);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

static double *red_scratch(opaw_ctx *c) { return (double *)c->red.p; }

int nhat_step(opaw_ctx *c, int set) {
  OPAW_CHECK(ensure(c->red, sizeof(double) * (2 * kRedBlocks + 64 + 64 * (size_t)(c->natom + 1) * 2)));
  double *part = red_scratch(c);
  double *fac = part + 2 * kRedBlocks;
  double *w = fac + 64;
  OPAW_CUDA(cudaMemsetAsync(c->d_nhat[set], 0, sizeof(double) * c->nn, c->stream));
  if (c->natom > 0 && c->nlmmax > 0) {
    const int nt = c->natom * c->nlmmax;
    k_nhat_w<<<grid1((int64_t)nt * 32, 256), 256, 0, c->stream>>>(c->d_rhoij[set], c->d_qijlm, c->d_ms, c->d_nlm, c->d_doff,
                                                     c->d_qoff, c->natom, c->nlmmax, w);
    c->launches++;
    if (c->ncunion > 0) {
      k_nhat<<<grid1(c->ncunion, 256), 256, 0, c->stream>>>(c->d_cpt, c->d_cstart, c->d_catom, c->d_cig, c->ncunion,
                                                            w, c->nlmmax, c->d_ngrid, c->d_nlm, c->d_g3off, c->d_g3d,
                                                            c->d_nhat[set]);
      c->launches++;
    }
  }
  k_sum2<<<kRedBlocks, 256, 0, c->stream>>>(c->d_nhat[set], c->d_dens[set], c->nn, part);
  k_renorm_factor<<<1, 256, 0, c->stream>>>(part, kRedBlocks, c->dv, c->rnel, c->nn, fac);
  k_scale2<<<grid1(c->nn, 256), 256, 0, c->stream>>>(c->d_nhat[set], c->d_dens[set], c->nn, fac);
  c->launches += 3;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

__global__ void k_add(const double *a, const double *b, double *o, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) o[i] = a[i] + b[i];
}

int vks_step(opaw_ctx *c, int set, int fp32_hartree) {
  OPAW_CHECK(ensure(c->work[2], sizeof(double) * c->nn * 2));
  double *t = (double *)c->work[2].p;  // n~ + n^ for the Hartree solve
  k_vxc<<<grid1(c->nn, 256), 256, 0, c->stream>>>(c->d_dens[set], c->d_ncoret, c->d_vxc[set], c->nn);
  c->launches++;
  OPAW_CHECK(ensure(c->red, sizeof(double) * (2 * kRedBlocks + 64 + 64 * (size_t)(c->natom + 1) * 2)));
  // t = dens + nhat (tddft_pot.f90:39)
  k_add<<<grid1(c->nn, 256), 256, 0, c->stream>>>(c->d_dens[set], c->d_nhat[set], t, c->nn);
  c->launches++;
  if (fp32_hartree) OPAW_CHECK(hartree_t<float>(c, t, nullptr, c->d_vh[set], nullptr));
  else OPAW_CHECK(hartree_t<double>(c, t, nullptr, c->d_vh[set], nullptr));
  const double *mean = nullptr;
  if (c->periodic) {
    double *part = red_scratch(c);
    double *fac = part + 2 * kRedBlocks;
    k_sum2<<<kRedBlocks, 256, 0, c->stream>>>(c->d_vh[set], nullptr, c->nn, part);
    k_renorm_factor<<<1, 256, 0, c->stream>>>(part, kRedBlocks, c->dv, 1.0, c->nn, fac);
    c->launches += 2;
    mean = fac + 1;
  }
  k_vks<<<grid1(c->nn, 256), 256, 0, c->stream>>>(c->d_vh[set], c->d_vxc[set], c->d_vloc, mean, c->d_vks[set],
                                                  c->d_vks_f[set], c->nn);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

int dij_step(opaw_ctx *c, int set) {
  if (c->natom == 0) return OPAW_OK;
  OPAW_CHECK(ensure(c->red, sizeof(double) * (2 * kRedBlocks + 64 + 64 * (size_t)(c->natom + 1) * 2)));
  double *prod = red_scratch(c) + 2 * kRedBlocks + 64 + 64 * (size_t)(c->natom + 1);
  const int L = c->nlmmax > 0 ? c->nlmmax : 1;
  k_dhat_prod<<<c->natom, 256, 0, c->stream>>>(c->d_vks[set], c->d_vxc[set], c->d_gpt, c->d_goff, c->d_ngrid,
                                                c->d_nlm, c->d_g3off, c->d_g3d, L, c->dv, prod);
  OPAW_CHECK(onsite_xc_of(c, c->d_rhoij[set], c->oxc_dxc));
  k_dij<<<grid1((int64_t)c->nd * 32, 256), 256, 0, c->stream>>>(prod, L, c->d_rhoij[set], c->d_qijlm, c->d_dij0, c->d_eijkl,
                                                  c->d_ms, c->d_nlm, c->d_doff, c->d_qoff, c->d_eoff,
                                                  c->d_dslot_atom, c->nd, c->dij_max,
                                                  c->oxc_on ? c->oxc_dxc : nullptr, c->d_dij[set]);
  c->launches += 2;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

// ---- pointer-based pieces (used by the perturbation-difference propagation)
int rhoij_of(opaw_ctx *c, const double2 *coef, int norb, double *out) {
  if (c->nd == 0) return OPAW_OK;
  k_rhoij<<<grid1((int64_t)c->nd * 32, 256), 256, 0, c->stream>>>(coef, norb, c->ns, c->nd, c->d_dslot_atom, c->d_soff, c->d_doff,
                                                    c->d_ms, out);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

template <typename R> int density_raw(opaw_ctx *c, const typename Tr<R>::C *psit, int norb, double *out) {
  k_density<typename Tr<R>::C><<<grid1(c->nn, 256), 256, 0, c->stream>>>(psit, norb, c->nn, out);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}
template int density_raw<float>(opaw_ctx *, const float2 *, int, double *);
template int density_raw<double>(opaw_ctx *, const double2 *, int, double *);

// compensation charge of rho_ij without the renormalisation (nhat.f90:13-28)
int nhat_raw_of(opaw_ctx *c, const double *rhoij, double *out) {
  OPAW_CHECK(ensure(c->red, sizeof(double) * (2 * kRedBlocks + 64 + 64 * (size_t)(c->natom + 1) * 2)));
  double *w = red_scratch(c) + 2 * kRedBlocks + 64;
  OPAW_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * c->nn, c->stream));
  if (c->natom > 0 && c->nlmmax > 0) {
    const int nt = c->natom * c->nlmmax;
    k_nhat_w<<<grid1((int64_t)nt * 32, 256), 256, 0, c->stream>>>(rhoij, c->d_qijlm, c->d_ms, c->d_nlm, c->d_doff, c->d_qoff,
                                                     c->natom, c->nlmmax, w);
    c->launches++;
    if (c->ncunion > 0) {
      k_nhat<<<grid1(c->ncunion, 256), 256, 0, c->stream>>>(c->d_cpt, c->d_cstart, c->d_catom, c->d_cig, c->ncunion,
                                                            w, c->nlmmax, c->d_ngrid, c->d_nlm, c->d_g3off, c->d_g3d,
                                                            out);
      c->launches++;
    }
  }
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

// partial sums of a and b (kRedBlocks x 2 doubles)
int sums2(opaw_ctx *c, const double *a, const double *b, double *part) {
  k_sum2<<<kRedBlocks, 256, 0, c->stream>>>(a, b, c->nn, part);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

int vxc_of(opaw_ctx *c, const double *dens, const double *core, double *out) {
  k_vxc<<<grid1(c->nn, 256), 256, 0, c->stream>>>(dens, core, out, c->nn);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

// dxc_pre: the on-site XC term already computed for this rho_ij (the mixed
// step computes it on the side stream), else it is computed here
int dij_of(opaw_ctx *c, const double *rhoij, const double *vks, const double *vxc, double *out,
           const double *dxc_pre) {
  if (c->natom == 0) return OPAW_OK;
  OPAW_CHECK(ensure(c->red, sizeof(double) * (2 * kRedBlocks + 64 + 64 * (size_t)(c->natom + 1) * 2)));
  double *prod = red_scratch(c) + 2 * kRedBlocks + 64 + 64 * (size_t)(c->natom + 1);
  const int L = c->nlmmax > 0 ? c->nlmmax : 1;
  k_dhat_prod<<<c->natom, 256, 0, c->stream>>>(vks, vxc, c->d_gpt, c->d_goff, c->d_ngrid, c->d_nlm, c->d_g3off, c->d_g3d, L,
                                                c->dv, prod);
  if (!dxc_pre) OPAW_CHECK(onsite_xc_of(c, rhoij, c->oxc_dxc));
  const double *dxc = c->oxc_on ? (dxc_pre ? dxc_pre : c->oxc_dxc) : nullptr;
  k_dij<<<grid1((int64_t)c->nd * 32, 256), 256, 0, c->stream>>>(prod, L, rhoij, c->d_qijlm, c->d_dij0, c->d_eijkl, c->d_ms, c->d_nlm,
                                                  c->d_doff, c->d_qoff, c->d_eoff, c->d_dslot_atom, c->nd, c->dij_max,
                                                  dxc, out);
  c->launches += 2;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

template int hartree_t<float>(opaw_ctx *, const double *, const double *, double *, double *);
template int hartree_t<double>(opaw_ctx *, const double *, const double *, double *, double *);

// rebuild from orbitals psi_bar (device, dtype) of `set`: psi~ = S^-1/2 psi_bar,
// then rho_ij, density, nhat, v_ks, D_ij
template <typename R> int rebuild_from(opaw_ctx *c, int set, const typename Tr<R>::C *psibar, int norb) {
  typedef typename Tr<R>::C C;
  OPAW_CHECK(ensure(c->work[4], sizeof(C) * (size_t)c->nn * norb));
  C *pt = (C *)c->work[4].p;
  OPAW_CHECK(sn_apply<R>(c, -0.5, psibar, pt, norb));  // ncpaw_make_hamiltonian.f90:119-122
  OPAW_CHECK(ensure(c->coef[0], sizeof(double2) * (size_t)c->ns * norb + 16));
  double2 *co = (double2 *)c->coef[0].p;
  OPAW_CHECK(gather<R>(c, 0, pt, norb, co));
  OPAW_CHECK(rhoij_from_coef(c, set, co, norb));  // :125
  OPAW_CHECK(density_of<R>(c, set, pt, norb));    // :126
  OPAW_CHECK(nhat_step(c, set));                  // :127
  OPAW_CHECK(vks_step(c, set, sizeof(R) == 4));    // :128 (FP32 Hartree on the mixed path)
  OPAW_CHECK(dij_step(c, set));                   // :129
  return OPAW_OK;
}
template int rebuild_from<float>(opaw_ctx *, int, const float2 *, int);
template int rebuild_from<double>(opaw_ctx *, int, const double2 *, int);

template <typename R> int rhoij_density_from(opaw_ctx *c, int set, const typename Tr<R>::C *psit, int norb, int what) {
  OPAW_CHECK(ensure(c->coef[0], sizeof(double2) * (size_t)c->ns * norb + 16));
  double2 *co = (double2 *)c->coef[0].p;
  if (what == 0) {
    OPAW_CHECK(gather<R>(c, 0, psit, norb, co));
    OPAW_CHECK(rhoij_from_coef(c, set, co, norb));
  } else {
    OPAW_CHECK(density_of<R>(c, set, psit, norb));
  }
  return OPAW_OK;
}
template int rhoij_density_from<float>(opaw_ctx *, int, const float2 *, int, int);
template int rhoij_density_from<double>(opaw_ctx *, int, const double2 *, int, int);

}  // namespace opaw

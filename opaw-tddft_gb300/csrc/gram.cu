// gram.cu — orbital Gram matrices and subspace rotations (the "sij" / Gram
// row of the path): G = dv A^H B (orthog_phi.f90:76-111 Gram, diag.f90:78
// subspace Hamiltonian), Psi <- Psi M (orthog_phi.f90:148-156, diag.f90:118),
// and the canonical orthogonalisation of the resident orbitals
// (orthog_phi.f90, h_type = 1: G = V diag(l) V^H, Psi <- Psi V l^-1/2).
// The small Hermitian eigenproblem runs on the host (cyclic complex Jacobi,
// deterministic); the reference uses EISPACK `ch` (library_1_matrix_all.f90).
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "fft.cuh"

namespace opaw {

constexpr int kGramTile = 16;   // 16 x 16 output tile per CTA
constexpr int kGramK = 32;      // grid points per shared-memory sub-block
constexpr int kGramSplit = 152; // K splits (one wave of CTAs per output tile row)

// part[z][i][j] = sum over the z-th slice of the grid of conj(A_i) B_j,
// FP32 (or FP64) products summed per 32-point sub-block, FP64 across them
template <typename R>
__global__ void __launch_bounds__(256) k_gram(const typename Tr<R>::C *__restrict__ A, int na,
                                              const typename Tr<R>::C *__restrict__ B, int nb, int64_t nn,
                                              double2 *__restrict__ part, int herm) {
  typedef typename Tr<R>::C C;
  __shared__ C sa[kGramTile][kGramK + 1];
  __shared__ C sb[kGramTile][kGramK + 1];
  const int ti = threadIdx.x / kGramTile, tj = threadIdx.x % kGramTile;
  const int i0 = blockIdx.x * kGramTile, j0 = blockIdx.y * kGramTile;
  if (herm && i0 > j0) return;  // Hermitian result: the tiles below the diagonal are mirrored
  const int z = blockIdx.z, nz = gridDim.z;
  const int64_t k0 = nn * z / nz, k1 = nn * (z + 1) / nz;
  double accx = 0, accy = 0;
  for (int64_t kb = k0; kb < k1; kb += kGramK) {
    for (int e = threadIdx.x; e < kGramTile * kGramK; e += 256) {
      const int r = e / kGramK, k = e % kGramK;
      const int64_t g = kb + k;
      C va, vb;
      va.x = va.y = vb.x = vb.y = 0;
      if (g < k1) {
        if (i0 + r < na) va = A[(int64_t)(i0 + r) * nn + g];
        if (j0 + r < nb) vb = B[(int64_t)(j0 + r) * nn + g];
      }
      sa[r][k] = va;
      sb[r][k] = vb;
    }
    __syncthreads();
    R sx = 0, sy = 0;
#pragma unroll 8
    for (int k = 0; k < kGramK; k++) {
      const C a = sa[ti][k], b = sb[tj][k];
      sx += a.x * b.x + a.y * b.y;  // conj(a) b
      sy += a.x * b.y - a.y * b.x;
    }
    accx += (double)sx;
    accy += (double)sy;
    __syncthreads();
  }
  const int i = i0 + ti, j = j0 + tj;
  if (i < na && j < nb) part[((int64_t)z * na + i) * nb + j] = make_double2(accx, accy);
}

// G[i + na j] = dv sum_z part[z][i][j] (fixed order); herm: the entries of
// tiles below the diagonal are the conjugates of their mirror images
__global__ void k_gram_reduce(const double2 *__restrict__ part, int nz, int na, int nb, double dv,
                              double2 *__restrict__ G, int herm) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= na * nb) return;
  int i = t / nb, j = t % nb;
  bool cj = false;
  if (herm && (i / kGramTile) > (j / kGramTile)) {
    const int q = i;
    i = j;
    j = q;
    cj = true;
  }
  double sx = 0, sy = 0;
  for (int z = 0; z < nz; z++) {
    const double2 v = part[((int64_t)z * na + i) * nb + j];
    sx += v.x;
    sy += v.y;
  }
  if (cj) G[j + (int64_t)na * i] = make_double2(sx * dv, -sy * dv);
  else G[i + (int64_t)na * j] = make_double2(sx * dv, sy * dv);
}

// out_j = sum_i A_i M[i + na j]: 256 grid points x 16 output orbitals per CTA
template <typename R>
__global__ void __launch_bounds__(256) k_rotate(const typename Tr<R>::C *__restrict__ A, int na,
                                                const double2 *__restrict__ M, int nb, int64_t nn,
                                                typename Tr<R>::C *__restrict__ out) {
  typedef typename Tr<R>::C C;
  __shared__ C sm[kGramTile][kGramTile];
  const int64_t g = blockIdx.x * (int64_t)256 + threadIdx.x;
  const int j0 = blockIdx.y * kGramTile;
  R ax[kGramTile], ay[kGramTile];
#pragma unroll
  for (int jj = 0; jj < kGramTile; jj++) ax[jj] = ay[jj] = 0;
  for (int i0 = 0; i0 < na; i0 += kGramTile) {
    {
      const int r = threadIdx.x / kGramTile, q = threadIdx.x % kGramTile;
      C v;
      v.x = v.y = 0;
      if (i0 + r < na && j0 + q < nb) {
        const double2 d = M[(i0 + r) + (int64_t)na * (j0 + q)];
        v.x = (R)d.x;
        v.y = (R)d.y;
      }
      sm[r][q] = v;
    }
    __syncthreads();
    if (g < nn) {
      for (int ii = 0; ii < kGramTile && i0 + ii < na; ii++) {
        const C a = A[(int64_t)(i0 + ii) * nn + g];
#pragma unroll
        for (int jj = 0; jj < kGramTile; jj++) {
          const C m = sm[ii][jj];
          ax[jj] += a.x * m.x - a.y * m.y;
          ay[jj] += a.x * m.y + a.y * m.x;
        }
      }
    }
    __syncthreads();
  }
  if (g < nn) {
#pragma unroll
    for (int jj = 0; jj < kGramTile; jj++) {
      if (j0 + jj < nb) {
        C v;
        v.x = ax[jj];
        v.y = ay[jj];
        out[(int64_t)(j0 + jj) * nn + g] = v;
      }
    }
  }
}

template <typename R>
int gram_t(opaw_ctx *c, const typename Tr<R>::C *A, int na, const typename Tr<R>::C *B, int nb, double2 *Gdev,
           int herm = 0) {
  OPAW_CHECK(ensure(c->gram, sizeof(double2) * (size_t)kGramSplit * na * nb + 16));
  double2 *part = (double2 *)c->gram.p;
  dim3 grid((na + kGramTile - 1) / kGramTile, (nb + kGramTile - 1) / kGramTile, kGramSplit);
  k_gram<R><<<grid, 256, 0, c->stream>>>(A, na, B, nb, c->nn, part, herm);
  k_gram_reduce<<<grid1((int64_t)na * nb, 128), 128, 0, c->stream>>>(part, kGramSplit, na, nb, c->dv, Gdev, herm);
  c->launches += 2;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

template <typename R>
int rotate_t(opaw_ctx *c, const typename Tr<R>::C *A, int na, const double2 *Mdev, int nb, typename Tr<R>::C *out) {
  dim3 grid(grid1(c->nn, 256), (nb + kGramTile - 1) / kGramTile);
  k_rotate<R><<<grid, 256, 0, c->stream>>>(A, na, Mdev, nb, c->nn, out);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

// ---- complex128 contractions in double-FP32 arithmetic --------------------
// GB300's FP64 rate is 1/64 of its FP32 rate, so the complex128 Gram matrices
// and rotations of the eigensolver run on FP32 pairs: every complex128 input
// is split once into hi + lo complex64 arrays (hi = fl32(x), lo = fl32(x -
// hi), together ~48 significant bits), each real product is formed as
// hi_x hi_y exactly (FMA error term) plus the two cross terms, and sums are
// carried as an FP32 value with a compensation term (two-sum), flushed into
// FP64 every sub-block.  Relative accuracy about 1e-14 of the sum of |terms|,
// against 1e-16 for FP64 and 1e-7 for complex64, at about five times the
// FP64 speed.

// x -> (hi, lo) complex64
__global__ void k_split_dd(const double2 *__restrict__ x, int64_t n, float2 *__restrict__ hi,
                           float2 *__restrict__ lo) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 v = x[i];
  const float hx = __double2float_rn(v.x), hy = __double2float_rn(v.y);
  hi[i] = make_float2(hx, hy);
  lo[i] = make_float2(__double2float_rn(v.x - (double)hx), __double2float_rn(v.y - (double)hy));
}

// S += (xh + xl)(yh + yl) with S = sh + sl: the product's hi part exactly
// (ph + its FMA error), the xl yl term dropped (2^-48 relative); sh keeps
// the running FP32 sum and sl collects the two-sum errors and the small terms
__device__ __forceinline__ void dd_mac(float &sh, float &sl, float xh, float xl, float yh, float yl) {
  const float ph = __fmul_rn(xh, yh);
  float pl = __fmaf_rn(xh, yh, -ph);
  pl = __fmaf_rn(xh, yl, pl);
  pl = __fmaf_rn(xl, yh, pl);
  const float s = __fadd_rn(sh, ph);
  const float v = __fsub_rn(s, sh);
  const float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, v)), __fsub_rn(ph, v));
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(e, pl));
}

// part[z][i][j] = sum over the z-th slice of conj(A_i) B_j, as k_gram
__global__ void __launch_bounds__(256) k_gram_dd(const float2 *__restrict__ Ah, const float2 *__restrict__ Al,
                                                 int na, const float2 *__restrict__ Bh,
                                                 const float2 *__restrict__ Bl, int nb, int64_t nn,
                                                 double2 *__restrict__ part, int herm) {
  __shared__ float4 sa[kGramTile][kGramK + 1];
  __shared__ float4 sb[kGramTile][kGramK + 1];
  const int ti = threadIdx.x / kGramTile, tj = threadIdx.x % kGramTile;
  const int i0 = blockIdx.x * kGramTile, j0 = blockIdx.y * kGramTile;
  if (herm && i0 > j0) return;
  const int z = blockIdx.z, nz = gridDim.z;
  const int64_t k0 = nn * z / nz, k1 = nn * (z + 1) / nz;
  double accx = 0, accy = 0;
  for (int64_t kb = k0; kb < k1; kb += kGramK) {
    for (int e = threadIdx.x; e < kGramTile * kGramK; e += 256) {
      const int r = e / kGramK, k = e % kGramK;
      const int64_t g = kb + k;
      float4 va = make_float4(0.f, 0.f, 0.f, 0.f), vb = va;
      if (g < k1) {
        if (i0 + r < na) {
          const int64_t o = (int64_t)(i0 + r) * nn + g;
          const float2 h = Ah[o], l = Al[o];
          va = make_float4(h.x, h.y, l.x, l.y);
        }
        if (j0 + r < nb) {
          const int64_t o = (int64_t)(j0 + r) * nn + g;
          const float2 h = Bh[o], l = Bl[o];
          vb = make_float4(h.x, h.y, l.x, l.y);
        }
      }
      sa[r][k] = va;
      sb[r][k] = vb;
    }
    __syncthreads();
    float xh = 0.f, xl = 0.f, yh = 0.f, yl = 0.f;
#pragma unroll 4
    for (int k = 0; k < kGramK; k++) {
      const float4 a = sa[ti][k], b = sb[tj][k];
      // conj(a) b = (ar br + ai bi) + i (ar bi - ai br)
      dd_mac(xh, xl, a.x, a.z, b.x, b.z);
      dd_mac(xh, xl, a.y, a.w, b.y, b.w);
      dd_mac(yh, yl, a.x, a.z, b.y, b.w);
      dd_mac(yh, yl, -a.y, -a.w, b.x, b.z);
    }
    accx += (double)xh + (double)xl;
    accy += (double)yh + (double)yl;
    __syncthreads();
  }
  const int i = i0 + ti, j = j0 + tj;
  if (i < na && j < nb) part[((int64_t)z * na + i) * nb + j] = make_double2(accx, accy);
}

// out_j = sum_i A_i M[i + na j] (as k_rotate), complex128 output
__global__ void __launch_bounds__(256) k_rotate_dd(const float2 *__restrict__ Ah, const float2 *__restrict__ Al,
                                                   int na, const double2 *__restrict__ M, int nb, int64_t nn,
                                                   double2 *__restrict__ out) {
  __shared__ float4 sm[kGramTile][kGramTile];
  const int64_t g = blockIdx.x * (int64_t)256 + threadIdx.x;
  const int j0 = blockIdx.y * kGramTile;
  float rh[kGramTile], rl[kGramTile], ih[kGramTile], il[kGramTile];
#pragma unroll
  for (int jj = 0; jj < kGramTile; jj++) rh[jj] = rl[jj] = ih[jj] = il[jj] = 0.f;
  for (int i0 = 0; i0 < na; i0 += kGramTile) {
    {
      const int r = threadIdx.x / kGramTile, q = threadIdx.x % kGramTile;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (i0 + r < na && j0 + q < nb) {
        const double2 d = M[(i0 + r) + (int64_t)na * (j0 + q)];
        const float hx = __double2float_rn(d.x), hy = __double2float_rn(d.y);
        v = make_float4(hx, hy, __double2float_rn(d.x - (double)hx), __double2float_rn(d.y - (double)hy));
      }
      sm[r][q] = v;
    }
    __syncthreads();
    if (g < nn) {
      for (int ii = 0; ii < kGramTile && i0 + ii < na; ii++) {
        const int64_t o = (int64_t)(i0 + ii) * nn + g;
        const float2 ah = Ah[o], al = Al[o];
#pragma unroll
        for (int jj = 0; jj < kGramTile; jj++) {
          const float4 m = sm[ii][jj];
          // a m = (ar mr - ai mi) + i (ar mi + ai mr)
          dd_mac(rh[jj], rl[jj], ah.x, al.x, m.x, m.z);
          dd_mac(rh[jj], rl[jj], -ah.y, -al.y, m.y, m.w);
          dd_mac(ih[jj], il[jj], ah.x, al.x, m.y, m.w);
          dd_mac(ih[jj], il[jj], ah.y, al.y, m.x, m.z);
        }
      }
    }
    __syncthreads();
  }
  if (g < nn) {
#pragma unroll
    for (int jj = 0; jj < kGramTile; jj++)
      if (j0 + jj < nb)
        out[(int64_t)(j0 + jj) * nn + g] = make_double2((double)rh[jj] + (double)rl[jj], (double)ih[jj] + (double)il[jj]);
  }
}

// hi / lo complex64 copies of n complex128 values into c->ddsplit at
// offset `slot` (in units of n elements of one half)
static int split_dd(opaw_ctx *c, const double2 *x, int64_t n, float2 **hi, float2 **lo, size_t *used) {
  const size_t need = *used + 2 * (size_t)n;
  OPAW_CHECK(ensure(c->ddsplit, sizeof(float2) * need + 16));
  float2 *base = (float2 *)c->ddsplit.p;
  *hi = base + *used;
  *lo = *hi + n;
  *used = need;
  k_split_dd<<<grid1(n, 256), 256, 0, c->stream>>>(x, n, *hi, *lo);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

static int gram_dd(opaw_ctx *c, const double2 *A, int na, const double2 *B, int nb, double2 *Gdev, int herm) {
  // both splits first (ensure may move the split buffer), then the pointers
  const int64_t nA = (int64_t)na * c->nn, nB = (int64_t)nb * c->nn;
  const bool same = A == B && na == nb;
  OPAW_CHECK(ensure(c->ddsplit, sizeof(float2) * 2 * (size_t)(nA + (same ? 0 : nB)) + 16));
  size_t used = 0;
  float2 *ah, *al, *bh, *bl;
  OPAW_CHECK(split_dd(c, A, nA, &ah, &al, &used));
  if (same) {
    bh = ah;
    bl = al;
  } else {
    OPAW_CHECK(split_dd(c, B, nB, &bh, &bl, &used));
  }
  OPAW_CHECK(ensure(c->gram, sizeof(double2) * (size_t)kGramSplit * na * nb + 16));
  double2 *part = (double2 *)c->gram.p;
  dim3 grid((na + kGramTile - 1) / kGramTile, (nb + kGramTile - 1) / kGramTile, kGramSplit);
  k_gram_dd<<<grid, 256, 0, c->stream>>>(ah, al, na, bh, bl, nb, c->nn, part, herm);
  k_gram_reduce<<<grid1((int64_t)na * nb, 128), 128, 0, c->stream>>>(part, kGramSplit, na, nb, c->dv, Gdev, herm);
  c->launches += 2;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

static int rotate_dd(opaw_ctx *c, const double2 *A, int na, const double2 *Mdev, int nb, double2 *out) {
  const int64_t nA = (int64_t)na * c->nn;
  size_t used = 0;
  float2 *ah, *al;
  OPAW_CHECK(ensure(c->ddsplit, sizeof(float2) * 2 * (size_t)nA + 16));
  OPAW_CHECK(split_dd(c, A, nA, &ah, &al, &used));
  dim3 grid(grid1(c->nn, 256), (nb + kGramTile - 1) / kGramTile);
  k_rotate_dd<<<grid, 256, 0, c->stream>>>(ah, al, na, Mdev, nb, c->nn, out);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

// ---- FP64 orthonormalisation on the device -------------------------------
// Cholesky of the Hermitian positive definite Gram matrix G (n x n,
// column-major) in one CTA, G = L L^H (right-looking, a column at a time),
// then M = L^-H (columns of L^-1 by forward substitution, a thread per
// column): Psi M is orthonormal since M^H G M = I.  info[0] = k + 1 when the
// k-th pivot is not positive (M is then left unset), 0 otherwise.
__global__ void __launch_bounds__(256) k_chol_inv(double2 *__restrict__ G, int n, double2 *__restrict__ M,
                                                  int *__restrict__ info) {
  __shared__ int bad;
  __shared__ double piv;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int k = 0; k < n; k++) {
    if (threadIdx.x == 0) {
      const double d = G[k + (int64_t)n * k].x;
      if (!(d > 0.0)) bad = k + 1;
      piv = d > 0.0 ? sqrt(d) : 1.0;
      G[k + (int64_t)n * k] = make_double2(piv, 0.0);
    }
    __syncthreads();
    if (bad) break;
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) {
      double2 &g = G[i + (int64_t)n * k];
      g.x /= piv;
      g.y /= piv;
    }
    __syncthreads();
    // trailing update of the lower triangle: G[i][j] -= L[i][k] conj(L[j][k])
    const int m = n - k - 1;
    for (int64_t e = threadIdx.x; e < (int64_t)m * m; e += blockDim.x) {
      const int j = k + 1 + (int)(e / m), i = k + 1 + (int)(e % m);
      if (i < j) continue;
      const double2 a = G[i + (int64_t)n * k], b = G[j + (int64_t)n * k];
      double2 &g = G[i + (int64_t)n * j];
      g.x -= a.x * b.x + a.y * b.y;
      g.y -= a.y * b.x - a.x * b.y;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) info[0] = bad;
  if (bad) return;
  // column j of X = L^-1: X[i][j] = (delta_ij - sum_{j<=q<i} L[i][q] X[q][j]) / L[i][i]; M = X^H
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    for (int i = 0; i < j; i++) M[j + (int64_t)n * i] = make_double2(0.0, 0.0);  // M[j][i] = conj(X[i][j]) = 0
    for (int i = j; i < n; i++) {
      double sx = (i == j) ? 1.0 : 0.0, sy = 0.0;
      for (int q = j; q < i; q++) {
        const double2 l = G[i + (int64_t)n * q];
        const double2 x = M[j + (int64_t)n * q];  // conj(X[q][j]) stored at M[j][q]
        // L[i][q] X[q][j] with X[q][j] = conj(x)
        sx -= l.x * x.x + l.y * x.y;
        sy -= l.y * x.x - l.x * x.y;
      }
      const double d = G[i + (int64_t)n * i].x;
      M[j + (int64_t)n * i] = make_double2(sx / d, -sy / d);  // store conj(X[i][j])
    }
  }
}

// small dense complex products on the device: C = alpha A B + beta I
// (n x n column-major; a thread per output entry)
__global__ void k_small_gemm(const double2 *__restrict__ A, const double2 *__restrict__ B, int n, double alpha,
                             double beta, double2 *__restrict__ Cm) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * n) return;
  const int i = (int)(e % n), j = (int)(e / n);
  double sx = 0, sy = 0;
  for (int q = 0; q < n; q++) {
    const double2 a = A[i + (int64_t)n * q], b = B[q + (int64_t)n * j];
    sx += a.x * b.x - a.y * b.y;
    sy += a.x * b.y + a.y * b.x;
  }
  Cm[e] = make_double2(alpha * sx + (i == j ? beta : 0.0), alpha * sy);
}

// max |G - I| (one CTA) into out[0]
__global__ void k_offdiag(const double2 *__restrict__ G, int n, double *__restrict__ out) {
  __shared__ double sh[256];
  double m = 0;
  for (int64_t e = threadIdx.x; e < (int64_t)n * n; e += blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    const double2 g = G[e];
    m = fmax(m, hypot(g.x - (i == j ? 1.0 : 0.0), g.y));
  }
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

// ---- host: cyclic Jacobi for a complex Hermitian matrix (column-major).
// On return w holds the eigenvalues ascending and V the eigenvectors.
void herm_eig(int n, std::vector<std::complex<double>> &H, std::vector<double> &w,
              std::vector<std::complex<double>> &V) {
  typedef std::complex<double> cd;
  auto h = [&](int i, int j) -> cd & { return H[i + (size_t)n * j]; };
  V.assign((size_t)n * n, cd(0, 0));
  for (int i = 0; i < n; i++) V[i + (size_t)n * i] = 1.0;
  double fro = 0;
  for (auto &x : H) fro += std::norm(x);
  fro = std::sqrt(fro);
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) off += std::norm(h(p, q));
    if (std::sqrt(off) <= 1e-15 * (fro > 0 ? fro : 1.0)) break;
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        const cd bpq = h(p, q);
        const double r = std::abs(bpq);
        if (r == 0.0) continue;
        const cd ph = bpq / r;  // e^{i phi}
        const double a = h(p, p).real(), d = h(q, q).real();
        const double tau = (d - a) / (2.0 * r);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        const double cc = 1.0 / std::sqrt(1.0 + t * t), ss = t * cc;
        // R = [[c, s], [-s e^{-i phi}, c e^{-i phi}]] on columns p, q
        const cd em = std::conj(ph);
        for (int k = 0; k < n; k++) {
          const cd hp = h(k, p), hq = h(k, q);
          h(k, p) = cc * hp - ss * em * hq;
          h(k, q) = ss * hp + cc * em * hq;
        }
        for (int k = 0; k < n; k++) {
          const cd hp = h(p, k), hq = h(q, k);
          h(p, k) = cc * hp - ss * ph * hq;
          h(q, k) = ss * hp + cc * ph * hq;
        }
        h(p, q) = h(q, p) = 0.0;
        h(p, p) = h(p, p).real();
        h(q, q) = h(q, q).real();
        for (int k = 0; k < n; k++) {
          const cd vp = V[k + (size_t)n * p], vq = V[k + (size_t)n * q];
          V[k + (size_t)n * p] = cc * vp - ss * em * vq;
          V[k + (size_t)n * q] = ss * vp + cc * em * vq;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; i++) idx[i] = i;
  std::vector<double> ev(n);
  for (int i = 0; i < n; i++) ev[i] = h(i, i).real();
  std::sort(idx.begin(), idx.end(), [&](int x, int y) { return ev[x] < ev[y] || (ev[x] == ev[y] && x < y); });
  std::vector<cd> Vs((size_t)n * n);
  w.resize(n);
  for (int j = 0; j < n; j++) {
    w[j] = ev[idx[j]];
    for (int k = 0; k < n; k++) Vs[k + (size_t)n * j] = V[k + (size_t)n * idx[j]];
  }
  V.swap(Vs);
}

}  // namespace opaw

using namespace opaw;

extern "C" {

int opaw_gram_dev(opaw_ctx *c, int dtype, const void *A, int na, const void *B, int nb, double *G) {
  if (!c || !A || !B || !G || na <= 0 || nb <= 0) {
    set_error("bad arguments");
    return OPAW_ERR_ARG;
  }
  OPAW_CHECK(ensure(c->gramout, sizeof(double2) * (size_t)na * nb));
  double2 *Gd = (double2 *)c->gramout.p;
  if (dtype == OPAW_C128) OPAW_CHECK(gram_t<double>(c, (const double2 *)A, na, (const double2 *)B, nb, Gd));
  else if (dtype == OPAW_C128_DD) OPAW_CHECK(gram_dd(c, (const double2 *)A, na, (const double2 *)B, nb, Gd, 0));
  else if (dtype == OPAW_C64) OPAW_CHECK(gram_t<float>(c, (const float2 *)A, na, (const float2 *)B, nb, Gd));
  else {
    set_error("dtype must be OPAW_C128, OPAW_C128_DD or OPAW_C64");
    return OPAW_ERR_ARG;
  }
  OPAW_CUDA(cudaMemcpyAsync(G, Gd, sizeof(double2) * (size_t)na * nb, cudaMemcpyDeviceToHost, c->stream));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return OPAW_OK;
}

int opaw_gram_herm_dev(opaw_ctx *c, int dtype, const void *A, const void *B, int n, double *G) {
  if (!c || !A || !B || !G || n <= 0) {
    set_error("bad arguments");
    return OPAW_ERR_ARG;
  }
  OPAW_CHECK(ensure(c->gramout, sizeof(double2) * (size_t)n * n));
  double2 *Gd = (double2 *)c->gramout.p;
  if (dtype == OPAW_C128) OPAW_CHECK(gram_t<double>(c, (const double2 *)A, n, (const double2 *)B, n, Gd, 1));
  else if (dtype == OPAW_C128_DD) OPAW_CHECK(gram_dd(c, (const double2 *)A, n, (const double2 *)B, n, Gd, 1));
  else if (dtype == OPAW_C64) OPAW_CHECK(gram_t<float>(c, (const float2 *)A, n, (const float2 *)B, n, Gd, 1));
  else {
    set_error("dtype must be OPAW_C128 or OPAW_C64");
    return OPAW_ERR_ARG;
  }
  OPAW_CUDA(cudaMemcpyAsync(G, Gd, sizeof(double2) * (size_t)n * n, cudaMemcpyDeviceToHost, c->stream));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return OPAW_OK;
}

int opaw_rotate_dev(opaw_ctx *c, int dtype, const void *A, int na, const double *M, int nb, void *out) {
  if (!c || !A || !M || !out || na <= 0 || nb <= 0 || A == out) {
    set_error("bad arguments (out must differ from A)");
    return OPAW_ERR_ARG;
  }
  OPAW_CHECK(ensure(c->gramout, sizeof(double2) * (size_t)na * nb));
  double2 *Md = (double2 *)c->gramout.p;
  OPAW_CUDA(cudaMemcpyAsync(Md, M, sizeof(double2) * (size_t)na * nb, cudaMemcpyHostToDevice, c->stream));
  if (dtype == OPAW_C128) OPAW_CHECK(rotate_t<double>(c, (const double2 *)A, na, Md, nb, (double2 *)out));
  else if (dtype == OPAW_C128_DD) OPAW_CHECK(rotate_dd(c, (const double2 *)A, na, Md, nb, (double2 *)out));
  else if (dtype == OPAW_C64) OPAW_CHECK(rotate_t<float>(c, (const float2 *)A, na, Md, nb, (float2 *)out));
  else {
    set_error("dtype must be OPAW_C128 or OPAW_C64");
    return OPAW_ERR_ARG;
  }
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return OPAW_OK;
}

int opaw_orthog(opaw_ctx *c, int set, double *eig_out) {
  if (!c || (set != 0 && set != 1)) {
    set_error("bad arguments");
    return OPAW_ERR_ARG;
  }
  const int n = c->norb[set];
  if (n == 0) {
    set_error("no orbitals uploaded for this set");
    return OPAW_ERR_STATE;
  }
  std::vector<std::complex<double>> G((size_t)n * n), V;
  OPAW_CHECK(opaw_gram_dev(c, OPAW_C128, c->d_psi[set], n, c->d_psi[set], n, (double *)G.data()));
  for (int i = 0; i < n; i++)  // exact Hermitian symmetry before the eigensolve
    for (int j = i + 1; j < n; j++) {
      const std::complex<double> a = 0.5 * (G[i + (size_t)n * j] + std::conj(G[j + (size_t)n * i]));
      G[i + (size_t)n * j] = a;
      G[j + (size_t)n * i] = std::conj(a);
    }
  std::vector<double> w;
  herm_eig(n, G, w, V);
  for (int j = 0; j < n; j++) {
    if (!(w[j] > 0)) {
      set_error("orbitals are linearly dependent (Gram eigenvalue <= 0)");
      return OPAW_ERR_NONFINITE;
    }
    const double f = 1.0 / std::sqrt(w[j]);  // orthog_phi.f90: p1(:,i) / sqrt(eig(i))
    for (int k = 0; k < n; k++) V[k + (size_t)n * j] *= f;
  }
  if (eig_out)
    for (int j = 0; j < n; j++) eig_out[j] = w[j];
  OPAW_CHECK(ensure(c->work[7], sizeof(double2) * (size_t)c->nn * n));
  OPAW_CHECK(opaw_rotate_dev(c, OPAW_C128, c->d_psi[set], n, (const double *)V.data(), n, c->work[7].p));
  if (set == 0) c->psi0_gen++;
  OPAW_CUDA(cudaMemcpyAsync(c->d_psi[set], c->work[7].p, sizeof(double2) * (size_t)c->nn * n,
                            cudaMemcpyDeviceToDevice, c->stream));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return OPAW_OK;
}

// FP64 orthonormalisation of the resident orbitals of `set` on the device
// (no host eigensolve): method 0 Cholesky, Psi <- Psi L^-H with G = L L^H;
// method 1 Loewdin, Psi <- Psi G^-1/2 by the coupled Newton-Schulz iteration
// (Y <- Y T, Z <- T Z, T = (3 I - Z Y) / 2 from Y = G, Z = I), which
// converges when the orbitals are close to orthonormal (max |G - I| < 0.5 is
// required; further away use method 0).  offdiag (may be NULL) receives
// max |G - I| before the orthonormalisation.
int opaw_orthonormalize_dev(opaw_ctx *c, int set, int method, double *offdiag) {
  if (!c || (set != 0 && set != 1) || (method != 0 && method != 1)) {
    set_error("bad arguments");
    return OPAW_ERR_ARG;
  }
  const int n = c->norb[set];
  if (n == 0) {
    set_error("no orbitals uploaded for this set");
    return OPAW_ERR_STATE;
  }
  const size_t nm = (size_t)n * n;
  OPAW_CHECK(ensure(c->gramout, sizeof(double2) * 5 * nm + 64));
  double2 *G = (double2 *)c->gramout.p, *M = G + nm, *Y = M + nm, *Z = Y + nm, *T = Z + nm;
  int *info = (int *)(T + nm);
  double *off = (double *)(T + nm) + 2;
  OPAW_CHECK(gram_t<double>(c, c->d_psi[set], n, c->d_psi[set], n, G));
  k_offdiag<<<1, 256, 0, c->stream>>>(G, n, off);
  c->launches++;
  double hoff = 0.0;
  OPAW_CUDA(cudaMemcpyAsync(&hoff, off, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  if (offdiag) *offdiag = hoff;
  const int nb = grid1((int64_t)nm, 256);
  if (method == 0) {
    k_chol_inv<<<1, 256, 0, c->stream>>>(G, n, M, info);
    c->launches++;
    int hinfo = 0;
    OPAW_CUDA(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    OPAW_CUDA(cudaStreamSynchronize(c->stream));
    if (hinfo) {
      set_error("orbitals are linearly dependent (Cholesky pivot " + std::to_string(hinfo) + " not positive)");
      return OPAW_ERR_NONFINITE;
    }
  } else {
    if (!(hoff < 0.5)) {
      set_error("Loewdin by Newton-Schulz needs max |G - I| < 0.5: use the Cholesky method");
      return OPAW_ERR_ARG;
    }
    OPAW_CUDA(cudaMemcpyAsync(Y, G, sizeof(double2) * nm, cudaMemcpyDeviceToDevice, c->stream));
    // Z = I: 0 A B + 1 I
    k_small_gemm<<<nb, 256, 0, c->stream>>>(G, G, n, 0.0, 1.0, Z);
    c->launches++;
    for (int it = 0; it < 30; it++) {
      k_small_gemm<<<nb, 256, 0, c->stream>>>(Z, Y, n, -0.5, 1.5, T);  // T = (3 I - Z Y) / 2
      k_small_gemm<<<nb, 256, 0, c->stream>>>(Y, T, n, 1.0, 0.0, M);   // Y T
      OPAW_CUDA(cudaMemcpyAsync(Y, M, sizeof(double2) * nm, cudaMemcpyDeviceToDevice, c->stream));
      k_small_gemm<<<nb, 256, 0, c->stream>>>(T, Z, n, 1.0, 0.0, M);   // T Z
      OPAW_CUDA(cudaMemcpyAsync(Z, M, sizeof(double2) * nm, cudaMemcpyDeviceToDevice, c->stream));
      c->launches += 3;
      if (it % 4 == 3) {  // converged when Y (-> G^1/2 G^-1/2 ... ) Z -> I: check |T - I|
        k_offdiag<<<1, 256, 0, c->stream>>>(T, n, off);
        c->launches++;
        double d = 1.0;
        OPAW_CUDA(cudaMemcpyAsync(&d, off, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        OPAW_CUDA(cudaStreamSynchronize(c->stream));
        if (d < 1e-15) break;
      }
    }
    OPAW_CUDA(cudaMemcpyAsync(M, Z, sizeof(double2) * nm, cudaMemcpyDeviceToDevice, c->stream));  // G^-1/2
  }
  OPAW_CUDA(cudaGetLastError());
  OPAW_CHECK(ensure(c->work[7], sizeof(double2) * (size_t)c->nn * n));
  OPAW_CHECK(rotate_t<double>(c, c->d_psi[set], n, M, n, (double2 *)c->work[7].p));
  if (set == 0) c->psi0_gen++;
  OPAW_CUDA(cudaMemcpyAsync(c->d_psi[set], c->work[7].p, sizeof(double2) * (size_t)c->nn * n,
                            cudaMemcpyDeviceToDevice, c->stream));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return OPAW_OK;
}

int opaw_herm_eig(int n, double *H, double *w, double *V) {
  if (n <= 0 || !H || !w || !V) {
    set_error("bad arguments");
    return OPAW_ERR_ARG;
  }
  std::vector<std::complex<double>> h((std::complex<double> *)H, (std::complex<double> *)H + (size_t)n * n), v;
  std::vector<double> ww;
  herm_eig(n, h, ww, v);
  for (int i = 0; i < n; i++) w[i] = ww[i];
  std::copy(v.begin(), v.end(), (std::complex<double> *)V);
  return OPAW_OK;
}

}  // extern "C"

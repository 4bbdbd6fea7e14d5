// precond_net.cu — the learned correction of the ground-state eigensolver's
// kinetic preconditioner: a 3-layer 3D convolutional network (3^3 kernels,
// 16 channels, BF16 weights and activations, FP32 accumulation on the tensor
// cores with mma.sync m16n8k16), its backward pass and Adam training on the
// device, and its application inside the preconditioner.
//
// The reference has no counterpart: its ground state comes from a
// Chebyshev-filtered SCF without any preconditioner (chebyr_m.f90:1-48,
// main.f90:67-96).  The network maps, per orbital, the normalised residual
// r / |r| (two channels, real and imaginary part) and the shifted potential
// v_ks - eps (one channel) to a correction c (two channels); the search
// direction of the eigensolver is K r + |r| c, K the Teter-Payne-Allan
// kinetic preconditioner.
//
// Layout: activations are channels-last [batch][z][y][x][16] BF16 (channels
// beyond a layer's real count are zero); weights [layer][tap 27][ci 16][co 16]
// with tap = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1); convolutions are 'same'
// with zeros outside the box.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <random>

#include "common.cuh"

namespace opaw {

constexpr int kNetCh = 16;             // stored channels of every activation
constexpr int kNetTaps = 27;
constexpr int kNetLayers = 3;
constexpr int kNetWl = kNetTaps * kNetCh * kNetCh;  // weights of one layer
constexpr int kNetPl = kNetWl + kNetCh;             // + bias
// real input / output channels of layer l
__host__ __device__ constexpr int net_cin(int l) { return l == 0 ? 3 : 16; }
__host__ __device__ constexpr int net_cout(int l) { return l == 2 ? 2 : 16; }
constexpr int kConvX = 64;    // output voxels (along x) per CTA
constexpr int kConvVS = 24;   // shared-memory stride of one voxel's channels (bf16): conflict-free fragments
constexpr int kConvWS = 24;   // shared-memory stride of one output channel's weights (bf16)

__device__ __forceinline__ float silu(float x) { return x / (1.f + __expf(-x)); }
__device__ __forceinline__ float silu_grad(float x) {
  const float s = 1.f / (1.f + __expf(-x));
  return s * (1.f + x * (1.f - s));
}
__device__ __forceinline__ unsigned pack_bf16(float a, float b) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);  // .x = a (low half), .y = b
  return *reinterpret_cast<const unsigned *>(&v);
}

// two BF16 values of one channel at consecutive voxels v, v + 1 of a staged
// row (stride kConvVS), packed low = v
__device__ __forceinline__ unsigned pack2(const __nv_bfloat16 *base, int v, int ch) {
  const unsigned lo = reinterpret_cast<const unsigned short &>(base[v * kConvVS + ch]);
  const unsigned hi = reinterpret_cast<const unsigned short &>(base[(v + 1) * kConvVS + ch]);
  return lo | (hi << 16);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Epilogue modes of the convolution
enum ConvMode {
  kFwdAct = 0,    // out = silu(acc + bias) as BF16, pre = acc + bias (FP32) when pre != null
  kFwdLinear = 1, // out32 = acc + bias (FP32, the last layer)
  kBwdData = 2    // out = acc * silu'(pre_prev) as BF16 (gradient of the previous layer's pre-activation)
};

struct ConvDims {
  int batch, nz, ny, nx;
};

// One 'same' 3^3 convolution, 16 -> 16 stored channels.  CTA: 4 warps, a row
// segment of kConvX voxels at (batch, z, y); each warp 16 voxels x 16 output
// channels (two m16n8k16 tiles per tap and 16-channel slice).  The 3 x 3 input
// rows around the segment (with one voxel of halo each side) and the weights
// (transposed to [tap][co][ci]) are staged in shared memory first.
template <int MODE>
__global__ void __launch_bounds__(128) k_net_conv(ConvDims d, const __nv_bfloat16 *__restrict__ in,
                                                  const __nv_bfloat16 *__restrict__ wt, const float *__restrict__ bias,
                                                  __nv_bfloat16 *__restrict__ out, float *__restrict__ out32,
                                                  float *__restrict__ pre, const float *__restrict__ pre_prev) {
  extern __shared__ __align__(16) unsigned char smem[];
  __nv_bfloat16 *xs = reinterpret_cast<__nv_bfloat16 *>(smem);              // [9][kConvX + 2][kConvVS]
  __nv_bfloat16 *ws = xs + 9 * (kConvX + 2) * kConvVS;                      // [27][16 co][kConvWS]
  const int nseg = (d.nx + kConvX - 1) / kConvX;
  int64_t row = blockIdx.x;
  const int seg = (int)(row % nseg);
  row /= nseg;
  const int y = (int)(row % d.ny);
  row /= d.ny;
  const int z = (int)(row % d.nz);
  const int b = (int)(row / d.nz);
  const int x0 = seg * kConvX;
  // stage weights: global [tap][ci][co] -> shared [tap][co][ci]
  for (int e = threadIdx.x; e < kNetWl; e += blockDim.x) {
    const int tap = e / (kNetCh * kNetCh), r = e - tap * kNetCh * kNetCh, ci = r / kNetCh, co = r - ci * kNetCh;
    ws[(tap * kNetCh + co) * kConvWS + ci] = wt[e];
  }
  // stage the 9 input rows, 16-byte chunks (two per voxel), zeros outside the box
  constexpr int kRowV = kConvX + 2;
  for (int e = threadIdx.x; e < 9 * kRowV * 2; e += blockDim.x) {
    const int half = e & 1, v = (e >> 1) % kRowV, r = (e >> 1) / kRowV;
    const int zz = z + r / 3 - 1, yy = y + r % 3 - 1, xx = x0 + v - 1;
    uint4 val = make_uint4(0u, 0u, 0u, 0u);
    if (zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny && xx >= 0 && xx < d.nx) {
      const int64_t g = (((int64_t)b * d.nz + zz) * d.ny + yy) * d.nx + xx;
      val = reinterpret_cast<const uint4 *>(in + g * kNetCh)[half];
    }
    *reinterpret_cast<uint4 *>(xs + ((int64_t)r * kRowV + v) * kConvVS + half * 8) = val;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int mbase = warp * 16;  // first voxel of this warp within the segment
  float acc[2][4];
#pragma unroll
  for (int n = 0; n < 2; n++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc[n][q] = 0.f;
#pragma unroll 3
  for (int tap = 0; tap < kNetTaps; tap++) {
    const int r = tap / 3;          // (dz, dy) row of the staged tile
    const int dxo = tap % 3;        // dx + 1: voxel offset within the row
    const __nv_bfloat16 *arow = xs + ((int64_t)r * kRowV + mbase + dxo) * kConvVS;
    unsigned a[4];
    a[0] = *reinterpret_cast<const unsigned *>(arow + g * kConvVS + 2 * t);
    a[1] = *reinterpret_cast<const unsigned *>(arow + (g + 8) * kConvVS + 2 * t);
    a[2] = *reinterpret_cast<const unsigned *>(arow + g * kConvVS + 2 * t + 8);
    a[3] = *reinterpret_cast<const unsigned *>(arow + (g + 8) * kConvVS + 2 * t + 8);
#pragma unroll
    for (int n = 0; n < 2; n++) {
      const __nv_bfloat16 *wb = ws + (tap * kNetCh + n * 8 + g) * kConvWS;
      const unsigned b0 = *reinterpret_cast<const unsigned *>(wb + 2 * t);
      const unsigned b1 = *reinterpret_cast<const unsigned *>(wb + 2 * t + 8);
      mma_bf16(acc[n], a, b0, b1);
    }
  }
  // epilogue: voxel m = g or g + 8 of the warp, channels co = n 8 + 2 t, +1
#pragma unroll
  for (int hrow = 0; hrow < 2; hrow++) {
    const int x = x0 + mbase + g + 8 * hrow;
    if (x >= d.nx) continue;
    const int64_t gv = ((((int64_t)b * d.nz + z) * d.ny + y) * d.nx + x) * kNetCh;
#pragma unroll
    for (int n = 0; n < 2; n++) {
      const int co = n * 8 + 2 * t;
      float v0 = acc[n][2 * hrow], v1 = acc[n][2 * hrow + 1];
      if (MODE == kFwdAct || MODE == kFwdLinear) {
        v0 += bias[co];
        v1 += bias[co + 1];
      }
      if (MODE == kFwdAct) {
        if (pre) *reinterpret_cast<float2 *>(pre + gv + co) = make_float2(v0, v1);
        *reinterpret_cast<unsigned *>(out + gv + co) = pack_bf16(silu(v0), silu(v1));
      } else if (MODE == kFwdLinear) {
        *reinterpret_cast<float2 *>(out32 + gv + co) = make_float2(v0, v1);
      } else {
        const float2 p = *reinterpret_cast<const float2 *>(pre_prev + gv + co);
        *reinterpret_cast<unsigned *>(out + gv + co) = pack_bf16(v0 * silu_grad(p.x), v1 * silu_grad(p.y));
      }
    }
  }
}

// Weight gradient of one layer: dW[tap][ci][co] += sum_v in[v + off(tap)][ci] dpre[v][co],
// db[co] += sum_v dpre[v][co].  CTA: 9 warps, three taps each; it walks
// rows of kConvX voxels (grid-stride), staging the 3 x 3 input rows and the
// row of dpre, and adds its sums to dW / db once at the end.
__global__ void __launch_bounds__(288) k_net_wgrad(ConvDims d, const __nv_bfloat16 *__restrict__ in,
                                                   const __nv_bfloat16 *__restrict__ dpre, float *__restrict__ dw,
                                                   float *__restrict__ db) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int kRowV = kConvX + 2;
  __nv_bfloat16 *xs = reinterpret_cast<__nv_bfloat16 *>(smem);  // [9][kRowV][kConvVS]
  __nv_bfloat16 *ds = xs + 9 * kRowV * kConvVS;                   // [kConvX][kConvVS]
  __shared__ float dbs[kNetCh];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  if (threadIdx.x < kNetCh) dbs[threadIdx.x] = 0.f;
  float acc[3][2][4];
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int n = 0; n < 2; n++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[j][n][q] = 0.f;
  float dbl = 0.f;  // thread < 16: its channel's bias gradient
  const int nseg = (d.nx + kConvX - 1) / kConvX;
  const int64_t nrows = (int64_t)d.batch * d.nz * d.ny * nseg;
  for (int64_t rowi = blockIdx.x; rowi < nrows; rowi += gridDim.x) {
    int64_t row = rowi;
    const int seg = (int)(row % nseg);
    row /= nseg;
    const int y = (int)(row % d.ny);
    row /= d.ny;
    const int z = (int)(row % d.nz);
    const int b = (int)(row / d.nz);
    const int x0 = seg * kConvX;
    __syncthreads();  // the previous row's tiles are no longer read
    for (int e = threadIdx.x; e < 9 * kRowV * 2; e += blockDim.x) {
      const int half = e & 1, v = (e >> 1) % kRowV, r = (e >> 1) / kRowV;
      const int zz = z + r / 3 - 1, yy = y + r % 3 - 1, xx = x0 + v - 1;
      uint4 val = make_uint4(0u, 0u, 0u, 0u);
      if (zz >= 0 && zz < d.nz && yy >= 0 && yy < d.ny && xx >= 0 && xx < d.nx) {
        const int64_t gg = (((int64_t)b * d.nz + zz) * d.ny + yy) * d.nx + xx;
        val = reinterpret_cast<const uint4 *>(in + gg * kNetCh)[half];
      }
      *reinterpret_cast<uint4 *>(xs + ((int64_t)r * kRowV + v) * kConvVS + half * 8) = val;
    }
    for (int e = threadIdx.x; e < kConvX * 2; e += blockDim.x) {
      const int half = e & 1, v = e >> 1, xx = x0 + v;
      uint4 val = make_uint4(0u, 0u, 0u, 0u);
      if (xx < d.nx) {
        const int64_t gg = (((int64_t)b * d.nz + z) * d.ny + y) * d.nx + xx;
        val = reinterpret_cast<const uint4 *>(dpre + gg * kNetCh)[half];
      }
      *reinterpret_cast<uint4 *>(ds + (int64_t)v * kConvVS + half * 8) = val;
    }
    __syncthreads();
    if (threadIdx.x < kNetCh)
      for (int v = 0; v < kConvX; v++) dbl += __bfloat162float(ds[v * kConvVS + threadIdx.x]);
    // A = in^T (m = ci, k = voxel), B = dpre (k = voxel, n = co)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int tap = warp * 3 + j;
      const int r = tap / 3, dxo = tap % 3;
      const __nv_bfloat16 *arow = xs + ((int64_t)r * kRowV + dxo) * kConvVS;
#pragma unroll
      for (int k0 = 0; k0 < kConvX; k0 += 16) {
        unsigned a[4];
        const int ka = k0 + 2 * t;
        a[0] = pack2(arow, ka, g);
        a[1] = pack2(arow, ka, g + 8);
        a[2] = pack2(arow, ka + 8, g);
        a[3] = pack2(arow, ka + 8, g + 8);
#pragma unroll
        for (int n = 0; n < 2; n++) {
          const unsigned b0 = pack2(ds, ka, n * 8 + g), b1 = pack2(ds, ka + 8, n * 8 + g);
          mma_bf16(acc[j][n], a, b0, b1);
        }
      }
    }
  }
  // D fragment: (m = ci = g or g + 8, n = co = 2 t, 2 t + 1)
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int tap = warp * 3 + j;
#pragma unroll
    for (int n = 0; n < 2; n++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int ci = g + 8 * (q >> 1), co = n * 8 + 2 * t + (q & 1);
        atomicAdd(dw + (tap * kNetCh + ci) * kNetCh + co, acc[j][n][q]);
      }
  }
  if (threadIdx.x < kNetCh) atomicAdd(db + threadIdx.x, dbl);
}

// ------------------------------------------------------------ training --
__device__ __forceinline__ double net_block_sum(double v, double *sh) {
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

// loss of the interior voxels (margin m from every face of a P^3 patch):
// L = sum (out - target)^2 / count over the two output channels; dout =
// dL/dout as BF16 (zero outside the interior and in the padded channels);
// per-block partial sums of L into part[blockIdx.x]
__global__ void __launch_bounds__(256) k_net_loss(const float *__restrict__ out32, const float *__restrict__ tgt,
                                                  int64_t nvox, int P, int margin, float inv_count,
                                                  __nv_bfloat16 *__restrict__ dout, double *__restrict__ part) {
  __shared__ double sh[8];
  double acc = 0;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(v % P), y = (int)((v / P) % P), z = (int)((v / ((int64_t)P * P)) % P);
    const bool in = x >= margin && x < P - margin && y >= margin && y < P - margin && z >= margin && z < P - margin;
    float d0 = 0.f, d1 = 0.f;
    if (in) {
      d0 = out32[v * kNetCh] - tgt[2 * v];
      d1 = out32[v * kNetCh + 1] - tgt[2 * v + 1];
      acc += (double)d0 * d0 + (double)d1 * d1;
    }
    uint4 *o = reinterpret_cast<uint4 *>(dout + v * kNetCh);
    o[0] = make_uint4(pack_bf16(2.f * d0 * inv_count, 2.f * d1 * inv_count), 0u, 0u, 0u);
    o[1] = make_uint4(0u, 0u, 0u, 0u);
  }
  const double t = net_block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

constexpr int kLossBlocks = 256;
__global__ void k_net_loss_final(const double *__restrict__ part, double inv_count, double *__restrict__ out) {
  __shared__ double sh[8];
  double a = 0;
  for (int i = threadIdx.x; i < kLossBlocks; i += blockDim.x) a += part[i];
  a = net_block_sum(a, sh);
  if (threadIdx.x == 0) *out = a * inv_count;
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters of every layer;
// entries of padded channels stay zero.  Then the BF16 forward weights and
// the weights of the backward-data convolution (taps mirrored, ci <-> co).
__global__ void k_net_adam(float *__restrict__ w, const float *__restrict__ gr, float *__restrict__ m,
                           float *__restrict__ v, float lr, float b1, float b2, float c1, float c2, float eps,
                           __nv_bfloat16 *__restrict__ wbf, __nv_bfloat16 *__restrict__ wflip) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kNetLayers * kNetPl) return;
  const int l = e / kNetPl, r = e - l * kNetPl;
  bool live;
  if (r < kNetWl) {
    const int tap = r / (kNetCh * kNetCh), q = r - tap * kNetCh * kNetCh, ci = q / kNetCh, co = q - ci * kNetCh;
    live = ci < net_cin(l) && co < net_cout(l);
    (void)tap;
  } else {
    live = (r - kNetWl) < net_cout(l);
  }
  float x = 0.f;
  if (live) {
    const float gg = gr[e];
    const float mm = b1 * m[e] + (1.f - b1) * gg, vv = b2 * v[e] + (1.f - b2) * gg * gg;
    m[e] = mm;
    v[e] = vv;
    x = w[e] - lr * (mm * c1) / (sqrtf(vv * c2) + eps);
  }
  w[e] = x;
  if (r < kNetWl) {
    const int tap = r / (kNetCh * kNetCh), q = r - tap * kNetCh * kNetCh, ci = q / kNetCh, co = q - ci * kNetCh;
    const __nv_bfloat16 xb = __float2bfloat16_rn(x);
    wbf[l * kNetWl + r] = xb;
    wflip[l * kNetWl + ((kNetTaps - 1 - tap) * kNetCh + co) * kNetCh + ci] = xb;
  }
}

// BF16 copies (forward and mirrored) of given master weights
__global__ void k_net_cast(const float *__restrict__ w, __nv_bfloat16 *__restrict__ wbf,
                           __nv_bfloat16 *__restrict__ wflip) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kNetLayers * kNetPl) return;
  const int l = e / kNetPl, r = e - l * kNetPl;
  if (r >= kNetWl) return;
  const int tap = r / (kNetCh * kNetCh), q = r - tap * kNetCh * kNetCh, ci = q / kNetCh, co = q - ci * kNetCh;
  const __nv_bfloat16 xb = __float2bfloat16_rn(w[e]);
  wbf[l * kNetWl + r] = xb;
  wflip[l * kNetWl + ((kNetTaps - 1 - tap) * kNetCh + co) * kNetCh + ci] = xb;
}

// minibatch s of the stored patches: slot i <- patch (s batch + i) % npatch
__global__ void k_net_gather(const uint4 *__restrict__ sx, const float2 *__restrict__ st, int64_t P3, int npatch,
                             int64_t s, int batch, uint4 *__restrict__ bx, float2 *__restrict__ bt) {
  const int i = blockIdx.y;
  const int64_t pi = (s * batch + i) % npatch;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < P3; e += (int64_t)gridDim.x * blockDim.x) {
    bx[((int64_t)i * P3 + e) * 2] = sx[(pi * P3 + e) * 2];
    bx[((int64_t)i * P3 + e) * 2 + 1] = sx[(pi * P3 + e) * 2 + 1];
    bt[(int64_t)i * P3 + e] = st[pi * P3 + e];
  }
}

// ------------------------------------------------------------- features --
// network input of norb orbitals on the grid: (Re r, Im r) s_o and v - eps_o,
// s_o = 1 / |r_o|, as BF16 channels 0..2 of [orbital][point][16]
template <typename C>
__global__ void k_net_input(const C *__restrict__ r, const double *__restrict__ vks, const double *__restrict__ eps,
                            const double *__restrict__ scale, int64_t nn, __nv_bfloat16 *__restrict__ x) {
  const int o = blockIdx.y;
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= nn) return;
  const C z = r[(int64_t)o * nn + g];
  const float sc = (float)scale[o];
  uint4 *dst = reinterpret_cast<uint4 *>(x + ((int64_t)o * nn + g) * kNetCh);
  dst[0] = make_uint4(pack_bf16((float)z.x * sc, (float)z.y * sc), pack_bf16((float)(vks[g] - eps[o]), 0.f), 0u, 0u);
  dst[1] = make_uint4(0u, 0u, 0u, 0u);
}

// training patches P^3 at origins (orbital, z0, y0, x0) (periodic wrap of the
// grid): input channels as k_net_input, targets t s_o (complex128 fields)
__global__ void k_net_patches(const double2 *__restrict__ r, const double2 *__restrict__ t,
                              const double *__restrict__ vks, const double *__restrict__ eps,
                              const double *__restrict__ scale, const int4 *__restrict__ org, int P, int nx, int ny,
                              int nz, __nv_bfloat16 *__restrict__ x, float *__restrict__ tgt) {
  const int p = blockIdx.y;
  const int64_t P3 = (int64_t)P * P * P;
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= P3) return;
  const int4 q = org[p];
  const int px = (int)(v % P), py = (int)((v / P) % P), pz = (int)(v / ((int64_t)P * P));
  const int gx = (q.w + px) % nx, gy = (q.z + py) % ny, gz = (q.y + pz) % nz;
  const int64_t nn = (int64_t)nx * ny * nz;
  const int64_t g = ((int64_t)gz * ny + gy) * nx + gx;
  const int o = q.x;
  const double sc = scale[o];
  const double2 rv = r[(int64_t)o * nn + g], tv = t[(int64_t)o * nn + g];
  uint4 *dst = reinterpret_cast<uint4 *>(x + ((int64_t)p * P3 + v) * kNetCh);
  dst[0] = make_uint4(pack_bf16((float)(rv.x * sc), (float)(rv.y * sc)), pack_bf16((float)(vks[g] - eps[o]), 0.f),
                      0u, 0u);
  dst[1] = make_uint4(0u, 0u, 0u, 0u);
  tgt[2 * ((int64_t)p * P3 + v)] = (float)(tv.x * sc);
  tgt[2 * ((int64_t)p * P3 + v) + 1] = (float)(tv.y * sc);
}

// w_o += |r_o| (out0 + i out1): the learned correction added to the kinetic
// preconditioner's output
template <typename C>
__global__ void k_net_combine(const float *__restrict__ out32, const double *__restrict__ rnorm, int64_t nn,
                              C *__restrict__ w) {
  const int o = blockIdx.y;
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= nn) return;
  const int64_t i = (int64_t)o * nn + g;
  const float2 c = *reinterpret_cast<const float2 *>(out32 + i * kNetCh);
  const double s = rnorm[o];
  C z = w[i];
  z.x += s * (double)c.x;
  z.y += s * (double)c.y;
  w[i] = z;
}

// per orbital a = sqrt(dv sum |r|^2): scale[o] = 1 / a (0 for a zero
// residual) for the input, rn[o] = a for the output
__global__ void k_net_scales(const double *__restrict__ n2, double dv, int norb, double *__restrict__ scale,
                             double *__restrict__ rn) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= norb) return;
  const double a = sqrt(n2[o] * dv);
  scale[o] = a > 0.0 ? 1.0 / a : 0.0;
  rn[o] = a;
}

// per-orbital squared norms (one block per orbital)
template <typename C>
__global__ void k_net_norm2(const C *__restrict__ r, int64_t nn, double *__restrict__ out) {
  __shared__ double sh[8];
  const int o = blockIdx.x;
  double a = 0;
  for (int64_t g = threadIdx.x; g < nn; g += blockDim.x) {
    const C z = r[(int64_t)o * nn + g];
    a += (double)z.x * z.x + (double)z.y * z.y;
  }
  a = net_block_sum(a, sh);
  if (threadIdx.x == 0) out[o] = a;
}

}  // namespace opaw

// ------------------------------------------------------------------ C ABI --
struct opaw_net {
  float *w32 = nullptr;                // [layer][kNetPl] master parameters (weights, bias)
  float *grad = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16 *wbf = nullptr;        // [layer][kNetWl]
  __nv_bfloat16 *wflip = nullptr;      // [layer][kNetWl] mirrored taps, ci <-> co
  int64_t step = 0;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  // training scratch, grown on demand
  opaw::DeviceBuf x, a1, a2, pre0, pre1, out32, d2, d1, d0, tgt, part, loss, org;
};

namespace opaw {

static size_t conv_smem() { return sizeof(__nv_bfloat16) * (9 * (kConvX + 2) * kConvVS + kNetTaps * kNetCh * kConvWS); }
static size_t wgrad_smem() { return sizeof(__nv_bfloat16) * (9 * (kConvX + 2) * kConvVS + kConvX * kConvVS); }

template <int MODE>
static int conv_launch(cudaStream_t st, ConvDims d, const __nv_bfloat16 *in, const __nv_bfloat16 *wt,
                       const float *bias, __nv_bfloat16 *out, float *out32, float *pre, const float *pre_prev,
                       int64_t *launches) {
  static bool attr = false;
  if (!attr) {
    OPAW_CUDA(cudaFuncSetAttribute(k_net_conv<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)conv_smem()));
    attr = true;
  }
  const int64_t rows = (int64_t)d.batch * d.nz * d.ny * ((d.nx + kConvX - 1) / kConvX);
  if (rows == 0) return OPAW_OK;
  OPAW_ARG(rows < (int64_t)INT32_MAX, "convolution grid too large");
  k_net_conv<MODE><<<(unsigned)rows, 128, conv_smem(), st>>>(d, in, wt, bias, out, out32, pre, pre_prev);
  (*launches)++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

// the three layers on x (BF16 [batch][nz][ny][nx][16]) into out32; with
// keep = true the pre-activations and activations of the hidden layers stay
// in the net's buffers for a backward pass
static int net_forward(opaw_net *n, cudaStream_t st, ConvDims d, const __nv_bfloat16 *x, float *out32, bool keep,
                       opaw::DeviceBuf &a1b, opaw::DeviceBuf &a2b) {
  const size_t nv = (size_t)d.batch * d.nz * d.ny * d.nx;
  OPAW_CHECK(ensure(a1b, sizeof(__nv_bfloat16) * kNetCh * nv));
  OPAW_CHECK(ensure(a2b, sizeof(__nv_bfloat16) * kNetCh * nv));
  float *p0 = nullptr, *p1 = nullptr;
  if (keep) {
    OPAW_CHECK(ensure(n->pre0, sizeof(float) * kNetCh * nv));
    OPAW_CHECK(ensure(n->pre1, sizeof(float) * kNetCh * nv));
    p0 = (float *)n->pre0.p;
    p1 = (float *)n->pre1.p;
  }
  __nv_bfloat16 *a1 = (__nv_bfloat16 *)a1b.p, *a2 = (__nv_bfloat16 *)a2b.p;
  OPAW_CHECK(conv_launch<kFwdAct>(st, d, x, n->wbf, n->w32 + kNetWl, a1, nullptr, p0, nullptr, &n->launches));
  OPAW_CHECK(conv_launch<kFwdAct>(st, d, a1, n->wbf + kNetWl, n->w32 + kNetPl + kNetWl, a2, nullptr, p1, nullptr,
                                  &n->launches));
  OPAW_CHECK(conv_launch<kFwdLinear>(st, d, a2, n->wbf + 2 * kNetWl, n->w32 + 2 * kNetPl + kNetWl, nullptr, out32,
                                     nullptr, nullptr, &n->launches));
  return OPAW_OK;
}

// loss and gradients of a batch of P^3 patches (x, tgt already in the net's
// buffers); the loss stays on the device at n->loss
static int net_loss_grad(opaw_net *n, int batch, int P, int margin) {
  cudaStream_t st = n->stream;
  const ConvDims d{batch, P, P, P};
  const size_t nv = (size_t)batch * P * P * P;
  OPAW_CHECK(ensure(n->out32, sizeof(float) * kNetCh * nv));
  OPAW_CHECK(ensure(n->d2, sizeof(__nv_bfloat16) * kNetCh * nv));
  OPAW_CHECK(ensure(n->d1, sizeof(__nv_bfloat16) * kNetCh * nv));
  OPAW_CHECK(ensure(n->d0, sizeof(__nv_bfloat16) * kNetCh * nv));
  OPAW_CHECK(ensure(n->part, sizeof(double) * kLossBlocks));
  OPAW_CHECK(ensure(n->loss, sizeof(double) * 2));
  const __nv_bfloat16 *x = (const __nv_bfloat16 *)n->x.p;
  OPAW_CHECK(net_forward(n, st, d, x, (float *)n->out32.p, true, n->a1, n->a2));
  const int inner = P - 2 * margin;
  OPAW_ARG(inner > 0, "patch margin leaves no interior");
  const double count = 2.0 * batch * (double)inner * inner * inner;
  k_net_loss<<<kLossBlocks, 256, 0, st>>>((const float *)n->out32.p, (const float *)n->tgt.p, (int64_t)nv, P, margin,
                                           (float)(1.0 / count), (__nv_bfloat16 *)n->d2.p, (double *)n->part.p);
  k_net_loss_final<<<1, 256, 0, st>>>((const double *)n->part.p, 1.0 / count, (double *)n->loss.p);
  n->launches += 2;
  OPAW_CUDA(cudaGetLastError());
  OPAW_CUDA(cudaMemsetAsync(n->grad, 0, sizeof(float) * kNetLayers * kNetPl, st));
  static bool attr = false;
  if (!attr) {
    OPAW_CUDA(cudaFuncSetAttribute(k_net_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wgrad_smem()));
    attr = true;
  }
  const int wg_blocks = 2 * 152;
  const __nv_bfloat16 *a1 = (const __nv_bfloat16 *)n->a1.p, *a2 = (const __nv_bfloat16 *)n->a2.p;
  __nv_bfloat16 *d2 = (__nv_bfloat16 *)n->d2.p, *d1 = (__nv_bfloat16 *)n->d1.p, *d0 = (__nv_bfloat16 *)n->d0.p;
  // layer 2 (linear): dpre2 = dout
  k_net_wgrad<<<wg_blocks, 288, wgrad_smem(), st>>>(d, a2, d2, n->grad + 2 * kNetPl, n->grad + 2 * kNetPl + kNetWl);
  n->launches++;
  OPAW_CUDA(cudaGetLastError());
  OPAW_CHECK(conv_launch<kBwdData>(st, d, d2, n->wflip + 2 * kNetWl, nullptr, d1, nullptr, nullptr,
                                   (const float *)n->pre1.p, &n->launches));
  k_net_wgrad<<<wg_blocks, 288, wgrad_smem(), st>>>(d, a1, d1, n->grad + kNetPl, n->grad + kNetPl + kNetWl);
  n->launches++;
  OPAW_CUDA(cudaGetLastError());
  OPAW_CHECK(conv_launch<kBwdData>(st, d, d1, n->wflip + kNetWl, nullptr, d0, nullptr, nullptr,
                                   (const float *)n->pre0.p, &n->launches));
  k_net_wgrad<<<wg_blocks, 288, wgrad_smem(), st>>>(d, x, d0, n->grad, n->grad + kNetWl);
  n->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

}  // namespace opaw

using namespace opaw;

extern "C" {

int opaw_net_free(opaw_net *n);

int opaw_net_create(unsigned long long seed, opaw_net **out) {
  OPAW_ARG(out, "null output");
  opaw_net *n = new opaw_net();
  const size_t np = (size_t)kNetLayers * kNetPl;
  std::vector<float> w(np, 0.f);
  // He-style initialisation of the hidden layers' real channels, zero biases
  // and a zero output layer: the untrained network adds nothing to the kinetic
  // preconditioner, and training moves it away only as far as the data asks
  std::mt19937_64 rng(seed);
  for (int l = 0; l < kNetLayers - 1; l++) {
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (kNetTaps * net_cin(l))));
    for (int tap = 0; tap < kNetTaps; tap++)
      for (int ci = 0; ci < net_cin(l); ci++)
        for (int co = 0; co < net_cout(l); co++) w[(size_t)l * kNetPl + (tap * kNetCh + ci) * kNetCh + co] = nd(rng);
  }
  int st = OPAW_OK;
  do {
    if (cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&n->w32, sizeof(float) * np) != cudaSuccess ||
        cudaMalloc(&n->grad, sizeof(float) * np) != cudaSuccess ||
        cudaMalloc(&n->m, sizeof(float) * np) != cudaSuccess || cudaMalloc(&n->v, sizeof(float) * np) != cudaSuccess ||
        cudaMalloc(&n->wbf, sizeof(__nv_bfloat16) * kNetLayers * kNetWl) != cudaSuccess ||
        cudaMalloc(&n->wflip, sizeof(__nv_bfloat16) * kNetLayers * kNetWl) != cudaSuccess) {
      set_error("opaw_net_create: device allocation failed");
      st = OPAW_ERR_NOMEM;
      break;
    }
    if (cudaMemcpy(n->w32, w.data(), sizeof(float) * np, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(n->m, 0, sizeof(float) * np) != cudaSuccess || cudaMemset(n->v, 0, sizeof(float) * np) != cudaSuccess) {
      set_error("opaw_net_create: upload failed");
      st = OPAW_ERR_CUDA;
      break;
    }
    k_net_cast<<<grid1(np, 256), 256, 0, n->stream>>>(n->w32, n->wbf, n->wflip);
    if (cudaStreamSynchronize(n->stream) != cudaSuccess) {
      set_error("opaw_net_create: weight cast failed");
      st = OPAW_ERR_CUDA;
    }
  } while (0);
  if (st != OPAW_OK) {
    opaw_net_free(n);
    return st;
  }
  *out = n;
  return OPAW_OK;
}

int opaw_net_free(opaw_net *n) {
  if (!n) return OPAW_OK;
  if (n->stream) cudaStreamSynchronize(n->stream);
  void *ptrs[] = {n->w32, n->grad, n->m, n->v, n->wbf, n->wflip};
  for (void *p : ptrs) cudaFree(p);
  opaw::DeviceBuf *bufs[] = {&n->x, &n->a1, &n->a2, &n->pre0, &n->pre1, &n->out32, &n->d2, &n->d1, &n->d0,
                             &n->tgt, &n->part, &n->loss, &n->org};
  for (auto *b : bufs) cudaFree(b->p);
  if (n->stream) cudaStreamDestroy(n->stream);
  delete n;
  return OPAW_OK;
}

int opaw_net_params(opaw_net *n, float *w_out) {
  OPAW_ARG(n && w_out, "null argument");
  OPAW_CUDA(cudaMemcpyAsync(w_out, n->w32, sizeof(float) * kNetLayers * kNetPl, cudaMemcpyDeviceToHost, n->stream));
  OPAW_CUDA(cudaStreamSynchronize(n->stream));
  return OPAW_OK;
}

int opaw_net_set_params(opaw_net *n, const float *w) {
  OPAW_ARG(n && w, "null argument");
  OPAW_CUDA(cudaMemcpyAsync(n->w32, w, sizeof(float) * kNetLayers * kNetPl, cudaMemcpyHostToDevice, n->stream));
  k_net_cast<<<grid1((int64_t)kNetLayers * kNetPl, 256), 256, 0, n->stream>>>(n->w32, n->wbf, n->wflip);
  n->launches++;
  OPAW_CUDA(cudaGetLastError());
  OPAW_CUDA(cudaStreamSynchronize(n->stream));
  return OPAW_OK;
}

int64_t opaw_net_launches(opaw_net *n) { return n ? n->launches : 0; }

// a batch of P^3 patches from host arrays: x BF16 bits [batch][P^3][16],
// tgt [batch][P^3][2]
static int net_put_batch(opaw_net *n, int batch, int P, const uint16_t *x, const float *tgt) {
  const size_t nv = (size_t)batch * P * P * P;
  OPAW_CHECK(ensure(n->x, sizeof(uint16_t) * kNetCh * nv));
  OPAW_CHECK(ensure(n->tgt, sizeof(float) * 2 * nv));
  OPAW_CUDA(cudaMemcpyAsync(n->x.p, x, sizeof(uint16_t) * kNetCh * nv, cudaMemcpyHostToDevice, n->stream));
  OPAW_CUDA(cudaMemcpyAsync(n->tgt.p, tgt, sizeof(float) * 2 * nv, cudaMemcpyHostToDevice, n->stream));
  return OPAW_OK;
}

int opaw_net_loss_grad(opaw_net *n, int batch, int P, int margin, const uint16_t *x, const float *tgt, double *loss,
                       float *grad) {
  OPAW_ARG(n && x && tgt && batch > 0 && P > 2 * margin && margin >= 0, "bad arguments");
  OPAW_CHECK(net_put_batch(n, batch, P, x, tgt));
  OPAW_CHECK(net_loss_grad(n, batch, P, margin));
  if (loss) OPAW_CUDA(cudaMemcpyAsync(loss, n->loss.p, sizeof(double), cudaMemcpyDeviceToHost, n->stream));
  if (grad)
    OPAW_CUDA(cudaMemcpyAsync(grad, n->grad, sizeof(float) * kNetLayers * kNetPl, cudaMemcpyDeviceToHost, n->stream));
  OPAW_CUDA(cudaStreamSynchronize(n->stream));
  return OPAW_OK;
}

int opaw_net_forward(opaw_net *n, int batch, int nz, int ny, int nx, const uint16_t *x, float *out) {
  OPAW_ARG(n && x && out && batch > 0 && nz > 0 && ny > 0 && nx > 0, "bad arguments");
  const ConvDims d{batch, nz, ny, nx};
  const size_t nv = (size_t)batch * nz * ny * nx;
  OPAW_CHECK(ensure(n->x, sizeof(uint16_t) * kNetCh * nv));
  OPAW_CHECK(ensure(n->out32, sizeof(float) * kNetCh * nv));
  OPAW_CUDA(cudaMemcpyAsync(n->x.p, x, sizeof(uint16_t) * kNetCh * nv, cudaMemcpyHostToDevice, n->stream));
  OPAW_CHECK(net_forward(n, n->stream, d, (const __nv_bfloat16 *)n->x.p, (float *)n->out32.p, false, n->a1, n->a2));
  OPAW_CUDA(cudaMemcpyAsync(out, n->out32.p, sizeof(float) * kNetCh * nv, cudaMemcpyDeviceToHost, n->stream));
  OPAW_CUDA(cudaStreamSynchronize(n->stream));
  return OPAW_OK;
}

// Training patches from fields on a context's grid (device complex128
// residuals r and targets t, [orbital][point]; host eps, scale per orbital,
// origins [npatch][4] = orbital, z0, y0, x0), appended to the net's store at
// patch index `first` (the store grows to first + npatch patches).
int opaw_net_add_patches(opaw_net *n, opaw_ctx *c, const void *r, const void *t, int norb, const double *eps,
                         const double *scale, int npatch, const int *origins, int P, int first) {
  OPAW_ARG(n && c && r && t && eps && scale && origins && npatch > 0 && P > 0 && first >= 0, "bad arguments");
  OPAW_ARG(P <= c->nx && P <= c->ny && P <= c->nz, "patch larger than the grid");
  for (int i = 0; i < npatch; i++) OPAW_ARG(origins[4 * i] >= 0 && origins[4 * i] < norb, "patch orbital out of range");
  const int64_t P3 = (int64_t)P * P * P;
  const size_t tot = (size_t)(first + npatch) * P3;
  // grow the stores keeping the patches already there
  auto grow = [&](opaw::DeviceBuf &b, size_t bytes, size_t keep) -> int {
    if (b.bytes >= bytes) return OPAW_OK;
    void *q = nullptr;
    OPAW_CUDA(cudaMalloc(&q, bytes));
    if (b.p && keep) OPAW_CUDA(cudaMemcpyAsync(q, b.p, keep, cudaMemcpyDeviceToDevice, n->stream));
    OPAW_CUDA(cudaStreamSynchronize(n->stream));
    cudaFree(b.p);
    b.p = q;
    b.bytes = bytes;
    return OPAW_OK;
  };
  OPAW_CHECK(grow(n->x, sizeof(uint16_t) * kNetCh * tot, sizeof(uint16_t) * kNetCh * (size_t)first * P3));
  OPAW_CHECK(grow(n->tgt, sizeof(float) * 2 * tot, sizeof(float) * 2 * (size_t)first * P3));
  OPAW_CHECK(ensure(c->pre, sizeof(double) * 2 * (size_t)norb));
  OPAW_CHECK(ensure(n->org, sizeof(int4) * (size_t)npatch));
  // the context's stream produced r and t; the net's stream consumes them
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  double *es = (double *)c->pre.p;
  OPAW_CUDA(cudaMemcpyAsync(es, eps, sizeof(double) * norb, cudaMemcpyHostToDevice, n->stream));
  OPAW_CUDA(cudaMemcpyAsync(es + norb, scale, sizeof(double) * norb, cudaMemcpyHostToDevice, n->stream));
  OPAW_CUDA(cudaMemcpyAsync(n->org.p, origins, sizeof(int4) * (size_t)npatch, cudaMemcpyHostToDevice, n->stream));
  k_net_patches<<<dim3(grid1(P3, 256), npatch), 256, 0, n->stream>>>(
      (const double2 *)r, (const double2 *)t, c->d_vks[0], es, es + norb, (const int4 *)n->org.p, P, c->nx, c->ny,
      c->nz, (__nv_bfloat16 *)n->x.p + (size_t)first * P3 * kNetCh, (float *)n->tgt.p + (size_t)first * P3 * 2);
  n->launches++;
  OPAW_CUDA(cudaGetLastError());
  OPAW_CUDA(cudaStreamSynchronize(n->stream));
  return OPAW_OK;
}

// nsteps Adam steps on minibatches of the stored patches: batch b of step s
// is patches (s * batch + i) % npatch; losses[s] receives each step's loss
int opaw_net_train(opaw_net *n, int npatch, int P, int margin, int nsteps, int batch, double lr, double *losses) {
  OPAW_ARG(n && npatch > 0 && batch > 0 && nsteps >= 0 && P > 2 * margin && margin >= 0, "bad arguments");
  const int64_t P3 = (int64_t)P * P * P;
  OPAW_ARG(n->x.bytes >= sizeof(uint16_t) * kNetCh * (size_t)npatch * P3, "fewer stored patches than npatch");
  // the minibatch is gathered from the store into a contiguous block
  opaw::DeviceBuf store_x = n->x, store_t = n->tgt;
  opaw::DeviceBuf bx, bt;
  int st = OPAW_OK;
  std::vector<double> hl((size_t)nsteps);
  double *dl = nullptr;
  do {
    if (cudaMalloc(&bx.p, sizeof(uint16_t) * kNetCh * (size_t)batch * P3) != cudaSuccess ||
        cudaMalloc(&bt.p, sizeof(float) * 2 * (size_t)batch * P3) != cudaSuccess ||
        cudaMalloc(&dl, sizeof(double) * (size_t)(nsteps > 0 ? nsteps : 1)) != cudaSuccess) {
      set_error("opaw_net_train: device allocation failed");
      st = OPAW_ERR_NOMEM;
      break;
    }
    bx.bytes = sizeof(uint16_t) * kNetCh * (size_t)batch * P3;
    bt.bytes = sizeof(float) * 2 * (size_t)batch * P3;
    const float b1 = 0.9f, b2 = 0.999f;
    for (int s = 0; s < nsteps && st == OPAW_OK; s++) {
      k_net_gather<<<dim3((unsigned)std::min<int64_t>(grid1(P3, 256), 64), batch), 256, 0, n->stream>>>(
          (const uint4 *)store_x.p, (const float2 *)store_t.p, P3, npatch, s, batch, (uint4 *)bx.p, (float2 *)bt.p);
      n->launches++;
      if (cudaGetLastError() != cudaSuccess) {
        set_error("opaw_net_train: batch gather failed");
        st = OPAW_ERR_CUDA;
        break;
      }
      n->x = bx;
      n->tgt = bt;
      st = net_loss_grad(n, batch, P, margin);
      n->x = store_x;
      n->tgt = store_t;
      if (st != OPAW_OK) break;
      n->step++;
      const float c1 = 1.f / (1.f - std::pow(b1, (float)n->step)), c2 = 1.f / (1.f - std::pow(b2, (float)n->step));
      k_net_adam<<<grid1((int64_t)kNetLayers * kNetPl, 256), 256, 0, n->stream>>>(
          n->w32, n->grad, n->m, n->v, (float)lr, b1, b2, c1, c2, 1e-8f, n->wbf, n->wflip);
      n->launches++;
      if (cudaGetLastError() != cudaSuccess ||
          cudaMemcpyAsync(dl + s, n->loss.p, sizeof(double), cudaMemcpyDeviceToDevice, n->stream) != cudaSuccess) {
        set_error("opaw_net_train: update failed");
        st = OPAW_ERR_CUDA;
      }
    }
    if (st != OPAW_OK) break;
    if (nsteps > 0 && (cudaMemcpyAsync(hl.data(), dl, sizeof(double) * nsteps, cudaMemcpyDeviceToHost, n->stream) !=
                           cudaSuccess ||
                       cudaStreamSynchronize(n->stream) != cudaSuccess)) {
      set_error("opaw_net_train: loss copy failed");
      st = OPAW_ERR_CUDA;
    }
  } while (0);
  cudaStreamSynchronize(n->stream);
  n->x = store_x;
  n->tgt = store_t;
  cudaFree(bx.p);
  cudaFree(bt.p);
  cudaFree(dl);
  if (st == OPAW_OK && losses)
    for (int s = 0; s < nsteps; s++) losses[s] = hl[s];
  return st;
}

// The learned preconditioner on norb device orbitals of a context: w =
// K r + |r| N(r / |r|, v_ks - eps), K the Teter-Payne-Allan preconditioner
// (kinetic energies ekin), N the network; eps and ekin host arrays [norb]
// (consumed before the call returns).  Asynchronous on the context's stream;
// scratch in the net.
int opaw_precond_learned_dev(opaw_ctx *c, opaw_net *n, int dtype, const void *r, const double *eps,
                             const double *ekin, void *w, int norb) {
  OPAW_ARG(c && n && r && eps && ekin && w && norb >= 0, "bad arguments");
  OPAW_ARG(dtype == OPAW_C128 || dtype == OPAW_C64, "dtype must be OPAW_C128 or OPAW_C64");
  if (norb == 0) return OPAW_OK;
  OPAW_ARG(r != w, "the residual and the output must differ");
  std::vector<double> h(3 * (size_t)norb);
  for (int i = 0; i < norb; i++) {
    OPAW_ARG(ekin[i] > 0.0 && std::isfinite(ekin[i]) && std::isfinite(eps[i]), "bad eps or ekin");
    h[i] = 1.0 / ekin[i];
    h[norb + i] = eps[i];
  }
  OPAW_CHECK(ensure(c->pre, sizeof(double) * 5 * (size_t)norb));
  double *dinv = (double *)c->pre.p, *deps = dinv + norb, *dn2 = deps + norb, *dsc = dn2 + norb, *dnrm = dsc + norb;
  OPAW_CUDA(cudaMemcpyAsync(dinv, h.data(), sizeof(double) * 2 * norb, cudaMemcpyHostToDevice, c->stream));
  if (dtype == OPAW_C128) k_net_norm2<double2><<<norb, 256, 0, c->stream>>>((const double2 *)r, c->nn, dn2);
  else k_net_norm2<float2><<<norb, 256, 0, c->stream>>>((const float2 *)r, c->nn, dn2);
  k_net_scales<<<grid1(norb, 128), 128, 0, c->stream>>>(dn2, c->dv, norb, dsc, dnrm);
  c->launches += 2;
  OPAW_CUDA(cudaGetLastError());
  // K r first (it reads r, writes w)
  if (dtype == OPAW_C128) OPAW_CHECK(precond_kinetic<double>(c, (const double2 *)r, dinv, (double2 *)w, norb));
  else OPAW_CHECK(precond_kinetic<float>(c, (const float2 *)r, dinv, (float2 *)w, norb));
  // the network on the whole grid of every orbital
  const size_t nv = (size_t)norb * c->nn;
  OPAW_CHECK(ensure(n->d0, sizeof(__nv_bfloat16) * kNetCh * nv));  // input features
  OPAW_CHECK(ensure(n->out32, sizeof(float) * kNetCh * nv));
  const dim3 g(grid1(c->nn, 256), norb);
  if (dtype == OPAW_C128)
    k_net_input<double2><<<g, 256, 0, c->stream>>>((const double2 *)r, c->d_vks[0], deps, dsc, c->nn,
                                                  (__nv_bfloat16 *)n->d0.p);
  else
    k_net_input<float2><<<g, 256, 0, c->stream>>>((const float2 *)r, c->d_vks[0], deps, dsc, c->nn,
                                                 (__nv_bfloat16 *)n->d0.p);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  const ConvDims d{norb, c->nz, c->ny, c->nx};
  OPAW_CHECK(net_forward(n, c->stream, d, (const __nv_bfloat16 *)n->d0.p, (float *)n->out32.p, false, n->d1, n->d2));
  c->launches += 3;
  if (dtype == OPAW_C128)
    k_net_combine<double2><<<g, 256, 0, c->stream>>>((const float *)n->out32.p, dnrm, c->nn, (double2 *)w);
  else
    k_net_combine<float2><<<g, 256, 0, c->stream>>>((const float *)n->out32.p, dnrm, c->nn, (float2 *)w);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

}  // extern "C"

// fft.cuh — batched 3D FFT building block: one kernel per axis that stages a
// tile of lines in shared memory and runs a mixed-radix Stockham autosort
// transform on it (radices 2, 3, 4, 5, 7, 8).  Element-wise work that belongs
// next to an FFT (kinetic scaling, v_ks multiply, Hartree kernel, embedding
// and cropping of the 2x box) is fused into the load / mid / store hooks of
// an operation functor, so it costs no extra pass over HBM.
//
// Conventions follow FFTW as the reference calls it
// (lib/library_fftw_v3.f90:56-83): unnormalised, forward sign -1, backward +1.
#pragma once

#include <algorithm>
#include <string>
#include <type_traits>
#include <typeinfo>
#include <utility>

#include "common.cuh"

namespace opaw {

struct AxisDev {
  int n;
  int nstage;
  int radix[16];
};

// n0,n1,n2: array extents (x fastest)
struct Dims3 {
  int n0, n1, n2;
};
// a subset of the lines of an axis pass (see ct_tile_geom); full() = all
struct LineSub {
  int a0, na, b0, nb;
  static LineSub full(const Dims3 &d) { return LineSub{0, d.n1, 0, d.n2}; }
};


template <typename C> struct CplxOf;
template <> struct CplxOf<float2> { typedef float R; };
template <> struct CplxOf<double2> { typedef double R; };

// multiply by sign*i (sign = -1 forward): (a+ib)*(s*i) = -s*b + i*s*a
template <typename C> __device__ __forceinline__ C mul_si(C z, int sign) {
  C r;
  r.x = -sign * z.y;
  r.y = sign * z.x;
  return r;
}

// twiddle W_n^t for the transform direction (table holds exp(-2 pi i t/n))
template <typename C> __device__ __forceinline__ C twid(const C *tw, int t, int sign) {
  C w = tw[t];
  if (sign > 0) w.y = -w.y;
  return w;
}

template <typename C, int R> struct Butterfly;

template <typename C> struct Butterfly<C, 2> {
  static __device__ __forceinline__ void run(C *u, const C *, int, int) {
    C a = u[0], b = u[1];
    u[0] = cadd(a, b);
    u[1] = csub(a, b);
  }
};

template <typename C> struct Butterfly<C, 4> {
  static __device__ __forceinline__ void run(C *u, const C *, int, int sign) {
    C a = cadd(u[0], u[2]), b = csub(u[0], u[2]);
    C c = cadd(u[1], u[3]), d = mul_si(csub(u[1], u[3]), sign);
    u[0] = cadd(a, c);
    u[2] = csub(a, c);
    u[1] = cadd(b, d);
    u[3] = csub(b, d);
  }
};

template <typename C> struct Butterfly<C, 8> {
  static __device__ __forceinline__ void run(C *u, const C *, int, int sign) {
    typedef typename CplxOf<C>::R R;
    const R h = (R)0.70710678118654752440084436210485;  // 1/sqrt(2)
    C e[4] = {u[0], u[2], u[4], u[6]};
    C o[4] = {u[1], u[3], u[5], u[7]};
    Butterfly<C, 4>::run(e, nullptr, 0, sign);
    Butterfly<C, 4>::run(o, nullptr, 0, sign);
    // W8^1 = (1 + s i)/sqrt2, W8^2 = s i, W8^3 = (-1 + s i)/sqrt2
    C o1 = o[1], o3 = o[3];
    C w1o1, w3o3;
    w1o1.x = h * (o1.x - sign * o1.y);
    w1o1.y = h * (o1.y + sign * o1.x);
    w3o3.x = h * (-o3.x - sign * o3.y);
    w3o3.y = h * (-o3.y + sign * o3.x);
    C w2o2 = mul_si(o[2], sign);
    u[0] = cadd(e[0], o[0]);
    u[4] = csub(e[0], o[0]);
    u[1] = cadd(e[1], w1o1);
    u[5] = csub(e[1], w1o1);
    u[2] = cadd(e[2], w2o2);
    u[6] = csub(e[2], w2o2);
    u[3] = cadd(e[3], w3o3);
    u[7] = csub(e[3], w3o3);
  }
};

// radix 3 with the constants of W3 = -1/2 + s i sqrt(3)/2
template <typename C> struct Butterfly<C, 3> {
  static __device__ __forceinline__ void run(C *u, const C *, int, int sign) {
    typedef typename CplxOf<C>::R R;
    const R h3 = (R)0.86602540378443864676372317075294;  // sqrt(3)/2
    const C t1 = cadd(u[1], u[2]);
    C t2;
    t2.x = u[0].x - (R)0.5 * t1.x;
    t2.y = u[0].y - (R)0.5 * t1.y;
    const C t3 = cscale(mul_si(csub(u[1], u[2]), sign), h3);
    u[0] = cadd(u[0], t1);
    u[1] = cadd(t2, t3);
    u[2] = csub(t2, t3);
  }
};

// radix 6 = 3 x 2: two 3-point DFTs, twiddles W6^c, then 2-point DFTs
template <typename C> struct Butterfly<C, 6> {
  static __device__ __forceinline__ void run(C *u, const C *, int, int sign) {
    typedef typename CplxOf<C>::R R;
    const R h3 = (R)0.86602540378443864676372317075294;
    C a[3] = {u[0], u[2], u[4]};
    C b[3] = {u[1], u[3], u[5]};
    Butterfly<C, 3>::run(a, nullptr, 0, sign);
    Butterfly<C, 3>::run(b, nullptr, 0, sign);
    // W6^1 = 1/2 + s i sqrt3/2, W6^2 = -1/2 + s i sqrt3/2
    C w1, w2;
    w1.x = (R)0.5 * b[1].x - sign * h3 * b[1].y;
    w1.y = (R)0.5 * b[1].y + sign * h3 * b[1].x;
    w2.x = (R)-0.5 * b[2].x - sign * h3 * b[2].y;
    w2.y = (R)-0.5 * b[2].y + sign * h3 * b[2].x;
    u[0] = cadd(a[0], b[0]);
    u[3] = csub(a[0], b[0]);
    u[1] = cadd(a[1], w1);
    u[4] = csub(a[1], w1);
    u[2] = cadd(a[2], w2);
    u[5] = csub(a[2], w2);
  }
};

// radix 16 = 4 x 4: four 4-point DFTs over q = 4a + b, twiddles W16^{bc},
// four 4-point DFTs over b
template <typename C> struct Butterfly<C, 16> {
  static __device__ __forceinline__ C rot(C z, int e, int sign) {
    // z * W16^e for e in 0..9 (W16 = exp(s 2 pi i / 16))
    typedef typename CplxOf<C>::R R;
    const R c1 = (R)0.92387953251128675612818318939679;  // cos(pi/8)
    const R s1 = (R)0.38268343236508977172845998403040;  // sin(pi/8)
    const R h = (R)0.70710678118654752440084436210485;
    R cr, ci;
    switch (e) {
      case 0: return z;
      case 1: cr = c1; ci = s1; break;
      case 2: cr = h; ci = h; break;
      case 3: cr = s1; ci = c1; break;
      case 4: return mul_si(z, sign);
      case 6: cr = -h; ci = h; break;
      case 9: cr = -c1; ci = -s1; break;
      default: cr = 1; ci = 0; break;
    }
    ci *= sign;
    C r;
    r.x = z.x * cr - z.y * ci;
    r.y = z.x * ci + z.y * cr;
    return r;
  }
  static __device__ __forceinline__ void run(C *u, const C *, int, int sign) {
    C A[4][4];
#pragma unroll
    for (int b = 0; b < 4; b++) {
      C t[4] = {u[b], u[4 + b], u[8 + b], u[12 + b]};
      Butterfly<C, 4>::run(t, nullptr, 0, sign);
#pragma unroll
      for (int c = 0; c < 4; c++) A[b][c] = rot(t[c], b * c, sign);
    }
#pragma unroll
    for (int c = 0; c < 4; c++) {
      C t[4] = {A[0][c], A[1][c], A[2][c], A[3][c]};
      Butterfly<C, 4>::run(t, nullptr, 0, sign);
#pragma unroll
      for (int d = 0; d < 4; d++) u[c + 4 * d] = t[d];
    }
  }
};

// generic odd radix (5, 7, 11, 13) from the twiddle table: y_s = sum_q u_q W_r^{qs}
template <typename C, int R> struct Butterfly {
  static __device__ __forceinline__ void run(C *u, const C *tw, int n, int sign) {
    C y[R];
    const int step = n / R;
#pragma unroll
    for (int s = 0; s < R; s++) {
      C acc = u[0];
#pragma unroll
      for (int q = 1; q < R; q++) acc = cadd(acc, cmul(u[q], twid(tw, ((q * s) % R) * step, sign)));
      y[s] = acc;
    }
#pragma unroll
    for (int s = 0; s < R; s++) u[s] = y[s];
  }
};

// One Stockham stage over all lines of the tile.  Element (l, j) of the tile
// sits at l*ls + j*js.  linefast selects the thread mapping (lines fastest
// for strided axes, butterflies fastest for the contiguous axis).
template <typename C, int R>
__device__ __forceinline__ void stage(const C *in, C *out, int n, int p, int TL, int ls, int js, bool linefast,
                                      const C *tw, int sign) {
  const int m = n / R;
  const int nb = TL * m;
  const int tstep = n / (p * R);
  for (int idx = threadIdx.x; idx < nb; idx += blockDim.x) {
    int l, i;
    if (linefast) {
      l = idx % TL;
      i = idx / TL;
    } else {
      i = idx % m;
      l = idx / m;
    }
    const int k = i % p;
    C u[R];
#pragma unroll
    for (int q = 0; q < R; q++) u[q] = in[l * ls + (i + q * m) * js];
    if (p > 1) {
#pragma unroll
      for (int q = 1; q < R; q++) u[q] = cmul(u[q], twid(tw, q * k * tstep, sign));
    }
    Butterfly<C, R>::run(u, tw, n, sign);
    const int j = (i - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; q++) out[l * ls + (j + q * p) * js] = u[q];
  }
}

// full transform of the tile: ping-pong between a and b, returns the buffer
// holding the result
template <typename C>
__device__ C *tile_fft(C *a, C *b, const AxisDev &ax, int TL, int ls, int js, bool linefast, const C *tw, int sign) {
  int p = 1;
  for (int s = 0; s < ax.nstage; s++) {
    const int r = ax.radix[s];
    switch (r) {
      case 2: stage<C, 2>(a, b, ax.n, p, TL, ls, js, linefast, tw, sign); break;
      case 3: stage<C, 3>(a, b, ax.n, p, TL, ls, js, linefast, tw, sign); break;
      case 4: stage<C, 4>(a, b, ax.n, p, TL, ls, js, linefast, tw, sign); break;
      case 5: stage<C, 5>(a, b, ax.n, p, TL, ls, js, linefast, tw, sign); break;
      case 7: stage<C, 7>(a, b, ax.n, p, TL, ls, js, linefast, tw, sign); break;
      case 11: stage<C, 11>(a, b, ax.n, p, TL, ls, js, linefast, tw, sign); break;
      case 13: stage<C, 13>(a, b, ax.n, p, TL, ls, js, linefast, tw, sign); break;
      default: stage<C, 8>(a, b, ax.n, p, TL, ls, js, linefast, tw, sign); break;
    }
    __syncthreads();
    C *t = a;
    a = b;
    b = t;
    p *= r;
  }
  return a;
}

// Axis kernel.  AXIS 0: lines along x (contiguous tiles); AXIS 1: lines along
// y, tiles of TL consecutive x at one z; AXIS 2: lines along z, tiles of TL
// consecutive (x,y) positions.  Op supplies load/store (by linear element
// index g and batch b) and, when Op::kMid, a k-space hook between a forward
// and an inverse transform in the same kernel.
template <typename C, int AXIS, class Op>
__global__ void __launch_bounds__(256) k_fft_axis(AxisDev ax, Dims3 d, int TL, int sign, const C *__restrict__ twg, Op op) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *tw = reinterpret_cast<C *>(smem_raw);
  const int n = ax.n;
  C *bufa = tw + n;
  C *bufb = bufa + (size_t)TL * n;
  for (int t = threadIdx.x; t < n; t += blockDim.x) tw[t] = twg[t];

  const int b = blockIdx.y;
  const int64_t tile = blockIdx.x;
  int64_t base;       // linear index of element (l=0, j=0)
  int64_t lstride;    // linear stride between consecutive lines of the tile
  int64_t jstride;    // linear stride between consecutive elements of a line
  int nl;             // valid lines in this tile
  if (AXIS == 0) {
    const int64_t nlines = (int64_t)d.n1 * d.n2;
    const int64_t l0 = tile * TL;
    nl = (int)min((int64_t)TL, nlines - l0);
    base = l0 * d.n0;
    lstride = d.n0;
    jstride = 1;
  } else if (AXIS == 1) {
    const int tpz = (d.n0 + TL - 1) / TL;
    const int z = (int)(tile / tpz);
    const int x0 = (int)(tile % tpz) * TL;
    nl = min(TL, d.n0 - x0);
    base = x0 + (int64_t)d.n0 * d.n1 * z;
    lstride = 1;
    jstride = d.n0;
  } else {
    const int64_t nlines = (int64_t)d.n0 * d.n1;
    const int64_t t0 = tile * TL;
    nl = (int)min((int64_t)TL, nlines - t0);
    base = t0;
    lstride = 1;
    jstride = (int64_t)d.n0 * d.n1;
  }
  const bool linefast = (AXIS != 0);
  const int ls = linefast ? 1 : n;
  const int js = linefast ? TL : 1;
  const int tot = TL * n;
  for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
    int l, j;
    if (linefast) { j = idx / TL; l = idx % TL; } else { l = idx / n; j = idx % n; }
    C v;
    if (l < nl) v = op.load(b, base + l * lstride + j * jstride);
    else { v.x = 0; v.y = 0; }
    bufa[l * ls + j * js] = v;
  }
  __syncthreads();
  C *res;
  if (Op::kMid) {
    res = tile_fft(bufa, bufb, ax, TL, ls, js, linefast, tw, -1);
    C *other = (res == bufa) ? bufb : bufa;
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
      int l, j;
      if (linefast) { j = idx / TL; l = idx % TL; } else { l = idx / n; j = idx % n; }
      if (l < nl) res[l * ls + j * js] = op.mid(b, base + l * lstride + j * jstride, op.line(base + l * lstride), j, res[l * ls + j * js]);
    }
    __syncthreads();
    res = tile_fft(res, other, ax, TL, ls, js, linefast, tw, +1);
  } else {
    res = tile_fft(bufa, bufb, ax, TL, ls, js, linefast, tw, sign);
  }
  for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
    int l, j;
    if (linefast) { j = idx / TL; l = idx % TL; } else { l = idx / n; j = idx % n; }
    if (l < nl) op.store(b, base + l * lstride + j * jstride, res[l * ls + j * js]);
  }
}

// plain load/store between two batched arrays (may alias)
// ---- staging helpers shared by the shared-memory FFT kernels
// Ops whose load is a plain read of array raw(b) at g stage their tile with
// cp.async (global -> shared, no registers, every copy of a thread in flight
// at once); ops with a prefetch/finish split (pre + fin) have their epilogue
// operands loaded in chunks before any store.
template <class Op, class = void> struct HasRaw : std::false_type {};
template <class Op>
struct HasRaw<Op, std::void_t<decltype(std::declval<const Op &>().raw(0))>> : std::true_type {};
template <class Op, class = void> struct HasPre : std::false_type {};
template <class Op>
struct HasPre<Op, std::void_t<decltype(std::declval<const Op &>().pre(0, int64_t(0)))>> : std::true_type {};

template <typename C> __device__ __forceinline__ void cp_async_elem(C *smem, const C *gmem) {
  static_assert(sizeof(C) == 8 || sizeof(C) == 16, "complex64 or complex128 elements");
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (sizeof(C) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
// asynchronous prefetch of a contiguous range into L2 (16-byte aligned start,
// size a multiple of 16 bytes); no data reaches the SM
__device__ __forceinline__ void l2_prefetch_bulk(const void *gmem, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(gmem), "r"(bytes) : "memory");
}


// a readable name of an operation functor for the autotuner's keys: its
// kName when it has one, else the type's name
template <class Op, class = void> struct OpNameOf {
  static std::string get() { return typeid(Op).name(); }
};
template <class Op> struct OpNameOf<Op, std::void_t<decltype(Op::kName)>> {
  static std::string get() { return Op::kName; }
};

template <typename C> struct OpCopy {
  static constexpr const char *kName = "copy";
  const C *src;
  C *dst;
  int64_t bstride;
  static constexpr bool kMid = false;
  __device__ C load(int b, int64_t g) const { return src[b * bstride + g]; }
  __device__ const C *raw(int b) const { return src + b * bstride; }
  __device__ void store(int b, int64_t g, C v) const { dst[b * bstride + g] = v; }
  __device__ double line(int64_t) const { return 0.0; }
  __device__ C mid(int, int64_t, double, int, C v) const { return v; }
};

template <typename C> inline int tile_lines(int axis, int n, int nlines_hint) {
  const int budget = sizeof(C) == 8 ? 4096 : 2048;  // elements per ping-pong buffer
  int tl = budget / n;
  if (tl < 1) tl = 1;
  if (tl > 32) tl = 32;
  (void)axis;
  (void)nlines_hint;
  return tl;
}

template <typename C> inline const C *axis_tw(const FFTAxis &a);
template <> inline const float2 *axis_tw<float2>(const FFTAxis &a) { return a.tw32; }
template <> inline const double2 *axis_tw<double2>(const FFTAxis &a) { return a.tw64; }

inline AxisDev axis_dev(const FFTAxis &a) {
  AxisDev d;
  d.n = a.n;
  d.nstage = a.nstage;
  for (int i = 0; i < 16; i++) d.radix[i] = a.radix[i];
  return d;
}

// ------------------------------------------------------------------------
// Specialised transform: the line length N, its radix plan and the tile
// width TL are compile-time constants, so every index of the butterfly loops
// is a multiply/shift and the stages unroll.  All axes stage the tile as
// [element][line] with an odd line stride TL+1: threads of a warp take
// consecutive lines of the same butterfly, which keeps shared memory free of
// bank conflicts for every stage and every axis.
// ------------------------------------------------------------------------
constexpr int kRadixPref[8] = {16, 8, 6, 4, 2, 3, 5, 7};
constexpr int ct_nstage(int n) {
  int c = 0;
  for (int k = 0; k < 8; k++)
    while (n % kRadixPref[k] == 0) { n /= kRadixPref[k]; c++; }
  return n == 1 ? c : -1;
}
constexpr int ct_radix(int n, int s) {
  int c = 0;
  for (int k = 0; k < 8; k++)
    while (n % kRadixPref[k] == 0) {
      if (c == s) return kRadixPref[k];
      n /= kRadixPref[k];
      c++;
    }
  return 1;
}
constexpr int ct_pre(int n, int s) {  // product of the radices before stage s
  int p = 1;
  for (int t = 0; t < s; t++) p *= ct_radix(n, t);
  return p;
}

template <typename C, int N, int TL, int NT, int S>
__device__ __forceinline__ void ct_stage(const C *__restrict__ in, C *__restrict__ out, const C *tw, int sign) {
  constexpr int R = ct_radix(N, S);
  constexpr int P = ct_pre(N, S);
  constexpr int M = N / R;
  constexpr int NB = TL * M;
  constexpr int TSTEP = N / (P * R);
  constexpr int LS = TL + 1;
#pragma unroll 1
  for (int idx = threadIdx.x; idx < NB; idx += NT) {
    const int l = idx % TL;
    const int i = idx / TL;
    const int k = i % P;
    C u[R];
#pragma unroll
    for (int q = 0; q < R; q++) u[q] = in[(i + q * M) * LS + l];
    if (P > 1) {
#pragma unroll
      for (int q = 1; q < R; q++) u[q] = cmul(u[q], twid(tw, q * k * TSTEP, sign));
    }
    Butterfly<C, R>::run(u, tw, N, sign);
    const int j = (i - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; q++) out[(j + q * P) * LS + l] = u[q];
  }
}

// ---- stages with explicit element accessors (shared tile or global memory)
// Element j (along the transformed axis) of line l of the tile.
template <typename C, int TL> struct SmemAcc {
  C *p;
  __device__ __forceinline__ C get(int j, int l) const { return p[j * (TL + 1) + l]; }
  __device__ __forceinline__ void put(int j, int l, C v) const { p[j * (TL + 1) + l] = v; }
};
template <typename C, class Op> struct GlobIn {  // the op's load; lines past nl read zero
  Op op;
  int b, lstride, jstride, nl;
  int64_t base;
  __device__ __forceinline__ C get(int j, int l) const {
    C v;
    v.x = 0;
    v.y = 0;
    if (l < nl) v = op.load(b, base + (int64_t)l * lstride + (int64_t)j * jstride);
    return v;
  }
};
template <typename C, int TL, class Op, typename L> struct MidAcc {  // k-space hook on the way into the tile
  C *p;
  Op op;
  int b, lstride, jstride, nl;
  int64_t base;
  const L *lvs;
  __device__ __forceinline__ void put(int j, int l, C v) const {
    if (l < nl) v = op.mid(b, base + (int64_t)l * lstride + (int64_t)j * jstride, lvs[l], j, v);
    p[j * (TL + 1) + l] = v;
  }
};
template <typename C, class Op> struct GlobOut {  // the op's store; lines past nl skipped
  Op op;
  int b, lstride, jstride, nl;
  int64_t base;
  __device__ __forceinline__ void put(int j, int l, C v) const {
    if (l < nl) op.store(b, base + (int64_t)l * lstride + (int64_t)j * jstride, v);
  }
};

template <typename C, int N, int TL, int NT, int S, class In, class Out>
__device__ __forceinline__ void ct_stage_io(const In &in, const Out &out, const C *tw, int sign) {
  constexpr int R = ct_radix(N, S);
  constexpr int P = ct_pre(N, S);
  constexpr int M = N / R;
  constexpr int NB = TL * M;
  constexpr int TSTEP = N / (P * R);
#pragma unroll 1
  for (int idx = threadIdx.x; idx < NB; idx += NT) {
    const int l = idx % TL;
    const int i = idx / TL;
    const int k = i % P;
    C u[R];
#pragma unroll
    for (int q = 0; q < R; q++) u[q] = in.get(i + q * M, l);
    if (P > 1) {
#pragma unroll
      for (int q = 1; q < R; q++) u[q] = cmul(u[q], twid(tw, q * k * TSTEP, sign));
    }
    Butterfly<C, R>::run(u, tw, N, sign);
    const int j = (i - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; q++) out.put(j + q * P, l, u[q]);
  }
}

// forward stages S..: the first reads `in`, the last writes through the
// k-space hook into buffer `dst`; returns the buffer holding the result
template <typename C, int N, int TL, int NT, int S, class In, class Mid>
__device__ __forceinline__ C *ct_fwd_mid(const In &in, C *dst, C *oth, const C *tw, Mid mo) {
  if constexpr (S == ct_nstage(N) - 1) {
    mo.p = dst;
    ct_stage_io<C, N, TL, NT, S>(in, mo, tw, -1);
    __syncthreads();
    return dst;
  } else {
    ct_stage_io<C, N, TL, NT, S>(in, SmemAcc<C, TL>{dst}, tw, -1);
    __syncthreads();
    return ct_fwd_mid<C, N, TL, NT, S + 1>(SmemAcc<C, TL>{dst}, oth, dst, tw, mo);
  }
}

// inverse stages S.. from shared buffer src; the last writes through `out`
template <typename C, int N, int TL, int NT, int S, class Out>
__device__ __forceinline__ void ct_inv_out(C *src, C *oth, const C *tw, const Out &out) {
  if constexpr (S == ct_nstage(N) - 1) {
    ct_stage_io<C, N, TL, NT, S>(SmemAcc<C, TL>{src}, out, tw, +1);
  } else {
    ct_stage_io<C, N, TL, NT, S>(SmemAcc<C, TL>{src}, SmemAcc<C, TL>{oth}, tw, +1);
    __syncthreads();
    ct_inv_out<C, N, TL, NT, S + 1>(oth, src, tw, out);
  }
}

template <typename C, int N, int TL, int NT, int S> struct CtStages {
  // runs stages S.. and returns the buffer holding the result
  static __device__ __forceinline__ C *run(C *a, C *b, const C *tw, int sign) {
    if constexpr (S >= ct_nstage(N)) {
      return a;
    } else {
      ct_stage<C, N, TL, NT, S>(a, b, tw, sign);
      __syncthreads();
      return CtStages<C, N, TL, NT, S + 1>::run(b, a, tw, sign);
    }
  }
};

// the lines of tile `tile` of an axis pass: first element, strides, count.
// sub restricts the lines: x lines with y in [a0, a0+na) and z in [b0, b0+nb);
// y lines with z in [b0, b0+nb); z lines are always all of them.
template <int N, int TL, int AXIS>
__device__ __forceinline__ void ct_tile_geom(const Dims3 &d, const LineSub &sub, int tile, int64_t &base,
                                             int &lstride, int &jstride, int &nl) {
  if (AXIS == 0) {
    const int tpy = (sub.na + TL - 1) / TL;
    const int zr = tile / tpy;
    const int y0 = (tile - zr * tpy) * TL;
    nl = min(TL, sub.na - y0);
    base = ((int64_t)(sub.a0 + y0) + (int64_t)d.n1 * (sub.b0 + zr)) * N;
    lstride = N;
    jstride = 1;
  } else if (AXIS == 1) {
    const int tpz = (d.n0 + TL - 1) / TL;
    const int zr = tile / tpz;
    const int x0 = (tile - zr * tpz) * TL;
    nl = min(TL, d.n0 - x0);
    base = x0 + (int64_t)d.n0 * d.n1 * (sub.b0 + zr);
    lstride = 1;
    jstride = d.n0;
  } else {
    const int nlines = d.n0 * d.n1;
    const int t0 = tile * TL;
    nl = min(TL, nlines - t0);
    base = t0;
    lstride = 1;
    jstride = d.n0 * d.n1;
  }
}

template <typename C, int N, int TL, int AXIS, class Op>
__global__ void __launch_bounds__(256) k_fft_ct(Dims3 d, LineSub sub, int sign, const C *__restrict__ twg, Op op) {
  constexpr int NT = 256;
  constexpr int LS = TL + 1;
  static_assert(ct_nstage(N) > 0, "unsupported length");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *tw = reinterpret_cast<C *>(smem_raw);
  C *bufa = tw + N;
  C *bufb = bufa + N * LS;
  for (int t = threadIdx.x; t < N; t += NT) tw[t] = twg[t];
  const int b = blockIdx.y;
  const int tile = blockIdx.x;
  int64_t base;
  int lstride, jstride, nl;
  ct_tile_geom<N, TL, AXIS>(d, sub, tile, base, lstride, jstride, nl);
  constexpr int TOT = TL * N;
  if constexpr (Op::kMid) {
    // forward transform -> k-space hook -> inverse transform: the first stage
    // reads global memory, the hook rides on the last forward stage's
    // writes, the last inverse stage writes global memory
    typedef decltype(op.line(0)) L;
    __shared__ L lvs[TL];
    if (threadIdx.x < nl) lvs[threadIdx.x] = op.line(base + threadIdx.x * lstride);
    __syncthreads();  // twiddles and line values
    GlobIn<C, Op> gin{op, b, lstride, jstride, nl, base};
    MidAcc<C, TL, Op, L> mo{bufa, op, b, lstride, jstride, nl, base, lvs};
    C *res = ct_fwd_mid<C, N, TL, NT, 0>(gin, bufa, bufb, tw, mo);
    ct_inv_out<C, N, TL, NT, 0>(res, res == bufa ? bufb : bufa, tw, GlobOut<C, Op>{op, b, lstride, jstride, nl, base});
    return;
  }
  if constexpr (HasRaw<Op>::value) {
    const C *src = op.raw(b);
#pragma unroll 4
    for (int e = threadIdx.x; e < TOT; e += NT) {
      int l, j;
      if (AXIS == 0) { l = e / N; j = e - l * N; } else { j = e / TL; l = e - j * TL; }
      if (l < nl) cp_async_elem(&bufa[j * LS + l], src + base + l * lstride + j * jstride);
      else { bufa[j * LS + l].x = 0; bufa[j * LS + l].y = 0; }
    }
    cp_async_wait_all();
  } else {
#pragma unroll 4
    for (int e = threadIdx.x; e < TOT; e += NT) {
      int l, j;
      if (AXIS == 0) { l = e / N; j = e - l * N; } else { j = e / TL; l = e - j * TL; }
      C v;
      if (l < nl) v = op.load(b, base + l * lstride + j * jstride);
      else { v.x = 0; v.y = 0; }
      bufa[j * LS + l] = v;
    }
  }
  __syncthreads();
  C *res;
  res = CtStages<C, N, TL, NT, 0>::run(bufa, bufb, tw, sign);
#pragma unroll 4
  for (int e = threadIdx.x; e < TOT; e += NT) {
    int l, j;
    if (AXIS == 0) { l = e / N; j = e - l * N; } else { j = e / TL; l = e - j * TL; }
    if (l < nl) op.store(b, base + l * lstride + j * jstride, res[j * LS + l]);
  }
}

template <typename C, int N> constexpr int ct_tile() {
  // ~24 KB per ping-pong buffer, power of two, at most 32 lines
  constexpr int budget = (sizeof(C) == 8 ? 3072 : 1536);
  return budget / N >= 32 ? 32 : (budget / N >= 16 ? 16 : (budget / N >= 8 ? 8 : 4));
}

template <typename C, int N, int TL, int AXIS, class Op>
int launch_ct_tl(opaw_ctx *c, const FFTAxis &a, Dims3 d, int batch, int sign, const Op &op, const LineSub *lsub) {
  const LineSub sub = lsub ? *lsub : LineSub::full(d);
  int64_t tiles;
  if (AXIS == 0) tiles = (int64_t)((sub.na + TL - 1) / TL) * sub.nb;
  else if (AXIS == 1) tiles = (int64_t)((d.n0 + TL - 1) / TL) * sub.nb;
  else tiles = ((int64_t)d.n0 * d.n1 + TL - 1) / TL;
  if (tiles == 0) return OPAW_OK;
  const size_t smem = sizeof(C) * ((size_t)N + 2 * (size_t)N * (TL + 1));
  auto kern = k_fft_ct<C, N, TL, AXIS, Op>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error(std::string("fft smem attribute: ") + cudaGetErrorString(e));
      return OPAW_ERR_CUDA;
    }
  }
  dim3 grid((unsigned)tiles, (unsigned)batch);
  kern<<<grid, 256, smem, c->stream>>>(d, sub, sign, axis_tw<C>(a), op);
  c->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("fft axis launch: ") + cudaGetErrorString(e));
    return OPAW_ERR_CUDA;
  }
  return OPAW_OK;
}

// ---- z pass with the tile staged by the Tensor Memory Accelerator --------
// The k-space-hook z pass (forward transform, kinetic factor, inverse
// transform of 32 consecutive (x, y) lines) with its input tile brought into
// shared memory by one cp.async.bulk.tensor load (32 lines x N planes, 8-byte
// elements, completion on an mbarrier) instead of per-thread global loads in
// the first stage.  The tile lands dense ([plane][line], stride 32: a warp's
// lanes read 32 consecutive lines of one plane, so no bank conflicts) in the
// buffer the first stage does not write; the stages and the hook are those
// of k_fft_ct.  Lines past the end of the grid are zero-filled by the TMA
// unit.  The wait on the barrier is bounded: after kTmaSpin polls the CTA
// records the failure in *err and leaves.
template <typename C, int TL> struct DenseAcc {  // [element][line] with line stride TL
  const C *p;
  __device__ __forceinline__ C get(int j, int l) const { return p[j * TL + l]; }
};
constexpr int kTmaSpin = 1 << 20;

template <class Op, class = void> struct HasBufStride : std::false_type {};
template <class Op>
struct HasBufStride<Op, std::void_t<decltype(std::declval<Op>().buf), decltype(std::declval<Op>().bstride)>>
    : std::true_type {};

template <int N, class Op>
__global__ void __launch_bounds__(256) k_fft_z_tma(const __grid_constant__ CUtensorMap tmap, Dims3 d,
                                                  const float2 *__restrict__ twg, Op op, int *__restrict__ err) {
  typedef float2 C;
  constexpr int TL = 32, NT = 256, LS = TL + 1;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar;
  typedef decltype(op.line(0)) L;
  __shared__ L lvs[TL];
  C *tw = reinterpret_cast<C *>(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
  C *bufa = tw + N;
  C *bufb = bufa + N * LS;  // 128-byte aligned: N (1 + LS) 8 bytes is a multiple of 128 for N % 16 == 0
  const int b = blockIdx.y;
  const int nlines = d.n0 * d.n1;
  const int64_t base = (int64_t)blockIdx.x * TL;
  const int nl = min(TL, nlines - (int)base);
  const uint32_t sbar = (uint32_t)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(sbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t sdst = (uint32_t)__cvta_generic_to_shared(bufb);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(sbar), "r"(TL * N * 8) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
            sdst),
        "l"(reinterpret_cast<uint64_t>(&tmap)), "r"((int)base), "r"(0), "r"(b), "r"(sbar)
        : "memory");
  }
  // twiddles and the hook's line values while the tile is in flight
  for (int t = threadIdx.x; t < N; t += NT) tw[t] = twg[t];
  if (threadIdx.x < nl) lvs[threadIdx.x] = op.line(base + threadIdx.x);
  uint32_t done = 0;
  for (int it = 0; it < kTmaSpin && !done; it++)
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(sbar)
        : "memory");
  // one decision for the whole CTA (a thread that gave up leaves with all)
  if (__syncthreads_or(!done)) {  // also orders the twiddles and line values
    if (threadIdx.x == 0) atomicExch(err, 1);
    return;
  }
  MidAcc<C, TL, Op, L> mo{bufa, op, b, 1, nlines, nl, base, lvs};
  C *res = ct_fwd_mid<C, N, TL, NT, 0>(DenseAcc<C, TL>{bufb}, bufa, bufb, tw, mo);
  ct_inv_out<C, N, TL, NT, 0>(res, res == bufa ? bufb : bufa, tw, GlobOut<C, Op>{op, b, 1, nlines, nl, base});
}

template <int N, class Op>
int launch_z_tma(opaw_ctx *c, const FFTAxis &a, Dims3 d, int batch, const Op &op) {
  constexpr int TL = 32;
  CUtensorMap m;
  OPAW_CHECK(tma_map_lines(&m, op.buf, (uint64_t)d.n0 * d.n1, (uint64_t)d.n2, (uint64_t)batch,
                           (uint64_t)op.bstride, TL, N));
  const int64_t tiles = ((int64_t)d.n0 * d.n1 + TL - 1) / TL;
  const size_t smem = sizeof(float2) * ((size_t)N + 2 * (size_t)N * (TL + 1)) + 128;
  auto kern = k_fft_z_tma<N, Op>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error(std::string("fft smem attribute: ") + cudaGetErrorString(e));
      return OPAW_ERR_CUDA;
    }
  }
  kern<<<dim3((unsigned)tiles, (unsigned)batch), 256, smem, c->stream>>>(m, d, a.tw32, op, c->d_tma_err);
  c->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("fft z TMA launch: ") + cudaGetErrorString(e));
    return OPAW_ERR_CUDA;
  }
  return OPAW_OK;
}

// z pass: the tile width (lines per CTA) is tuned between the default and
// half of it (the lines are transformed the same way in either); the other
// axes take the default
template <typename C, int N, int AXIS, class Op>
int launch_ct(opaw_ctx *c, const FFTAxis &a, Dims3 d, int batch, int sign, const Op &op, const LineSub *lsub) {
  constexpr int TL = ct_tile<C, N>();
  // a third candidate for the complex64 k-space-hook pass over a plain batch:
  // the tile staged by the TMA unit
  constexpr bool kTma = AXIS == 2 && TL == 32 && sizeof(C) == 8 && Op::kMid && HasBufStride<Op>::value &&
                        N % 16 == 0;
  if constexpr (AXIS == 2 && TL >= 16) {
    static const std::vector<std::string> labels =
        kTma ? std::vector<std::string>{std::to_string(TL) + " lines per CTA", std::to_string(TL / 2) + " lines per CTA",
                                        "32 lines per CTA, tile staged by TMA"}
             : std::vector<std::string>{std::to_string(TL) + " lines per CTA",
                                        std::to_string(TL / 2) + " lines per CTA"};
    const std::string key = std::string("z pass ") + (sizeof(C) == 8 ? "c64" : "c128") + " n " + std::to_string(N) +
                            " lines " + std::to_string((int64_t)d.n0 * d.n1) + " batch " + std::to_string(batch) +
                            " op " + OpNameOf<Op>::get();
    TuneSite *ts = nullptr;
    const int cand = tune_begin(c, key, labels, 0, &ts);
    int st;
    if constexpr (kTma) {
      const bool tma_ok = !lsub && ((uintptr_t)op.buf & 15) == 0 && ((int64_t)d.n0 * d.n1) % 2 == 0 &&
                          op.bstride % 2 == 0;
      if (cand == 2 && tma_ok) st = launch_z_tma<N, Op>(c, a, d, batch, op);
      else if (cand == 1) st = launch_ct_tl<C, N, TL / 2, AXIS>(c, a, d, batch, sign, op, lsub);
      else st = launch_ct_tl<C, N, TL, AXIS>(c, a, d, batch, sign, op, lsub);
    } else {
      st = cand == 1 ? launch_ct_tl<C, N, TL / 2, AXIS>(c, a, d, batch, sign, op, lsub)
                     : launch_ct_tl<C, N, TL, AXIS>(c, a, d, batch, sign, op, lsub);
    }
    OPAW_CHECK(st);
    return tune_end(c, ts);
  } else {
    return launch_ct_tl<C, N, TL, AXIS>(c, a, d, batch, sign, op, lsub);
  }
}

// ------------------------------------------------------------------------
// XY-plane kernel: one CTA transforms a whole z-plane (nx x ny) of one
// orbital in shared memory, x lines then y lines (inverse: y then x), so a 3D
// transform needs this pass plus one z pass instead of three axis passes.
// The plane is stored [y][x] with an odd row stride; every stage keeps its
// butterfly inputs in registers between two barriers and writes in place.
// ------------------------------------------------------------------------
template <typename C, int N, int NLINES, int LSL, int LSE, int NT, int S>
__device__ __forceinline__ void xy_stage(C *__restrict__ buf, const C *tw, int sign, int tid) {
  constexpr int R = ct_radix(N, S);
  constexpr int P = ct_pre(N, S);
  constexpr int M = N / R;
  constexpr int TOT = NLINES * M;
  constexpr int B = (TOT + NT - 1) / NT;
  constexpr int TSTEP = N / (P * R);
  C u[B][R];
#pragma unroll
  for (int k = 0; k < B; k++) {
    const int bf = tid + k * NT;
    if (bf < TOT) {
      const int line = bf % NLINES, i = bf / NLINES;
#pragma unroll
      for (int q = 0; q < R; q++) u[k][q] = buf[line * LSL + (i + q * M) * LSE];
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < B; k++) {
    const int bf = tid + k * NT;
    if (bf < TOT) {
      const int line = bf % NLINES, i = bf / NLINES;
      const int kk = i % P;
      if (P > 1) {
#pragma unroll
        for (int q = 1; q < R; q++) u[k][q] = cmul(u[k][q], twid(tw, q * kk * TSTEP, sign));
      }
      Butterfly<C, R>::run(u[k], tw, N, sign);
      const int j = (i - kk) * R + kk;
#pragma unroll
      for (int q = 0; q < R; q++) buf[line * LSL + (j + q * P) * LSE] = u[k][q];
    }
  }
  __syncthreads();
}

template <typename C, int N, int NLINES, int LSL, int LSE, int NT, int S> struct XyStages {
  static __device__ __forceinline__ void run(C *buf, const C *tw, int sign, int tid = threadIdx.x) {
    if constexpr (S < ct_nstage(N)) {
      xy_stage<C, N, NLINES, LSL, LSE, NT, S>(buf, tw, sign, tid);
      XyStages<C, N, NLINES, LSL, LSE, NT, S + 1>::run(buf, tw, sign, tid);
    }
  }
};

// stages [S, END) of one axis (see XyStages)
template <typename C, int N, int NLINES, int LSL, int LSE, int NT, int S, int END> struct XyStagesTo {
  static __device__ __forceinline__ void run(C *buf, const C *tw, int sign, int tid = threadIdx.x) {
    if constexpr (S < END) {
      xy_stage<C, N, NLINES, LSL, LSE, NT, S>(buf, tw, sign, tid);
      XyStagesTo<C, N, NLINES, LSL, LSE, NT, S + 1, END>::run(buf, tw, sign, tid);
    }
  }
};

// The last x stage of an inverse plane transform with the epilogue of Op
// applied on the way out: outputs go straight to global memory (no write-back
// to shared memory, no barrier after it).  Lanes take consecutive butterflies
// of a row, so the shared-memory reads and, for a first stage radix that
// leaves P > 1, the global accesses run along x.  The epilogue operands of a
// butterfly's outputs are loaded before its shared-memory reads.
template <typename C, int NX, int NY, int LX, int NT, class Op>
__device__ __forceinline__ void xy_last_x_epi(const C *__restrict__ pl, const C *tw, int sign, const Op &op, int b,
                                              int64_t base) {
  constexpr int S = ct_nstage(NX) - 1;
  constexpr int R = ct_radix(NX, S), P = ct_pre(NX, S), M = NX / R;
  constexpr int TOT = NY * M, TSTEP = NX / (P * R);
#pragma unroll 1
  for (int bf = threadIdx.x; bf < TOT; bf += NT) {
    const int i = bf % M, row = bf / M;
    const int kk = i % P;
    const int j = (i - kk) * R + kk;
    const int64_t g0 = base + (int64_t)row * NX + j;
    decltype(op.pre(0, int64_t(0))) pr[R];
#pragma unroll
    for (int q = 0; q < R; q++) pr[q] = op.pre(b, g0 + q * P);
    C u[R];
#pragma unroll
    for (int q = 0; q < R; q++) u[q] = pl[row * LX + i + q * M];
    if (P > 1) {
#pragma unroll
      for (int q = 1; q < R; q++) u[q] = cmul(u[q], twid(tw, q * kk * TSTEP, sign));
    }
    Butterfly<C, R>::run(u, tw, NX, sign);
#pragma unroll
    for (int q = 0; q < R; q++) op.fin(b, g0 + q * P, u[q], pr[q]);
  }
}

template <typename C, int NX, int NY, class Op>
__global__ void __launch_bounds__(384, 2)
    k_fft_xy(int sign, const C *__restrict__ twx, const C *__restrict__ twy, Op op, int ahead) {
  constexpr int NT = 384;
  constexpr int LX = NX + 1;  // odd row stride
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *tx = reinterpret_cast<C *>(smem_raw);
  C *ty = tx + NX;
  C *pl = ty + NY;
  for (int t = threadIdx.x; t < NX; t += NT) tx[t] = twx[t];
  for (int t = threadIdx.x; t < NY; t += NT) ty[t] = twy[t];
  const int b = blockIdx.y;
  const int64_t base = (int64_t)blockIdx.x * NX * NY;
  constexpr int TOT = NX * NY;
  constexpr int CH = 8;  // elements per thread whose loads are issued together
  if (threadIdx.x == 0) {
    // L2 prefetch of the plane of the CTA that starts one resident wave later
    // (CTAs start roughly in linear order)
    if constexpr (HasRaw<Op>::value && !HasPre<Op>::value) {  // measured: helps plain copies only
      const int nxt = blockIdx.y * gridDim.x + blockIdx.x + ahead;
      if (ahead > 0 && nxt < (int)(gridDim.x * gridDim.y)) {
        const int bn = nxt / gridDim.x;
        const C *q = op.raw(bn) + (int64_t)(nxt - bn * gridDim.x) * TOT;
        if (((uintptr_t)q & 15) == 0 && (TOT * sizeof(C)) % 16 == 0) l2_prefetch_bulk(q, TOT * sizeof(C));
      }
    }
  }
  if constexpr (HasRaw<Op>::value) {
    const C *src = op.raw(b) + base;
#pragma unroll 8
    for (int e = threadIdx.x; e < TOT; e += NT) {
      const int y = e / NX, x = e - y * NX;
      cp_async_elem(&pl[y * LX + x], src + e);
    }
    cp_async_wait_all();
  } else {
    for (int e0 = threadIdx.x; e0 < TOT; e0 += NT * CH) {
      C r[CH];
#pragma unroll
      for (int j = 0; j < CH; j++) {
        const int e = e0 + j * NT;
        if (e < TOT) r[j] = op.load(b, base + e);
      }
#pragma unroll
      for (int j = 0; j < CH; j++) {
        const int e = e0 + j * NT;
        if (e < TOT) {
          const int y = e / NX, x = e - y * NX;
          pl[y * LX + x] = r[j];
        }
      }
    }
  }
  __syncthreads();
  if constexpr (HasPre<Op>::value) {
    // y lines, then x lines with the epilogue riding on the last x stage
    // (either direction: the two axes' transforms commute)
    XyStages<C, NY, NX, 1, LX, NT, 0>::run(pl, ty, sign);
    XyStagesTo<C, NX, NY, LX, 1, NT, 0, ct_nstage(NX) - 1>::run(pl, tx, sign);
    xy_last_x_epi<C, NX, NY, LX, NT>(pl, tx, sign, op, b, base);
    return;
  } else if (sign < 0) {
    XyStages<C, NX, NY, LX, 1, NT, 0>::run(pl, tx, sign);   // x lines (rows)
    XyStages<C, NY, NX, 1, LX, NT, 0>::run(pl, ty, sign);   // y lines (columns)
  } else {
    XyStages<C, NY, NX, 1, LX, NT, 0>::run(pl, ty, sign);
    XyStages<C, NX, NY, LX, 1, NT, 0>::run(pl, tx, sign);
  }
#pragma unroll 4
  for (int e = threadIdx.x; e < TOT; e += NT) {
    const int y = e / NX, x = e - y * NX;
    op.store(b, base + e, pl[y * LX + x]);
  }
}

template <typename C, int NX, int NY, class Op>
int launch_xy(opaw_ctx *c, const FFTAxis &ax, const FFTAxis &ay, int nz, int batch, int sign, const Op &op) {
  const size_t smem = sizeof(C) * ((size_t)NX + NY + (size_t)NY * (NX + 1));
  auto kern = k_fft_xy<C, NX, NY, Op>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error(std::string("xy smem attribute: ") + cudaGetErrorString(e));
      return OPAW_ERR_CUDA;
    }
  }
  dim3 grid((unsigned)nz, (unsigned)batch);
  // L2 prefetch distance of the plain copy pass, in resident waves (tuned)
  int ahead = 2 * c->nsm;
  TuneSite *ts = nullptr;
  if constexpr (HasRaw<Op>::value && !HasPre<Op>::value) {
    static const std::vector<std::string> labels = {"no prefetch", "prefetch 1 wave ahead", "prefetch 2 waves ahead",
                                                    "prefetch 4 waves ahead"};
    const int waves[4] = {0, 1, 2, 4};
    const std::string key = "xy copy " + std::to_string(NX) + "x" + std::to_string(NY) + " nz " +
                            std::to_string(nz) + " batch " + std::to_string(batch);
    ahead = waves[tune_begin(c, key, labels, 2, &ts)] * c->nsm;
  }
  kern<<<grid, 384, smem, c->stream>>>(sign, axis_tw<C>(ax), axis_tw<C>(ay), op, ahead);
  c->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("xy launch: ") + cudaGetErrorString(e));
    return OPAW_ERR_CUDA;
  }
  return tune_end(c, ts);
}

// both x and y transforms of every z-plane in one pass when the plane has a
// specialised kernel (complex64 planes that fit shared memory); returns 1 if
// it ran, 0 if the caller must run the two axis passes
template <typename C, class Op>
int launch_xy_if(opaw_ctx *c, const FFT3 &f, int batch, int sign, const Op &op, int *st) {
  *st = OPAW_OK;
  if constexpr (sizeof(C) != 8) {
    return 0;
  } else {
    const int nx = f.n[0], ny = f.n[1], nz = f.n[2];
    if (nx == 96 && ny == 96) { *st = launch_xy<C, 96, 96>(c, f.ax[0], f.ax[1], nz, batch, sign, op); return 1; }
    if (nx == 48 && ny == 48) { *st = launch_xy<C, 48, 48>(c, f.ax[0], f.ax[1], nz, batch, sign, op); return 1; }
    if (nx == 96 && ny == 64) { *st = launch_xy<C, 96, 64>(c, f.ax[0], f.ax[1], nz, batch, sign, op); return 1; }
    if (nx == 64 && ny == 48) { *st = launch_xy<C, 64, 48>(c, f.ax[0], f.ax[1], nz, batch, sign, op); return 1; }
    if (nx == 32 && ny == 48) { *st = launch_xy<C, 32, 48>(c, f.ax[0], f.ax[1], nz, batch, sign, op); return 1; }
    return 0;
  }
}

// launch one axis pass over `batch` arrays of dims d
template <typename C, int AXIS, class Op>
// sub: only these lines are needed (their results), the others may be left
// unwritten; the generic kernel ignores it and transforms every line
int launch_axis(opaw_ctx *c, const FFTAxis &a, Dims3 d, int batch, int sign, const Op &op,
                const LineSub *sub = nullptr) {
  const int n = a.n;  // n == 1 runs zero stages: the fused operations still apply
  switch (n) {  // specialised lengths of the production grids and their 2x boxes
    case 32: return launch_ct<C, 32, AXIS>(c, a, d, batch, sign, op, sub);
    case 48: return launch_ct<C, 48, AXIS>(c, a, d, batch, sign, op, sub);
    case 64: return launch_ct<C, 64, AXIS>(c, a, d, batch, sign, op, sub);
    case 96: return launch_ct<C, 96, AXIS>(c, a, d, batch, sign, op, sub);
    case 128: return launch_ct<C, 128, AXIS>(c, a, d, batch, sign, op, sub);
    case 192: return launch_ct<C, 192, AXIS>(c, a, d, batch, sign, op, sub);
    default: break;
  }
  const int TL = tile_lines<C>(AXIS, n, 0);
  int64_t tiles;
  if (AXIS == 0) tiles = ((int64_t)d.n1 * d.n2 + TL - 1) / TL;
  else if (AXIS == 1) tiles = (int64_t)((d.n0 + TL - 1) / TL) * d.n2;
  else tiles = ((int64_t)d.n0 * d.n1 + TL - 1) / TL;
  size_t smem = sizeof(C) * ((size_t)n + 2 * (size_t)TL * n);
  auto kern = k_fft_axis<C, AXIS, Op>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error(std::string("fft smem attribute: ") + cudaGetErrorString(e));
      return OPAW_ERR_CUDA;
    }
  }
  dim3 grid((unsigned)tiles, (unsigned)batch);
  kern<<<grid, 256, smem, c->stream>>>(axis_dev(a), d, TL, sign, axis_tw<C>(a), op);
  c->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("fft axis launch: ") + cudaGetErrorString(e));
    return OPAW_ERR_CUDA;
  }
  return OPAW_OK;
}

}  // namespace opaw

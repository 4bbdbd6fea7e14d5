// hamiltonian.cu — the OPAW operators on batches of orbitals:
//   gather   <p|psi> over each atom's projector box       (proj.f90, proj1.f90)
//   scatter  psi += sum_i p_i coef_i over the box union    (hphi.f90:31-64, snphi.f90:29-46)
//   h_apply  F^-1[ek F psi] + v_ks psi + sum p D <p|psi>   (hphi.f90:1-66)
//   sn_apply psi + sum p1 ((1+s)^n - 1) <p1|psi>           (snphi.f90:1-49)
//   shs      S^-1/2 H S^-1/2                               (shs.f90:3-23)
// Every reduction runs in a fixed order (one warp per atom and orbital for
// the box sums; one thread per grid point, atoms in order, for the scatter),
// so FP64 results are bit-reproducible run to run.
#include <algorithm>

#include <vector>

#include "fft.cuh"

namespace opaw {

template <typename R> struct ProjTab;
template <> struct ProjTab<float> {
  static const float *get(const opaw_ctx *c, int which) { return which ? c->d_p3d1_f : c->d_p3d_f; }
};
template <> struct ProjTab<double> {
  static const double *get(const opaw_ctx *c, int which) { return which ? c->d_p3d1 : c->d_p3d; }
};

__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------- gather --
// Warp reduction of NV register values by recursive halving: at each level a
// lane keeps one half of its values and receives the partner's sums for that
// half, so NV values cost NV-1 shuffles in total instead of 5 NV.  Afterwards
// lane L holds the warp sums of values L*(NV/32) .. L*(NV/32) + NV/32 - 1.
template <int NV, int LEVEL = 0> struct Halve {
  template <typename T> static __device__ __forceinline__ void run(T *v, int lane) {
    constexpr int OFF = 16 >> LEVEL;
    constexpr int HALF = (NV >> LEVEL) / 2;
    if constexpr (OFF >= 1 && HALF >= 1) {
      const bool up = (lane & OFF) != 0;
#pragma unroll
      for (int k = 0; k < HALF; k++) {
        const T send = up ? v[k] : v[k + HALF];
        const T keep = up ? v[k + HALF] : v[k];
        v[k] = keep + __shfl_xor_sync(0xffffffffu, send, OFF);
      }
      Halve<NV, LEVEL + 1>::run(v, lane);
    }
  }
};

// out[o*ns + soff[a] + i] = dv * sum_box P_a[i][b] * psi_o[g(b)]   (p real: Gamma point)
// One warp per orbital and kGatherWarps orbitals per CTA over one atom's box:
// lane l sums the points l, l+32, ... (U per iteration, their loads issued
// together) into 2*MSMAX registers, then a shuffle tree adds the lanes.  The
// warps of a CTA read the same projector rows, which L1 serves once, so the
// projector tables cost one L2 read per atom and orbital group.  The order of
// every sum is fixed (bit-reproducible).
constexpr int kGatherWarps = 8;

template <typename R, int MSMAX>
__global__ void __launch_bounds__(32 * kGatherWarps)
    k_gather(const typename Tr<R>::C *__restrict__ psi, int64_t nn, int norb, const R *__restrict__ P,
             const int64_t *__restrict__ poff, const int *__restrict__ boxg, const int64_t *__restrict__ boff,
             const int *__restrict__ nrough, const int *__restrict__ ms, const int64_t *__restrict__ soff, double dv,
             double *__restrict__ out, int ns) {
  typedef typename Tr<R>::C C;
  constexpr int NV = 2 * MSMAX;  // value index 2 i + re/im
  static_assert(NV == 16 || NV == 32, "8 or 16 projectors per atom");
  const int a = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int o = blockIdx.y * kGatherWarps + warp;
  if (o >= norb) return;  // whole warps leave: no block-wide barrier follows
  const int m = ms[a];
  const int nbox = nrough[3 * a] * nrough[3 * a + 1] * nrough[3 * a + 2];
  const int *bg = boxg + boff[a];  // wrapped grid index of each box point (proj.f90:27-37)
  const R *Pa = P + poff[a];
  const C *po = psi + (int64_t)o * nn;
  R v[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) v[k] = 0;
  // U points per lane and iteration: their index loads, then their orbital
  // loads, are all in flight before the first product
  constexpr int U = (sizeof(R) == 4 && MSMAX <= 8) ? 8 : 4;
  for (int b0 = lane; b0 < nbox; b0 += 32 * U) {
    int gg[U];
    C z[U];
#pragma unroll
    for (int k = 0; k < U; k++) gg[k] = (b0 + 32 * k < nbox) ? bg[b0 + 32 * k] : -1;
#pragma unroll
    for (int k = 0; k < U; k++) {
      if (gg[k] >= 0) z[k] = po[gg[k]];
      else z[k].x = z[k].y = (R)0;
    }
#pragma unroll
    for (int k = 0; k < U; k++) {
      const int b = b0 + 32 * k;
      if (b < nbox) {
#pragma unroll
        for (int i = 0; i < MSMAX; i++) {
          const R p = (i < m) ? Pa[(int64_t)i * nbox + b] : (R)0;
          v[2 * i] += p * z[k].x;
          v[2 * i + 1] += p * z[k].y;
        }
      }
    }
  }
  Halve<NV>::run(v, lane);  // lane L: value L * NV / 32 (NV = 16: lanes L, L^1 hold halves of it)
  R sum = v[0];
  int idx = lane;
  if constexpr (NV == 16) {
    sum += __shfl_xor_sync(0xffffffffu, sum, 1);
    idx = lane >> 1;
  }
  const int i = idx >> 1;
  if (i < m && (NV == 32 || (lane & 1) == 0)) out[2 * ((int64_t)o * ns + soff[a] + i) + (idx & 1)] = (double)sum * dv;
}

template <typename R>
int gather(opaw_ctx *c, int which, const typename Tr<R>::C *pin, int norb, double2 *coef) {
  if (c->natom == 0) return OPAW_OK;
  if constexpr (sizeof(R) == 4) {
    // complex64: the pipelined two-table pass (k_gather2) is faster than the
    // warp-per-orbital one even with the other table's sums discarded
    if (c->msmax <= 8) {
      OPAW_CHECK(ensure(c->g2other, sizeof(double2) * (size_t)c->ns * norb + 16));
      double2 *o = (double2 *)c->g2other.p;
      return which == 0 ? gather2<R>(c, pin, norb, coef, o) : gather2<R>(c, pin, norb, o, coef);
    }
  }
  const R *P = ProjTab<R>::get(c, which);
  const dim3 grid(c->natom, (norb + kGatherWarps - 1) / kGatherWarps);
  if (c->msmax <= 8) {
    k_gather<R, 8><<<grid, 32 * kGatherWarps, 0, c->stream>>>(pin, c->nn, norb, P, c->d_poff, c->d_boxg, c->d_boff,
                                                              c->d_nrough, c->d_ms, c->d_soff, c->dv,
                                                              (double *)coef, c->ns);
  } else if (c->msmax <= 16) {
    k_gather<R, 16><<<grid, 32 * kGatherWarps, 0, c->stream>>>(pin, c->nn, norb, P, c->d_poff, c->d_boxg, c->d_boff,
                                                               c->d_nrough, c->d_ms, c->d_soff, c->dv,
                                                               (double *)coef, c->ns);
  } else {
    set_error("more than 16 projectors per atom");
    return OPAW_ERR_ARG;
  }
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

// both projector families in one pass over the boxes: out0 = <p~|psi>,
// out1 = <p~1|psi>.  CTA = one atom and kG2Warps orbitals (a warp each); the
// box is walked in chunks of 256 (FP64: 128) points whose projector rows of both
// tables are staged once in shared memory for all the CTA's warps, while
// each lane's orbital loads for the chunk are already in flight.  Lane L ends
// with values L*PER .. L*PER+PER-1 of the shuffle tree (fixed order).
constexpr int kG2Warps = 16;

// rows i < m of both tables for box points [c0, c0 + CH) into dst
// [table][i][point] by cp.async, zeros past the segment end or past m
template <typename R, int MSMAX, int CH, int NT>
__device__ __forceinline__ void g2_stage_rows(R *dst, const R *Pa, const R *Qa, int m, int nbox, int c0, int b1) {
  for (int e = threadIdx.x; e < 2 * MSMAX * CH; e += NT) {
    const int tab = e / (MSMAX * CH), r = e - tab * (MSMAX * CH);
    const int i = r / CH, j = r - i * CH;
    const int b = c0 + j;
    const bool ok = i < m && b < b1;
    const R *src = ok ? (tab ? Qa : Pa) + (int64_t)i * nbox + b : Pa;
    const unsigned sa = (unsigned)__cvta_generic_to_shared(dst + e);
    const int n = ok ? (int)sizeof(R) : 0;  // 0: the destination is zero-filled
    if constexpr (sizeof(R) == 4)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(src), "r"(n) : "memory");
    else
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(src), "r"(n) : "memory");
  }
}

template <typename R, int MSMAX>
__global__ void __launch_bounds__(32 * kG2Warps, (sizeof(R) == 4 && MSMAX <= 8) ? 2 : 1)
    k_gather2(const typename Tr<R>::C *__restrict__ psi, int64_t nn, int norb, const R *__restrict__ P0,
              const R *__restrict__ P1, const int64_t *__restrict__ poff, const int *__restrict__ boxg,
              const int64_t *__restrict__ boff, const int *__restrict__ nrough, const int *__restrict__ ms,
              const int64_t *__restrict__ soff, double dv, double *__restrict__ out0, double *__restrict__ out1,
              int ns, int nseg) {
  typedef typename Tr<R>::C C;
  constexpr int H = 2 * MSMAX;  // values per table: 2 i + re/im
  constexpr int NV = 2 * H;
  constexpr int PER = NV / 32;
  constexpr int kG2Chunk = sizeof(R) == 4 ? 128 : 64;  // points per chunk
  constexpr int U = kG2Chunk / 32;  // points per lane and chunk
  constexpr int NT = 32 * kG2Warps;
  constexpr int RV = 2 * MSMAX * kG2Chunk;  // staged row values per chunk
  static_assert(NV == 32 || NV == 64, "8 or 16 projectors per atom");
  // the rows of two chunks: chunk c + 1 is copied in (cp.async) while chunk c is summed
  __shared__ __align__(16) R sp[2][2][MSMAX][kG2Chunk];
  const int a = blockIdx.x / nseg, seg = blockIdx.x - a * nseg;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int o = blockIdx.y * kG2Warps + warp;
  const bool live = o < norb;  // idle warps still take part in the staging
  const int m = ms[a];
  const int nbox = nrough[3 * a] * nrough[3 * a + 1] * nrough[3 * a + 2];
  // this CTA's segment of the box, whole chunks
  const int seglen = (nbox + nseg * kG2Chunk - 1) / (nseg * kG2Chunk) * kG2Chunk;
  const int b0 = seg * seglen, b1 = min(nbox, b0 + seglen);
  const int *bg = boxg + boff[a];
  const R *Pa = P0 + poff[a];
  const R *Qa = P1 + poff[a];
  const C *po = psi + (int64_t)(live ? o : 0) * nn;
  R v[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) v[k] = 0;
  // software pipeline: grid indices two chunks ahead, orbital values one ahead
  C zn[U];   // the orbital at the lane's points of the next chunk
  int gn[U]; // grid indices of the lane's points of the chunk after it (-1: none)
#pragma unroll
  for (int k = 0; k < U; k++) {
    const int b = b0 + lane + 32 * k, b2 = b + kG2Chunk;
    zn[k].x = zn[k].y = (R)0;
    if (live && b < b1) zn[k] = po[bg[b]];
    gn[k] = (live && b2 < b1) ? bg[b2] : -1;
  }
  if (b0 < b1) g2_stage_rows<R, MSMAX, kG2Chunk, NT>(&sp[0][0][0][0], Pa, Qa, m, nbox, b0, b1);
  int buf = 0;
  for (int c0 = b0; c0 < b1; c0 += kG2Chunk, buf ^= 1) {
    C z[U];
#pragma unroll
    for (int k = 0; k < U; k++) z[k] = zn[k];
    cp_async_wait_all();
    __syncthreads();  // this chunk's rows landed; the other buffer's last reader is done
    const int c1 = c0 + kG2Chunk;
    if (c1 < b1) {
#pragma unroll
      for (int k = 0; k < U; k++) {
        zn[k].x = zn[k].y = (R)0;
        if (gn[k] >= 0) zn[k] = po[gn[k]];
        const int b2 = c1 + kG2Chunk + lane + 32 * k;
        gn[k] = (live && b2 < b1) ? bg[b2] : -1;
      }
      g2_stage_rows<R, MSMAX, kG2Chunk, NT>(&sp[buf ^ 1][0][0][0], Pa, Qa, m, nbox, c1, b1);
    }
#pragma unroll
    for (int k = 0; k < U; k++) {
      const int j = lane + 32 * k;
#pragma unroll
      for (int i = 0; i < MSMAX; i++) {
        const R p = sp[buf][0][i][j], q = sp[buf][1][i][j];
        v[2 * i] += p * z[k].x;
        v[2 * i + 1] += p * z[k].y;
        v[H + 2 * i] += q * z[k].x;
        v[H + 2 * i + 1] += q * z[k].y;
      }
    }
  }
  if (!live) return;  // no block-wide barrier follows
  Halve<NV>::run(v, lane);
#pragma unroll
  for (int k = 0; k < PER; k++) {
    const int idx = lane * PER + k;
    const int tab = idx / H, r = idx - tab * H;
    const int i = r >> 1;
    if (i < m) {
      // segment partial: [seg][table][orbital][slot] (nseg = 1: the result itself)
      double *dst = nseg == 1 ? (tab ? out1 : out0) : out0 + (int64_t)(2 * seg + tab) * 2 * norb * ns;
      dst[2 * ((int64_t)o * ns + soff[a] + i) + (r & 1)] = (double)v[k] * dv;
    }
  }
}

// sum of the segment partials in segment order
__global__ void k_gather2_sum(const double2 *__restrict__ part, int nseg, int64_t n, double2 *__restrict__ out0,
                              double2 *__restrict__ out1) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= 2 * n) return;
  const int tab = (int)(t / n);
  const int64_t j = t - tab * n;
  double sx = 0, sy = 0;
  for (int q = 0; q < nseg; q++) {
    const double2 v = part[(int64_t)(2 * q + tab) * n + j];
    sx += v.x;
    sy += v.y;
  }
  (tab ? out1 : out0)[j] = make_double2(sx, sy);
}

template <typename R>
int gather2(opaw_ctx *c, const typename Tr<R>::C *pin, int norb, double2 *c0, double2 *c1) {
  if (c->natom == 0) return OPAW_OK;
  const R *P0 = ProjTab<R>::get(c, 0), *P1 = ProjTab<R>::get(c, 1);
  // segments of about 1024 points per box: enough CTAs to fill the GPU
  const int nseg = std::max(1, std::min(8, c->maxbox / 1024));
  const int64_t n = (int64_t)c->ns * norb;
  double *o0 = (double *)c0, *o1 = (double *)c1;
  if (nseg > 1) {
    OPAW_CHECK(ensure(c->g2part, sizeof(double2) * 2 * (size_t)nseg * n + 64));
    o0 = (double *)c->g2part.p;
    o1 = nullptr;
  }
  const dim3 grid(c->natom * nseg, (norb + kG2Warps - 1) / kG2Warps);
  if (c->msmax <= 8)
    k_gather2<R, 8><<<grid, 32 * kG2Warps, 0, c->stream>>>(pin, c->nn, norb, P0, P1, c->d_poff, c->d_boxg,
                                                           c->d_boff, c->d_nrough, c->d_ms, c->d_soff, c->dv, o0, o1,
                                                           c->ns, nseg);
  else
    k_gather2<R, 16><<<grid, 32 * kG2Warps, 0, c->stream>>>(pin, c->nn, norb, P0, P1, c->d_poff, c->d_boxg,
                                                            c->d_boff, c->d_nrough, c->d_ms, c->d_soff, c->dv, o0,
                                                            o1, c->ns, nseg);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  if (nseg > 1) {
    k_gather2_sum<<<grid1(2 * n, 256), 256, 0, c->stream>>>((const double2 *)c->g2part.p, nseg, n, c0, c1);
    c->launches++;
    OPAW_CUDA(cudaGetLastError());
  }
  return OPAW_OK;
}

// --------------------------------------------------------------- scatter --
// out_o[upt[u]] += sum over the (atom, box point) entries of u of
//                  sum_i P_a[i][b] * coef[o][soff[a] + i]
// One thread per grid point of the box union: the projector values of the
// point are loaded once into registers and reused for every orbital; the
// entries of a point are summed in atom order (deterministic).
constexpr int kScatterOrb = 16;  // orbitals per thread of the box scatter

template <typename R, int EMAX, int MSMAX>
__global__ void __launch_bounds__(256) k_union_scatter(typename Tr<R>::C *__restrict__ out, int64_t nn, int nunion,
                                                       int norb, const int *__restrict__ upt,
                                                       const int *__restrict__ ustart, const int *__restrict__ uatom,
                                                       const int *__restrict__ ubox, const R *__restrict__ P,
                                                       const int64_t *__restrict__ poff,
                                                       const int *__restrict__ nrough, const int *__restrict__ ms,
                                                       const int64_t *__restrict__ soff,
                                                       const typename Tr<R>::C *__restrict__ coef, int ns) {
  typedef typename Tr<R>::C C;
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nunion) return;
  const int e0 = ustart[u], ne = ustart[u + 1] - e0;
  C *dst = out + upt[u];
  if (ne <= EMAX) {
    R pv[EMAX][MSMAX];
    int so[EMAX], mm[EMAX];
#pragma unroll
    for (int e = 0; e < EMAX; e++) {
      mm[e] = 0;
      so[e] = 0;
      if (e < ne) {
        const int a = uatom[e0 + e], b = ubox[e0 + e];
        const int nbox = nrough[3 * a] * nrough[3 * a + 1] * nrough[3 * a + 2];
        mm[e] = ms[a];
        so[e] = (int)soff[a];
        const R *Pa = P + poff[a] + b;
#pragma unroll
        for (int i = 0; i < MSMAX; i++) pv[e][i] = (i < mm[e]) ? Pa[(int64_t)i * nbox] : (R)0;
      }
    }
    const int oa = blockIdx.y * kScatterOrb, ob = min(norb, oa + kScatterOrb);
    constexpr int Q = 8;  // orbitals whose values are loaded together
    for (int o0 = oa; o0 < ob; o0 += Q) {
      C cur[Q];
#pragma unroll
      for (int q = 0; q < Q; q++)
        if (o0 + q < ob) cur[q] = dst[(int64_t)(o0 + q) * nn];
#pragma unroll
      for (int q = 0; q < Q; q++) {
        if (o0 + q < ob) {
          const C *co = coef + (int64_t)(o0 + q) * ns;
          R sx = 0, sy = 0;
#pragma unroll
          for (int e = 0; e < EMAX; e++) {
            if (e < ne) {
#pragma unroll
              for (int i = 0; i < MSMAX; i++) {
                if (i < mm[e]) {
                  const C cf = co[so[e] + i];
                  sx += pv[e][i] * cf.x;
                  sy += pv[e][i] * cf.y;
                }
              }
            }
          }
          cur[q].x += sx;
          cur[q].y += sy;
        }
      }
#pragma unroll
      for (int q = 0; q < Q; q++)
        if (o0 + q < ob) dst[(int64_t)(o0 + q) * nn] = cur[q];
    }
    return;
  }
  for (int o = blockIdx.y * kScatterOrb; o < min(norb, (int)(blockIdx.y + 1) * kScatterOrb); o++) {
    const C *co = coef + (int64_t)o * ns;
    R sx = 0, sy = 0;
    for (int e = e0; e < e0 + ne; e++) {
      const int a = uatom[e], b = ubox[e];
      const int nbox = nrough[3 * a] * nrough[3 * a + 1] * nrough[3 * a + 2];
      const R *Pa = P + poff[a] + b;
      const C *ca = co + soff[a];
      const int m = ms[a];
      for (int i = 0; i < m; i++) {
        const R p = Pa[(int64_t)i * nbox];
        sx += p * ca[i].x;
        sy += p * ca[i].y;
      }
    }
    C v = dst[(int64_t)o * nn];
    v.x += sx;
    v.y += sy;
    dst[(int64_t)o * nn] = v;
  }
}

template <typename R> struct CoefIn;
template <> struct CoefIn<double> {
  static const double2 *get(opaw_ctx *, const double2 *coef, int) { return coef; }
};
__global__ void k_coef_to_f(const double2 *__restrict__ a, float2 *__restrict__ b, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = make_float2(d2f(a[i].x), d2f(a[i].y));
}
template <> struct CoefIn<float> {
  // the scatter's coefficients in single precision, converted once
  static const float2 *get(opaw_ctx *c, const double2 *coef, int norb) {
    const int64_t n = (int64_t)c->ns * norb;
    if (ensure(c->coefr, sizeof(float2) * n + 16) != OPAW_OK) return nullptr;
    k_coef_to_f<<<grid1(n, 256), 256, 0, c->stream>>>(coef, (float2 *)c->coefr.p, n);
    c->launches++;
    return (const float2 *)c->coefr.p;
  }
};

template <typename R>
int union_scatter(opaw_ctx *c, int which, typename Tr<R>::C *out, int norb, const double2 *coef) {
  if (c->nunion == 0) return OPAW_OK;
  const R *P = ProjTab<R>::get(c, which);
  const typename Tr<R>::C *cf = CoefIn<R>::get(c, coef, norb);
  if (!cf) return OPAW_ERR_NOMEM;
  const dim3 grid(grid1(c->nunion, 128), (norb + kScatterOrb - 1) / kScatterOrb);
  if (c->msmax <= 8)
    k_union_scatter<R, 2, 8><<<grid, 128, 0, c->stream>>>(out, c->nn, c->nunion, norb, c->d_upt, c->d_ustart,
                                                          c->d_uatom, c->d_ubox, P, c->d_poff, c->d_nrough, c->d_ms,
                                                          c->d_soff, cf, c->ns);
  else
    k_union_scatter<R, 1, 16><<<grid, 128, 0, c->stream>>>(out, c->nn, c->nunion, norb, c->d_upt, c->d_ustart,
                                                           c->d_uatom, c->d_ubox, P, c->d_poff, c->d_nrough, c->d_ms,
                                                           c->d_soff, cf, c->ns);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

// ----------------------------------------------------- coefficient algebra --
// arr[o][a][i] = sum_j D_a(i,j) c[o][a][j]   (hphi.f90:43-47, FP64)
__global__ void k_coef_dij(const double2 *__restrict__ cin, double2 *__restrict__ cout, int norb, int ns,
                           const int *__restrict__ slot_atom, const int64_t *__restrict__ soff,
                           const int64_t *__restrict__ doff, const int *__restrict__ ms,
                           const double *__restrict__ dij) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int o = blockIdx.y;
  if (t >= ns || o >= norb) return;
  const int a = slot_atom[t];
  const int m = ms[a];
  const int i = t - (int)soff[a];
  const double *D = dij + doff[a];
  const double2 *ci = cin + (int64_t)o * ns + soff[a];
  double sx = 0, sy = 0;
  for (int j = 0; j < m; j++) {
    const double d = D[i + m * j];
    sx += d * ci[j].x;
    sy += d * ci[j].y;
  }
  cout[(int64_t)o * ns + t] = make_double2(sx, sy);
}

// arr = D c + dD c0: the nonlocal coefficients of H' applied to the
// difference plus those of (H' - H) applied to the unperturbed vector
__global__ void k_coef_dij2(const double2 *__restrict__ cin, const double2 *__restrict__ c0,
                            double2 *__restrict__ cout, int norb, int ns, const int *__restrict__ slot_atom,
                            const int64_t *__restrict__ soff, const int64_t *__restrict__ doff,
                            const int *__restrict__ ms, const double *__restrict__ dij,
                            const double *__restrict__ ddij) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int o = blockIdx.y;
  if (t >= ns || o >= norb) return;
  const int a = slot_atom[t];
  const int m = ms[a];
  const int i = t - (int)soff[a];
  const double *D = dij + doff[a];
  const double *dD = ddij + doff[a];
  const double2 *ci = cin + (int64_t)o * ns + soff[a];
  const double2 *c0i = c0 + (int64_t)o * ns + soff[a];
  double sx = 0, sy = 0;
  for (int j = 0; j < m; j++) {
    const double d = D[i + m * j], e = dD[i + m * j];
    sx += d * ci[j].x + e * c0i[j].x;
    sy += d * ci[j].y + e * c0i[j].y;
  }
  cout[(int64_t)o * ns + t] = make_double2(sx, sy);
}

// coef[o][t] = sigma[t] * c[o][t]   (snphi.f90:24-28)
__global__ void k_coef_scale(const double2 *__restrict__ cin, double2 *__restrict__ cout, int norb, int ns,
                             const double *__restrict__ sigma) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int o = blockIdx.y;
  if (t >= ns || o >= norb) return;
  const double s = sigma[t];
  const double2 v = cin[(int64_t)o * ns + t];
  cout[(int64_t)o * ns + t] = make_double2(s * v.x, s * v.y);
}

// ------------------------------------------------------------ FFT ops --
// kinetic hook on z-lines: v *= min((kx^2 + ky^2 + kz^2)/2, ekcut) / N   (ek.f90:40-50)
template <typename R> struct OpKin;
template <> struct OpKin<double> {
  static constexpr const char *kName = "kinetic";
  double2 *buf;
  int64_t bstride;
  const double *k2x, *k2y, *k2z;
  int nx, ny;
  double ekcut, ntot;
  static constexpr bool kMid = true;
  __device__ double2 load(int b, int64_t g) const { return buf[b * bstride + g]; }
  __device__ const double2 *raw(int b) const { return buf + b * bstride; }
  __device__ void store(int b, int64_t g, double2 v) const { buf[b * bstride + g] = v; }
  // z-lines: the line index is the (x, y) position
  __device__ double line(int64_t gl) const {
    const int t = (int)gl;
    return __dadd_rn(k2x[t % nx], k2y[t / nx]);
  }
  __device__ double2 mid(int, int64_t, double kxy, int z, double2 v) const {
    double e = __dadd_rn(kxy, k2z[z]) * 0.5;
    if (ekcut > 0.0 && e > ekcut) e = ekcut;
    e = __ddiv_rn(e, ntot);
    return make_double2(v.x * e, v.y * e);
  }
};
template <> struct OpKin<float> {
  static constexpr const char *kName = "kinetic";
  float2 *buf;
  int64_t bstride;
  const float *k2x, *k2y, *k2z;
  int nx, ny;
  float ekcut, invn;
  static constexpr bool kMid = true;
  __device__ float2 load(int b, int64_t g) const { return buf[b * bstride + g]; }
  __device__ const float2 *raw(int b) const { return buf + b * bstride; }
  __device__ void store(int b, int64_t g, float2 v) const { buf[b * bstride + g] = v; }
  __device__ float line(int64_t gl) const {
    const int t = (int)gl;
    return k2x[t % nx] + k2y[t / nx];
  }
  __device__ float2 mid(int, int64_t, float kxy, int z, float2 v) const {
    float e = (kxy + k2z[z]) * 0.5f;
    if (ekcut > 0.f && e > ekcut) e = ekcut;
    e *= invn;
    return make_float2(v.x * e, v.y * e);
  }
};

// Teter-Payne-Allan kinetic preconditioner (Phys. Rev. B 40, 12255 (1989))
// as the k-space hook of the z pass: with x = (|k|^2 / 2) / Ekin_b, the
// kinetic energy of orbital b,
//   K(x) = (27 + 18 x + 12 x^2 + 8 x^3) / (27 + 18 x + 12 x^2 + 8 x^3 + 16 x^4),
// applied with the 1/N of the unnormalised inverse transform folded in
template <typename R> struct OpTPA {
  static constexpr const char *kName = "kinetic preconditioner";
  typedef typename Tr<R>::C C;
  C *buf;
  int64_t bstride;
  const R *k2x, *k2y, *k2z;
  int nx;
  const double *inv_ekin;  // [batch] 1 / Ekin
  R invn;
  static constexpr bool kMid = true;
  __device__ C load(int b, int64_t g) const { return buf[b * bstride + g]; }
  __device__ const C *raw(int b) const { return buf + b * bstride; }
  __device__ void store(int b, int64_t g, C v) const { buf[b * bstride + g] = v; }
  __device__ R line(int64_t gl) const {
    const int t = (int)gl;
    return k2x[t % nx] + k2y[t / nx];
  }
  __device__ C mid(int b, int64_t, R kxy, int z, C v) const {
    const R x = (R)0.5 * (kxy + k2z[z]) * (R)inv_ekin[b];
    const R num = (R)27 + x * ((R)18 + x * ((R)12 + x * (R)8));
    const R f = num / (num + (R)16 * x * x * x * x) * invn;
    v.x *= f;
    v.y *= f;
    return v;
  }
};

// last inverse pass of h_phi: hp = F^-1[...] + pin * v_ks   (hphi.f90:21);
// with t0/dv set it also adds the local part of (H' - H) t0 = dv * t0 (the
// source term of the perturbation-difference propagation)
template <typename R> struct OpHFinal {
  typedef typename Tr<R>::C C;
  const C *src;
  const C *pin;
  const R *vks;
  C *hp;
  int64_t bstride;
  const C *t0;
  const R *dv;
  static constexpr bool kMid = false;
  __device__ C load(int b, int64_t g) const { return src[b * bstride + g]; }
  __device__ const C *raw(int b) const { return src + b * bstride; }
  // the epilogue operands of one element, loaded ahead of the stores
  struct Pre {
    C p, t;
    R w, d;
  };
  __device__ Pre pre(int b, int64_t g) const {
    Pre q;
    q.p = pin[b * bstride + g];
    q.w = vks[g];
    if (t0) {
      q.t = t0[b * bstride + g];
      q.d = dv[g];
    }
    return q;
  }
  __device__ void fin(int b, int64_t g, C v, const Pre &q) const {
    C r;
    r.x = v.x + q.p.x * q.w;
    r.y = v.y + q.p.y * q.w;
    if (t0) {
      r.x += q.t.x * q.d;
      r.y += q.t.y * q.d;
    }
    hp[b * bstride + g] = r;
  }
  __device__ void store(int b, int64_t g, C v) const { fin(b, g, v, pre(b, g)); }
  __device__ double line(int64_t) const { return 0.0; }
  __device__ C mid(int, int64_t, double, int, C v) const { return v; }
};

// All orbital sets of a stage in one batch, interleaved: batch entry
// b = nset o + X, X = 0 the unperturbed set, X = 1 + k the difference of kick
// k.  The forward plane pass reads t (set 0) or t_d of kick k (X > 0) of
// orbital o; the epilogue of a difference set reads t_0 of the same orbital
// and plane that the set-0 CTA a few rows of CTAs earlier has just read, so
// that read is served by L2.
template <typename C> struct OpCopyK {
  const C *src0, *src1;  // t_0 [orbital][point], t_d [kick][orbital][point]
  C *dst;
  int64_t nn;
  int nset, norb;
  static constexpr bool kMid = false;
  __device__ const C *raw(int b) const {
    const int o = b / nset, X = b - o * nset;
    return X == 0 ? src0 + (int64_t)o * nn : src1 + ((int64_t)(X - 1) * norb + o) * nn;
  }
  __device__ C load(int b, int64_t g) const { return raw(b)[g]; }
  __device__ void store(int b, int64_t g, C v) const { dst[b * nn + g] = v; }
  __device__ double line(int64_t) const { return 0.0; }
  __device__ C mid(int, int64_t, double, int, C v) const { return v; }
};

template <typename R> struct OpHFinalK {
  typedef typename Tr<R>::C C;
  const C *src;        // the transformed batch, nset norb entries
  const C *p0, *pd;    // t_0, t_d of every kick
  const R *v0, *v1;    // v_ks of set 0, of every kicked set [kick][point]
  C *h0, *hd;          // outputs u'_0, u'_d of every kick
  const R *dv;         // v_1 - v_0 of every kick [kick][point]
  int64_t nn;
  int nset, norb;
  static constexpr bool kMid = false;
  __device__ C load(int b, int64_t g) const { return src[b * nn + g]; }
  __device__ const C *raw(int b) const { return src + b * nn; }
  struct Pre {
    C p, t;
    R w, d;
  };
  __device__ Pre pre(int b, int64_t g) const {
    Pre q;
    const int o = b / nset, X = b - o * nset;
    const int64_t i = (int64_t)o * nn + g;
    if (X) {
      const int64_t kp = (int64_t)(X - 1) * nn;
      q.p = pd[kp * norb + i];
      q.w = v1[kp + g];
      q.t = p0[i];
      q.d = dv[kp + g];
    } else {
      q.p = p0[i];
      q.w = v0[g];
    }
    return q;
  }
  __device__ void fin(int b, int64_t g, C v, const Pre &q) const {
    C r;
    r.x = v.x + q.p.x * q.w;
    r.y = v.y + q.p.y * q.w;
    const int o = b / nset, X = b - o * nset;
    const int64_t i = (int64_t)o * nn + g;
    if (X) {
      r.x += q.t.x * q.d;
      r.y += q.t.y * q.d;
      hd[(int64_t)(X - 1) * norb * nn + i] = r;
    } else {
      h0[i] = r;
    }
  }
  __device__ void store(int b, int64_t g, C v) const { fin(b, g, v, pre(b, g)); }
  __device__ double line(int64_t) const { return 0.0; }
  __device__ C mid(int, int64_t, double, int, C v) const { return v; }
};

template <typename R> struct VksOf;
template <> struct VksOf<float> {
  static const float *get(const opaw_ctx *c, int set) { return c->d_vks_f[set]; }
};
template <> struct VksOf<double> {
  static const double *get(const opaw_ctx *c, int set) { return c->d_vks[set]; }
};

template <typename R> static OpKin<R> make_kin(opaw_ctx *c, typename Tr<R>::C *buf);
template <> OpKin<double> make_kin<double>(opaw_ctx *c, double2 *buf) {
  OpKin<double> k;
  k.buf = buf;
  k.bstride = c->nn;
  k.k2x = c->d_k2[0];
  k.k2y = c->d_k2[1];
  k.k2z = c->d_k2[2];
  k.nx = c->nx;
  k.ny = c->ny;
  k.ekcut = c->ekcut;
  k.ntot = (double)c->nx * (double)c->ny * (double)c->nz;
  return k;
}
template <> OpKin<float> make_kin<float>(opaw_ctx *c, float2 *buf) {
  OpKin<float> k;
  k.buf = buf;
  k.bstride = c->nn;
  k.k2x = c->d_k2f[0];
  k.k2y = c->d_k2f[1];
  k.k2z = c->d_k2f[2];
  k.nx = c->nx;
  k.ny = c->ny;
  k.ekcut = (float)c->ekcut;
  k.invn = (float)(1.0 / ((double)c->nx * (double)c->ny * (double)c->nz));
  return k;
}

template <typename R>
int h_apply(opaw_ctx *c, int set, const typename Tr<R>::C *pin, typename Tr<R>::C *hp, int norb) {
  typedef typename Tr<R>::C C;
  if (norb <= 0) return OPAW_OK;
  OPAW_CHECK(ensure(c->coef[0], sizeof(double2) * (size_t)c->ns * norb + 16));
  OPAW_CHECK(ensure(c->coef[1], sizeof(double2) * (size_t)c->ns * norb + 16));
  double2 *c0 = (double2 *)c->coef[0].p, *c1 = (double2 *)c->coef[1].p;
  // <p~|psi> and D c (addvnl, hphi.f90:40-47), from the unmodified input
  OPAW_CHECK(gather<R>(c, 0, pin, norb, c0));
  if (c->ns > 0) {
    dim3 g(grid1(c->ns, 128), norb);
    k_coef_dij<<<g, 128, 0, c->stream>>>(c0, c1, norb, c->ns, c->d_slot_atom, c->d_soff, c->d_doff, c->d_ms,
                                         c->d_dij[set]);
    c->launches++;
    OPAW_CUDA(cudaGetLastError());
  }
  // kinetic term through the 3D FFT (hphi.f90:14-18) and v_ks psi (:21)
  OPAW_CHECK(h_fft<R>(c, VksOf<R>::get(c, set), pin, hp, norb, nullptr, nullptr));
  // nonlocal term (hphi.f90:42-60)
  OPAW_CHECK(union_scatter<R>(c, 0, hp, norb, c1));
  return OPAW_OK;
}

// H applied with explicit potential / D_ij, optionally with the projections
// <p~|pin> already known (cpre) and with the perturbation-difference extras
// (t0, dv, c0, ddij): hp = H[vks, dij] pin + dv t0 + sum p~ ddij c0
template <typename R>
int h_apply_ex(opaw_ctx *c, const R *vks, const double *dij, const typename Tr<R>::C *pin, typename Tr<R>::C *hp,
               int norb, const double2 *cpre, const typename Tr<R>::C *t0, const R *dv, const double2 *c0,
               const double *ddij) {
  if (norb <= 0) return OPAW_OK;
  OPAW_CHECK(ensure(c->coef[0], sizeof(double2) * (size_t)c->ns * norb + 16));
  OPAW_CHECK(ensure(c->coef[1], sizeof(double2) * (size_t)c->ns * norb + 16));
  const double2 *cp = cpre;
  if (!cp) {
    OPAW_CHECK(gather<R>(c, 0, pin, norb, (double2 *)c->coef[0].p));
    cp = (const double2 *)c->coef[0].p;
  }
  double2 *c1 = (double2 *)c->coef[1].p;
  if (c->ns > 0) {
    dim3 g(grid1(c->ns, 128), norb);
    if (t0)
      k_coef_dij2<<<g, 128, 0, c->stream>>>(cp, c0, c1, norb, c->ns, c->d_slot_atom, c->d_soff, c->d_doff, c->d_ms,
                                            dij, ddij);
    else
      k_coef_dij<<<g, 128, 0, c->stream>>>(cp, c1, norb, c->ns, c->d_slot_atom, c->d_soff, c->d_doff, c->d_ms, dij);
    c->launches++;
    OPAW_CUDA(cudaGetLastError());
  }
  OPAW_CHECK(h_fft<R>(c, vks, pin, hp, norb, t0, dv));
  OPAW_CHECK(union_scatter<R>(c, 0, hp, norb, c1));
  return OPAW_OK;
}

// the grid part of h_phi: hp = F^-1[ek F pin] + v_ks pin (+ dv t0)
// (hphi.f90:16-21), without the projector term
template <typename R>
int h_fft(opaw_ctx *c, const R *vks, const typename Tr<R>::C *pin, typename Tr<R>::C *hp, int norb,
          const typename Tr<R>::C *t0, const R *dv) {
  typedef typename Tr<R>::C C;
  if (norb <= 0) return OPAW_OK;
  OPAW_CHECK(ensure(c->work[0], sizeof(C) * (size_t)c->nn * norb));
  C *w = (C *)c->work[0].p;
  Dims3 d{c->nx, c->ny, c->nz};
  OpCopy<C> x_in{pin, w, c->nn};
  OpCopy<C> inplace{w, w, c->nn};
  OpHFinal<R> fin{w, pin, vks, hp, c->nn, t0, dv};
  int st;
  if (launch_xy_if<C>(c, c->fft, norb, -1, x_in, &st)) {
    // three passes: xy planes, z lines with the kinetic factor, xy planes + v_ks psi
    OPAW_CHECK(st);
    OPAW_CHECK((launch_axis<C, 2>(c, c->fft.ax[2], d, norb, 0, make_kin<R>(c, w))));
    launch_xy_if<C>(c, c->fft, norb, +1, fin, &st);
    OPAW_CHECK(st);
  } else {
    OPAW_CHECK((launch_axis<C, 0>(c, c->fft.ax[0], d, norb, -1, x_in)));
    OPAW_CHECK((launch_axis<C, 1>(c, c->fft.ax[1], d, norb, -1, inplace)));
    OPAW_CHECK((launch_axis<C, 2>(c, c->fft.ax[2], d, norb, 0, make_kin<R>(c, w))));
    OPAW_CHECK((launch_axis<C, 1>(c, c->fft.ax[1], d, norb, +1, inplace)));
    OPAW_CHECK((launch_axis<C, 0>(c, c->fft.ax[0], d, norb, +1, fin)));
  }
  return OPAW_OK;
}

// the grid part of H of every set of a stage (the kicked sets in the
// difference form H' t_d + dv t_0) in one interleaved batch of (1 + nkick)
// norb; returns 0 when the grid has no plane kernel (the caller then runs
// h_fft per set)
template <typename R>
int h_fftk(opaw_ctx *c, const R *v0, const R *v1, const typename Tr<R>::C *t0, const typename Tr<R>::C *td,
           typename Tr<R>::C *u0, typename Tr<R>::C *ud, const R *dv, int norb, int nkick, int *ran) {
  typedef typename Tr<R>::C C;
  *ran = 0;
  if (norb <= 0) return OPAW_OK;
  const int nset = 1 + nkick;
  OPAW_CHECK(ensure(c->work[0], sizeof(C) * (size_t)c->nn * nset * norb));
  C *w = (C *)c->work[0].p;
  Dims3 d{c->nx, c->ny, c->nz};
  OpCopyK<C> fwd{t0, td, w, c->nn, nset, norb};
  OpHFinalK<R> fin{w, t0, td, v0, v1, u0, ud, dv, c->nn, nset, norb};
  int st;
  if (!launch_xy_if<C>(c, c->fft, nset * norb, -1, fwd, &st)) return OPAW_OK;
  OPAW_CHECK(st);
  OPAW_CHECK((launch_axis<C, 2>(c, c->fft.ax[2], d, nset * norb, 0, make_kin<R>(c, w))));
  launch_xy_if<C>(c, c->fft, nset * norb, +1, fin, &st);
  OPAW_CHECK(st);
  *ran = 1;
  return OPAW_OK;
}

// out = F^-1 [K(x) F pin] per orbital (OpTPA); inv_ekin: device [norb]
template <typename R>
int precond_kinetic(opaw_ctx *c, const typename Tr<R>::C *pin, const double *inv_ekin, typename Tr<R>::C *out,
                    int norb) {
  typedef typename Tr<R>::C C;
  if (norb <= 0) return OPAW_OK;
  Dims3 d{c->nx, c->ny, c->nz};
  OpCopy<C> x_in{pin, out, c->nn};
  OpCopy<C> inplace{out, out, c->nn};
  OpTPA<R> tpa{out, c->nn, nullptr, nullptr, nullptr, c->nx, inv_ekin,
               (R)(1.0 / ((double)c->nx * (double)c->ny * (double)c->nz))};
  if constexpr (sizeof(R) == 8) {
    tpa.k2x = c->d_k2[0];
    tpa.k2y = c->d_k2[1];
    tpa.k2z = c->d_k2[2];
  } else {
    tpa.k2x = c->d_k2f[0];
    tpa.k2y = c->d_k2f[1];
    tpa.k2z = c->d_k2f[2];
  }
  int st;
  if (launch_xy_if<C>(c, c->fft, norb, -1, x_in, &st)) {
    OPAW_CHECK(st);
    OPAW_CHECK((launch_axis<C, 2>(c, c->fft.ax[2], d, norb, 0, tpa)));
    launch_xy_if<C>(c, c->fft, norb, +1, inplace, &st);
    OPAW_CHECK(st);
  } else {
    OPAW_CHECK((launch_axis<C, 0>(c, c->fft.ax[0], d, norb, -1, x_in)));
    OPAW_CHECK((launch_axis<C, 1>(c, c->fft.ax[1], d, norb, -1, inplace)));
    OPAW_CHECK((launch_axis<C, 2>(c, c->fft.ax[2], d, norb, 0, tpa)));
    OPAW_CHECK((launch_axis<C, 1>(c, c->fft.ax[1], d, norb, +1, inplace)));
    OPAW_CHECK((launch_axis<C, 0>(c, c->fft.ax[0], d, norb, +1, inplace)));
  }
  return OPAW_OK;
}
template int precond_kinetic<float>(opaw_ctx *, const float2 *, const double *, float2 *, int);
template int precond_kinetic<double>(opaw_ctx *, const double2 *, const double *, double2 *, int);

// per orbital sum over k of min(|k|^2 / 2, ekcut) |F x|^2 and of |F x|^2 (one
// block per orbital); their ratio is the kinetic energy <x|T|x> / <x|x> of
// the Hamiltonian's kinetic operator (ek.f90)
template <typename C, typename R>
__global__ void k_ekin_sums(const C *__restrict__ fx, int nx, int ny, int nz, const R *__restrict__ k2x,
                            const R *__restrict__ k2y, const R *__restrict__ k2z, double ekcut,
                            double *__restrict__ out) {
  __shared__ double sh[2][8];
  const int o = blockIdx.x;
  const int64_t nn = (int64_t)nx * ny * nz;
  double a = 0, b = 0;
  for (int64_t g = threadIdx.x; g < nn; g += blockDim.x) {
    const int x = (int)(g % nx), y = (int)((g / nx) % ny), z = (int)(g / ((int64_t)nx * ny));
    double e = 0.5 * ((double)k2x[x] + (double)k2y[y] + (double)k2z[z]);
    if (ekcut > 0.0 && e > ekcut) e = ekcut;
    const C v = fx[(int64_t)o * nn + g];
    const double m = (double)v.x * v.x + (double)v.y * v.y;
    a += e * m;
    b += m;
  }
#pragma unroll
  for (int q = 16; q > 0; q >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, q);
    b += __shfl_down_sync(0xffffffffu, b, q);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = a;
    sh[1][w] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sa = 0, sb = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
      sa += sh[0][i];
      sb += sh[1][i];
    }
    out[2 * o] = sa;
    out[2 * o + 1] = sb;
  }
}

// kinetic energies <x_o|T|x_o> / <x_o|x_o> of norb device orbitals (host out)
template <typename R>
int kinetic_energy(opaw_ctx *c, const typename Tr<R>::C *x, int norb, double *ekin) {
  typedef typename Tr<R>::C C;
  if (norb <= 0) return OPAW_OK;
  OPAW_CHECK(ensure(c->work[0], sizeof(C) * (size_t)c->nn * norb));
  OPAW_CHECK(ensure(c->pre, sizeof(double) * 2 * (size_t)norb));
  C *w = (C *)c->work[0].p;
  OPAW_CUDA(cudaMemcpyAsync(w, x, sizeof(C) * (size_t)c->nn * norb, cudaMemcpyDeviceToDevice, c->stream));
  OPAW_CHECK(fft3d<R>(c, c->fft, w, norb, -1));
  const R *k2[3];
  for (int k = 0; k < 3; k++) k2[k] = sizeof(R) == 8 ? (const R *)c->d_k2[k] : (const R *)c->d_k2f[k];
  k_ekin_sums<C, R><<<norb, 256, 0, c->stream>>>(w, c->nx, c->ny, c->nz, k2[0], k2[1], k2[2], c->ekcut,
                                                 (double *)c->pre.p);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  std::vector<double> h(2 * (size_t)norb);
  OPAW_CUDA(cudaMemcpyAsync(h.data(), c->pre.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  for (int o = 0; o < norb; o++) ekin[o] = h[2 * o + 1] > 0.0 ? h[2 * o] / h[2 * o + 1] : 0.0;
  return OPAW_OK;
}
template int kinetic_energy<float>(opaw_ctx *, const float2 *, int, double *);
template int kinetic_energy<double>(opaw_ctx *, const double2 *, int, double *);

// sigma table for sn_phi's exponent n: cached for n = -1, -1/2, 1/2, 1
static int sigma_table(opaw_ctx *c, double n, const double **out) {
  int slot;
  if (n == -1.0) slot = 0;
  else if (n == -0.5) slot = 1;
  else if (n == 0.5) slot = 2;
  else if (n == 1.0) slot = 3;
  else {
    set_error("sn_phi exponent must be -1, -0.5, 0.5 or 1");
    return OPAW_ERR_ARG;
  }
  *out = c->d_sigma[slot];
  return OPAW_OK;
}

template <typename R>
int sn_apply(opaw_ctx *c, double n, const typename Tr<R>::C *pin, typename Tr<R>::C *sp, int norb) {
  typedef typename Tr<R>::C C;
  if (norb <= 0) return OPAW_OK;
  const double *sigma;
  OPAW_CHECK(sigma_table(c, n, &sigma));
  OPAW_CHECK(ensure(c->coef[2], sizeof(double2) * (size_t)c->ns * norb + 16));
  OPAW_CHECK(ensure(c->coef[3], sizeof(double2) * (size_t)c->ns * norb + 16));
  double2 *c0 = (double2 *)c->coef[2].p, *c1 = (double2 *)c->coef[3].p;
  OPAW_CHECK(gather<R>(c, 1, pin, norb, c0));  // proj1 of the unmodified input (snphi.f90:23)
  if (c->ns > 0) {
    dim3 g(grid1(c->ns, 128), norb);
    k_coef_scale<<<g, 128, 0, c->stream>>>(c0, c1, norb, c->ns, sigma);
    c->launches++;
    OPAW_CUDA(cudaGetLastError());
  }
  if (sp != pin) OPAW_CUDA(cudaMemcpyAsync(sp, pin, sizeof(C) * (size_t)c->nn * norb, cudaMemcpyDeviceToDevice, c->stream));
  OPAW_CHECK(union_scatter<R>(c, 1, sp, norb, c1));
  return OPAW_OK;
}

template <typename R>
int shs_apply(opaw_ctx *c, int set, const typename Tr<R>::C *pin, typename Tr<R>::C *pout, int norb) {
  typedef typename Tr<R>::C C;
  if (norb <= 0) return OPAW_OK;
  OPAW_CHECK(ensure(c->work[1], sizeof(C) * (size_t)c->nn * norb));
  C *t = (C *)c->work[1].p;
  OPAW_CHECK(sn_apply<R>(c, -0.5, pin, t, norb));   // shs.f90:19
  OPAW_CHECK(h_apply<R>(c, set, t, pout, norb));    // :20
  OPAW_CHECK(sn_apply<R>(c, -0.5, pout, pout, norb)); // :21-22
  return OPAW_OK;
}

#define OPAW_INST(R)                                                                                   \
  template int gather<R>(opaw_ctx *, int, const Tr<R>::C *, int, double2 *);                        \
  template int union_scatter<R>(opaw_ctx *, int, Tr<R>::C *, int, const double2 *);                 \
  template int h_apply<R>(opaw_ctx *, int, const Tr<R>::C *, Tr<R>::C *, int);                      \
  template int sn_apply<R>(opaw_ctx *, double, const Tr<R>::C *, Tr<R>::C *, int);                  \
  template int shs_apply<R>(opaw_ctx *, int, const Tr<R>::C *, Tr<R>::C *, int);                    \
  template int h_apply_ex<R>(opaw_ctx *, const R *, const double *, const Tr<R>::C *, Tr<R>::C *, int,  \
                             const double2 *, const Tr<R>::C *, const R *, const double2 *, const double *); \
  template int h_fft<R>(opaw_ctx *, const R *, const Tr<R>::C *, Tr<R>::C *, int, const Tr<R>::C *, const R *); \
  template int h_fftk<R>(opaw_ctx *, const R *, const R *, const Tr<R>::C *, const Tr<R>::C *, Tr<R>::C *,         \
                         Tr<R>::C *, const R *, int, int, int *);                                                   \
  template int gather2<R>(opaw_ctx *, const Tr<R>::C *, int, double2 *, double2 *);
OPAW_INST(float)
OPAW_INST(double)

}  // namespace opaw

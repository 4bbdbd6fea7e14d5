// common.cuh — context, error plumbing and precision traits shared by the
// translation units of libopaw_gb300.so (the sm_103a OPAW-TDDFT path).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <deque>
#include <string>
#include <vector>

#include "../../include/opaw_gb300.h"

namespace opaw {

// union points per tile of the box-coefficient pass
constexpr int kUTile = 128;

// ---------------------------------------------------------------- errors --
void set_error(const std::string &msg);
const char *get_error();

#define OPAW_CUDA(call)                                                                 \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      ::opaw::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));          \
      return OPAW_ERR_CUDA;                                                             \
    }                                                                                   \
  } while (0)

#define OPAW_CHECK(call)         \
  do {                           \
    int s_ = (call);             \
    if (s_ != OPAW_OK) return s_; \
  } while (0)

#define OPAW_ARG(cond, msg)                  \
  do {                                       \
    if (!(cond)) {                           \
      ::opaw::set_error(msg);                \
      return OPAW_ERR_ARG;                   \
    }                                        \
  } while (0)

// ------------------------------------------------------- precision traits --
template <typename R> struct Tr;
template <> struct Tr<float> {
  typedef float2 C;
  static constexpr int dtype = OPAW_C64;
};
template <> struct Tr<double> {
  typedef double2 C;
  static constexpr int dtype = OPAW_C128;
};

__host__ __device__ inline float2 cmake(float a, float b) { return make_float2(a, b); }
__host__ __device__ inline double2 cmake(double a, double b) { return make_double2(a, b); }

template <typename C> __host__ __device__ inline C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __host__ __device__ inline C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __host__ __device__ inline C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename C, typename R> __host__ __device__ inline C cscale(C a, R s) { C r; r.x = a.x * s; r.y = a.y * s; return r; }
template <typename C> __host__ __device__ inline C cconj(C a) { C r; r.x = a.x; r.y = -a.y; return r; }

#ifdef __CUDACC__
// IEEE double -> float with round-to-nearest-even done on the integer pipe.
// GB300 runs 64-bit type conversions at its (low) FP64 rate; the bulk
// kernels of the mixed path convert every grid point, so they use these.
// Magnitudes below 2^-126 flush to a signed zero, above FLT_MAX give inf;
// NaN stays NaN.
__device__ __forceinline__ float d2f(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned sign = hi & 0x80000000u;
  const unsigned ex = (hi >> 20) & 0x7ffu;
  if (ex == 0x7ffu) return __uint_as_float(sign | 0x7f800000u | (((hi & 0xfffffu) | lo) ? 0x400000u : 0u));
  const int e = (int)ex - 1023 + 127;
  if (e <= 0) return __uint_as_float(sign);
  if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
  const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned rest = lo & 0x1fffffffu;
  unsigned r = sign | ((unsigned)e << 23) | m;
  if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) r += 1u;  // a carry rolls into the exponent
  return __uint_as_float(r);
}
// Fixed-order sum over a block of 256 threads: thread t adds elements
// t, t+256, ... of a strided sequence, then a shuffle/shared-memory tree.
// Returns the total in thread 0 (deterministic for a given n).
__device__ __forceinline__ double block_sum_seq(const double *__restrict__ v, int n, int stride, double *sh) {
  double acc = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += v[(int64_t)i * stride];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = acc;
  __syncthreads();
  double r = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) r += sh[i];
  return r;
}

// exact float -> double on the integer pipe (subnormal floats flush to zero)
__device__ __forceinline__ double f2d(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  unsigned hi, lo;
  if (e == 0) {
    hi = sign;
    lo = 0;
  } else if (e == 0xffu) {
    hi = sign | 0x7ff00000u | (m >> 3);
    lo = m << 29;
  } else {
    hi = sign | ((e + 896u) << 20) | (m >> 3);
    lo = m << 29;
  }
  return __hiloint2double((int)hi, (int)lo);
}
#endif

// ---------------------------------------------------------- FFT planning --
struct FFTAxis {
  int n = 0;
  int nstage = 0;
  int radix[16];
  // twiddle table exp(-2 pi i t / n), t in [0, n)
  double2 *tw64 = nullptr;
  float2 *tw32 = nullptr;
};

struct FFT3 {
  int n[3] = {0, 0, 0};
  FFTAxis ax[3];
};

int fft3_init(FFT3 &f, int nx, int ny, int nz);
void fft3_free(FFT3 &f);

// ------------------------------------------------------------- context --
struct DeviceBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

// One launch site of the autotuner (autotune.cu): its candidates are timed
// with CUDA events on the launches the computation makes anyway (every
// candidate computes bit-identical results), kTuneRounds times each in turn;
// then the fastest is kept for the context's lifetime.
struct TuneSite {
  std::vector<std::string> labels;
  std::vector<cudaEvent_t> ev;  // [round][candidate][start, stop]
  std::vector<float> ms;        // best time per candidate
  int next = 0;                 // timed launches so far
  int chosen = -1;
};

}  // namespace opaw

struct opaw_ctx {
  // scalars of the system
  int nx, ny, nz;
  int64_t nn;
  double dx, dy, dz, dv, ekcut, rnel, dij_max;
  int scale_vh, periodic;
  int nsm = 0;  // multiprocessors of the context's device
  // live timing of the fused dense pass (opaw_ktime_begin / _end)
  bool ktime_on = false;
  // autotuner state: launch site key -> site (autotune.cu)
  int tune_on = 1;  // 1 timing, 2 frozen (decided sites kept, no timing), 0 off (defaults)
  std::deque<std::pair<std::string, opaw::TuneSite>> tune;
  std::vector<cudaEvent_t> kev;  // start/stop pairs, reused
  int kev_used = 0;
  double kbytes = 0.0;
  int nxb, nyb, nzb;
  int64_t nnb;
  int natom;
  int ns;   // sum of ms
  int nd;   // sum of ms^2
  int msmax;

  cudaStream_t stream = nullptr;
  int64_t launches = 0;

  // host copies of small tables
  std::vector<int> h_ms, h_nrough, h_ir0;  // ir0 is 0-based
  std::vector<int64_t> h_poff, h_soff, h_doff;

  // atom tables (device)
  int *d_ms = nullptr, *d_nrough = nullptr, *d_ir0 = nullptr;
  int64_t *d_poff = nullptr, *d_soff = nullptr, *d_doff = nullptr;
  double *d_p3d = nullptr, *d_p3d1 = nullptr;
  float *d_p3d_f = nullptr, *d_p3d1_f = nullptr;
  double *d_s = nullptr, *d_sinv = nullptr;
  double *d_sigma[4] = {nullptr, nullptr, nullptr, nullptr};  // (1+s)^n - 1 for n = -1(sinv), -1/2, 1/2, 1
  int *d_slot_atom = nullptr;    // [ns] atom of each projector slot
  int *d_dslot_atom = nullptr;   // [nd] atom of each ms x ms matrix entry
  // union of projector boxes: CSR over grid points
  int nunion = 0, nuent = 0;
  int *d_upt = nullptr, *d_ustart = nullptr, *d_uatom = nullptr, *d_ubox = nullptr;
  // per union entry: {projector-table offset of the box point, index of the
  // atom among the distinct atoms of its tile of kUTile union points,
  // projector count, box size}; per tile its atoms' first slots and projector
  // counts (utile_na atoms, at most uamax); null when the table offsets
  // exceed int32
  int4 *d_uent = nullptr;
  int2 *d_utile = nullptr;
  int *d_utile_na = nullptr;
  int uamax = 0;
  int *d_boxg = nullptr;         // per atom and box point: the wrapped linear grid index
  int64_t *d_boff = nullptr;     // per atom offset into d_boxg
  int *d_uidx = nullptr;         // per grid point: its union index, -1 outside every box
  int maxbox = 0;                // largest projector box (points)
  // projector overlaps <p_x|p_y> (x, y = p~ or p~1; FP64, dv included) as
  // dense ms_a x ms_b blocks for every pair of atoms whose boxes share a
  // grid point: block k of row atom a is (a, ovl_atom[k]) for k in
  // [ovl_start[a], ovl_start[a+1]), stored row-major at ovl_off[k]
  int novl = 0;
  int *d_ovl_start = nullptr, *d_ovl_atom = nullptr;
  int64_t *d_ovl_off = nullptr;
  double *d_ovl[4] = {nullptr, nullptr, nullptr, nullptr};  // <p~|p~>, <p~|p~1>, <p~1|p~>, <p~1|p~1>

  // compensation charge tables
  int ncomp = 0;             // total sphere points
  int nlmmax = 0;
  std::vector<int64_t> h_goff, h_g3off, h_qoff, h_eoff;
  std::vector<int> h_ngrid, h_nlm;
  int *d_ngrid = nullptr, *d_nlm = nullptr;
  int64_t *d_goff = nullptr, *d_g3off = nullptr, *d_qoff = nullptr, *d_eoff = nullptr;
  int *d_gpt = nullptr;      // linear grid index per sphere point
  double *d_g3d = nullptr, *d_qijlm = nullptr, *d_dij0 = nullptr, *d_eijkl = nullptr;
  // union of sphere points: CSR
  int ncunion = 0;
  int *d_cpt = nullptr, *d_cstart = nullptr, *d_catom = nullptr, *d_cig = nullptr;

  // on-site XC term of D_ij (onsite_xc.cu): radial tables per atom, the
  // Gaunt coefficients per atom [9][ms][ms], scratch [2][9][radial points]
  // and the result [nd]
  int oxc_on = 0;
  int *oxc_rad_n = nullptr, *oxc_pwave = nullptr, *oxc_nphi = nullptr;
  int oxc_nchunk = 1;
  int64_t *oxc_roff = nullptr, *oxc_phioff = nullptr;
  double *oxc_r = nullptr, *oxc_w = nullptr, *oxc_core = nullptr, *oxc_tcore = nullptr;
  double *oxc_phi = nullptr, *oxc_tphi = nullptr, *oxc_gaunt = nullptr;
  short *oxc_live = nullptr;  // per atom: (L, pair) entries with non-zero Gaunt coefficients
  int *oxc_nlive = nullptr;
  opaw::DeviceBuf oxc_part;  // partial radial integrals [set][atom][part][chunk][L][pair]
  opaw::DeviceBuf oxc_sets;  // D_xc of the unperturbed and every kicked set (mixed step)
  // a second stream of the context: the on-site XC term of the mixed step
  // runs there while the Hartree solves run on `stream` (fork / join events)
  cudaStream_t side = nullptr;
  cudaEvent_t side_fork = nullptr, side_join = nullptr;
  double *oxc_dxc = nullptr;

  // kinetic separable tables: k^2 per axis (double, exact copies of the
  // reference's kx*kx) and float twins
  double *d_k2[3] = {nullptr, nullptr, nullptr};
  float *d_k2f[3] = {nullptr, nullptr, nullptr};

  // potentials
  double *d_vloc = nullptr, *d_ncoret = nullptr;
  double *d_vk = nullptr;        // MT kernel on the big box, 1/Nb folded in
  float *d_vk_f = nullptr;       // its FP32 copy for the mixed-precision Hartree solve
  double *d_vks[2] = {nullptr, nullptr};
  float *d_vks_f[2] = {nullptr, nullptr};
  double *d_dij[2] = {nullptr, nullptr};
  double *d_rhoij[2] = {nullptr, nullptr};
  double *d_dens[2] = {nullptr, nullptr};
  double *d_nhat[2] = {nullptr, nullptr};
  double *d_vh[2] = {nullptr, nullptr};
  double *d_vxc[2] = {nullptr, nullptr};

  // FFT plans
  opaw::FFT3 fft, fftb;

  // resident orbitals (complex128); set 1 holds nkick kicked sets of
  // norb[1] orbitals each, [kick][orbital][point], all propagated against the
  // one unperturbed set 0; the per-set state arrays of set 1 (d_vks[1],
  // d_vks_f[1], d_dij[1], d_rhoij[1], d_dens[1], d_nhat[1], d_vh[1],
  // d_vxc[1]) have room for kcap kicks, [kick][...]
  double2 *d_psi[2] = {nullptr, nullptr};
  int norb[2] = {0, 0};
  int nkick = 1, kcap = 1;
  double *d_kgamma = nullptr;     // [kcap] kick strengths on the device
  std::vector<double> h_kgamma;   // [nkick] and on the host

  // scratch (grown on demand)
  // 0 FFT work, 1 shs intermediate, 2 Hartree source, 3 Hartree 2x box,
  // 4 rebuild psi~, 5-6 host-twin staging, 7 RK4 k, 8 RK4 y, 9 RK4 ksum
  opaw::DeviceBuf work[12];
  opaw::DeviceBuf coef[4];       // [norb][ns] double2
  opaw::DeviceBuf coefr;         // single-precision copy of the scatter coefficients
  opaw::DeviceBuf gram, gramout; // Gram partials, small matrices
  opaw::DeviceBuf mix[16];       // buffers of the mixed-precision difference step
  opaw::DeviceBuf href;          // FP64 reference source and Hartree potential of the unperturbed set
  // generation of set 0's contents, bumped whenever they are replaced from
  // outside the propagation (upload, orthogonalisation, device pointer handed
  // out); the Hartree reference is reused by later mixed calls of the same
  // generation
  int64_t psi0_gen = 0, href_gen = -1;
  opaw::DeviceBuf red;           // reductions
  opaw::DeviceBuf pre;           // per-orbital arguments of the preconditioners
  opaw::DeviceBuf g2part;        // segment partials of the two-table gather
  opaw::DeviceBuf g2other;       // the unused table's sums when one table is wanted
  opaw::DeviceBuf ddsplit;       // hi / lo complex64 halves of complex128 operands (gram.cu)
  int *d_tma_err = nullptr;      // set by a TMA-staged kernel whose barrier wait ran out
  double *h_red = nullptr;       // pinned host mirror of small reductions
};

namespace opaw {

int ensure(DeviceBuf &b, size_t bytes);
// room for K kicked sets in the set-1 state arrays (ctx.cu); the contents of
// kick 0 are kept
int kick_capacity(opaw_ctx *c, int K);
// the kick strengths of the context's kicked sets, to the device (ctx.cu)
int upload_kgamma(opaw_ctx *c);

inline int grid1(int64_t n, int t) { return (int)((n + t - 1) / t); }

// ---------------------------------------------------- operator building blocks --
// (hamiltonian.cu)
template <typename R>
int gather(opaw_ctx *c, int which, const typename Tr<R>::C *pin, int norb, double2 *coef);
template <typename R>
int union_scatter(opaw_ctx *c, int which, typename Tr<R>::C *out, int norb, const double2 *coef);
template <typename R>
int h_apply(opaw_ctx *c, int set, const typename Tr<R>::C *pin, typename Tr<R>::C *hp, int norb);
template <typename R>
int sn_apply(opaw_ctx *c, double n, const typename Tr<R>::C *pin, typename Tr<R>::C *sp, int norb);
template <typename R>
int shs_apply(opaw_ctx *c, int set, const typename Tr<R>::C *pin, typename Tr<R>::C *pout, int norb);

template <typename R>
int h_apply_ex(opaw_ctx *c, const R *vks, const double *dij, const typename Tr<R>::C *pin, typename Tr<R>::C *hp,
               int norb, const double2 *cpre, const typename Tr<R>::C *t0, const R *dv, const double2 *c0,
               const double *ddij);
// projector coefficient algebra (hamiltonian.cu): cout = D cin, and
// cout = D cin + dD c0 (hphi.f90:43-47)
__global__ void k_coef_dij(const double2 *__restrict__ cin, double2 *__restrict__ cout, int norb, int ns,
                           const int *__restrict__ slot_atom, const int64_t *__restrict__ soff,
                           const int64_t *__restrict__ doff, const int *__restrict__ ms,
                           const double *__restrict__ dij);
__global__ void k_coef_dij2(const double2 *__restrict__ cin, const double2 *__restrict__ c0,
                            double2 *__restrict__ cout, int norb, int ns, const int *__restrict__ slot_atom,
                            const int64_t *__restrict__ soff, const int64_t *__restrict__ doff,
                            const int *__restrict__ ms, const double *__restrict__ dij,
                            const double *__restrict__ ddij);
// the grid part of h_phi (kinetic + local, + dv t0 when t0 is given)
template <typename R>
int h_fft(opaw_ctx *c, const R *vks, const typename Tr<R>::C *pin, typename Tr<R>::C *hp, int norb,
          const typename Tr<R>::C *t0, const R *dv);
template <typename R>
int h_fftk(opaw_ctx *c, const R *v0, const R *v1, const typename Tr<R>::C *t0, const typename Tr<R>::C *td,
           typename Tr<R>::C *u0, typename Tr<R>::C *ud, const R *dv, int norb, int nkick, int *ran);
// Teter-Payne-Allan kinetic preconditioner of norb orbitals (inv_ekin: device
// [norb] inverse kinetic energies); out may equal pin
template <typename R>
int precond_kinetic(opaw_ctx *c, const typename Tr<R>::C *pin, const double *inv_ekin, typename Tr<R>::C *out,
                    int norb);
// kinetic energies <x_o|T|x_o> / <x_o|x_o> of norb device orbitals into a host array
template <typename R>
int kinetic_energy(opaw_ctx *c, const typename Tr<R>::C *x, int norb, double *ekin);
// <p~|pin> and <p~1|pin> in one pass over the boxes
template <typename R>
int gather2(opaw_ctx *c, const typename Tr<R>::C *pin, int norb, double2 *c0, double2 *c1);

// (fft.cu) batched 3D FFT of `batch` arrays; sign -1 forward, +1 backward
template <typename R>
int fft3d(opaw_ctx *c, const FFT3 &f, typename Tr<R>::C *data, int batch, int sign);

// (rebuild.cu)
int hartree(opaw_ctx *c, const double *dens0, const double *dens1, double *vh0, double *vh1);
template <typename R>
int hartree_t(opaw_ctx *c, const double *dens0, const double *dens1, double *vh0, double *vh1);
template <typename R>
int hartree_pair_t(opaw_ctx *c, const double *dens0, const double *dens1, double *vh0, double *vh1);
// nsrc independent sources src[b] = src + b nn in one batch of complex
// transforms (each keeps its own relative precision): vh + b nn
template <typename R>
int hartree_batch_t(opaw_ctx *c, const double *src, int nsrc, double *vh);
int rhoij_of(opaw_ctx *c, const double2 *coef, int norb, double *out);
template <typename R> int density_raw(opaw_ctx *c, const typename Tr<R>::C *psit, int norb, double *out);
int nhat_raw_of(opaw_ctx *c, const double *rhoij, double *out);
int sums2(opaw_ctx *c, const double *a, const double *b, double *part);
constexpr int kRedBlocks = 1024;
int vxc_of(opaw_ctx *c, const double *dens, const double *core, double *out);
// (onsite_xc.cu) the on-site XC term of D_ij: set-up from the system's
// radial tables (none given: the term is off), release, and D_xc of rho_ij
int onsite_init(opaw_ctx *c, const opaw_system *s);
void onsite_free(opaw_ctx *c);
int onsite_xc_of(opaw_ctx *c, const double *rhoij, double *dxc);
int onsite_xc_sets(opaw_ctx *c, const double *rhoij, int nsets, double *dxc, cudaStream_t st);
// D_ij (get_dij.f90) from rho_ij and the potential v_ks - v_xc of Dhat (vxc may be null)
int dij_of(opaw_ctx *c, const double *rhoij, const double *vks, const double *vxc, double *out,
           const double *dxc_pre = nullptr);
// (mixed.cu) nsteps mixed-precision TDDFT steps of the unperturbed set and
// the c->nkick kicked sets (strengths gamma_dev[k]); 3 + 6 nkick doubles per
// step into dd_dev: dip, then dip'_k and d_dip_k of every kick
int mixed_steps(opaw_ctx *c, int nsteps, double dt, const double *gamma_dev, double *dd_dev);
int ensemble_steps(opaw_ctx *const *cs, int n, int nsteps, double dt, double *const *dd, double *const *fixed);
// autotuner: the candidate to launch at site `key` (labels: one per
// candidate; dflt when tuning is off, finished or the stream is capturing);
// *timed != nullptr: the launch is being timed, close it with tune_end
int tune_begin(opaw_ctx *c, const std::string &key, const std::vector<std::string> &labels, int dflt,
               TuneSite **timed);
int tune_end(opaw_ctx *c, TuneSite *timed);
// 3D tensor map of a batch of nlines x nz arrays of 8-byte elements (tma.cu)
int tma_map_lines(CUtensorMap *m, const void *base, uint64_t nlines, uint64_t nz, uint64_t batch, uint64_t bstride,
                  uint32_t box_lines, uint32_t box_z);
// after a stream synchronisation: OPAW_ERR_CUDA when a TMA-staged kernel's
// barrier wait ran out (the flag is cleared)
int tma_status(opaw_ctx *c);
void tune_free(opaw_ctx *c);
// LDA potential of n points (device arrays)
int vxc_points(opaw_ctx *c, const double *dens, double *vxc, int64_t n);
// gout = 1/N ifft(bk fft(a)) on the context's main FFT plan; a is overwritten
int rconv_device(opaw_ctx *c, double2 *a, const double *bk, double *gout, int n0, int n1, int n2);

}  // namespace opaw

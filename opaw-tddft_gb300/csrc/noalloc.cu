// noalloc.cu — the r2c Hartree-type convolution (rconv) for callers that
// cannot allocate device memory.
//
// opaw_rconv allocates its work arrays and FFT tables on every call.  Some
// callers cannot do that: a host program that hands this library a device
// memory budget fixed at start-up (for example a Fortran code that sized all
// device memory once and runs close to it), or a process whose allocator a
// library must not touch (a memory pool owned by another runtime).
// opaw_rconv_noalloc takes caller-allocated device buffers for the input, the
// kernel and the output, and keeps its scratch (the complex work array and
// the twiddle tables) in file-scope device arrays of fixed size that every
// GPU which loads this library holds until the process exits.  The twiddles
// are computed on the device by a kernel, so nothing is copied from host
// memory; the call waits for its stream before it returns, so the scratch is
// free for the next call once it has returned.
#include <cuda.h>

#include <mutex>

#include "fft.cuh"

namespace opaw {

constexpr int64_t kNoAllocMaxPoints = int64_t(1) << 18;  // 262,144 grid points: 4 MiB of complex128
constexpr int kNoAllocMaxExtent = 256;                   // per axis
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double2 g_noalloc_work[kNoAllocMaxPoints];
static __device__ __align__(256) double2 g_noalloc_tw[3 * kNoAllocMaxExtent];

// Device addresses of the two arrays, looked up once per device and context
// (host code must not use the symbols themselves): a device reset or a new
// primary context gives the arrays new addresses, so the context handle the
// lookup was made under is kept with them.
struct NoAllocPtrs {
  CUcontext ctx = nullptr;
  double2 *work = nullptr;
  double2 *tw = nullptr;
};
static NoAllocPtrs g_na_ptrs[kNoAllocMaxDevices];
static std::mutex g_na_mutex;

// cuCtxGetCurrent through the runtime's driver entry-point query, so that
// the library does not link libcuda itself (it loads on hosts without a GPU)
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
static CUcontext current_context() {
  static CtxGetCurrentFn fn = nullptr;
  if (!fn) {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !f)
      return nullptr;
    fn = (CtxGetCurrentFn)f;
  }
  CUcontext cur = nullptr;
  if (fn(&cur) != CUDA_SUCCESS) return nullptr;
  return cur;
}

// set-up with device `dev` current: the lookup is repeated only when the
// thread's current context differs from the one the cached addresses were
// taken under (none bound yet on this thread, another context, a reset)
static int noalloc_setup(int dev, NoAllocPtrs *out) {
  std::lock_guard<std::mutex> lock(g_na_mutex);
  CUcontext cur = current_context();
  NoAllocPtrs &p = g_na_ptrs[dev];
  if (!p.work || !cur || p.ctx != cur) {
    void *w = nullptr, *t = nullptr;
    // the runtime binds the device's primary context first if none is current
    cudaError_t e = cudaGetSymbolAddress(&w, g_noalloc_work);
    if (e != cudaSuccess) {
      set_error(std::string("cudaGetSymbolAddress(work): ") + cudaGetErrorString(e));
      return OPAW_ERR_CUDA;
    }
    e = cudaGetSymbolAddress(&t, g_noalloc_tw);
    if (e != cudaSuccess) {
      set_error(std::string("cudaGetSymbolAddress(twiddles): ") + cudaGetErrorString(e));
      return OPAW_ERR_CUDA;
    }
    cur = current_context();
    p.tw = (double2 *)t;
    p.work = (double2 *)w;
    p.ctx = cur;
  }
  *out = p;
  return OPAW_OK;
}

__global__ void k_na_real_to_complex(const double *__restrict__ g, double2 *__restrict__ a, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) a[i] = make_double2(g[i], 0.0);
}

// twiddle tables exp(-2 pi i t / n_k) of the three axes, axis k at k * 256
__global__ void k_na_twiddles(double2 *__restrict__ tw, int n0, int n1, int n2) {
  const int k = blockIdx.x, t = threadIdx.x;
  const int n = k == 0 ? n0 : (k == 1 ? n1 : n2);
  if (t >= n) return;
  double s, c;
  sincospi(2.0 * (double)t / (double)n, &s, &c);
  tw[k * kNoAllocMaxExtent + t] = make_double2(c, -s);
}

static bool radix_ok(int n) {
  for (int r : {2, 3, 5, 7})
    while (n % r == 0) n /= r;
  return n == 1;
}

}  // namespace opaw

using namespace opaw;

extern "C" int opaw_rconv_noalloc(int n0, int n1, int n2, const double *gin, const double *bk, double *gout,
                                  void *stream) {
  if (!gin || !bk || !gout || n0 <= 0 || n1 <= 0 || n2 <= 0) {
    set_error("opaw_rconv_noalloc: null buffer or non-positive extent");
    return OPAW_ERR_ARG;
  }
  const int ext[3] = {n0, n1, n2};
  for (int k = 0; k < 3; k++) {
    if (ext[k] > kNoAllocMaxExtent || !radix_ok(ext[k])) {
      set_error("opaw_rconv_noalloc: each extent must be <= 256 with prime factors 2, 3, 5, 7");
      return OPAW_ERR_ARG;
    }
  }
  const int64_t n = (int64_t)n0 * n1 * n2;
  if (n > kNoAllocMaxPoints) {
    set_error("opaw_rconv_noalloc: " + std::to_string(n) + " grid points exceed the fixed scratch of " +
              std::to_string(kNoAllocMaxPoints));
    return OPAW_ERR_ARG;
  }
  int dev = 0;
  OPAW_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) {
    set_error("opaw_rconv_noalloc: device ordinal out of range");
    return OPAW_ERR_ARG;
  }
  NoAllocPtrs p;
  OPAW_CHECK(noalloc_setup(dev, &p));

  opaw_ctx c;  // launch plumbing only: no tables, no buffers
  c.stream = (cudaStream_t)stream;
  for (int k = 0; k < 3; k++) {
    FFTAxis &a = c.fft.ax[k];
    a.n = ext[k];
    a.nstage = 0;
    int m = ext[k];
    for (int r : {8, 4, 2, 3, 5, 7})
      while (m % r == 0) {
        a.radix[a.nstage++] = r;
        m /= r;
      }
    a.tw64 = p.tw + (size_t)k * kNoAllocMaxExtent;
    a.tw32 = nullptr;
    c.fft.n[k] = ext[k];
  }
  k_na_twiddles<<<3, kNoAllocMaxExtent, 0, c.stream>>>(p.tw, n0, n1, n2);
  OPAW_CUDA(cudaGetLastError());
  k_na_real_to_complex<<<grid1(n, 256), 256, 0, c.stream>>>(gin, p.work, n);
  OPAW_CUDA(cudaGetLastError());
  OPAW_CHECK(rconv_device(&c, p.work, bk, gout, n0, n1, n2));
  // every call shares the scratch: it is free again once this call's work ended
  OPAW_CUDA(cudaStreamSynchronize(c.stream));
  return OPAW_OK;
}

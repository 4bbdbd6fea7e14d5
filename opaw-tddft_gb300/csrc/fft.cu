// fft.cu — FFT plans (radix schedule + twiddle tables) and the plain batched
// 3D transform.
#include <cmath>

#include "fft.cuh"

namespace opaw {

static int plan_axis(FFTAxis &a, int n) {
  a.n = n;
  a.nstage = 0;
  int m = n;
  const int pref[] = {8, 4, 2, 3, 5, 7, 11, 13};
  for (int r : pref) {
    while (m % r == 0 && a.nstage < 16) {
      a.radix[a.nstage++] = r;
      m /= r;
    }
  }
  if (m != 1) {
    set_error("grid extent " + std::to_string(n) + " has a prime factor other than 2, 3, 5, 7, 11, 13");
    return OPAW_ERR_ARG;
  }
  std::vector<double2> t64(n);
  std::vector<float2> t32(n);
  for (int t = 0; t < n; t++) {
    // exp(-2 pi i t / n), evaluated in double on the host
    double ang = 2.0 * M_PI * (double)t / (double)n;
    t64[t] = make_double2(cos(ang), -sin(ang));
    t32[t] = make_float2((float)cos(ang), (float)-sin(ang));
  }
  OPAW_CUDA(cudaMalloc(&a.tw64, sizeof(double2) * n));
  OPAW_CUDA(cudaMalloc(&a.tw32, sizeof(float2) * n));
  OPAW_CUDA(cudaMemcpy(a.tw64, t64.data(), sizeof(double2) * n, cudaMemcpyHostToDevice));
  OPAW_CUDA(cudaMemcpy(a.tw32, t32.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
  return OPAW_OK;
}

int fft3_init(FFT3 &f, int nx, int ny, int nz) {
  f.n[0] = nx;
  f.n[1] = ny;
  f.n[2] = nz;
  OPAW_CHECK(plan_axis(f.ax[0], nx));
  OPAW_CHECK(plan_axis(f.ax[1], ny));
  OPAW_CHECK(plan_axis(f.ax[2], nz));
  return OPAW_OK;
}

void fft3_free(FFT3 &f) {
  for (int i = 0; i < 3; i++) {
    cudaFree(f.ax[i].tw64);
    cudaFree(f.ax[i].tw32);
    f.ax[i].tw64 = nullptr;
    f.ax[i].tw32 = nullptr;
  }
}

template <typename R>
int fft3d(opaw_ctx *c, const FFT3 &f, typename Tr<R>::C *data, int batch, int sign) {
  typedef typename Tr<R>::C C;
  Dims3 d{f.n[0], f.n[1], f.n[2]};
  OpCopy<C> op{data, data, (int64_t)d.n0 * d.n1 * d.n2};
  int st;
  if (sign < 0 && launch_xy_if<C>(c, f, batch, sign, op, &st)) {
    OPAW_CHECK(st);
    OPAW_CHECK((launch_axis<C, 2>(c, f.ax[2], d, batch, sign, op)));
    return OPAW_OK;
  }
  if (sign > 0) {
    OPAW_CHECK((launch_axis<C, 2>(c, f.ax[2], d, batch, sign, op)));
    if (launch_xy_if<C>(c, f, batch, sign, op, &st)) return st;
    OPAW_CHECK((launch_axis<C, 1>(c, f.ax[1], d, batch, sign, op)));
    OPAW_CHECK((launch_axis<C, 0>(c, f.ax[0], d, batch, sign, op)));
    return OPAW_OK;
  }
  OPAW_CHECK((launch_axis<C, 0>(c, f.ax[0], d, batch, sign, op)));
  OPAW_CHECK((launch_axis<C, 1>(c, f.ax[1], d, batch, sign, op)));
  OPAW_CHECK((launch_axis<C, 2>(c, f.ax[2], d, batch, sign, op)));
  return OPAW_OK;
}

template int fft3d<float>(opaw_ctx *, const FFT3 &, float2 *, int, int);
template int fft3d<double>(opaw_ctx *, const FFT3 &, double2 *, int, int);

}  // namespace opaw

// tma.cu — tensor maps for the Tensor Memory Accelerator (cp.async.bulk.tensor)
// loads of the FFT passes, encoded through the runtime's driver entry-point
// query so that the library does not link libcuda itself.
#include <cudaTypedefs.h>

#include <mutex>

#include "common.cuh"

namespace opaw {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  if (!fn) {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess && f)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
  }
  return fn;
}

// A batch of arrays of nlines x nz 8-byte elements (lines fastest, batch
// stride bstride elements) as a 3D tensor map with boxes of box_lines lines x
// box_z planes x 1 array, no swizzle, zero fill outside.  Returns OPAW_OK, or
// OPAW_ERR_ARG when the layout breaks a TMA rule (16-byte aligned base, strides
// and inner box extent multiples of 16 bytes, box extents <= 256).
int tma_map_lines(CUtensorMap *m, const void *base, uint64_t nlines, uint64_t nz, uint64_t batch, uint64_t bstride,
                  uint32_t box_lines, uint32_t box_z) {
  if (((uintptr_t)base & 15) || (nlines * 8) % 16 || (bstride * 8) % 16 || (box_lines * 8) % 16 || box_lines > 256 ||
      box_z > 256 || box_lines == 0 || box_z == 0) {
    set_error("TMA layout rule not met");
    return OPAW_ERR_ARG;
  }
  auto fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available");
    return OPAW_ERR_CUDA;
  }
  const cuuint64_t dims[3] = {nlines, nz, batch};
  const cuuint64_t strides[2] = {nlines * 8, bstride * 8};
  const cuuint32_t box[3] = {box_lines, box_z, 1};
  const cuuint32_t es[3] = {1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void *>(base), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return OPAW_ERR_CUDA;
  }
  return OPAW_OK;
}

int tma_status(opaw_ctx *c) {
  int h = 0;
  OPAW_CUDA(cudaMemcpy(&h, c->d_tma_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    OPAW_CUDA(cudaMemset(c->d_tma_err, 0, sizeof(int)));
    set_error("a TMA-staged FFT pass did not see its tile arrive (barrier wait ran out)");
    return OPAW_ERR_CUDA;
  }
  return OPAW_OK;
}

}  // namespace opaw

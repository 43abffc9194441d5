// Host-side TMA descriptor encoding through the driver entry point of
// cuTensorMapEncodeTiled (no link-time dependency on libcuda).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <mutex>

#include "tc_common.cuh"

namespace numc_k {

namespace {
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_once;
}  // namespace

cudaError_t make_tmap_2d(CUtensorMap *m, const void *base, CUtensorMapDataType dtype,
                         int elem_bytes, uint64_t rows, uint64_t cols, uint64_t pitch_elems,
                         uint32_t box_rows, uint32_t box_cols) {
  std::call_once(g_once, [] {
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  });
  if (!g_encode) return cudaErrorNotSupported;
  // TMA requires a 16-byte aligned base and 16-byte multiple pitch.
  if (((uintptr_t)base & 15) || ((pitch_elems * elem_bytes) & 15)) return cudaErrorInvalidValue;
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {pitch_elems * (cuuint64_t)elem_bytes};
  cuuint32_t box[2] = {box_cols, box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(m, dtype, 2, const_cast<void *>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace numc_k

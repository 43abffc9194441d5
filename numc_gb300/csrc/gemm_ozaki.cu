// float64 Ozaki-scheme GEMM (placeholder until the kernel lands).
#include "kernels.h"

namespace numc_k {
size_t ozaki_workspace(int64_t, int64_t, int64_t, int) { return 0; }
cudaError_t launch_ozaki(const Gemm &, int, void *, size_t, cudaStream_t) {
  return cudaErrorNotSupported;
}
}  // namespace numc_k

// Optional per-phase timing of multi-kernel GEMMs with CUDA events recorded
// on the launching stream: phase 0 = operand preparation (split/slice
// passes), phase 1 = the tensor-core GEMM kernel.  Off unless enabled with
// numc_cuda_phase_timing(1); must stay off during CUDA graph capture.
#pragma once

#include <cuda_runtime.h>

namespace numc_k {

bool phase_timing_on();
// Records the start of a call; split_done()/gemm_done() record phase ends.
class PhaseMark {
 public:
  explicit PhaseMark(cudaStream_t s);
  void split_done();
  void gemm_done();

 private:
  cudaStream_t s_;
  int slot_;
};

}  // namespace numc_k

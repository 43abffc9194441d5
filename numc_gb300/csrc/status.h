// Per-device status word written by kernels that abandon a bounded wait.
#pragma once

#include <cstdint>

namespace numc_k {

// Device address of the current device's status word (allocated on first
// use), or nullptr if it could not be allocated.
unsigned *status_word();

// Codes written to the status word (first writer wins).
enum StatusCode : unsigned {
  kStatusOk = 0,
  kStatusTimeoutProducer = 1,  // TMA producer waited too long for a free slot
  kStatusTimeoutMma = 2,       // MMA issuer waited too long for a full slot
  kStatusTimeoutEpilogue = 3,  // epilogue waited too long for the accumulator
  kStatusTimeoutDrain = 4,     // issued MMAs did not complete before TMEM release
};

// How long a bounded wait spins before it gives up, and whether the TMA
// producers of the tensor-core kernels issue their loads.  Defaults: 2 s,
// loads on.  numc_cuda_debug_wait_timeout changes both for tests of the
// give-up path: with loads off no barrier ever completes, every wait runs
// out after the limit, and no TMA copy or MMA is in flight when the kernel
// leaves.
struct WaitCfg {
  unsigned long long limit_ns;
  int starve;
};
WaitCfg wait_cfg();

// The allocation-free split GEMM's own status word (used when its caller
// passes none): read and cleared into *status, 0 if that entry point has
// not run on the current device with a NULL status.
int static_status_read_and_clear(unsigned *status, void *stream);

}  // namespace numc_k

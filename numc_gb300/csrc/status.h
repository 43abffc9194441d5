// Per-device status word written by kernels that abandon a bounded wait.
#pragma once

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
};

}  // namespace numc_k

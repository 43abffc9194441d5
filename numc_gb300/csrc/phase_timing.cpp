// Event pool behind numc_cuda_phase_timing / numc_cuda_phase_times.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "numc/cuda.h"
#include "numc/error.h"
#include "phase_timing.h"

namespace numc_k {

namespace {
std::atomic<bool> g_on{false};
std::mutex g_mu;
struct Rec {
  cudaEvent_t ev[3];
  int n;   // events recorded (3 when complete)
};
std::vector<Rec> g_recs;
size_t g_used = 0;
}  // namespace

bool phase_timing_on() { return g_on.load(std::memory_order_relaxed); }

PhaseMark::PhaseMark(cudaStream_t s) : s_(s), slot_(-1) {
  if (!phase_timing_on()) return;
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_used == g_recs.size()) {
    Rec r;
    for (auto &e : r.ev)
      if (cudaEventCreate(&e) != cudaSuccess) return;
    r.n = 0;
    g_recs.push_back(r);
  }
  slot_ = (int)g_used++;
  g_recs[slot_].n = 0;
  if (cudaEventRecord(g_recs[slot_].ev[0], s_) == cudaSuccess) g_recs[slot_].n = 1;
}

void PhaseMark::split_done() {
  if (slot_ < 0) return;
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_recs[slot_].n == 1 && cudaEventRecord(g_recs[slot_].ev[1], s_) == cudaSuccess)
    g_recs[slot_].n = 2;
}

void PhaseMark::gemm_done() {
  if (slot_ < 0) return;
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_recs[slot_].n == 2 && cudaEventRecord(g_recs[slot_].ev[2], s_) == cudaSuccess)
    g_recs[slot_].n = 3;
}

}  // namespace numc_k

extern "C" int numc_cuda_phase_timing(int enable) {
  std::lock_guard<std::mutex> lock(numc_k::g_mu);
  numc_k::g_used = 0;
  numc_k::g_on = enable != 0;
  return 0;
}

extern "C" int numc_cuda_phase_times(double *prep_ms, double *gemm_ms, uint64_t *calls) {
  std::lock_guard<std::mutex> lock(numc_k::g_mu);
  double p = 0, g = 0;
  uint64_t n = 0;
  for (size_t i = 0; i < numc_k::g_used; i++) {
    auto &r = numc_k::g_recs[i];
    if (r.n != 3) continue;
    float a = 0, b = 0;
    if (cudaEventSynchronize(r.ev[2]) != cudaSuccess ||
        cudaEventElapsedTime(&a, r.ev[0], r.ev[1]) != cudaSuccess ||
        cudaEventElapsedTime(&b, r.ev[1], r.ev[2]) != cudaSuccess)
      return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "phase timing events failed");
    p += a;
    g += b;
    n++;
  }
  if (prep_ms) *prep_ms = p;
  if (gemm_ms) *gemm_ms = g;
  if (calls) *calls = n;
  return 0;
}

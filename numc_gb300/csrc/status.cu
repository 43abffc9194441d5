// Device status word and launch counter shared by all kernels.
//
// Kernels that spin on an mbarrier give up after a bounded time, record a
// nonzero code in a per-device status word and return, so that a broken
// pipeline surfaces as NUMC_ERR_INTERNAL instead of a hung GPU.
#include <cuda_runtime.h>
#include <atomic>
#include <mutex>

#include "kernels.h"
#include "status.h"

namespace numc_k {

namespace {
std::atomic<uint64_t> g_launches{0};
std::atomic<unsigned long long> g_wait_limit_ns{2000000000ull};
std::atomic<int> g_wait_starve{0};
std::atomic<int> g_fail_mallocs{0};
std::mutex g_status_mu;
unsigned *g_status_dev[64] = {nullptr};
}  // namespace

void count_launch(unsigned n) { g_launches.fetch_add(n); }

WaitCfg wait_cfg() { return WaitCfg{g_wait_limit_ns.load(), g_wait_starve.load()}; }

cudaError_t dev_malloc(void **p, size_t bytes) {
  // numc_cuda_debug_fail_malloc: fail the next n allocations as the device
  // would when out of memory.
  int n = g_fail_mallocs.load();
  while (n > 0) {
    if (g_fail_mallocs.compare_exchange_weak(n, n - 1)) {
      *p = nullptr;
      return cudaErrorMemoryAllocation;
    }
  }
  return cudaMalloc(p, bytes);
}
uint64_t launches() { return g_launches.load(); }

unsigned *status_word() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_status_mu);
  if (!g_status_dev[dev]) {
    unsigned *p = nullptr;
    if (dev_malloc((void **)&p, sizeof(unsigned)) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, sizeof(unsigned)) != cudaSuccess) {
      cudaFree(p);
      return nullptr;
    }
    g_status_dev[dev] = p;
  }
  return g_status_dev[dev];
}

cudaError_t read_and_clear_status(unsigned *status, cudaStream_t s) {
  *status = 0;
  unsigned *p = status_word();
  if (!p) return cudaErrorMemoryAllocation;
  cudaError_t e = cudaMemcpyAsync(status, p, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, sizeof(unsigned), s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

}  // namespace numc_k

extern "C" int numc_cuda_debug_wait_timeout(unsigned long long limit_ns, int starve) {
  numc_k::g_wait_limit_ns = limit_ns ? limit_ns : 2000000000ull;
  numc_k::g_wait_starve = limit_ns ? (starve != 0) : 0;
  return 0;
}

extern "C" int numc_cuda_debug_fail_malloc(int count) {
  numc_k::g_fail_mallocs = count > 0 ? count : 0;
  return 0;
}

// CUDA-core GEMM for all ten numc dtypes: the single-problem launcher of
// the tile in simt_common.cuh (arithmetic per dtype documented there).
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>

#include "kernels.h"
#include "simt_common.cuh"

namespace numc_k {
namespace {

using simt::kThreads;

// Two CTAs per SM (at most 128 registers) except for the int8/uint8 kernel,
// whose per-block store rule keeps 64 partial sums and 64 stored bytes per
// thread.
template <typename T, int BM, int BN, int BK, int TM, int TN, int KIND>
__global__ void __launch_bounds__(kThreads, KIND == simt::kByte ? 1 : 2)
simt_gemm(Gemm g, int rule8) {
  simt::simt_tile<T, BM, BN, BK, TM, TN, KIND>(g, rule8, (int64_t)blockIdx.y * BM,
                                               (int64_t)blockIdx.x * BN);
}

// 16 remainder groups (one a half-warp) per 256-thread block.
template <typename T>
__global__ void __launch_bounds__(256) float_edges(Gemm g, int64_t r0, int64_t c0, int64_t n) {
  for (int64_t g0 = (int64_t)blockIdx.x * 16; g0 < n; g0 += (int64_t)gridDim.x * 16) {
    const int64_t gi = g0 + threadIdx.x / 16;
    if (gi < n) simt::float_edge_output<T>(g, gi, threadIdx.x % 16, r0, c0);
  }
}

// kEdgeLanes lanes per remainder output, 32 outputs per 256-thread block;
// the loop bound is uniform over the block, so every warp reaches the
// fold's shuffles together.
template <typename T>
__global__ void __launch_bounds__(256) float_edges_lanes(Gemm g, int64_t r0, int64_t c0,
                                                         int64_t n) {
  constexpr int64_t per_block = 256 / simt::kEdgeLanes;
  for (int64_t e0 = (int64_t)blockIdx.x * per_block; e0 < n; e0 += (int64_t)gridDim.x * per_block) {
    const int64_t e = e0 + threadIdx.x / simt::kEdgeLanes;
    simt::float_edge_output_lanes<T>(g, e, e < n, r0, c0);
  }
}

// numc's packed-path remainder tiles of g, after the GEMM kernel.  With 4 or
// more K blocks an output, 8 lanes share each output's blocks (a single
// problem has few remainder outputs, each a long chain); with fewer, one
// lane an output in column groups (coalesced).  Measured: 2048^3 (4096
// remainder outputs, 8 blocks each) one lane an output 357 us, 8 lanes
// 39 us; 2048 grouped problems with K <= 1024 (plain float32 plan) 9.1 ms
// with 8 lanes, 4.5 ms with one.
template <typename T>
cudaError_t launch_float_edges(const Gemm &g, cudaStream_t s) {
  if (!simt::float_edges_needed<T>(g.K)) return cudaSuccess;
  const int64_t r0 = simt::edge_row<T>(g.M, g.isa), c0 = simt::edge_col<T>(g.N, g.isa);
  // K blocks on separate lanes when there are enough of them, or when the
  // outputs are too few to fill the GPU one lane each (the chains are then
  // the whole latency)
  const int64_t nkb = (g.K + simt::kNumcKC - 1) / simt::kNumcKC;
  if (nkb >= 4 || simt::float_edge_count<T>(g.M, g.N, g.isa) <= 152 * 128) {
    const int64_t n = simt::float_edge_count<T>(g.M, g.N, g.isa);
    if (n == 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((n + 31) / 32, 152 * 16);
    float_edges_lanes<T><<<(unsigned)blocks, 256, 0, s>>>(g, r0, c0, n);
  } else {
    const int64_t n = simt::float_edge_groups<T>(g.M, g.N, g.isa);
    if (n == 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((n + 15) / 16, 152 * 16);
    float_edges<T><<<(unsigned)blocks, 256, 0, s>>>(g, r0, c0, n);
  }
  count_launch();
  return cudaGetLastError();
}

template <typename T, int BM, int BN, int TM, int TN, int KIND, int BK = 8>
cudaError_t launch_tile(const Gemm &g, int rule8, cudaStream_t s) {
  if (g.M == 0 || g.N == 0) return cudaSuccess;
  int64_t gx = (g.N + BN - 1) / BN, gy = (g.M + BM - 1) / BM;
  if (gy > 65535 || gx > 0x7FFFFFFF) return cudaErrorInvalidConfiguration;
  simt_gemm<T, BM, BN, BK, TM, TN, KIND><<<dim3((unsigned)gx, (unsigned)gy), kThreads, 0, s>>>(g, rule8);
  count_launch();
  return cudaGetLastError();
}

// SMs of the current device (cached per device).
int sms() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (!cache[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
    cache[dev] = n;
  }
  return cache[dev];
}

// Square tile for a problem: the largest of `big`, big/2, ... 32 whose grid
// still gives every SM a CTA (a 512 x 512 output is 16 tiles of 128 but 256
// of 32).  Each output's arithmetic does not depend on the tile.
template <typename T, int KIND, int BIG>
cudaError_t launch_sized(const Gemm &g, int rule8, cudaStream_t s) {
  int t = BIG;
  while (t > 32 && ((g.M + t - 1) / t) * ((g.N + t - 1) / t) < sms()) t /= 2;
  if constexpr (BIG >= 128)
    if (t == 128) return launch_tile<T, 128, 128, 8, 8, KIND>(g, rule8, s);
  if (t >= 64) return launch_tile<T, 64, 64, 4, 4, KIND>(g, rule8, s);
  return launch_tile<T, 32, 32, 2, 2, KIND, 32>(g, rule8, s);
}

// numc's packed float path: 64- and 32-wide tiles sum the remainder-tile
// outputs per K block in the tile kernel (kFloatEdges); 128-wide tiles
// (8 x 8 outputs a thread, no registers to spare) leave them to the
// float_edges pass.
template <typename T, int BIG>
cudaError_t launch_float_packed(const Gemm &g, cudaStream_t s) {
  int t = BIG;
  while (t > 32 && ((g.M + t - 1) / t) * ((g.N + t - 1) / t) < sms()) t /= 2;
  cudaError_t e;
  if constexpr (BIG >= 128) {
    if (t == 128) {
      e = launch_tile<T, 128, 128, 8, 8, simt::kFloat>(g, 0, s);
      return e != cudaSuccess || g.K == 0 ? e : launch_float_edges<T>(g, s);
    }
  }
  if (t >= 64) return launch_tile<T, 64, 64, 4, 4, simt::kFloatEdges>(g, 0, s);
  return launch_tile<T, 32, 32, 2, 2, simt::kFloatEdges, 32>(g, 0, s);
}

}  // namespace

int float_rule(NumcDType dt, const Gemm &g, int rule) {
  const int kind = rule & kFloatKindMask;
  if (kind != kFloatNumc) return rule;
  // numc_matmul's gemmsup threshold (src/matmul/matmul.c:241-256; the same
  // table on every ISA)
  const double thr = dt == NUMC_DTYPE_FLOAT32 ? 96.0 * 96 * 96 : 48.0 * 48 * 48;
  return (rule & ~kFloatKindMask) |
         ((double)g.M * g.K * g.N > thr ? kFloatNumcPacked : kFloatNumcSmall);
}

cudaError_t launch_simt(NumcDType dt, const Gemm &g_in, int rule8, cudaStream_t s) {
  Gemm g = g_in;
  if (dt == NUMC_DTYPE_FLOAT32 || dt == NUMC_DTYPE_FLOAT64) {
    // the float variant's ISA bit selects numc's tile geometry
    g.isa = (rule8 & kFloatIsaNeon) ? kIsaNeon : kIsaX86;
    rule8 = float_rule(dt, g, rule8) & kFloatKindMask;
  }
  switch (dt) {
  case NUMC_DTYPE_FLOAT32:
    switch (rule8) {
    case kFloatNaive: return launch_sized<float, simt::kFloatUnfused, 128>(g, 0, s);
    case kFloatNumcSmall: return launch_sized<float, simt::kFloatSmall, 128>(g, 0, s);
    default: return launch_float_packed<float, 128>(g, s);
    }
  case NUMC_DTYPE_FLOAT64:
    switch (rule8) {
    case kFloatNaive: return launch_sized<double, simt::kFloatUnfused, 64>(g, 0, s);
    case kFloatNumcSmall: return launch_sized<double, simt::kFloatSmall, 64>(g, 0, s);
    default: return launch_float_packed<double, 64>(g, s);
    }
  case NUMC_DTYPE_INT16: return launch_sized<int16_t, simt::kWrapInt, 128>(g, 0, s);
  case NUMC_DTYPE_UINT16: return launch_sized<uint16_t, simt::kWrapInt, 128>(g, 0, s);
  case NUMC_DTYPE_INT32: return launch_sized<int32_t, simt::kWrapInt, 128>(g, 0, s);
  case NUMC_DTYPE_UINT32: return launch_sized<uint32_t, simt::kWrapInt, 128>(g, 0, s);
  case NUMC_DTYPE_INT64: return launch_sized<int64_t, simt::kWrapInt, 64>(g, 0, s);
  case NUMC_DTYPE_UINT64: return launch_sized<uint64_t, simt::kWrapInt, 64>(g, 0, s);
  case NUMC_DTYPE_INT8: return launch_tile<int8_t, 128, 128, 8, 8, simt::kByte>(g, rule8, s);
  case NUMC_DTYPE_UINT8: return launch_tile<uint8_t, 128, 128, 8, 8, simt::kByte>(g, rule8, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace numc_k

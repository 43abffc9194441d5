// Splitting float32 operands into bfloat16 planes (shared by the single and
// grouped split-BF16 GEMMs).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace numc_k {

// ---- pass 1: split float32 into bf16 planes -------------------------------
//
// dst_p(row, k) for row < R, k < Kp: plane p of src[row * rs_row + k * rs_k]
// (zero for k >= K).  Plane p starts at planes + p * R * Kp.  A 32-row x
// 128-k tile per block goes through shared memory; reads are float4 along
// whichever source dimension is contiguous (scalar otherwise), writes are 4
// bf16 (8 bytes) per thread per plane along k.
//
// Non-finite inputs cannot go through the split (inf * x1 with x1 = 0 gives
// NaN where the true product is infinite), so the block records them: the
// flag word of the row group (row / flag_rows, flag_rows a multiple of 32)
// is set to `gen`, the call's generation number, and the GEMM recomputes
// the affected output tiles with plain FMA chains.  Stale flags from
// earlier calls hold other numbers, so the flags never need clearing.
constexpr int kSplitRows = 32, kSplitK = 128;

// One 32-row x 128-k tile at (r0, k0), executed by a 256-thread block;
// `tile` is the block's shared staging buffer.
template <int PLANES>
__device__ __forceinline__ void split_tile(const float *__restrict__ src, int64_t rs_row,
                                           int64_t rs_k, int64_t R, int64_t K, int64_t Kp,
                                           __nv_bfloat16 *__restrict__ planes,
                                           unsigned long long *flags, int flag_rows,
                                           unsigned long long gen, int mode, int64_t r0,
                                           int64_t k0, float (*tile)[kSplitK + 4]) {
  const int tid = threadIdx.x;
  bool bad = false;
  if (mode == 1) {            // k contiguous, 16-byte aligned rows
#pragma unroll
    for (int q = 0; q < 4; q++) {
      int e = tid + 256 * q, r = e / 32, k4 = (e % 32) * 4;
      int64_t gr = r0 + r, gk = k0 + k4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gr < R) {
        const float *p = src + gr * rs_row + gk;
        if (gk + 3 < K) v = *reinterpret_cast<const float4 *>(p);
        else {
          if (gk < K) v.x = p[0];
          if (gk + 1 < K) v.y = p[1];
          if (gk + 2 < K) v.z = p[2];
        }
      }
      bad |= !isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z) || !isfinite(v.w);
      *reinterpret_cast<float4 *>(&tile[r][k4]) = v;
    }
  } else if (mode == 2) {     // rows contiguous, 16-byte aligned columns
#pragma unroll
    for (int q = 0; q < 4; q++) {
      int e = tid + 256 * q, rq = (e % 8) * 4, k = e / 8;
      int64_t gr = r0 + rq, gk = k0 + k;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gk < K) {
        const float *p = src + gr + gk * rs_k;
        if (gr + 3 < R) v = *reinterpret_cast<const float4 *>(p);
        else {
          if (gr < R) v.x = p[0];
          if (gr + 1 < R) v.y = p[1];
          if (gr + 2 < R) v.z = p[2];
        }
      }
      bad |= !isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z) || !isfinite(v.w);
      tile[rq][k] = v.x;
      tile[rq + 1][k] = v.y;
      tile[rq + 2][k] = v.z;
      tile[rq + 3][k] = v.w;
    }
  } else {                    // general strides
    const bool kfast = rs_k == 1 || rs_row != 1;
#pragma unroll 4
    for (int q = 0; q < 16; q++) {
      int e = tid + 256 * q;
      int r = kfast ? e / kSplitK : e % kSplitRows;
      int k = kfast ? e % kSplitK : e / kSplitRows;
      int64_t gr = r0 + r, gk = k0 + k;
      float x = (gr < R && gk < K) ? src[gr * rs_row + gk * rs_k] : 0.0f;
      bad |= !isfinite(x);
      tile[r][k] = x;
    }
  }
  if (__syncthreads_or(bad) && tid == 0) flags[r0 / flag_rows] = gen;

  const int warp = tid >> 5, lane = tid & 31;
  const int64_t plane_elems = R * Kp;
#pragma unroll
  for (int rr = 0; rr < kSplitRows / 8; rr++) {
    const int r = warp + 8 * rr;
    const int64_t gr = r0 + r, gk = k0 + 4 * lane;
    if (gr >= R || gk >= Kp) continue;
    const float4 v = *reinterpret_cast<const float4 *>(&tile[r][4 * lane]);
    float rem[4] = {v.x, v.y, v.z, v.w};
    __nv_bfloat16 out[PLANES][4];
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const bool finite = isfinite(rem[t]);
#pragma unroll
      for (int p = 0; p < PLANES; p++) {
        __nv_bfloat16 h = __float2bfloat16_rn(rem[t]);
        float hf = __bfloat162float(h);
        if (isinf(hf) && finite) {       // rounding overflowed: truncate
          h = __float2bfloat16_rz(rem[t]);
          hf = __bfloat162float(h);
        }
        out[p][t] = (p == 0 || finite) ? h : __float2bfloat16_rn(0.0f);
        rem[t] = finite ? rem[t] - hf : 0.0f;
      }
    }
    const int64_t off = gr * Kp + gk;
#pragma unroll
    for (int p = 0; p < PLANES; p++) {
      uint2 w;
      w.x = (uint32_t)__bfloat16_as_ushort(out[p][0]) | ((uint32_t)__bfloat16_as_ushort(out[p][1]) << 16);
      w.y = (uint32_t)__bfloat16_as_ushort(out[p][2]) | ((uint32_t)__bfloat16_as_ushort(out[p][3]) << 16);
      *reinterpret_cast<uint2 *>(planes + p * plane_elems + off) = w;
    }
  }
}

// Read mode of a split source: 1 = k contiguous (float4 along k), 2 = rows
// contiguous (float4 along rows), 0 = general strides.
inline int split_mode(const float *p, int64_t rs_row, int64_t rs_k) {
  if ((uintptr_t)p % 16) return 0;
  if (rs_k == 1 && rs_row % 4 == 0) return 1;
  if (rs_row == 1 && rs_k % 4 == 0) return 2;
  return 0;
}

}  // namespace numc_k

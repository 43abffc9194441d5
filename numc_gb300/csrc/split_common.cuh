// Splitting float32 operands into 16-bit planes (shared by the single and
// grouped split GEMMs).
//
// Two plane formats:
//  * bfloat16 (8 significant bits, float32's exponent range): x is cut by
//    repeated rounding, x0 = bf16(x), x1 = bf16(x - x0), ...
//  * scaled float16 (11 significant bits, exponents -24..15): each row of A
//    and each column of B is first multiplied by a power of two 2^s that
//    puts its largest magnitude in [2^14, 2^15), then cut the same way,
//    h0 = f16(x 2^s), h1 = f16(x 2^s - h0).  h0 + h1 holds 22 bits of x;
//    the GEMM multiplies the float32 sum by 2^-(s_row + s_col).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace numc_k {

// Scale exponent of a row whose largest magnitude has float32 bits
// `maxbits`: s with max * 2^s in [2^14, 2^15), or 0 for an all-zero or
// non-finite row (a non-finite row is recomputed by the fallback anyway).
// 2^e as a double, exactly, for |e| <= 1022.
__device__ __forceinline__ double exp2_dbl(int e) {
  return __longlong_as_double((long long)(e + 1023) << 52);
}

__host__ __device__ inline int f16_scale_exp(unsigned maxbits) {
  if (maxbits == 0 || maxbits >= 0x7f800000u) return 0;
  int e;   // floor(log2(max))
  if (maxbits >> 23) {
    e = (int)(maxbits >> 23) - 127;
  } else {   // subnormal: position of the leading bit
    int lead = 31;
    while (!((maxbits >> lead) & 1u)) lead--;
    e = lead - 149;
  }
  return 14 - e;   // in [-113, 163]
}

// 2^e as a float32 for e in [-126, 127].
__host__ __device__ inline float exp2_int(int e) {
  union { unsigned u; float f; } v;
  v.u = (unsigned)(e + 127) << 23;
  return v.f;
}

// x * 2^s exactly for |x * 2^s| < 2^15 (s in [-113, 163]; two steps keep
// each factor a normal float32).
__device__ __forceinline__ float scale_pow2(float x, int s) {
  const int s1 = s > 126 ? 126 : s;
  return (x * exp2_int(s1)) * exp2_int(s - s1);
}

// Largest magnitude of each row r < R of src[r * rs_row + k * rs_k] over
// k < K, as float32 bits, merged into maxbits[r] with atomicMax (maxbits
// starts at zero).  A 256-thread block covers
//   mode 1 (k contiguous):    8 rows x 1024 k, one warp per row;
//   mode 3 (k contiguous, rows not 16-byte aligned): the same, scalar loads;
//   mode 2 (rows contiguous): 1024 rows x 64 k, 4 rows per thread;
//   mode 0 (general):         256 rows x 64 k, one row per thread.
constexpr int kMaxRows1 = 8, kMaxK1 = 1024, kMaxRows2 = 1024, kMaxK2 = 64, kMaxRows0 = 256,
              kMaxK0 = 64;

__device__ __forceinline__ unsigned absbits(float x) { return __float_as_uint(x) & 0x7fffffffu; }

// K extent of a block in read mode 2 (rows contiguous, 1024 rows a block):
// 64 on large operands; on small ones halved down to 8 until the grid has
// about four blocks per SM, so the pass is not a few long load chains.
__host__ __device__ inline int64_t absmax_k2(int64_t R, int64_t K) {
  int64_t kk = kMaxK2;
  while (kk > 8 && ((K + kk - 1) / kk) * ((R + kMaxRows2 - 1) / kMaxRows2) < 608) kk /= 2;
  return kk;
}

// Block (bk, br) of the grid below, executed by a 256-thread block.
__device__ __forceinline__ void absmax_block(const float *__restrict__ src, int64_t rs_row,
                                             int64_t rs_k, int64_t R, int64_t K, int mode,
                                             unsigned *__restrict__ maxbits, int64_t bk,
                                             int64_t br) {
  const int tid = threadIdx.x;
  if (mode == 3) {
    const int64_t r = br * kMaxRows1 + (tid >> 5);
    const int64_t k0 = bk * kMaxK1;
    const int lane = tid & 31;
    unsigned m = 0;
    if (r < R) {
      const float *row = src + r * rs_row;
      const int64_t k1 = k0 + kMaxK1 < K ? k0 + kMaxK1 : K;
#pragma unroll 4
      for (int64_t k = k0 + lane; k < k1; k += 32) m = max(m, absbits(row[k]));
    }
    m = __reduce_max_sync(0xffffffffu, m);
    if (lane == 0 && r < R && m) atomicMax(&maxbits[r], m);
  } else if (mode == 1) {
    const int64_t r = br * kMaxRows1 + (tid >> 5);
    const int64_t k0 = bk * kMaxK1;
    const int lane = tid & 31;
    unsigned m = 0;
    if (r < R) {
      const float *row = src + r * rs_row;
#pragma unroll
      for (int q = 0; q < kMaxK1 / 128; q++) {
        const int64_t k = k0 + 128 * q + 4 * lane;
        if (k + 3 < K) {
          const float4 v = *reinterpret_cast<const float4 *>(row + k);
          m = max(max(m, absbits(v.x)), max(absbits(v.y), max(absbits(v.z), absbits(v.w))));
        } else {
          for (int t = 0; t < 4; t++)
            if (k + t < K) m = max(m, absbits(row[k + t]));
        }
      }
    }
    m = __reduce_max_sync(0xffffffffu, m);
    if (lane == 0 && r < R && m) atomicMax(&maxbits[r], m);
  } else if (mode == 2) {
    const int64_t r = br * kMaxRows2 + 4 * tid;
    const int64_t kk = absmax_k2(R, K);
    const int64_t k0 = bk * kk;
    unsigned m[4] = {0, 0, 0, 0};
    if (r < R) {
      const int n = (int)((k0 + kk < K ? k0 + kk : K) - k0);
      const float *p = src + r + k0 * rs_k;
      if (r + 3 < R) {
        // 8 independent 16-byte loads in flight a thread
#pragma unroll 8
        for (int k = 0; k < n; k++, p += rs_k) {
          const float4 v = *reinterpret_cast<const float4 *>(p);
          m[0] = max(m[0], absbits(v.x));
          m[1] = max(m[1], absbits(v.y));
          m[2] = max(m[2], absbits(v.z));
          m[3] = max(m[3], absbits(v.w));
        }
      } else {
        for (int k = 0; k < n; k++, p += rs_k)
          for (int t = 0; t < 4; t++)
            if (r + t < R) m[t] = max(m[t], absbits(p[t]));
      }
    }
    for (int t = 0; t < 4; t++)
      if (r + t < R && m[t]) atomicMax(&maxbits[r + t], m[t]);
  } else {
    const int64_t r = br * kMaxRows0 + tid;
    const int64_t k0 = bk * kMaxK0;
    unsigned m = 0;
    if (r < R) {
      const int64_t k1 = k0 + kMaxK0 < K ? k0 + kMaxK0 : K;
      const float *p = src + r * rs_row + k0 * rs_k;
#pragma unroll 8
      for (int64_t k = k0; k < k1; k++, p += rs_k) m = max(m, absbits(*p));
    }
    if (r < R && m) atomicMax(&maxbits[r], m);
  }
}

static __global__ void __launch_bounds__(256)
absmax_rows_f32(const float *__restrict__ src, int64_t rs_row, int64_t rs_k, int64_t R,
                int64_t K, int mode, unsigned *__restrict__ maxbits) {
  absmax_block(src, rs_row, rs_k, R, K, mode, maxbits, blockIdx.x, blockIdx.y);
}

// Grid of absmax_rows_f32 for R rows, K columns, read mode `mode`.
__host__ __device__ inline dim3 absmax_grid(int64_t R, int64_t K, int mode) {
  const bool rowwise = mode == 1 || mode == 3;
  const int64_t kk = rowwise ? kMaxK1 : mode == 2 ? absmax_k2(R, K) : kMaxK0;
  const int64_t rr = rowwise ? kMaxRows1 : mode == 2 ? kMaxRows2 : kMaxRows0;
  return dim3((unsigned)((K + kk - 1) / kk), (unsigned)((R + rr - 1) / rr));
}

// ---- pass 1: split float32 into 16-bit planes -----------------------------
//
// dst_p(row, k) for row < R, k < Kp: plane p of src[row * rs_row + k * rs_k]
// (zero for k >= K); bfloat16 planes, or with F16 scaled float16 planes
// whose row scale comes from maxbits[row].  Plane p starts at planes + p * R * Kp.  A 32-row x
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
// MODE >= 0 fixes the read mode at compile time (one read path per kernel,
// fewer registers); -1 takes `mode` at run time (grouped passes).
template <int PLANES, bool F16 = false, int MODE = -1>
__device__ __forceinline__ void split_tile(const float *__restrict__ src, int64_t rs_row,
                                           int64_t rs_k, int64_t R, int64_t K, int64_t Kp,
                                           void *__restrict__ planes_v,
                                           unsigned long long *flags, int flag_rows,
                                           unsigned long long gen, int mode, int64_t r0,
                                           int64_t k0, float (*tile)[kSplitK + 4],
                                           const unsigned *maxbits = nullptr) {
  uint16_t *planes = (uint16_t *)planes_v;
  const int tid = threadIdx.x;
  bool bad = false;
  if (MODE >= 0) mode = MODE;
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
  } else if (rs_k == 1) {     // k contiguous, rows not 16-byte aligned
    // thread: column k0 + tid % 128 of rows r0 + tid / 128 + 2q
    const int k = tid % kSplitK, rr = tid / kSplitK;
    const int64_t gk = k0 + k;
    const float *p = src + (r0 + rr) * rs_row + gk;
    float x[16];
#pragma unroll
    for (int q = 0; q < 16; q++)
      x[q] = (r0 + rr + 2 * q < R && gk < K) ? p[2 * q * rs_row] : 0.0f;
#pragma unroll
    for (int q = 0; q < 16; q++) {
      bad |= !isfinite(x[q]);
      tile[rr + 2 * q][k] = x[q];
    }
  } else if (rs_row == 1) {   // rows contiguous, k not 16-byte aligned
    // thread: row r0 + tid % 32 of k0 + tid / 32 + 8q
    const int r = tid % kSplitRows, kk = tid / kSplitRows;
    const int64_t gr = r0 + r;
    const float *p = src + gr + (k0 + kk) * rs_k;
    float x[16];
#pragma unroll
    for (int q = 0; q < 16; q++)
      x[q] = (gr < R && k0 + kk + 8 * q < K) ? p[8 * q * rs_k] : 0.0f;
#pragma unroll
    for (int q = 0; q < 16; q++) {
      bad |= !isfinite(x[q]);
      tile[r][kk + 8 * q] = x[q];
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
    uint16_t out[PLANES][4];
    if (F16) {
      const int sexp = f16_scale_exp(maxbits[gr]);
#pragma unroll
      for (int t = 0; t < 4; t++) {
        const bool finite = isfinite(rem[t]);
        float x = finite ? scale_pow2(rem[t], sexp) : 0.0f;   // |x| < 2^15
#pragma unroll
        for (int p = 0; p < PLANES; p++) {
          const __half h = __float2half_rn(x);
          out[p][t] = __half_as_ushort(h);
          x -= __half2float(h);   // exact
        }
      }
    } else {
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
          out[p][t] = __bfloat16_as_ushort((p == 0 || finite) ? h : __float2bfloat16_rn(0.0f));
          rem[t] = finite ? rem[t] - hf : 0.0f;
        }
      }
    }
    const int64_t off = gr * Kp + gk;
#pragma unroll
    for (int p = 0; p < PLANES; p++) {
      uint2 w;
      w.x = (uint32_t)out[p][0] | ((uint32_t)out[p][1] << 16);
      w.y = (uint32_t)out[p][2] | ((uint32_t)out[p][3] << 16);
      *reinterpret_cast<uint2 *>(planes + p * plane_elems + off) = w;
    }
  }
}

// Read mode of the scale pass for a source of split mode `mode`: k-contiguous
// rows that are not 16-byte aligned are read one warp per row (3), not one
// thread per row.
// ---- fused scale and split (float16 planes) ----------------------------------
//
// One 256-thread block: kFusedRows rows of one operand (A's rows, or B's
// columns as B^T's rows).  Pass 1 reads the rows for their maxima; pass 2
// reads them again (from L2: a block's rows are at most kFusedRows x K
// elements) and writes the two float16 planes — one launch and one DRAM read
// of the operand instead of the absmax and split passes.  No shared-memory
// staging, so many blocks fit on an SM and K is unbounded.  Writes
// maxbits[row] directly (no zeroing first) and, for a non-finite value,
// flags[r0 / flag_rows] = gen.  Same arithmetic as split_tile<2, true>.
// Pass 1 layout: k contiguous (rs_k == 1): 16 threads per row along k;
// otherwise 16 consecutive rows per k step, 16 k steps a pass (coalesced
// reads of B's rows; the 16 threads per row reduce through shared memory).
// Pass 2: 16 threads per row along k for both, so each row's planes are
// written in 128-byte runs (B's second read comes from L2 in 4-byte pieces).
constexpr int kFusedRows = 16;

template <bool STASH>
__device__ __forceinline__ void fused_scale_split_rows(
    const float *__restrict__ src, int64_t rs_row, int64_t rs_k, int R, int K, int Kp, int r0,
    uint16_t *__restrict__ planes, unsigned long long *flags, int flag_rows,
    unsigned *__restrict__ maxbits, unsigned long long gen) {
  constexpr int kPlanes = 2;
  __shared__ unsigned red[16][16];
  __shared__ unsigned rowmax[kFusedRows];
  const int tid = threadIdx.x;
  const bool along_k = rs_k == 1;
  const int r = along_k ? tid / 16 : tid % 16, sub = along_k ? tid % 16 : tid / 16;
  const bool live = r0 + r < R;
  const float *p = src + (int64_t)(r0 + (live ? r : 0)) * rs_row;

  // Pass 1: the row's largest magnitude (float32 bits) and non-finite values.
  unsigned m = 0;
  bool bad = false;
  // rows contiguous and 16-byte aligned: float4 loads, k = 4 sub + 64 i
  const bool vec = along_k && (rs_row & 3) == 0 && (reinterpret_cast<uintptr_t>(src) & 15) == 0;
  if (live && vec) {
    const int K4 = K & ~3;
#pragma unroll 4
    for (int k = 4 * sub; k < K4; k += 64) {
      const float4 x = *reinterpret_cast<const float4 *>(p + k);
      bad |= !isfinite(x.x) || !isfinite(x.y) || !isfinite(x.z) || !isfinite(x.w);
      m = max(m, max(max(absbits(x.x), absbits(x.y)), max(absbits(x.z), absbits(x.w))));
    }
    for (int k = K4 + sub; k < K; k += 16) {   // the last K % 4 columns
      const float x = p[k];
      bad |= !isfinite(x);
      m = max(m, absbits(x));
    }
  } else if (live) {
#pragma unroll 8
    for (int k = sub; k < K; k += 16) {
      const float x = p[(int64_t)k * rs_k];
      bad |= !isfinite(x);
      m = max(m, absbits(x));
    }
  }
  if (along_k) {
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  } else {
    m = max(m, __shfl_xor_sync(0xffffffffu, m, 16));   // lanes r and r + 16
    if ((tid & 31) < 16) red[tid >> 5][r] = m;
    __syncthreads();
    m = 0;
#pragma unroll
    for (int w = 0; w < 8; w++) m = max(m, red[w][r]);
  }
  if (sub == 0) {
    rowmax[r] = m;
    if (live) maxbits[r0 + r] = m;
  }
  if (__syncthreads_or(bad) && tid == 0) flags[r0 / flag_rows] = gen;

  // Pass 2: thread (r2, q) converts k = 4 q + 64 i .. +3 of row r2.  Rows
  // contiguous along k are read in place; otherwise (the columns of a
  // row-major B) with STASH each 64-deep chunk of the 16 rows is first read
  // with the lanes along the rows (64 contiguous bytes per k) into shared
  // memory (measured faster for one large problem: 512^3 split 18.2 ->
  // 17.8 us), without it read in place (faster for the grouped launch of
  // many small problems, whose blocks then sync less: 1.77 -> 1.70 ms).
  const int r2 = tid / 16, q = tid % 16;
  const bool live2 = r0 + r2 < R;
  const int sexp = f16_scale_exp(rowmax[r2]);
  const int64_t plane_elems = (int64_t)R * Kp;
  uint16_t *dst = planes + (int64_t)(r0 + r2) * Kp;
  auto convert_store = [&](const float (&rem)[4], int k) {
    uint16_t out[kPlanes][4];
#pragma unroll
    for (int t = 0; t < 4; t++) {
      float x = isfinite(rem[t]) ? scale_pow2(rem[t], sexp) : 0.0f;
#pragma unroll
      for (int pl = 0; pl < kPlanes; pl++) {
        const __half h = __float2half_rn(x);
        out[pl][t] = __half_as_ushort(h);
        x -= __half2float(h);
      }
    }
#pragma unroll
    for (int pl = 0; pl < kPlanes; pl++) {
      uint2 w;
      w.x = (uint32_t)out[pl][0] | ((uint32_t)out[pl][1] << 16);
      w.y = (uint32_t)out[pl][2] | ((uint32_t)out[pl][3] << 16);
      *reinterpret_cast<uint2 *>(dst + pl * plane_elems + k) = w;
    }
  };
  if (STASH && !along_k) {
    __shared__ float stash[kFusedRows][64 + 1];
    for (int k0 = 0; k0 < Kp; k0 += 64) {
      __syncthreads();   // the previous chunk's reads of the stash are done
#pragma unroll
      for (int t = 0; t < 4; t++) {
        const int kk = (tid >> 4) + 16 * t, k = k0 + kk;
        stash[r][kk] = live && k < K ? p[(int64_t)k * rs_k] : 0.0f;
      }
      __syncthreads();
      float rem[4];
#pragma unroll
      for (int t = 0; t < 4; t++) rem[t] = stash[r2][4 * q + t];
      if (live2) convert_store(rem, k0 + 4 * q);
    }
  } else if (live2) {
    const float *p2 = src + (int64_t)(r0 + r2) * rs_row;
#pragma unroll 2
    for (int k = 4 * q; k < Kp; k += 64) {
      float rem[4];
      if (vec && k + 4 <= K) {
        const float4 x = *reinterpret_cast<const float4 *>(p2 + k);
        rem[0] = x.x; rem[1] = x.y; rem[2] = x.z; rem[3] = x.w;
      } else {
#pragma unroll
        for (int t = 0; t < 4; t++) rem[t] = k + t < K ? p2[(int64_t)(k + t) * rs_k] : 0.0f;
      }
      convert_store(rem, k);
    }
  }
}

// ---- one k-contiguous row per block, held in registers -----------------------
//
// Scale and split of row `r` of an operand whose rows are contiguous along k
// and 16-byte aligned (split read mode 1), by a 256-thread block: thread t
// loads k = 4 t + 1024 i, i < V, as float4 (V * 1024 >= Kp), the block
// reduces the row's largest magnitude, and the same registers are converted
// to the two float16 planes — each float32 read from HBM once, no second
// read and no shared-memory staging.  Writes maxbits[r] directly and, for a
// non-finite value, flags[r / flag_rows] = gen.  Same arithmetic as
// split_tile<2, true> after absmax_rows_f32, so the planes are the same bits.
template <int V>
__device__ __forceinline__ void scale_split_row_regs(const float *__restrict__ src,
                                                     int64_t rs_row, int64_t R, int K, int Kp,
                                                     int64_t r, uint16_t *__restrict__ planes,
                                                     unsigned long long *flags, int flag_rows,
                                                     unsigned *__restrict__ maxbits,
                                                     unsigned long long gen) {
  __shared__ unsigned wmax[8], wbad[8];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const float *row = src + r * rs_row;
  float4 v[V];
  unsigned m = 0;
  bool bad = false;
#pragma unroll
  for (int i = 0; i < V; i++) {
    const int k = 4 * tid + 1024 * i;
    v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (k + 4 <= K) {
      v[i] = __ldcs(reinterpret_cast<const float4 *>(row + k));
    } else if (k < K) {
      v[i].x = row[k];
      if (k + 1 < K) v[i].y = row[k + 1];
      if (k + 2 < K) v[i].z = row[k + 2];
    }
  }
#pragma unroll
  for (int i = 0; i < V; i++) {
    bad |= !isfinite(v[i].x) || !isfinite(v[i].y) || !isfinite(v[i].z) || !isfinite(v[i].w);
    m = max(m, max(max(absbits(v[i].x), absbits(v[i].y)), max(absbits(v[i].z), absbits(v[i].w))));
  }
  m = __reduce_max_sync(0xffffffffu, m);
  const unsigned b = __any_sync(0xffffffffu, bad);
  if (lane == 0) {
    wmax[warp] = m;
    wbad[warp] = b;
  }
  __syncthreads();
  m = wmax[0];
  unsigned anybad = wbad[0];
#pragma unroll
  for (int w = 1; w < 8; w++) {
    m = max(m, wmax[w]);
    anybad |= wbad[w];
  }
  if (tid == 0) {
    maxbits[r] = m;
    if (anybad) flags[r / flag_rows] = gen;
  }
  const int sexp = f16_scale_exp(m);
  const int64_t plane_elems = R * Kp;
  uint16_t *dst = planes + r * Kp;
#pragma unroll
  for (int i = 0; i < V; i++) {
    const int k = 4 * tid + 1024 * i;
    if (k >= Kp) continue;
    const float rem[4] = {v[i].x, v[i].y, v[i].z, v[i].w};
    uint16_t out[2][4];
#pragma unroll
    for (int t = 0; t < 4; t++) {
      float x = isfinite(rem[t]) ? scale_pow2(rem[t], sexp) : 0.0f;   // |x| < 2^15
#pragma unroll
      for (int pl = 0; pl < 2; pl++) {
        const __half h = __float2half_rn(x);
        out[pl][t] = __half_as_ushort(h);
        x -= __half2float(h);   // exact
      }
    }
#pragma unroll
    for (int pl = 0; pl < 2; pl++) {
      uint2 w;
      w.x = (uint32_t)out[pl][0] | ((uint32_t)out[pl][1] << 16);
      w.y = (uint32_t)out[pl][2] | ((uint32_t)out[pl][3] << 16);
      *reinterpret_cast<uint2 *>(dst + pl * plane_elems + k) = w;
    }
  }
}

// ---- coalesced epilogue stores ------------------------------------------------
//
// The tensor-memory drain (tcgen05.ld 32x32b) leaves one output row per lane,
// so a direct store instruction of a warp touches 32 rows.  This writes the
// warp's 32 rows x W columns (v[c] of row row0 + lane, column col0 + c) to a
// row-major C with unit column stride through `stage`, the warp's 2 KiB of
// shared memory, 16 columns at a time: each lane writes its row's 16 values
// as four 16-byte chunks (chunk q at position q ^ ((row >> 1) & 3): the 8
// lanes of a store phase hit 32 distinct banks), then every load / store
// instruction covers two rows of 16 consecutive columns (two 64-byte
// segments).  Rows >= M and columns >= N are not written.  All 32 lanes
// must call it.
constexpr int kEpiStageFloats = 32 * 16;

template <int W>
__device__ __forceinline__ void store_rows_coalesced(const float (&v)[W], float *stage, float *C,
                                                     int64_t rso, int row0, int col0, int M,
                                                     int N, int lane) {
  static_assert(W % 16 == 0, "16-column blocks");
#pragma unroll
  for (int c0 = 0; c0 < W; c0 += 16) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int qs = q ^ ((lane >> 1) & 3);
      *reinterpret_cast<float4 *>(stage + lane * 16 + qs * 4) =
          make_float4(v[c0 + 4 * q], v[c0 + 4 * q + 1], v[c0 + 4 * q + 2], v[c0 + 4 * q + 3]);
    }
    __syncwarp();
    const int c = lane & 15, r1 = lane >> 4;
    // rows r1, r1 + 2, ...: one running pointer, valid rows counted down
    float *dst = C + (int64_t)(row0 + r1) * rso + (col0 + c0 + c);
    int rows_left = M - (row0 + r1);
    const bool col_ok = col0 + c0 + c < N;
#pragma unroll 1
    for (int rr = 0; rr < 32; rr += 2, dst += 2 * rso, rows_left -= 2) {
      const int r = rr + r1;
      const float x = stage[r * 16 + (((c >> 2) ^ ((r >> 1) & 3)) << 2) + (c & 3)];
      if (rows_left > 0 && col_ok) *dst = x;
    }
    __syncwarp();
  }
}

__host__ __device__ inline int absmax_mode(int mode, int64_t rs_k) {
  return mode == 0 && rs_k == 1 ? 3 : mode;
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

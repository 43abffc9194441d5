// numc_dot's non-GEMM cases (src/reduction/dot.c of numc): the 0-D case
// (multiply by a scalar) and the 1-D inner product, with numc's arithmetic.
//
// 0-D (dot.c:339-346 -> numc_mul_scalar): the scalar element goes to double
// and back to the dtype (elemwise/arithmetic.c:193-203), then each output is
// one product in the dtype: rounded once for floats, modulo 2^bits for
// integers.
//
// 1-D (dot.c:348-365): integers give the exact sum modulo 2^bits in any
// order.  Contiguous float operands follow numc's SIMD dot
// (intrinsics/dot_avx2.h:106-158): thread t of an 8W-thread block (W = 8
// lanes for float32, 4 for float64) owns lane t of the 8W-element blocks and
// chains fma(a, b, acc) over the full blocks of its chunk; the 8
// accumulators are then added pairwise (0+1, 2+3, 4+5, 6+7, 0+2, 4+6, 0+4),
// the lanes by numc's horizontal-sum order, the tail as `tail + a * b`
// unfused, result + tail.  Above 1 MiB of operand bytes numc splits the sum
// into nt = min(4, bytes / 512 KiB) OpenMP chunks (dot.c:235-258), one
// block each here, added to 0 in chunk order.  Strided float operands use
// numc's reduction (reduction/kernel.h:48-78): one unfused chain from 0.
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#include "kernels.h"

namespace numc_k {
namespace {

template <typename T> struct Unsigned { using type = T; };
template <> struct Unsigned<int8_t> { using type = uint8_t; };
template <> struct Unsigned<int16_t> { using type = uint16_t; };
template <> struct Unsigned<int32_t> { using type = uint32_t; };
template <> struct Unsigned<int64_t> { using type = uint64_t; };

template <typename T>
__device__ __forceinline__ T mul_rn(T a, T b) {
  if constexpr (std::is_same<T, float>::value) return __fmul_rn(a, b);
  else if constexpr (std::is_same<T, double>::value) return __dmul_rn(a, b);
  else {
    using U = typename Unsigned<T>::type;
    // widen to 64 bits so 8/16-bit products are not promoted to signed int
    return (T)(U)((uint64_t)(U)a * (uint64_t)(U)b);
  }
}

template <typename T>
__device__ __forceinline__ T add_rn(T a, T b) {
  if constexpr (std::is_same<T, float>::value) return __fadd_rn(a, b);
  else return __dadd_rn(a, b);
}

template <typename T>
__device__ __forceinline__ T fma_rn(T a, T b, T c) {
  if constexpr (std::is_same<T, float>::value) return __fmaf_rn(a, b, c);
  else return __fma_rn(a, b, c);
}

// ---- 0-D ------------------------------------------------------------------

template <typename T>
__global__ void dot_scalar_kernel(const T *__restrict__ x, const T *__restrict__ sp,
                                  T *__restrict__ out, DotNd ix, int64_t total) {
  const double sd = (double)*sp;   // numc's _to_double
  const T s = (T)sd;               // numc's _double_to_dtype
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = e, xo = 0, oo = 0;
    for (int d = ix.dim - 1; d >= 0; d--) {
      const int64_t q = rem % ix.shape[d];
      rem /= ix.shape[d];
      xo += q * ix.xs[d];
      oo += q * ix.os[d];
    }
    out[oo] = mul_rn<T>(x[xo], s);
  }
}

// ---- 1-D: integers ----------------------------------------------------------

constexpr int kIntBlocks = 256, kIntThreads = 256;

// Partial sums modulo 2^64 (hence modulo 2^bits) of a grid-stride slice.
template <typename T>
__global__ void dot1d_int_partial(const T *__restrict__ a, int64_t sa, const T *__restrict__ b,
                                  int64_t sb, int64_t n, uint64_t *__restrict__ part) {
  __shared__ uint64_t red[kIntThreads];
  uint64_t acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t x = std::is_signed<T>::value ? (uint64_t)(int64_t)a[i * sa] : (uint64_t)a[i * sa];
    const uint64_t y = std::is_signed<T>::value ? (uint64_t)(int64_t)b[i * sb] : (uint64_t)b[i * sb];
    acc += x * y;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kIntThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

template <typename T>
__global__ void dot1d_int_final(const uint64_t *__restrict__ part, int nparts, T *out) {
  uint64_t acc = 0;
  for (int i = 0; i < nparts; i++) acc += part[i];
  *out = (T)acc;
}

// ---- 1-D: floats ------------------------------------------------------------

// numc's SIMD dot as 8W independent FMA chains per OpenMP chunk: chain t
// of chunk c runs over elements s_c + t, s_c + t + 8W, ... of the chunk's
// full 8W-element blocks.  Each chain is sequential, so the parallelism is
// the chains: a block takes 32 bytes' worth of consecutive chains of one
// chunk (8 float32 / 4 float64 — whole DRAM sectors), and while its first
// warp runs the chains over one stage of kDotRows blocks held in shared
// memory, the other seven warps load the stage after next.  16 Mi float32
// (4 chunks, 64 chains of 65536 FMAs each): 0.64 ms, against 6.8 ms with one
// 64-thread block a chunk reading its operands directly.
constexpr int kDotRows = 256, kDotStages = 3;   // 3 x 2 operands: 48 KiB of shared memory

template <typename T, int W>
__global__ void __launch_bounds__(256)
dot1d_simd_chains(const T *__restrict__ a, const T *__restrict__ b, int64_t n, int nt,
                  T *__restrict__ lanes_out) {
  constexpr int CG = 32 / (int)sizeof(T);        // chains a block
  constexpr int GROUPS = 8 * W / CG;             // blocks a chunk (8)
  __shared__ T sa[kDotStages][kDotRows][CG], sb[kDotStages][kDotRows][CG];
  const int c = blockIdx.x / GROUPS, grp = blockIdx.x % GROUPS;
  const int64_t per = n / nt;
  const int64_t s = (int64_t)c * per, e = (c == nt - 1) ? n : s + per;
  const int64_t rows = (e - s) / (8 * W);        // full 8W-element blocks
  const int64_t stages = (rows + kDotRows - 1) / kDotRows;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t col0 = s + grp * CG;             // element of chain grp*CG, row 0

  // loaders (warps 1-7): rows r0 .. r0 + kDotRows of this block's chains
  auto load = [&](int buf, int64_t r0) {
    const int lt = tid - 32;                     // 0 .. 223
    const int ch = lt % CG;
    for (int r = lt / CG; r < kDotRows; r += 224 / CG) {
      const int64_t row = r0 + r;
      T x = T(0), y = T(0);
      if (row < rows) {
        const int64_t idx = col0 + row * 8 * W + ch;
        x = a[idx];
        y = b[idx];
      }
      sa[buf][r][ch] = x;
      sb[buf][r][ch] = y;
    }
  };
  if (warp > 0) {
    load(0, 0);
    if (stages > 1) load(1, kDotRows);
  }
  __syncthreads();
  T acc = T(0);
  for (int64_t st = 0; st < stages; st++) {
    const int buf = (int)(st % kDotStages);
    if (warp > 0) {
      if (st + 2 < stages) load((int)((st + 2) % kDotStages), (st + 2) * kDotRows);
    } else if (lane < CG) {
      const int nr = (int)min((int64_t)kDotRows, rows - st * kDotRows);
#pragma unroll 8
      for (int r = 0; r < nr; r++) acc = fma_rn<T>(sa[buf][r][lane], sb[buf][r][lane], acc);
    }
    __syncthreads();
  }
  if (warp == 0 && lane < CG) lanes_out[(int64_t)c * 8 * W + grp * CG + lane] = acc;
}

// Chunk c's result from its 8W chain values: numc's pairwise accumulator
// sums, horizontal lane sum and unfused tail.
template <typename T, int W>
__global__ void dot1d_simd_combine(const T *__restrict__ a, const T *__restrict__ b, int64_t n,
                                   int nt, const T *__restrict__ lanes, T *__restrict__ part) {
  const int c = blockIdx.x;
  const int64_t per = n / nt;
  const int64_t s = (int64_t)c * per, e = (c == nt - 1) ? n : s + per;
  const int64_t full_end = s + ((e - s) / (8 * W)) * (8 * W);
  T v[8][W];
  for (int j = 0; j < 8; j++)
    for (int l = 0; l < W; l++) v[j][l] = lanes[(int64_t)c * 8 * W + W * j + l];
  for (int l = 0; l < W; l++) {
    v[0][l] = add_rn<T>(v[0][l], v[1][l]);
    v[2][l] = add_rn<T>(v[2][l], v[3][l]);
    v[4][l] = add_rn<T>(v[4][l], v[5][l]);
    v[6][l] = add_rn<T>(v[6][l], v[7][l]);
    v[0][l] = add_rn<T>(v[0][l], v[2][l]);
    v[4][l] = add_rn<T>(v[4][l], v[6][l]);
    v[0][l] = add_rn<T>(v[0][l], v[4][l]);
  }
  T result;
  if constexpr (W == 8) {   // _hsum_ps_avx2
    const T s0 = add_rn<T>(v[0][0], v[0][4]), s1 = add_rn<T>(v[0][1], v[0][5]);
    const T s2 = add_rn<T>(v[0][2], v[0][6]), s3 = add_rn<T>(v[0][3], v[0][7]);
    result = add_rn<T>(add_rn<T>(s0, s2), add_rn<T>(s1, s3));
  } else {                  // _hsum_pd_avx2
    result = add_rn<T>(add_rn<T>(v[0][0], v[0][2]), add_rn<T>(v[0][1], v[0][3]));
  }
  T tail = T(0);
  for (int64_t i = full_end; i < e; i++) tail = add_rn<T>(tail, mul_rn<T>(a[i], b[i]));
  part[c] = add_rn<T>(result, tail);
}

template <typename T>
__global__ void dot1d_float_final(const T *__restrict__ part, int nt, T *out) {
  T g = T(0);
  for (int c = 0; c < nt; c++) g = add_rn<T>(g, part[c]);
  *out = g;
}

// numc's strided reduction: one unfused chain in order (sequential).
template <typename T>
__global__ void dot1d_naive(const T *__restrict__ a, int64_t sa, const T *__restrict__ b,
                            int64_t sb, int64_t n, T *out) {
  T acc = T(0);
  for (int64_t i = 0; i < n; i++) acc = add_rn<T>(acc, mul_rn<T>(a[i * sa], b[i * sb]));
  *out = acc;
}

template <typename T>
cudaError_t scalar_t(const void *x, const void *sp, void *out, const DotNd &ix, cudaStream_t s) {
  int64_t total = 1;
  for (int d = 0; d < ix.dim; d++) total *= ix.shape[d];
  if (total == 0) return cudaSuccess;
  const int64_t blocks = (total + 255) / 256;
  dot_scalar_kernel<T><<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, s>>>(
      (const T *)x, (const T *)sp, (T *)out, ix, total);
  count_launch();
  return cudaGetLastError();
}

template <typename T>
cudaError_t dot1d_t(const void *a, int64_t sa, const void *b, int64_t sb, int64_t n,
                    bool contiguous, void *out, void *scratch, cudaStream_t s) {
  if constexpr (std::is_floating_point<T>::value) {
    constexpr int W = sizeof(T) == 4 ? 8 : 4;
    if (!contiguous) {
      dot1d_naive<T><<<1, 1, 0, s>>>((const T *)a, sa, (const T *)b, sb, n, (T *)out);
      count_launch();
      return cudaGetLastError();
    }
    const uint64_t bytes = (uint64_t)n * sizeof(T) * 2;
    int nt = (int)(bytes / (1u << 19));
    if (nt > 4) nt = 4;
    if (!(bytes > (1u << 20) && nt >= 2)) nt = 1;
    T *lanes = (T *)scratch, *part = lanes + 4 * 8 * W;   // nt <= 4 chunks
    constexpr int GROUPS = 8 * W / (32 / (int)sizeof(T));
    dot1d_simd_chains<T, W><<<nt * GROUPS, 256, 0, s>>>((const T *)a, (const T *)b, n, nt, lanes);
    dot1d_simd_combine<T, W><<<nt, 1, 0, s>>>((const T *)a, (const T *)b, n, nt, lanes, part);
    dot1d_float_final<T><<<1, 1, 0, s>>>(part, nt, (T *)out);
    count_launch(3);
    return cudaGetLastError();
  } else {
    uint64_t *part = (uint64_t *)scratch;
    dot1d_int_partial<T><<<kIntBlocks, kIntThreads, 0, s>>>((const T *)a, sa, (const T *)b, sb,
                                                            n, part);
    dot1d_int_final<T><<<1, 1, 0, s>>>(part, kIntBlocks, (T *)out);
    count_launch(2);
    return cudaGetLastError();
  }
}

}  // namespace

// integer partial sums, or float chain values (4 chunks x 64) and chunk sums
size_t dot1d_scratch_bytes() {
  const size_t f = (4 * 64 + 4) * 8;
  return (size_t)kIntBlocks * 8 > f ? (size_t)kIntBlocks * 8 : f;
}

cudaError_t launch_dot_scalar(NumcDType dt, const void *x, const void *scalar, void *out,
                              const DotNd &ix, cudaStream_t s) {
  switch (dt) {
  case NUMC_DTYPE_INT8: return scalar_t<int8_t>(x, scalar, out, ix, s);
  case NUMC_DTYPE_INT16: return scalar_t<int16_t>(x, scalar, out, ix, s);
  case NUMC_DTYPE_INT32: return scalar_t<int32_t>(x, scalar, out, ix, s);
  case NUMC_DTYPE_INT64: return scalar_t<int64_t>(x, scalar, out, ix, s);
  case NUMC_DTYPE_UINT8: return scalar_t<uint8_t>(x, scalar, out, ix, s);
  case NUMC_DTYPE_UINT16: return scalar_t<uint16_t>(x, scalar, out, ix, s);
  case NUMC_DTYPE_UINT32: return scalar_t<uint32_t>(x, scalar, out, ix, s);
  case NUMC_DTYPE_UINT64: return scalar_t<uint64_t>(x, scalar, out, ix, s);
  case NUMC_DTYPE_FLOAT32: return scalar_t<float>(x, scalar, out, ix, s);
  case NUMC_DTYPE_FLOAT64: return scalar_t<double>(x, scalar, out, ix, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_dot_1d(NumcDType dt, const void *a, int64_t sa, const void *b, int64_t sb,
                          int64_t n, bool contiguous, void *out, void *scratch,
                          cudaStream_t s) {
  switch (dt) {
  case NUMC_DTYPE_INT8: return dot1d_t<int8_t>(a, sa, b, sb, n, contiguous, out, scratch, s);
  case NUMC_DTYPE_INT16: return dot1d_t<int16_t>(a, sa, b, sb, n, contiguous, out, scratch, s);
  case NUMC_DTYPE_INT32: return dot1d_t<int32_t>(a, sa, b, sb, n, contiguous, out, scratch, s);
  case NUMC_DTYPE_INT64: return dot1d_t<int64_t>(a, sa, b, sb, n, contiguous, out, scratch, s);
  case NUMC_DTYPE_UINT8: return dot1d_t<uint8_t>(a, sa, b, sb, n, contiguous, out, scratch, s);
  case NUMC_DTYPE_UINT16: return dot1d_t<uint16_t>(a, sa, b, sb, n, contiguous, out, scratch, s);
  case NUMC_DTYPE_UINT32: return dot1d_t<uint32_t>(a, sa, b, sb, n, contiguous, out, scratch, s);
  case NUMC_DTYPE_UINT64: return dot1d_t<uint64_t>(a, sa, b, sb, n, contiguous, out, scratch, s);
  case NUMC_DTYPE_FLOAT32: return dot1d_t<float>(a, sa, b, sb, n, contiguous, out, scratch, s);
  case NUMC_DTYPE_FLOAT64: return dot1d_t<double>(a, sa, b, sb, n, contiguous, out, scratch, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace numc_k


// CUDA-core GEMM tile shared by the single-problem and grouped launchers.
//
// One templated tile kernel: a BM x BN output tile per 256-thread CTA, a
// BK-deep K slab staged through double-buffered shared memory (next slab
// prefetched into registers while the current one is consumed), and a
// TM x TN register tile per thread split into two halves BM/2 (BN/2) apart
// so shared-memory reads are conflict-free float4-width rows.
//
// Arithmetic per dtype reproduces numc (src/intrinsics/gemm_avx2.h):
//   float32/float64  one fused multiply-add chain per output in k order
//                    from +0, exactly numc's full-tile micro-kernels
//                    (gemm_ukernel_f32_6x16_avx2.S keeps one FMA
//                    accumulator per output and reloads it between K
//                    blocks); only numc's remainder tiles round differently.
//   int16..uint64    products and sums wrap in 32 (16- and 32-bit types)
//                    or 64 bits, then truncate: the exact sum modulo 2^bits,
//                    as numc's vpmullw/vpmulld/emulated-64-bit kernels give.
//   int8/uint8       exact int32 partial sums per K block of 512 with numc's
//                    store rule applied at each block end (Rule8).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#include "kernels.h"

namespace numc_k {
namespace simt {


constexpr int kThreads = 256;

// kFloat: one fused multiply-add chain per output (numc's register tiles);
// kFloatUnfused: `acc = acc + a * b`, product and sum each rounded (numc's
// naive kernels, compiled without contraction).
enum Kind : int { kFloat = 0, kWrapInt = 1, kByte = 2, kFloatUnfused = 3 };

// ---- numc's int8/uint8 store rules ---------------------------------------

__device__ __forceinline__ int32_t sat_s8(int32_t v) {
  return v < -128 ? -128 : (v > 127 ? 127 : v);
}
// packusdw then packuswb (x86): clamp to [0,65535], view as int16, clamp
// to [0,255].
__device__ __forceinline__ int32_t sat_u8_x86(int32_t v) {
  int32_t u16 = v < 0 ? 0 : (v > 65535 ? 65535 : v);
  int32_t s16 = u16 >= 32768 ? u16 - 65536 : u16;
  return s16 < 0 ? 0 : (s16 > 255 ? 255 : s16);
}
__device__ __forceinline__ int32_t wrap8(int32_t v, bool is_signed) {
  uint32_t byte = (uint32_t)v & 0xFFu;
  return is_signed ? (int32_t)(int8_t)byte : (int32_t)byte;
}
// Full 6x16 register tile of numc's x86 packed int8 path: M blocked by
// MC=72 (MR=6), N by NC=4080 (NR=16) — gemm_avx2.h:2741-2880.
__device__ __forceinline__ bool x86_full(int64_t i, int64_t j, int64_t M,
                                         int64_t N) {
  int64_t ic = (i / 72) * 72, mc = min((int64_t)72, M - ic);
  int64_t ir = ((i - ic) / 6) * 6, mr = min((int64_t)6, mc - ir);
  int64_t jc = (j / 4080) * 4080, nc = min((int64_t)4080, N - jc);
  int64_t jr = ((j - jc) / 16) * 16, nr = min((int64_t)16, nc - jr);
  return mr == 6 && nr == 16;
}
// Full 6x8 tile of numc's NEON int8 path (gemm_neon.h:1509-1535).
__device__ __forceinline__ bool neon_full(int64_t i, int64_t j, int64_t M,
                                          int64_t N) {
  int64_t ic = (i / 72) * 72, mc = min((int64_t)72, M - ic);
  return (i - ic) < (mc / 6) * 6 && j < (N / 8) * 8;
}

// One K-block end for element (i, j): fold the block's partial sum P into
// the stored value d according to the rule.  `first` marks block 0.
__device__ __forceinline__ int32_t fold8(int32_t d, int32_t P, bool first,
                                         int rule, bool is_signed, int64_t i,
                                         int64_t j, int64_t M, int64_t N) {
  if (rule == kRuleX86Packed) {
    if (x86_full(i, j, M, N)) {
      int32_t v = d + P;
      return is_signed ? sat_s8(v) : sat_u8_x86(v);
    }
    int32_t t = is_signed ? sat_s8(P) : sat_u8_x86(P);
    return first ? t : wrap8(d + t, is_signed);
  }
  if (rule == kRuleNeon) {
    if (neon_full(i, j, M, N))
      return is_signed ? sat_s8(P) : ((uint32_t)P > 255u ? 255 : P);
    return wrap8(P, is_signed);
  }
  return wrap8((int32_t)((uint32_t)d + (uint32_t)P), is_signed);
}

template <typename T> struct AccOf { using type = uint32_t; };
template <> struct AccOf<float> { using type = float; };
template <> struct AccOf<double> { using type = double; };
template <> struct AccOf<int64_t> { using type = uint64_t; };
template <> struct AccOf<uint64_t> { using type = uint64_t; };

template <typename Acc>
__device__ __forceinline__ Acc madd(Acc a, Acc b, Acc c) { return c + a * b; }
template <> __device__ __forceinline__ float madd(float a, float b, float c) {
  return __fmaf_rn(a, b, c);
}
template <> __device__ __forceinline__ double madd(double a, double b, double c) {
  return __fma_rn(a, b, c);
}
// The _rn intrinsics are never contracted into a fused multiply-add.
__device__ __forceinline__ float madd_unfused(float a, float b, float c) {
  return __fadd_rn(c, __fmul_rn(a, b));
}
__device__ __forceinline__ double madd_unfused(double a, double b, double c) {
  return __dadd_rn(c, __dmul_rn(a, b));
}

// Widen one element to the accumulation type: sign-extend signed integers,
// zero-extend unsigned ones (then wrap in the unsigned accumulator).
template <typename T, typename Acc>
__device__ __forceinline__ Acc widen(T v) {
  if constexpr (std::is_floating_point<T>::value) return (Acc)v;
  else if constexpr (std::is_signed<T>::value) return (Acc)(int64_t)v;
  else return (Acc)v;
}

// One BM x BN output tile at (m0, n0) of problem g, by a kThreads-thread
// block.
template <typename T, int BM, int BN, int BK, int TM, int TN, int KIND>
__device__ __forceinline__ void simt_tile(const Gemm &g, int rule8, int64_t m0, int64_t n0) {
  using Acc = typename AccOf<T>::type;
  constexpr int LA = BM * BK / kThreads;   // A elements loaded per thread
  constexpr int LB = BK * BN / kThreads;   // B elements loaded per thread
  constexpr int TX = BN / TN;              // threads along N
  static_assert(TX * (BM / TM) == kThreads, "thread grid");
  __shared__ __align__(16) Acc As[2][BK][BM];
  __shared__ __align__(16) Acc Bs[2][BK][BN];

  const T *__restrict__ A = (const T *)g.a;
  const T *__restrict__ B = (const T *)g.b;
  T *__restrict__ C = (T *)g.c;
  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  const bool a_kfast = g.csa == 1, b_nfast = g.csb == 1 || g.rsb != 1;

  Acc ra[LA], rb[LB];
  auto load_tiles = [&](int64_t k0) {
#pragma unroll
    for (int q = 0; q < LA; q++) {
      int e = tid + kThreads * q;
      int r = a_kfast ? e / BK : e % BM;
      int kk = a_kfast ? e % BK : e / BM;
      int64_t gi = m0 + r, gk = k0 + kk;
      ra[q] = (gi < g.M && gk < g.K) ? widen<T, Acc>(A[gi * g.rsa + gk * g.csa]) : Acc(0);
    }
#pragma unroll
    for (int q = 0; q < LB; q++) {
      int e = tid + kThreads * q;
      int c = b_nfast ? e % BN : e / BK;
      int kk = b_nfast ? e / BN : e % BK;
      int64_t gj = n0 + c, gk = k0 + kk;
      rb[q] = (gj < g.N && gk < g.K) ? widen<T, Acc>(B[gk * g.rsb + gj * g.csb]) : Acc(0);
    }
  };
  auto store_tiles = [&](int buf) {
#pragma unroll
    for (int q = 0; q < LA; q++) {
      int e = tid + kThreads * q;
      int r = a_kfast ? e / BK : e % BM;
      int kk = a_kfast ? e % BK : e / BM;
      As[buf][kk][r] = ra[q];
    }
#pragma unroll
    for (int q = 0; q < LB; q++) {
      int e = tid + kThreads * q;
      int c = b_nfast ? e % BN : e / BK;
      int kk = b_nfast ? e / BN : e % BK;
      Bs[buf][kk][c] = rb[q];
    }
  };

  // Rows/columns of this thread's register tile: two halves BM/2 apart.
  auto row_of = [&](int i) {
    return i < TM / 2 ? ty * (TM / 2) + i : BM / 2 + ty * (TM / 2) + (i - TM / 2);
  };
  auto col_of = [&](int j) {
    return j < TN / 2 ? tx * (TN / 2) + j : BN / 2 + tx * (TN / 2) + (j - TN / 2);
  };

  Acc acc[TM][TN];
  int32_t dst[KIND == kByte ? TM : 1][KIND == kByte ? TN : 1];
#pragma unroll
  for (int i = 0; i < TM; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) acc[i][j] = Acc(0);
  if constexpr (KIND == kByte) {
#pragma unroll
    for (int i = 0; i < TM; i++)
#pragma unroll
      for (int j = 0; j < TN; j++) dst[i][j] = 0;
  }

  const int64_t ntiles = (g.K + BK - 1) / BK;
  // int8/uint8: K-block length over which partial sums are exact before the
  // store rule folds them (512 for numc's x86 packed path, all of K else).
  const int64_t kblock = (KIND == kByte && rule8 == kRuleX86Packed) ? 512 : (int64_t)1 << 62;
  int64_t block_idx = 0;

  load_tiles(0);
  store_tiles(0);
  __syncthreads();
  for (int64_t t = 0; t < ntiles; t++) {
    const int buf = (int)(t & 1);
    if (t + 1 < ntiles) load_tiles((t + 1) * BK);
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      Acc av[TM], bv[TN];
#pragma unroll
      for (int i = 0; i < TM; i++) av[i] = As[buf][kk][row_of(i)];
#pragma unroll
      for (int j = 0; j < TN; j++) bv[j] = Bs[buf][kk][col_of(j)];
#pragma unroll
      for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) {
          if constexpr (KIND == kFloatUnfused) acc[i][j] = madd_unfused(av[i], bv[j], acc[i][j]);
          else acc[i][j] = madd<Acc>(av[i], bv[j], acc[i][j]);
        }
    }
    if constexpr (KIND == kByte) {
      const int64_t kend = (t + 1) * BK;
      if (kend % kblock == 0 || t + 1 == ntiles) {
        const bool is_signed = (T)(-1) < (T)0;
#pragma unroll
        for (int i = 0; i < TM; i++)
#pragma unroll
          for (int j = 0; j < TN; j++) {
            dst[i][j] = fold8(dst[i][j], (int32_t)acc[i][j], block_idx == 0, rule8,
                              is_signed, m0 + row_of(i), n0 + col_of(j), g.M, g.N);
            acc[i][j] = 0;
          }
        block_idx++;
      }
    }
    if (t + 1 < ntiles) store_tiles(buf ^ 1);
    __syncthreads();
  }
  if constexpr (KIND == kByte) {
    if (ntiles == 0) {   // K == 0: every stored value is zero
#pragma unroll
      for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) dst[i][j] = 0;
    }
  }

#pragma unroll
  for (int i = 0; i < TM; i++) {
    int64_t gi = m0 + row_of(i);
    if (gi >= g.M) continue;
#pragma unroll
    for (int j = 0; j < TN; j++) {
      int64_t gj = n0 + col_of(j);
      if (gj >= g.N) continue;
      T v;
      if constexpr (KIND == kByte) v = (T)dst[i][j];
      else v = (T)acc[i][j];
      C[gi * g.rso + gj * g.cso] = v;
    }
  }
}

}  // namespace simt
}  // namespace numc_k

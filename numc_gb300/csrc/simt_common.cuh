// CUDA-core GEMM tile shared by the single-problem and grouped launchers.
//
// One templated tile kernel: a BM x BN output tile per 256-thread CTA, a
// BK-deep K slab staged through double-buffered shared memory (next slab
// prefetched into registers while the current one is consumed; for
// row-major operands and inner tiles from fixed per-thread offsets, with
// no index arithmetic), and a TM x TN register tile per thread split into
// two halves BM/2 (BN/2) apart so shared-memory reads are conflict-free
// float4-width rows (2 x 2 tiles: one adjacent pair).
//
// Arithmetic per dtype reproduces numc (src/intrinsics/gemm_avx2.h):
//   float32/float64  one fused multiply-add chain per output in k order
//                    from +0, exactly numc's full-tile micro-kernels
//                    (gemm_ukernel_f32_6x16_avx2.S keeps one FMA
//                    accumulator per output and reloads it between K
//                    blocks); numc's remainder tiles sum each 256-deep K
//                    block separately (kFloatEdges, or the float_edges
//                    pass after 128-wide tiles).
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

// kFloat: one fused multiply-add chain per output (numc's full register
// tiles; numc_float_edges then redoes the packed path's remainder tiles);
// kFloatEdges: kFloat with the remainder-tile outputs summed per 256-deep K
// block inside the tile kernel (chain from zero each block, added in order);
// kFloatSmall: numc's unpacked (gemmsup) float path;
// kFloatUnfused: `acc = acc + a * b`, product and sum each rounded (numc's
// naive kernels, compiled without contraction).
enum Kind : int { kFloat = 0, kWrapInt = 1, kByte = 2, kFloatUnfused = 3, kFloatSmall = 4,
                  kFloatEdges = 5 };

// ---- numc's float register tiles ------------------------------------------
//
// Packed path: M in blocks of MC rows cut into MR-row register tiles, N in
// panels of NC columns cut into NR-column tiles, K in blocks of 256.  An
// output of a full MR x NR tile is one FMA chain over all K (the
// micro-kernel reloads C between K blocks); an output of a remainder tile
// sums each K block as an FMA chain from zero and adds it to the stored
// value.  Unpacked path (M K N at most 96^3 float32 / 48^3 float64): 6 x NR
// tiles from the origin; in a tile narrower than NR the first
// (width / VW) x VW columns are vector FMA chains and the rest scalar
// `c += a * b`, unfused (numc is ISO C without contraction).
// The geometry depends on the ISA numc was built for (Gemm::isa):
//   x86-64 AVX2 (gemm_avx2.h:852-950, 1377-1475; gemmsup_avx2.h:97-147,
//   221-270): float32 MC 144, MR 6, NR 16, NC 4080, VW 8; float64 MC 72,
//   MR 6, NR 8, NC 4080, VW 4;
//   aarch64 NEON (gemm_neon.h:610-740, 951-1080; gemmsup_neon.h:28-155,
//   163-300): float32 MC 128, MR 8, NR 12, NC 4080, VW 4; float64 MC 96,
//   MR 6, NR 8, NC 2048, VW 2.
struct FloatGeom {
  int mc, mr, nc, nr, vw;
};
template <typename T> __host__ __device__ inline FloatGeom numc_geom(int isa) {
  if constexpr (std::is_same<T, float>::value)
    return isa == kIsaNeon ? FloatGeom{128, 8, 4080, 12, 4} : FloatGeom{144, 6, 4080, 16, 8};
  else
    return isa == kIsaNeon ? FloatGeom{96, 6, 2048, 8, 2} : FloatGeom{72, 6, 4080, 8, 4};
}
constexpr int kNumcKC = 256;

// First row / column of numc's remainder register tiles: rows from
// edge_row(M) (the last MC block's partial MR tile), and, above them,
// columns from edge_col(N) (the last NC-column panel's partial NR tile).
// MC and NC are multiples of MR and NR on every ISA, so no other tile is
// partial.
template <typename T> __host__ __device__ inline int64_t edge_row(int64_t M, int isa) {
  if (M == 0) return 0;
  const FloatGeom G = numc_geom<T>(isa);
  const int64_t ic = ((M - 1) / G.mc) * G.mc;
  return ic + ((M - ic) / G.mr) * G.mr;
}
template <typename T> __host__ __device__ inline int64_t edge_col(int64_t N, int isa) {
  if (N == 0) return 0;
  const FloatGeom G = numc_geom<T>(isa);
  const int64_t jc = ((N - 1) / G.nc) * G.nc;
  return jc + ((N - jc) / G.nr) * G.nr;
}

// Unpacked path: column j is one of a narrow tile's scalar (unfused) columns.
template <typename T>
__device__ __forceinline__ bool small_col_unfused(int64_t j, int64_t N, int isa) {
  const FloatGeom G = numc_geom<T>(isa);
  const int64_t j0 = (j / G.nr) * G.nr, nr = min((int64_t)G.nr, N - j0);
  return nr < G.nr && (j - j0) >= (nr / G.vw) * G.vw;
}

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
// x86_full split into its row and column halves, in 32-bit arithmetic
// (dimensions below 2^31): x86_full(i, j) == x86_row_full(i) && x86_col_full(j).
__device__ __forceinline__ bool x86_row_full(int i, int M) {
  const int ic = i / 72 * 72, mc = min(72, M - ic);
  return i - ic < mc / 6 * 6;
}
__device__ __forceinline__ bool x86_col_full(int j, int N) {
  const int jc = j / 4080 * 4080, nc = min(4080, N - jc);
  return j - jc < nc / 16 * 16;
}
// x86_col_full of columns j0 .. j0 + W - 1 (W <= 64) as a bit mask (bit c
// for column j0 + c): the full columns of an NC block are a prefix of it,
// and W columns touch at most two NC blocks.
__device__ __forceinline__ uint64_t x86_col_mask(int j0, int N, int W) {
  auto prefix = [](int64_t n) -> uint64_t {   // bits [0, n), n clamped to [0, 64]
    return n <= 0 ? 0ull : n >= 64 ? ~0ull : (1ull << n) - 1;
  };
  const int jc0 = j0 / 4080 * 4080;
  const int64_t end0 = jc0 + min(4080, N - jc0) / 16 * 16;   // first non-full column of block 0
  const int64_t jc1 = (int64_t)jc0 + 4080;
  const int64_t end1 = jc1 + (N > jc1 ? min((int64_t)4080, N - jc1) / 16 * 16 : 0);
  uint64_t m = prefix(end0 - j0);
  if (jc1 < (int64_t)j0 + W) m |= prefix(end1 - j0) & ~prefix(jc1 - j0);
  return m & prefix(W);
}
// Full MR x NR tile of a clamp-once int8 path that blocks M by MC (a
// multiple of MR) and N by NR from column 0: numc's NEON build (72, 6, 8;
// gemm_neon.h:1509-1535) and its AVX-512 build (240, 12, 16;
// gemm_avx512.h:1315-1341).
__device__ __forceinline__ bool clamp_full(int64_t i, int64_t j, int64_t M, int64_t N,
                                           int rule) {
  const int64_t MC = rule == kRuleNeon ? 72 : 240, MR = rule == kRuleNeon ? 6 : 12;
  const int64_t NR = rule == kRuleNeon ? 8 : 16;
  int64_t ic = (i / MC) * MC, mc = min(MC, M - ic);
  return (i - ic) < (mc / MR) * MR && j < (N / NR) * NR;
}

// The clamp-once rules' final narrowing of a row's outputs, with the tile
// class split into its row and column halves in 32-bit arithmetic
// (dimensions below 2^31): for every column j of the row,
// narrow_once(...)[j] == fold8(0, P[j], true, rule, ...) for the NEON,
// AVX-512 and wrap rules.
__device__ __forceinline__ int32_t narrow_once(int32_t P, bool full, bool is_signed) {
  if (full) return is_signed ? sat_s8(P) : ((uint32_t)P > 255u ? 255 : P);
  return wrap8(P, is_signed);
}
__device__ __forceinline__ bool clamp_row_full(int i, int M, int rule) {
  if (rule != kRuleNeon && rule != kRuleAvx512) return false;
  const int MC = rule == kRuleNeon ? 72 : 240, MR = rule == kRuleNeon ? 6 : 12;
  const int ic = i / MC * MC, mc = min(MC, M - ic);
  return i - ic < mc / MR * MR;
}
// Columns below this are inside full tiles (with a full row).
__device__ __forceinline__ int clamp_col_limit(int N, int rule) {
  const int NR = rule == kRuleNeon ? 8 : 16;
  return N / NR * NR;
}

// One K-block end for element (i, j): fold the block's partial sum P into
// the stored value d according to the rule.  `first` marks block 0.
// x86 packed rule with the element's tile class known (`full`: inside a
// full 6x16 register tile).
__device__ __forceinline__ int32_t fold8_x86(int32_t d, int32_t P, bool first,
                                             bool full, bool is_signed) {
  if (full) {
    int32_t v = d + P;
    return is_signed ? sat_s8(v) : sat_u8_x86(v);
  }
  int32_t t = is_signed ? sat_s8(P) : sat_u8_x86(P);
  return first ? t : wrap8(d + t, is_signed);
}
__device__ __forceinline__ int32_t fold8(int32_t d, int32_t P, bool first,
                                         int rule, bool is_signed, int64_t i,
                                         int64_t j, int64_t M, int64_t N) {
  if (rule == kRuleX86Packed)
    return fold8_x86(d, P, first, x86_full(i, j, M, N), is_signed);
  if (rule == kRuleNeon || rule == kRuleAvx512) {
    // one block over all K: the wrapped int32 sum narrowed once with
    // saturation (uint8: the lane read as unsigned, min(u32, 255)), or
    // truncated in remainder tiles
    if (clamp_full(i, j, M, N, rule))
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
template <typename T>
__device__ __forceinline__ T add_rn(T a, T b) {
  if constexpr (std::is_same<T, float>::value) return __fadd_rn(a, b);
  else return __dadd_rn(a, b);
}
// numc's elementwise a + b in the dtype: rounded once for floats, modulo
// 2^bits for integers.
template <typename T>
__device__ __forceinline__ T add_elem(T a, T b) {
  if constexpr (std::is_floating_point<T>::value) return add_rn<T>(a, b);
  else return (T)((uint64_t)(int64_t)a + (uint64_t)(int64_t)b);
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
  // A is stored transposed (k-major): rows padded so that the lanes of a
  // warp, which load along k for row-major A, store to distinct banks
  constexpr int APAD = BK >= 32 ? 2 : 4;
  __shared__ __align__(16) Acc As[2][BK][BM + APAD];
  __shared__ __align__(16) Acc Bs[2][BK][BN];

  const T *__restrict__ A = (const T *)g.a;
  const T *__restrict__ B = (const T *)g.b;
  T *__restrict__ C = (T *)g.c;
  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  const bool a_kfast = g.csa == 1, b_nfast = g.csb == 1 || g.rsb != 1;

  Acc ra[LA], rb[LB];
  // A and B with unit column stride (numc's contiguous arrays) and a tile
  // inside the matrix: each thread's operand elements sit at fixed offsets
  // from two pointers, so they load without index arithmetic or checks.
  static_assert(kThreads % BK == 0 && kThreads % BN == 0, "load mapping");
  const bool inner_mn = g.csa == 1 && g.csb == 1 && m0 + BM <= g.M && n0 + BN <= g.N;
  const T *pa = A + (m0 + tid / BK) * g.rsa + tid % BK;          // row tid/BK + q*256/BK
  const T *pb = B + (int64_t)(tid / BN) * g.rsb + n0 + tid % BN;  // k tid/BN + q*256/BN
  const int64_t a_step = (int64_t)(kThreads / BK) * g.rsa;
  const int64_t b_step = (int64_t)(kThreads / BN) * g.rsb;
  auto load_tiles = [&](int64_t k0) {
    if (inner_mn && k0 + BK <= g.K) {
      const T *a0 = pa + k0, *b0 = pb + k0 * g.rsb;
#pragma unroll
      for (int q = 0; q < LA; q++) ra[q] = widen<T, Acc>(a0[q * a_step]);
#pragma unroll
      for (int q = 0; q < LB; q++) rb[q] = widen<T, Acc>(b0[q * b_step]);
      return;
    }
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

  // Rows/columns of this thread's register tile: two halves BM/2 apart,
  // or, for 2 x 2 tiles, one adjacent pair (one 8-byte shared load each).
  auto row_of = [&](int i) {
    if constexpr (TM == 2) return ty * 2 + i;
    return i < TM / 2 ? ty * (TM / 2) + i : BM / 2 + ty * (TM / 2) + (i - TM / 2);
  };
  auto col_of = [&](int j) {
    if constexpr (TN == 2) return tx * 2 + j;
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

  // kFloatEdges: bit i*TN+j: output (i, j) lies in a remainder tile and K
  // spans several blocks; its block sums accumulate in bsum.
  static_assert(KIND != kFloatEdges || TM * TN <= 32, "edge mask");
  constexpr bool kEdges = KIND == kFloatEdges;
  Acc bsum[kEdges ? TM : 1][kEdges ? TN : 1];
  uint32_t edge_mask = 0;
  if constexpr (kEdges) {
    if (g.K > kNumcKC) {
      const int64_t er = edge_row<T>(g.M, g.isa), ec = edge_col<T>(g.N, g.isa);
#pragma unroll
      for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) {
          bsum[i][j] = Acc(0);
          if (m0 + row_of(i) >= er || n0 + col_of(j) >= ec) edge_mask |= 1u << (i * TN + j);
        }
    }
  }
  int64_t edge_blk = 0;

  uint32_t unf_mask = 0;   // kFloatSmall: bit j: column j is an unfused one
  if constexpr (KIND == kFloatSmall) {
#pragma unroll
    for (int j = 0; j < TN; j++)
      if (small_col_unfused<T>(n0 + col_of(j), g.N, g.isa)) unf_mask |= 1u << j;
  }

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
          if constexpr (KIND == kFloatUnfused) {
            acc[i][j] = madd_unfused(av[i], bv[j], acc[i][j]);
          } else if constexpr (KIND == kFloatSmall) {
            acc[i][j] = ((unf_mask >> j) & 1u) ? madd_unfused(av[i], bv[j], acc[i][j])
                                               : madd<Acc>(av[i], bv[j], acc[i][j]);
          } else {
            acc[i][j] = madd<Acc>(av[i], bv[j], acc[i][j]);
          }
        }
    }
    if constexpr (kEdges) {
      const int64_t kend = (t + 1) * BK;
      if (edge_mask && (kend % kNumcKC == 0 || t + 1 == ntiles)) {
#pragma unroll
        for (int i = 0; i < TM; i++)
#pragma unroll
          for (int j = 0; j < TN; j++)
            if ((edge_mask >> (i * TN + j)) & 1u) {
              bsum[i][j] = edge_blk == 0 ? acc[i][j] : add_rn<Acc>(bsum[i][j], acc[i][j]);
              acc[i][j] = Acc(0);
            }
        edge_blk++;
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
      else if constexpr (kEdges) v = (T)(((edge_mask >> (i * TN + j)) & 1u) ? bsum[i][j] : acc[i][j]);
      else v = (T)acc[i][j];
      if (g.bias) v = add_elem<T>(v, ((const T *)g.bias)[gj * g.bias_stride]);
      C[gi * g.rso + gj * g.cso] = v;
    }
  }
}

// ---- numc's packed-path remainder tiles (floats) --------------------------
//
// Only the last, partial MC block of rows and the last, partial NR tile of
// the last NC-column panel hold remainder tiles (MC and NC are multiples of
// the tile sizes): rows from edge_row(M), columns from edge_col(N).  Their outputs are recomputed after the GEMM kernel: each
// 256-deep K block as an FMA chain from zero, added to the running value.

// Short K or many problems: remainder outputs in groups of 16 consecutive
// columns of one row: first
// the rows >= r0 (all columns, ceil(N / 16) groups a row), then the rows
// < r0 (columns c0..N-1, at most 15: one group a row).  A half-warp takes a
// group, one output a lane, so its loads of B are consecutive and its loads
// of A one address.
template <typename T>
__host__ __device__ inline int64_t float_edge_groups(int64_t M, int64_t N, int isa) {
  const int64_t r0 = edge_row<T>(M, isa), c0 = edge_col<T>(N, isa);
  return (M - r0) * ((N + 15) / 16) + (c0 < N ? r0 : 0);
}

// Output `sub` (0..15) of remainder group `gi`: each 256-deep K block as an
// FMA chain from zero, the block sums added in K order (numc's remainder
// tiles).  Lanes past the last column return.
// One numc K block of an output as an FMA chain from zero, k = pc .. pe-1
// in order.  The operands are fetched 32 steps ahead into registers so the
// chain waits for memory once per 32 steps, not once per step (for the
// few-output, latency-bound fix-up; 232 registers a thread).
template <typename T>
__device__ __forceinline__ T chain_block(const T *A, int64_t csa, const T *B, int64_t rsb,
                                         int64_t pc, int64_t pe) {
  constexpr int U = 32;
  T t = T(0);
#pragma unroll 1
  for (int64_t k0 = pc; k0 < pe; k0 += U) {
    T av[U], bv[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const bool in = k0 + u < pe;
      av[u] = in ? A[(k0 + u) * csa] : T(0);
      bv[u] = in ? B[(k0 + u) * rsb] : T(0);
    }
#pragma unroll
    for (int u = 0; u < U; u++)
      if (k0 + u < pe) t = madd<T>(av[u], bv[u], t);
  }
  return t;
}

template <typename T>
__device__ __forceinline__ void float_edge_output(const Gemm &g, int64_t gi, int sub, int64_t r0,
                                                  int64_t c0) {
  const int64_t nb = (g.N + 15) / 16, nbottom = (g.M - r0) * nb;
  int64_t i, j;
  if (gi < nbottom) {
    i = r0 + gi / nb;
    j = (gi % nb) * 16 + sub;
  } else {
    i = gi - nbottom;
    j = c0 + sub;
  }
  if (j >= g.N) return;
  const T *A = (const T *)g.a + i * g.rsa, *B = (const T *)g.b + j * g.csb;
  T d = T(0);
  for (int64_t pc = 0; pc < g.K; pc += kNumcKC) {
    const int64_t pe = min(pc + (int64_t)kNumcKC, g.K);
    T t = T(0);
#pragma unroll 8
    for (int64_t k = pc; k < pe; k++) t = madd<T>(A[k * g.csa], B[k * g.rsb], t);
    d = pc == 0 ? t : add_rn<T>(d, t);
  }
  if (g.bias) d = add_elem<T>(d, ((const T *)g.bias)[j * g.bias_stride]);
  ((T *)g.c)[i * g.rso + j * g.cso] = d;
}

// Lanes per remainder output: lane l of a group sums K blocks l, l + 8, ...
constexpr int kEdgeLanes = 8;

// Long K (several blocks an output, few outputs): output e of the
// remainder set (rows >= r0: all columns; then rows < r0: columns >= c0),
// computed by a group of kEdgeLanes lanes of one warp: each
// lane runs its K blocks as FMA chains from zero and the group folds the
// block sums in K order (d = t0, then d = d + t1, ...) — numc's per-block
// accumulation with the blocks computed in parallel.  Every lane of the
// warp calls this with the same K (the fold shuffles across the warp);
// `valid` is false for lanes past the last output.
template <typename T>
__device__ __forceinline__ void float_edge_output_lanes(const Gemm &g, int64_t e, bool valid, int64_t r0,
                                                  int64_t c0) {
  const int lane = threadIdx.x & 31, sub = lane & (kEdgeLanes - 1), base = lane & ~(kEdgeLanes - 1);
  int64_t i = 0, j = 0;
  if (valid) {
    const int64_t nbottom = (g.M - r0) * g.N;
    if (e < nbottom) {
      i = r0 + e / g.N;
      j = e % g.N;
    } else {
      const int64_t w = g.N - c0;
      i = (e - nbottom) / w;
      j = c0 + (e - nbottom) % w;
    }
  }
  const T *A = (const T *)g.a + i * g.rsa, *B = (const T *)g.b + j * g.csb;
  const int64_t nkb = (g.K + kNumcKC - 1) / kNumcKC;
  T d = T(0);
  for (int64_t r = 0; r < nkb; r += kEdgeLanes) {
    const int64_t kb = r + sub;
    T t = T(0);
    if (valid && kb < nkb) {
      const int64_t pc = kb * kNumcKC, pe = min(pc + (int64_t)kNumcKC, g.K);
      t = chain_block<T>(A, g.csa, B, g.rsb, pc, pe);
    }
#pragma unroll
    for (int q = 0; q < kEdgeLanes; q++) {
      const T v = __shfl_sync(0xffffffffu, t, base + q);
      if (r + q < nkb) d = r + q == 0 ? v : add_rn<T>(d, v);
    }
  }
  if (valid && sub == 0) {
    if (g.bias) d = add_elem<T>(d, ((const T *)g.bias)[j * g.bias_stride]);
    ((T *)g.c)[i * g.rso + j * g.cso] = d;
  }
}

// Remainder outputs exist only where the packed path ran more than one K
// block: with K <= 256 every remainder output is a single FMA chain from
// zero, which the tile kernel already produced.
template <typename T>
__host__ __device__ inline bool float_edges_needed(int64_t K) { return K > kNumcKC; }

template <typename T>
__host__ __device__ inline int64_t float_edge_count(int64_t M, int64_t N, int isa) {
  const int64_t r0 = edge_row<T>(M, isa), c0 = edge_col<T>(N, isa);
  return (M - r0) * N + r0 * (N - c0);
}

}  // namespace simt
}  // namespace numc_k

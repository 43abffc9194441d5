// float64 GEMM by Ozaki slicing on the tcgen05 tensor cores — the fast
// alternative to numc's FP64 FMA GEMM (src/intrinsics/gemm_avx2.h:1377
// gemm_f64_avx2); GB300's FP64 pipes run at ~1.2 TFLOP/s.
//
// Ozaki, Ogita, Oishi and Rump, "Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59 (2012): split each operand into
// slices whose pairwise products are computed exactly, then recombine.
//
// Slicing (per row i of A, per column j of B): e_i is the binary exponent
// with max_k |a_ik| < 2^e_i; x = a_ik 2^-e_i lies in (-1, 1) and is cut into
// s slices of 8 bits by truncation, x = sum_p sigma_p 2^-8(p+1) + r with
// integer |sigma_p| <= 255 (exact in bfloat16's 8-bit significand,
// |r| < 2^-8s).  B likewise.  The slice product matrices
// sum_k sigma^A_p sigma^B_q are integers: bf16 x bf16 products are exact in
// FP32 and so is every partial sum below 2^24, so each TMEM accumulation
// chain is limited to 4 K slabs of 64 (at most 256 * 255^2 < 2^24).
// Products are kept for p + q <= s - 1 (s(s+1)/2 of them, the usual
// triangular truncation).
//
// Recombination is done in integers: products with the same diagonal
// D = p + q share the weight 2^-8(D+2), so T = sum_D S_D 2^8(s-1-D) is an
// integer and the result is T 2^(e_i + f_j - 8(s+1)).  The accumulator
// warps evaluate T by Horner's rule, diagonal by diagonal from the top,
// in one int64 per output: acc = acc * 2^8 + S_D, exactly, while the
// thread's largest |acc| stays below 2^53; past that the thread instead
// drops 8 more low bits of the incoming diagonals (acc stays, later S_D are
// added rounded to multiples of 2^d, d counted per thread).  So every
// output keeps at least 53 bits relative to the largest output of its
// 32-column group, whatever K and s.  The only floating-point steps are the
// final int64 -> float64 conversion (one rounding) and the exact
// power-of-two rescale by 2^(d + e_i + f_j - 8(s+1)).
//
// Kernels: row/column absolute maxima (atomicMax on the bit patterns),
// slicing into s K-major bf16 planes per operand (B transposed), and the
// GEMM.  The default (ozaki_pair_gemm): persistent clusters of two CTAs on
// 256 x 128 output tiles, one (A_p, B_q) 64-deep slab pair per ring stage,
// cta_group::2 MMAs into two TMEM chunk buffers, the int64 Horner
// accumulators held in TMEM and each diagonal's chunk sums kept as exact
// FP32 partials (see the kernel).  ozaki_gemm (NUMC_CUDA_OZAKI_CTAS=1): one
// 128 x 128 output tile per CTA; warp 0 streams one slab pair per ring
// stage with TMA; warp 1 issues 4 tcgen05.mma (M = N = 128) per stage into
// one of four TMEM buffers (one buffer per chunk); warps 2-17 (four per
// TMEM lane quarter, 32 columns each) fold finished chunks into int64
// accumulators in registers and store.  Both are bound by the L2 -> shared
// memory operand stream: every diagonal fetches its slab pairs again.
// Non-finite inputs are flagged and their tiles recomputed with FP64 FMA
// chains (numc's arithmetic).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <atomic>
#include <cstdlib>
#include <algorithm>
#include <cmath>
#include <cstdint>

#include "kernels.h"
#include "phase_timing.h"
#include "status.h"
#include "tc_common.cuh"

namespace numc_k {
namespace {

constexpr int kBM = 128, kBN = 128, kBK = 64;
constexpr int kStages = 6;             // 32 KiB a stage
constexpr int kChunkSlabs = 4;         // 4 * 64 * 255^2 < 2^24
constexpr int kAccWarps = 16;          // 4 per TMEM lane quarter, 32 columns each
constexpr int kThreads = 64 + 32 * kAccWarps;
constexpr int kNumBuf = 4;             // 4 x 128 TMEM columns
constexpr int kMaxSlices = 8;

inline int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

// Bit tests on float64 values: GB300's FP64 pipe is slow, so compares on
// doubles are done on their IEEE bit patterns in the integer pipes.
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ bool finite_bits(unsigned long long a) {
  return a < 0x7FF0000000000000ull;
}
// frexp exponent of a non-negative finite double given as bits (0 for 0):
// x = m 2^e with m in [0.5, 1).
__device__ __forceinline__ int frexp_exp_bits(unsigned long long a) {
  if (a == 0) return 0;
  const int field = (int)(a >> 52);
  if (field) return field - 1022;
  return (64 - __clzll((long long)a)) - 1074;   // subnormal: a * 2^-1074
}

// ---- pass 1: row maxima of |A|, column maxima of |B| -----------------------
// out[row] = max over k of |src[row * rs_row + k * rs_k]| as IEEE bits
// (atomicMax on the bit pattern orders non-negative doubles).  Non-finite
// values set the row group's flag to `gen`.
__global__ void __launch_bounds__(256)
absmax_rows(const double *__restrict__ src, int64_t rs_row, int64_t rs_k, int64_t R, int64_t K,
            unsigned long long *out, unsigned long long *flags, int flag_rows,
            unsigned long long gen) {
  __shared__ unsigned long long rmax[32];
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 128;
  const int tid = threadIdx.x;
  if (tid < 32) rmax[tid] = 0;
  __syncthreads();
  const bool kfast = rs_k == 1 || rs_row != 1;
  bool bad = false;
#pragma unroll 4
  for (int q = 0; q < 16; q++) {
    int e = tid + 256 * q;
    int r = kfast ? e / 128 : e % 32;
    int k = kfast ? e % 128 : e / 32;
    int64_t gr = r0 + r, gk = k0 + k;
    if (gr < R && gk < K) {
      const unsigned long long ax = abs_bits(src[gr * rs_row + gk * rs_k]);
      if (!finite_bits(ax)) bad = true;
      else if (ax) atomicMax(&rmax[r], ax);
    }
  }
  if (__syncthreads_or(bad) && tid == 0) flags[r0 / flag_rows] = gen;
  if (tid < 32 && r0 + tid < R && rmax[tid]) atomicMax(&out[r0 + tid], rmax[tid]);
}

// ---- pass 2: slices ------------------------------------------------------------
// planes[p][row][k] = sigma_p of src(row, k) 2^-e_row, K-major, zero for
// k >= K.  32 rows x 64 k per block through shared memory.
//
// Integer extraction instead of FP64 arithmetic (GB300's FP64 pipes are
// slow): with |a| = m 2^(ea - 52) (m the 53-bit significand), the fixed-point
// value X = trunc(|a| 2^(8s - e)) = m shifted by (ea - 52 - e + 8s) bits,
// and sigma_p = +-((X >> 8(s-1-p)) & 255).  Truncating |x| and restoring the
// sign equals slicing x by truncation toward zero.
__device__ __forceinline__ uint64_t fixed_point(double a, int e, int s) {
  const uint64_t bits = (uint64_t)__double_as_longlong(a) & 0x7FFFFFFFFFFFFFFFull;
  const int field = (int)(bits >> 52);
  if (field == 0 && bits == 0) return 0;
  uint64_t m = bits & 0xFFFFFFFFFFFFFull;
  int ea = field - 1023;
  if (field) m |= 1ull << 52;
  else ea = -1022;                       // subnormal: no implicit bit
  const int sh = ea - 52 - e + 8 * s;    // X = m * 2^sh, X < 2^(8s) <= 2^64
  if (sh >= 0) return m << sh;
  return -sh >= 64 ? 0 : (m >> -sh);
}

__global__ void __launch_bounds__(256)
slice_f64(const double *__restrict__ src, int64_t rs_row, int64_t rs_k, int64_t R, int64_t K,
          int64_t Kp, const unsigned long long *__restrict__ maxbits, int slices,
          __nv_bfloat16 *__restrict__ planes) {
  __shared__ double tile[32][65];
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 64;
  const int tid = threadIdx.x;
  const bool kfast = rs_k == 1 || rs_row != 1;
#pragma unroll
  for (int q = 0; q < 8; q++) {
    int e = tid + 256 * q;
    int r = kfast ? e / 64 : e % 32;
    int k = kfast ? e % 64 : e / 32;
    int64_t gr = r0 + r, gk = k0 + k;
    double x = (gr < R && gk < K) ? src[gr * rs_row + gk * rs_k] : 0.0;
    tile[r][k] = finite_bits(abs_bits(x)) ? x : 0.0;
  }
  __syncthreads();
  const int64_t plane = R * Kp;
  const int warp = tid >> 5, lane = tid & 31;
#pragma unroll
  for (int rr = 0; rr < 4; rr++) {
    const int r = warp + 8 * rr;
    const int64_t gr = r0 + r;
    if (gr >= R) continue;
    const int ex = frexp_exp_bits(maxbits[gr]);
    const int64_t gk = k0 + 2 * lane;
    const double x0 = tile[r][2 * lane], x1 = tile[r][2 * lane + 1];
    const uint64_t X0 = fixed_point(x0, ex, slices), X1 = fixed_point(x1, ex, slices);
    const bool n0 = __double_as_longlong(x0) < 0, n1 = __double_as_longlong(x1) < 0;
    for (int p = 0; p < slices; p++) {
      const int sh = 8 * (slices - 1 - p);
      const int s0 = (int)((X0 >> sh) & 255), s1 = (int)((X1 >> sh) & 255);
      *reinterpret_cast<__nv_bfloat162 *>(planes + p * plane + gr * Kp + gk) =
          __halves2bfloat162(__int2bfloat16_rn(n0 ? -s0 : s0), __int2bfloat16_rn(n1 ? -s1 : s1));
    }
  }
}

// ---- pass 3: the slice-product GEMM --------------------------------------------

struct OzParams {
  const unsigned long long *amax, *bmax;   // max |a| per row, max |b| per column (bits)
  const unsigned long long *flags_a, *flags_b;
  unsigned long long gen;
  const double *A, *B;                     // originals, for non-finite tiles
  int64_t rsa, csa, rsb, csb, K;
  int slices;
};

__device__ __forceinline__ int exponent_of(unsigned long long bits) {
  return frexp_exp_bits(bits);
}

// 320 threads: registers are granted per group of four warps, so at most 168
// per thread; an accumulator thread holds 32 int64 sums (64 registers).
__global__ void __launch_bounds__(kThreads, 1)
ozaki_gemm(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB,
           double *__restrict__ C, int64_t rso, int64_t cso, int M, int N, int num_kb,
           int tiles_m, int tiles_n, unsigned *status, OzParams op, WaitCfg wc) {
  constexpr uint32_t A_BYTES = kBM * kBK * 2, B_BYTES = kBN * kBK * 2;
  constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *bars = (uint64_t *)(smem + kStages * STAGE_BYTES);
  uint64_t *full = bars, *empty = bars + kStages;
  uint64_t *tfull = bars + 2 * kStages, *tempty = tfull + kNumBuf;
  uint64_t *drain = tempty + kNumBuf;   // all issued MMAs complete
  uint32_t *tmem_slot = (uint32_t *)(drain + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = op.slices;

  const int tile = blockIdx.x;
  constexpr int GM = 16;
  const int group = tile / (GM * tiles_n);
  const int first_m = group * GM;
  const int gm = min(tiles_m - first_m, GM);
  const int local = tile - group * GM * tiles_n;
  const int m0 = (first_m + local % gm) * kBM;
  const int n0 = (local / gm) * kBN;

  if (threadIdx.x == 0) {
    for (int i = 0; i < kStages; i++) {
      tc::mbar_init(tc::smem_u32(&full[i]), 1);
      tc::mbar_init(tc::smem_u32(&empty[i]), 1);
    }
    for (int b = 0; b < kNumBuf; b++) {
      tc::mbar_init(tc::smem_u32(&tfull[b]), 1);
      tc::mbar_init(tc::smem_u32(&tempty[b]), kAccWarps);
    }
    tc::mbar_init(tc::smem_u32(drain), 1);
    tc::fence_barrier_init();
    tc::tma_prefetch_desc(&tA);
    tc::tma_prefetch_desc(&tB);
  }
  if (warp == 1) tc::tmem_alloc(tc::smem_u32(tmem_slot), kNumBuf * kBN);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  // Stage sequence: diagonal D = 0..s-1, K slab kb, pair (p, D - p); a chunk
  // is up to kChunkSlabs consecutive stages of one diagonal.
  if (warp == 0) {
    if (lane == 0) {
      int g = 0;   // global stage counter
      bool live = true;
      for (int D = 0; D < s && live; D++)
        for (int kb = 0; kb < num_kb && live; kb++)
          for (int p = 0; p <= D; p++, g++) {
            const int st = g % kStages;
            if (g >= kStages &&
                !tc::mbar_wait_bounded(tc::smem_u32(&empty[st]), ((g / kStages) & 1) ^ 1,
                                       status, kStatusTimeoutProducer, wc.limit_ns)) {
              live = false;
              break;
            }
            if (wc.starve) continue;   // give-up test: no load, no barrier completes
            const uint32_t fbar = tc::smem_u32(&full[st]);
            const uint32_t sa = tc::smem_u32(smem + st * STAGE_BYTES);
            tc::mbar_arrive_expect_tx(fbar, STAGE_BYTES);
            tc::tma_load_3d(sa, &tA, fbar, kb * kBK, m0, p);
            tc::tma_load_3d(sa + A_BYTES, &tB, fbar, kb * kBK, n0, D - p);
          }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_bf16_f32(kBM, kBN);
      int g = 0, chunk = 0;
      bool live = true;
      for (int D = 0; D < s && live; D++) {
        const int stages_d = num_kb * (D + 1);
        for (int i = 0; i < stages_d && live; i++, g++) {
          const int st = g % kStages;
          const bool cstart = i % kChunkSlabs == 0;
          const bool cend = i % kChunkSlabs == kChunkSlabs - 1 || i == stages_d - 1;
          const int buf = chunk % kNumBuf;
          if (cstart && chunk >= kNumBuf &&
              !tc::mbar_wait_bounded(tc::smem_u32(&tempty[buf]), ((chunk / kNumBuf) & 1) ^ 1,
                                     status, kStatusTimeoutMma, wc.limit_ns)) {
            live = false;
            break;
          }
          if (!tc::mbar_wait_bounded(tc::smem_u32(&full[st]), (g / kStages) & 1, status,
                                     kStatusTimeoutMma, wc.limit_ns)) {
            live = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t sa = tc::smem_u32(smem + st * STAGE_BYTES), sb = sa + A_BYTES;
#pragma unroll
          for (int kk = 0; kk < kBK / 16; kk++) {
            const uint32_t acc = (!cstart || kk > 0) ? 1u : 0u;
            tc::mma_bf16(tmem + buf * kBN, tc::sdesc_k128(sa + kk * 32),
                         tc::sdesc_k128(sb + kk * 32), idesc, acc);
          }
          tc::mma_commit(tc::smem_u32(&empty[st]));
          if (cend) {
            tc::mma_commit(tc::smem_u32(&tfull[buf]));
            chunk++;
          }
        }
      }
      // Every MMA issued above completes before TMEM is released, also when
      // the loop gave up (a commit with none outstanding arrives at once).
      tc::mma_commit(tc::smem_u32(drain));
      tc::mbar_wait_bounded(tc::smem_u32(drain), 0, status, kStatusTimeoutDrain, wc.limit_ns);
    }
    __syncwarp();
  } else {
    constexpr int CW = kBN / 4;   // 32 columns per thread (the bit-drop group)
    const int quad = warp & 3, quarter = (warp - 2) >> 2;
    const int row = m0 + quad * 32 + lane;
    const int cbase = quarter * CW;
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    long long acc[CW];
#pragma unroll
    for (int j = 0; j < CW; j++) acc[j] = 0;
    bool ok = true;
    int chunk = 0;
    int drop = 0;   // low bits dropped so far (acc holds T / 2^drop)
    for (int D = 0; D < s && ok; D++) {
      const int stages_d = num_kb * (D + 1);
      const int nchunks = (stages_d + kChunkSlabs - 1) / kChunkSlabs;
      if (D > 0) {
        // Horner step: acc *= 2^8 if it stays exact, else drop 8 more bits.
        unsigned long long mx = 0;
#pragma unroll
        for (int j = 0; j < CW; j++) {
          const unsigned long long m = (unsigned long long)(acc[j] < 0 ? -acc[j] : acc[j]);
          mx = m > mx ? m : mx;
        }
        if (mx < (1ull << 53)) {
#pragma unroll
          for (int j = 0; j < CW; j++) acc[j] *= 256;
        } else {
          drop += 8;
        }
      }
      const int sh = drop;   // this diagonal's sums enter as round(S / 2^drop)
      for (int c = 0; c < nchunks; c++, chunk++) {
        const int buf = chunk % kNumBuf;
        ok = tc::mbar_wait_bounded(tc::smem_u32(&tfull[buf]), (chunk / kNumBuf) & 1, status,
                                   kStatusTimeoutEpilogue, wc.limit_ns);
        ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld below is warp-collective
        if (!ok) break;
        tc::tc_fence_after();
#pragma unroll
        for (int c0 = 0; c0 < CW; c0 += 16) {   // 16 columns a load: fewer live registers
          uint32_t r[16];
          tc::tmem_ld_32x32b_x16(tmem + lane_off + buf * kBN + cbase + c0, r);
          tc::tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 16; j++) {
            const long long v = (long long)__float2int_rn(__uint_as_float(r[j]));  // exact
            acc[c0 + j] += sh == 0 ? v : (sh >= 63 ? 0 : ((v + (1ll << (sh - 1))) >> sh));
          }
        }
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(tc::smem_u32(&tempty[buf]));
      }
    }

    bool nonfinite = op.flags_a[m0 / kBM] == op.gen;
#pragma unroll 1
    for (int c = n0 / 64; c < (n0 + kBN) / 64 && c * 64 < N; c++)
      nonfinite |= op.flags_b[c] == op.gen;
    if (ok && row < M) {
      if (nonfinite) {
        // numc's arithmetic: one FMA chain per output in k order.
#pragma unroll 1
        for (int j = 0; j < CW; j++) {
          const int col = n0 + cbase + j;
          if (col >= N) break;
          double f = 0.0;
#pragma unroll 1
          for (int64_t k = 0; k < op.K; k++)
            f = __fma_rn(op.A[(int64_t)row * op.rsa + k * op.csa],
                         op.B[k * op.rsb + (int64_t)col * op.csb], f);
          C[(int64_t)row * rso + (int64_t)col * cso] = f;
        }
      } else {
        const int ea = exponent_of(op.amax[row]);
        const int base = ea + drop - 8 * (s + 1);
#pragma unroll
        for (int j = 0; j < CW; j++) {
          const int col = n0 + cbase + j;
          if (col < N) {
            const int eb = exponent_of(op.bmax[col]);
            C[(int64_t)row * rso + (int64_t)col * cso] =
                ldexp(__ll2double_rn(acc[j]), base + eb);
          }
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, kNumBuf * kBN);
  }
}

// ---- CTA pairs -------------------------------------------------------------------
//
// The default GEMM: clusters of two CTAs walk 256 x 128 output tiles
// persistently; each CTA loads its 128 rows of A_p and 64 rows of B_q^T per
// 64-deep slab (24 KiB, against 32 KiB for the same multiply-adds on one
// CTA) and the even CTA's MMA thread multiplies both halves with
// cta_group::2 MMAs.  TMEM per CTA: two 128-column FP32 chunk buffers and
// 256 columns holding the 128 x 128 int64 Horner accumulators (low word,
// high word), so that the accumulator threads keep only a diagonal's
// partial sums in registers, as two FP32 integers per output: each chunk
// sum S (an integer below 2^24) is split as S = 4096 h + l with
// h = round(S / 4096) and |l| <= 2048 (one FMA and one add each, exact),
// and H += h, L += l stay exact for up to 2048 chunks.  The float-to-int
// conversions (a quarter of the FP32 rate) run once per diagonal instead
// of once per chunk.  At a diagonal's end: acc = acc * 2^8 + round((4096 H
// + L) / 2^drop), with the same bit-drop rule as the single-CTA kernel but
// rounding the diagonal's sum once (never less accurate).
constexpr int kPairBN = 128, kPairBNCta = 64;
constexpr int kPairStages = 8;              // 24 KiB a stage
constexpr int kPairNumBuf = 2;              // 2 x 128 TMEM columns of chunk sums
constexpr uint32_t kPairAccCol = 256;       // int64 accumulators: columns 256..511
constexpr int kPairFlushChunks = 2048;      // H, L exact up to here

__global__ void __launch_bounds__(kThreads, 1)
ozaki_pair_gemm(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB,
                double *__restrict__ C, int64_t rso, int64_t cso, int M, int N, int num_kb,
                int tiles_m, int tiles_n, unsigned *status, OzParams op, WaitCfg wc) {
  constexpr uint32_t A_BYTES = kBM * kBK * 2, B_BYTES = kPairBNCta * kBK * 2;
  constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
  constexpr int NBUF = kPairNumBuf;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *bars = (uint64_t *)(smem + kPairStages * STAGE_BYTES);
  uint64_t *full = bars, *empty = bars + kPairStages;
  uint64_t *tfull = bars + 2 * kPairStages, *tempty = tfull + NBUF;
  uint64_t *drain = tempty + NBUF;   // all issued MMAs complete
  uint32_t *tmem_slot = (uint32_t *)(drain + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = op.slices;
  const int ntiles = tiles_m * tiles_n;
  const uint32_t rank = tc::cluster_ctarank();
  const bool leader = rank == 0;
  const int first_tile = blockIdx.x / 2, tile_step = gridDim.x / 2;
  auto tile_origin = [&](int t, int &m0, int &n0) {
    constexpr int GM = 8;   // 2048 rows of pair tiles
    const int group = t / (GM * tiles_n);
    const int first_m = group * GM;
    const int gm = min(tiles_m - first_m, GM);
    const int local = t - group * GM * tiles_n;
    m0 = (first_m + local % gm) * (2 * kBM);
    n0 = (local / gm) * kPairBN;
  };

  if (threadIdx.x == 0) {
    for (int i = 0; i < kPairStages; i++) {
      tc::mbar_init(tc::smem_u32(&full[i]), 1);
      tc::mbar_init(tc::smem_u32(&empty[i]), 1);
    }
    for (int b = 0; b < NBUF; b++) {
      tc::mbar_init(tc::smem_u32(&tfull[b]), 1);
      tc::mbar_init(tc::smem_u32(&tempty[b]), kAccWarps * 2);   // both CTAs' warps
    }
    tc::mbar_init(tc::smem_u32(drain), 1);
    tc::fence_barrier_init();
    tc::tma_prefetch_desc(&tA);
    tc::tma_prefetch_desc(&tB);
  }
  if (warp == 1) tc::tmem_alloc_pair(tc::smem_u32(tmem_slot), 512);
  tc::tc_fence_before();
  __syncthreads();
  tc::cluster_sync();   // peer barriers initialised
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  tc::griddep_wait();   // the slicing passes have completed

  // Stage sequence per tile: diagonal D = 0..s-1, K slab kb, pair (p, D - p);
  // a chunk is up to kChunkSlabs consecutive stages of one diagonal.
  if (warp == 0) {
    if (lane == 0) {
      int g = 0;   // stage counter across tiles
      bool live = true;
      for (int t = first_tile; t < ntiles && live; t += tile_step) {
        int m0, n0;
        tile_origin(t, m0, n0);
        const int ma = m0 + (int)rank * kBM, nb = n0 + (int)rank * kPairBNCta;
        for (int D = 0; D < s && live; D++)
          for (int kb = 0; kb < num_kb && live; kb++)
            for (int p = 0; p <= D; p++, g++) {
              const int st = g % kPairStages;
              if (g >= kPairStages &&
                  !tc::mbar_wait_bounded(tc::smem_u32(&empty[st]), ((g / kPairStages) & 1) ^ 1,
                                         status, kStatusTimeoutProducer, wc.limit_ns)) {
                live = false;
                break;
              }
              if (wc.starve) continue;   // give-up test: no load, no barrier completes
              const uint32_t fbar = tc::smem_u32(&full[st]);
              const uint32_t sa = tc::smem_u32(smem + st * STAGE_BYTES);
              // the even CTA's full barrier counts the bytes of both CTAs
              if (leader) tc::mbar_arrive_expect_tx(fbar, 2 * STAGE_BYTES);
              const uint32_t fbar_leader = tc::mapa_shared(fbar, 0);
              tc::tma_load_3d_pair(sa, &tA, fbar_leader, kb * kBK, ma, p);
              tc::tma_load_3d_pair(sa + A_BYTES, &tB, fbar_leader, kb * kBK, nb, D - p);
            }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0 && leader) {
      constexpr uint32_t idesc = tc::idesc_bf16_f32(2 * kBM, kPairBN);
      int g = 0, chunk = 0;
      bool live = true;
      for (int t = first_tile; t < ntiles && live; t += tile_step) {
        for (int D = 0; D < s && live; D++) {
          const int stages_d = num_kb * (D + 1);
          for (int i = 0; i < stages_d && live; i++, g++) {
            const int st = g % kPairStages;
            const bool cstart = i % kChunkSlabs == 0;
            const bool cend = i % kChunkSlabs == kChunkSlabs - 1 || i == stages_d - 1;
            const int buf = chunk % NBUF;
            if (cstart && chunk >= NBUF &&
                !tc::mbar_wait_bounded(tc::smem_u32(&tempty[buf]), ((chunk / NBUF) & 1) ^ 1,
                                       status, kStatusTimeoutMma, wc.limit_ns)) {
              live = false;
              break;
            }
            if (!tc::mbar_wait_bounded(tc::smem_u32(&full[st]), (g / kPairStages) & 1, status,
                                       kStatusTimeoutMma, wc.limit_ns)) {
              live = false;
              break;
            }
            tc::tc_fence_after();
            const uint32_t sa = tc::smem_u32(smem + st * STAGE_BYTES), sb = sa + A_BYTES;
#pragma unroll
            for (int kk = 0; kk < kBK / 16; kk++)
              tc::mma_f16_pair(tmem + buf * kPairBN, tc::sdesc_k128(sa + kk * 32),
                               tc::sdesc_k128(sb + kk * 32), idesc,
                               (!cstart || kk > 0) ? 1u : 0u);
            tc::mma_commit_pair(tc::smem_u32(&empty[st]), 0x3);
            if (cend) {
              tc::mma_commit_pair(tc::smem_u32(&tfull[buf]), 0x3);
              chunk++;
            }
          }
        }
      }
      // Every MMA issued above completes before TMEM is released, also when
      // the loop gave up (a commit with none outstanding arrives at once).
      tc::mma_commit_pair(tc::smem_u32(drain), 0x1);
      tc::mbar_wait_bounded(tc::smem_u32(drain), 0, status, kStatusTimeoutDrain, wc.limit_ns);
    }
    __syncwarp();
  } else {
    constexpr int CW = kPairBN / 4;   // 32 columns per thread (the bit-drop group)
    const int quad = warp & 3, quarter = (warp - 2) >> 2;
    const int cbase = quarter * CW;
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    const uint32_t acc_addr = tmem + lane_off + kPairAccCol + 2 * cbase;
    constexpr float kMagic = 12582912.0f;   // 1.5 x 2^23: adding it rounds to an integer
    int chunk = 0;                          // across tiles
    bool ok = true;
    for (int t = first_tile; t < ntiles && ok; t += tile_step) {
      int m0, n0;
      tile_origin(t, m0, n0);
      const int mr = m0 + (int)rank * kBM;   // this CTA's 128 rows
      const int row = mr + quad * 32 + lane;
      int drop = 0;                  // low bits dropped so far (acc holds T / 2^drop)
      unsigned long long mx = 0;     // largest |acc| of the thread after the last update
      for (int D = 0; D < s && ok; D++) {
        const int stages_d = num_kb * (D + 1);
        const int nchunks = (stages_d + kChunkSlabs - 1) / kChunkSlabs;
        // Horner step: acc *= 2^8 if it stays exact, else drop 8 more bits
        // of this and every later diagonal.
        bool mul = D > 0;
        if (D > 0 && mx >= (1ull << 53)) {
          mul = false;
          drop += 8;
        }
        const int sh = drop;
        for (int c0 = 0; c0 < nchunks && ok; c0 += kPairFlushChunks) {
          float H[CW], L[CW];
#pragma unroll
          for (int j = 0; j < CW; j++) H[j] = L[j] = 0.0f;
          const int c1 = min(nchunks, c0 + kPairFlushChunks);
          for (int c = c0; c < c1; c++, chunk++) {
            const int buf = chunk % NBUF;
            ok = tc::mbar_wait_bounded(tc::smem_u32(&tfull[buf]), (chunk / NBUF) & 1, status,
                                       kStatusTimeoutEpilogue, wc.limit_ns);
            ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld below is warp-collective
            if (!ok) break;
            tc::tc_fence_after();
#pragma unroll
            for (int q0 = 0; q0 < CW; q0 += 8) {   // 8 columns a load: H, L hold 64 registers
              uint32_t r[8];
              tc::tmem_ld_32x32b_x8(tmem + lane_off + buf * kPairBN + cbase + q0, r);
              tc::tmem_ld_wait();
#pragma unroll
              for (int j = 0; j < 8; j++) {
                const float v = __uint_as_float(r[j]);               // integer, |v| < 2^24
                const float h = __fmaf_rn(v, 1.0f / 4096.0f, kMagic) - kMagic;
                L[q0 + j] += __fmaf_rn(-h, 4096.0f, v);               // exact, |.| <= 2048
                H[q0 + j] += h;
              }
            }
            tc::tc_fence_before();
            __syncwarp();
            if (lane == 0)   // the buffer's loads completed at tcgen05.wait::ld
              tc::mbar_arrive_cluster_relaxed(tc::mapa_shared(tc::smem_u32(&tempty[buf]), 0));
          }
          if (!ok) break;
          // Fold the partial sums into the int64 accumulators held in TMEM
          // (4 outputs, 8 words, per access); the first fold of a diagonal
          // applies its Horner step.
          const bool first_fold = c0 == 0;
          unsigned long long nmx = 0;
#pragma unroll
          for (int g4 = 0; g4 < CW / 4; g4++) {
            uint32_t w[8];
            if (D > 0 || !first_fold) {
              tc::tmem_ld_32x32b_x8(acc_addr + 8 * g4, w);
              tc::tmem_ld_wait();
            } else {
#pragma unroll
              for (int i = 0; i < 8; i++) w[i] = 0;
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
              const int q = 4 * g4 + j;
              long long acc = (long long)(((unsigned long long)w[2 * j + 1] << 32) | w[2 * j]);
              if (first_fold && mul) acc *= 256;
              const long long S = (long long)__float2int_rn(H[q]) * 4096 +
                                  (long long)__float2int_rn(L[q]);
              acc += sh == 0 ? S : (sh >= 63 ? 0 : ((S + (1ll << (sh - 1))) >> sh));
              const unsigned long long a = (unsigned long long)(acc < 0 ? -acc : acc);
              nmx = a > nmx ? a : nmx;
              w[2 * j] = (uint32_t)acc;
              w[2 * j + 1] = (uint32_t)((unsigned long long)acc >> 32);
            }
            tc::tmem_st_32x32b_x8(acc_addr + 8 * g4, w);
          }
          tc::tmem_st_wait();
          mx = nmx;
        }
      }
      if (!ok) break;

      // (a pair's odd CTA may lie wholly below the last row: no flag there)
      bool nonfinite = mr < M && op.flags_a[mr / kBM] == op.gen;
#pragma unroll 1
      for (int c = n0 / 64; c < (n0 + kPairBN) / 64 && c * 64 < N; c++)
        nonfinite |= op.flags_b[c] == op.gen;
      if (nonfinite) {
        if (row < M) {
          // numc's arithmetic: one FMA chain per output in k order.
#pragma unroll 1
          for (int j = 0; j < CW; j++) {
            const int col = n0 + cbase + j;
            if (col >= N) break;
            double f = 0.0;
#pragma unroll 1
            for (int64_t k = 0; k < op.K; k++)
              f = __fma_rn(op.A[(int64_t)row * op.rsa + k * op.csa],
                           op.B[k * op.rsb + (int64_t)col * op.csb], f);
            C[(int64_t)row * rso + (int64_t)col * cso] = f;
          }
        }
      } else {
        const int base = (row < M ? exponent_of(op.amax[row]) : 0) + drop - 8 * (s + 1);
#pragma unroll
        for (int g4 = 0; g4 < CW / 4; g4++) {
          uint32_t w[8];
          tc::tmem_ld_32x32b_x8(acc_addr + 8 * g4, w);   // warp-collective
          tc::tmem_ld_wait();
          if (row < M) {
#pragma unroll
            for (int j = 0; j < 4; j++) {
              const int col = n0 + cbase + 4 * g4 + j;
              if (col < N) {
                const long long acc =
                    (long long)(((unsigned long long)w[2 * j + 1] << 32) | w[2 * j]);
                C[(int64_t)row * rso + (int64_t)col * cso] =
                    ldexp(__ll2double_rn(acc), base + exponent_of(op.bmax[col]));
              }
            }
          }
        }
      }
      tc::tc_fence_before();
      __syncwarp();   // reconverge before the next tile's tcgen05.ld
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  // Neither CTA of a pair leaves while the other may still signal its
  // barriers or read its shared memory.
  tc::cluster_sync();
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc_pair(tmem, 512);
  }
}

struct OzLayout {
  int64_t Kp;
  size_t amax, bmax, flags_a, flags_b, a, b, total;
};

OzLayout oz_layout(int64_t M, int64_t K, int64_t N, int s) {
  OzLayout L;
  L.Kp = round_up(K > 0 ? K : 1, kBK);
  L.amax = 0;
  L.bmax = (size_t)round_up(M * 8, 256);
  L.flags_a = L.bmax + (size_t)round_up(N * 8, 256);
  L.flags_b = L.flags_a + (size_t)round_up(((M + kBM - 1) / kBM) * 8, 256);
  L.a = L.flags_b + (size_t)round_up(((N + 63) / 64) * 8, 256);
  L.b = L.a + (size_t)round_up((int64_t)s * M * L.Kp * 2, 256);
  L.total = L.b + (size_t)round_up((int64_t)s * N * L.Kp * 2, 256);
  return L;
}

std::atomic<unsigned long long> g_oz_gen{0x0a2a000000000000ull};

// CTA pairs unless NUMC_CUDA_OZAKI_CTAS=1 asks for the single-CTA kernel
// (read once).
int ozaki_ctas() {
  static const int v = [] {
    const char *e = getenv("NUMC_CUDA_OZAKI_CTAS");
    return (e && atoi(e) == 1) ? 1 : 2;
  }();
  return v;
}

cudaError_t launch_ozaki_pair(const Gemm &g, const OzLayout &L, const __nv_bfloat16 *pa,
                              const __nv_bfloat16 *pb, unsigned *status, const OzParams &op,
                              cudaStream_t s) {
  CUtensorMap ta, tb;
  cudaError_t e;
  if ((e = make_tmap_3d(&ta, pa, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, op.slices, g.M, L.Kp,
                        L.Kp, kBM, kBK)))
    return e;
  if ((e = make_tmap_3d(&tb, pb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, op.slices, g.N, L.Kp,
                        L.Kp, kPairBNCta, kBK)))
    return e;
  constexpr uint32_t SMEM = kPairStages * (kBM + kPairBNCta) * kBK * 2 + 1024 + 256;
  static_assert(SMEM <= 232448, "shared memory");
  static_assert((2 * kPairStages + 2 * kPairNumBuf + 1) * 8 + 4 <= 256, "barrier space");
  static LaunchCache lc;
  if ((e = smem_attr_once(lc, (const void *)ozaki_pair_gemm, SMEM))) return e;
  const int tiles_m = (int)((g.M + 2 * kBM - 1) / (2 * kBM));
  const int tiles_n = (int)((g.N + kPairBN - 1) / kPairBN);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = SMEM;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3((unsigned)(2 * std::max(1, sm_count() / 2)));
  int pairs = clusters_once(lc, (const void *)ozaki_pair_gemm, cfg);
  if (pairs <= 0) pairs = std::max(1, sm_count() / 2);
  pairs = std::min(pairs, tiles_m * tiles_n);
  cfg.gridDim = dim3((unsigned)(2 * pairs));
  cfg.numAttrs = 2;
  e = cudaLaunchKernelEx(&cfg, ozaki_pair_gemm, ta, tb, (double *)g.c, (int64_t)g.rso,
                         (int64_t)g.cso, (int)g.M, (int)g.N, (int)(L.Kp / kBK), tiles_m, tiles_n,
                         status, op, wait_cfg());
  if (e != cudaSuccess) return e;
  count_launch();
  return cudaGetLastError();
}

}  // namespace

size_t ozaki_workspace(int64_t M, int64_t K, int64_t N, int slices) {
  return oz_layout(M, K, N, slices).total;
}

cudaError_t launch_ozaki(const Gemm &g, int slices, void *ws_v, size_t ws_bytes, cudaStream_t s) {
  if (g.M == 0 || g.N == 0) return cudaSuccess;
  if (g.K == 0) return launch_simt(NUMC_DTYPE_FLOAT64, g, 0, s);   // C = 0
  if (slices < 1 || slices > kMaxSlices) return cudaErrorInvalidValue;
  if (g.M >= (1ll << 31) || g.N >= (1ll << 31) || g.K >= (1ll << 31))
    return cudaErrorInvalidValue;
  const OzLayout L = oz_layout(g.M, g.K, g.N, slices);
  if (ws_bytes < L.total || ((uintptr_t)ws_v & 255)) return cudaErrorInvalidValue;
  char *ws = (char *)ws_v;
  unsigned *status = status_word();
  if (!status) return cudaErrorMemoryAllocation;
  PhaseMark mark(s);
  const unsigned long long gen = ++g_oz_gen;
  auto *amax = (unsigned long long *)(ws + L.amax), *bmax = (unsigned long long *)(ws + L.bmax);
  auto *fa = (unsigned long long *)(ws + L.flags_a), *fb = (unsigned long long *)(ws + L.flags_b);
  cudaError_t e = cudaMemsetAsync(ws, 0, L.flags_a, s);   // maxima start at +0
  if (e) return e;
  const double *A = (const double *)g.a, *B = (const double *)g.b;
  dim3 ma((unsigned)((g.K + 127) / 128), (unsigned)((g.M + 31) / 32));
  dim3 mb((unsigned)((g.K + 127) / 128), (unsigned)((g.N + 31) / 32));
  dim3 sa((unsigned)(L.Kp / 64), (unsigned)((g.M + 31) / 32));
  dim3 sb((unsigned)(L.Kp / 64), (unsigned)((g.N + 31) / 32));
  if (ma.y > 65535 || mb.y > 65535) return cudaErrorInvalidConfiguration;
  absmax_rows<<<ma, 256, 0, s>>>(A, g.rsa, g.csa, g.M, g.K, amax, fa, kBM, gen);
  absmax_rows<<<mb, 256, 0, s>>>(B, g.csb, g.rsb, g.N, g.K, bmax, fb, 64, gen);
  auto *pa = (__nv_bfloat16 *)(ws + L.a), *pb = (__nv_bfloat16 *)(ws + L.b);
  slice_f64<<<sa, 256, 0, s>>>(A, g.rsa, g.csa, g.M, g.K, L.Kp, amax, slices, pa);
  slice_f64<<<sb, 256, 0, s>>>(B, g.csb, g.rsb, g.N, g.K, L.Kp, bmax, slices, pb);
  count_launch(4);
  if ((e = cudaGetLastError())) return e;
  mark.split_done();

  OzParams op;
  op.amax = amax; op.bmax = bmax; op.flags_a = fa; op.flags_b = fb; op.gen = gen;
  op.A = A; op.B = B; op.rsa = g.rsa; op.csa = g.csa; op.rsb = g.rsb; op.csb = g.csb;
  op.K = g.K; op.slices = slices;
  if (ozaki_ctas() == 2) {
    e = launch_ozaki_pair(g, L, pa, pb, status, op, s);
    mark.gemm_done();
    return e;
  }
  CUtensorMap ta, tb;
  if ((e = make_tmap_3d(&ta, pa, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, slices, g.M, L.Kp, L.Kp,
                        kBM, kBK)))
    return e;
  if ((e = make_tmap_3d(&tb, pb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, slices, g.N, L.Kp, L.Kp,
                        kBN, kBK)))
    return e;
  constexpr uint32_t SMEM = kStages * (kBM + kBN) * kBK * 2 + 1024 + 256;
  static_assert(SMEM <= 232448, "shared memory");
  static_assert((2 * kStages + 2 * kNumBuf + 1) * 8 + 4 <= 256, "barrier space");
  static LaunchCache lc1;
  if ((e = smem_attr_once(lc1, (const void *)ozaki_gemm, SMEM))) return e;
  const int tiles_m = (int)((g.M + kBM - 1) / kBM), tiles_n = (int)((g.N + kBN - 1) / kBN);
  ozaki_gemm<<<tiles_m * tiles_n, kThreads, SMEM, s>>>(ta, tb, (double *)g.c, g.rso, g.cso,
                                                       (int)g.M, (int)g.N, (int)(L.Kp / kBK),
                                                       tiles_m, tiles_n, status, op,
                                                       wait_cfg());
  count_launch();
  e = cudaGetLastError();
  mark.gemm_done();
  return e;
}

}  // namespace numc_k

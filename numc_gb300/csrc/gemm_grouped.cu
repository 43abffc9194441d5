// Grouped float32 GEMM: many independent matmuls of uneven shape in a few
// launches, capturable in a CUDA graph.  numc has no grouped entry point —
// its callers loop numc_matmul (src/matmul/matmul.c:347) once per problem;
// this is the batched form of that loop.
//
// A plan (numc_cuda_gemm_plan_create) fixes the problems, picks a kernel
// variant per problem from the committed autotune table, lays out an owned
// device workspace, encodes one TMA descriptor per operand per problem and
// uploads per-variant tile lists.  Running it enqueues only:
//   1. a memset of the non-finite flags (and row / column maxima),
//   2. for scaled float16 planes (NUMC_CUDA_ALGO_SPLIT_FP16, the default),
//      one grouped scale pass: row maxima of every A, column maxima of
//      every B,
//   3. one grouped split pass over every tensor-core problem (x -> two
//      16-bit planes; a block reads its problem from a job table),
//   4. one persistent split tcgen05 kernel per tile width (128 or 64
//      columns): each CTA walks a static share of the variant's tile list;
//      the TMA ring, the MMA chunk stream and the TMEM buffers run on
//      across tiles, so a tile's stores overlap the next tile's MMAs,
//   5. one grouped CUDA-core kernel (FP32 FMA chains, numc's arithmetic)
//      for problems too small for the tensor path, and for the plain
//      algorithm.
// The tile lists are ordered by K, largest first, so the static
// round-robin finishes with short tiles.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "kernels.h"
#include "numc/cuda.h"
#include "numc/error.h"
#include "simt_common.cuh"
#include "split_common.cuh"
#include "status.h"
#include "tc_common.cuh"

namespace numc_k {
namespace grouped {

constexpr int kBM = 128, kBK = 64, kPlanes = 2;

// Device-side description of one problem.
struct Prob {
  const float *A, *B;
  float *C;
  int64_t rsa, csa, rsb, csb, rso, cso;
  int M, N, K, num_kb, Kp;
  int split_mode_a, split_mode_b;
  int isa;                                // CUDA-core problems: numc's tile geometry
  uint16_t *pa, *pb;                      // planes (2 x M x Kp, 2 x N x Kp)
  unsigned long long *flags_a, *flags_b;  // per 128 rows of A, per 64 columns of B
  unsigned *max_a, *max_b;                // float16 planes: row / column maxima
  int splits;                             // K slices (split-K; 1 = none)
  float *part;                            // split-K: splits x M x N partial sums
};

// One output tile; with split-K, slice `ks` of the problem's K slabs.
struct Tile {
  int prob, m0, n0, ks;
};

// K slabs [kb0, kb1) of slice ks of P (slices differ by at most one slab).
__host__ __device__ inline void slice_range(const Prob &P, int ks, int &kb0, int &kb1) {
  kb0 = (int)((int64_t)ks * P.num_kb / P.splits);
  kb1 = (int)((int64_t)(ks + 1) * P.num_kb / P.splits);
}

// ---- grouped scale pass (float16 planes) -----------------------------------------

// Block b handles scale job jobs[b] = (problem p, job j of p): the blocks of
// absmax_grid(M, K) over A's rows, then those of absmax_grid(N, K) over B's
// columns.
__global__ void __launch_bounds__(256)
grouped_absmax(const Prob *__restrict__ probs, const int2 *__restrict__ jobs) {
  const int2 job = jobs[blockIdx.x];
  const Prob &P = probs[job.x];
  long long j = job.y;
  const int ma = absmax_mode(P.split_mode_a, P.csa);
  const dim3 ga = absmax_grid(P.M, P.K, ma);
  const long long a_jobs = (long long)ga.x * ga.y;
  if (j < a_jobs) {
    absmax_block(P.A, P.rsa, P.csa, P.M, P.K, ma, P.max_a, j % ga.x, j / ga.x);
  } else {
    j -= a_jobs;
    const int mb = absmax_mode(P.split_mode_b, P.rsb);
    const dim3 gb = absmax_grid(P.N, P.K, mb);
    absmax_block(P.B, P.csb, P.rsb, P.N, P.K, mb, P.max_b, j % gb.x, j / gb.x);
  }
}

// ---- grouped split pass --------------------------------------------------------

// Block b handles split job jobs[b] = (problem p, job j of p): A tiles
// (ceil(M/32) x ceil(Kp/128)) come first, then B tiles.
template <bool F16>
__global__ void __launch_bounds__(256)
grouped_split(const Prob *__restrict__ probs, const int2 *__restrict__ jobs,
              unsigned long long gen) {
  __shared__ __align__(16) float tile[kSplitRows][kSplitK + 4];
  const int2 job = jobs[blockIdx.x];
  const Prob &P = probs[job.x];
  long long j = job.y;
  const long long kt = (P.Kp + kSplitK - 1) / kSplitK;
  const long long a_jobs = (long long)((P.M + kSplitRows - 1) / kSplitRows) * kt;
  if (j < a_jobs) {
    split_tile<kPlanes, F16>(P.A, P.rsa, P.csa, P.M, P.K, P.Kp, P.pa, P.flags_a, kBM, gen,
                             P.split_mode_a, (j / kt) * kSplitRows, (j % kt) * kSplitK, tile,
                             P.max_a);
  } else {
    j -= a_jobs;
    split_tile<kPlanes, F16>(P.B, P.csb, P.rsb, P.N, P.K, P.Kp, P.pb, P.flags_b, 64, gen,
                             P.split_mode_b, (j / kt) * kSplitRows, (j % kt) * kSplitK, tile,
                             P.max_b);
  }
}

// ---- fused scale and split (float16 planes) --------------------------------------

// One block: kFusedRows rows of one operand (A's rows, or B's columns as the
// rows of B^T) over the whole of K: each row's largest magnitude (the scale
// pass's result, stored for the GEMM's final rescale), then the two float16
// planes, from one launch and one DRAM read of the operand.  jobs[b] =
// (problem, block), A's blocks first.  kFusedRows and the block body:
// split_common.cuh.

__global__ void __launch_bounds__(256)
grouped_scale_split(const Prob *__restrict__ probs, const int2 *__restrict__ jobs,
                    unsigned long long gen) {
  const int2 job = jobs[blockIdx.x];
  const Prob &P = probs[job.x];
  const int a_blocks = (P.M + kFusedRows - 1) / kFusedRows;
  const bool is_a = job.y < a_blocks;
  fused_scale_split_rows<false>(is_a ? P.A : P.B, is_a ? P.rsa : P.csb, is_a ? P.csa : P.rsb,
                         is_a ? P.M : P.N, P.K, P.Kp,
                         (is_a ? job.y : job.y - a_blocks) * kFusedRows,
                         is_a ? P.pa : P.pb, is_a ? P.flags_a : P.flags_b, is_a ? kBM : 64,
                         is_a ? P.max_a : P.max_b, gen);
}

// ---- persistent grouped split GEMM ----------------------------------------------

template <int BN, int STAGES, int FLUSH>
struct Cfg {
  static constexpr uint32_t A_BYTES = kBM * kBK * 2, B_BYTES = BN * kBK * 2;
  static constexpr uint32_t STAGE_BYTES = kPlanes * (A_BYTES + B_BYTES);
  static constexpr int ACC_WARPS = 8;
  // ring, barriers, and per accumulator warp a staging buffer for coalesced
  // stores
  static constexpr uint32_t SMEM =
      STAGES * STAGE_BYTES + 1024 + 256 + ACC_WARPS * kEpiStageFloats * 4;
  static constexpr int NBUF = 512 / BN;
  static constexpr int CW = BN / 2;
  static constexpr int THREADS = 64 + 32 * ACC_WARPS;
  static_assert(SMEM <= 232448, "shared memory");
  static_assert((2 * STAGES + 2 * NBUF + 1) * 8 + 4 <= 256, "barrier space");
};

template <int BN, int STAGES, int FLUSH, bool F16>
__global__ void __launch_bounds__(Cfg<BN, STAGES, FLUSH>::THREADS, 1)
grouped_split_gemm(const CUtensorMap *__restrict__ tmaps, const Prob *__restrict__ probs,
                   const Tile *__restrict__ tiles, int ntiles, unsigned *status,
                   unsigned long long gen, WaitCfg wc) {
  using C_ = Cfg<BN, STAGES, FLUSH>;
  constexpr int NBUF = C_::NBUF;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *bars = (uint64_t *)(smem + STAGES * C_::STAGE_BYTES);
  uint64_t *full = bars, *empty = bars + STAGES;
  uint64_t *tfull = bars + 2 * STAGES, *tempty = tfull + NBUF;
  uint64_t *drain = tempty + NBUF;   // all issued MMAs complete
  uint32_t *tmem_slot = (uint32_t *)(drain + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      tc::mbar_init(tc::smem_u32(&full[s]), 1);
      tc::mbar_init(tc::smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < NBUF; b++) {
      tc::mbar_init(tc::smem_u32(&tfull[b]), 1);
      tc::mbar_init(tc::smem_u32(&tempty[b]), C_::ACC_WARPS);
    }
    tc::mbar_init(tc::smem_u32(drain), 1);
    tc::fence_barrier_init();
  }
  if (warp == 1) tc::tmem_alloc(tc::smem_u32(tmem_slot), 512);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int g = 0;
      bool live = true;
      for (int t = blockIdx.x; t < ntiles && live; t += gridDim.x) {
        const Tile tl = tiles[t];
        int kb0, kb1;
        slice_range(probs[tl.prob], tl.ks, kb0, kb1);
        const CUtensorMap *ta = tmaps + 2 * tl.prob, *tb = ta + 1;
        tc::tensormap_acquire(ta);
        tc::tensormap_acquire(tb);
        for (int kb = kb0; kb < kb1; kb++, g++) {
          const int s = g % STAGES;
          if (g >= STAGES &&
              !tc::mbar_wait_bounded(tc::smem_u32(&empty[s]), ((g / STAGES) & 1) ^ 1, status,
                                     kStatusTimeoutProducer, wc.limit_ns)) {
            live = false;
            break;
          }
          if (wc.starve) continue;   // give-up test: no load, no barrier completes
          const uint32_t fbar = tc::smem_u32(&full[s]);
          const uint32_t st = tc::smem_u32(smem + s * C_::STAGE_BYTES);
          tc::mbar_arrive_expect_tx(fbar, C_::STAGE_BYTES);
#pragma unroll
          for (int p = 0; p < kPlanes; p++) {
            tc::tma_load_3d(st + p * C_::A_BYTES, ta, fbar, kb * kBK, tl.m0, p);
            tc::tma_load_3d(st + kPlanes * C_::A_BYTES + p * C_::B_BYTES, tb, fbar, kb * kBK,
                            tl.n0, p);
          }
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = F16 ? tc::idesc_f16_f32(kBM, BN) : tc::idesc_bf16_f32(kBM, BN);
      int g = 0, chunk = 0;
      bool live = true;
      for (int t = blockIdx.x; t < ntiles && live; t += gridDim.x) {
        int kb0, kb1;
        slice_range(probs[tiles[t].prob], tiles[t].ks, kb0, kb1);
        for (int kb = kb0; kb < kb1; kb++, g++) {
          const int s = g % STAGES, buf = chunk % NBUF;
          const bool cstart = (kb - kb0) % FLUSH == 0;
          const bool cend = (kb - kb0) % FLUSH == FLUSH - 1 || kb == kb1 - 1;
          if (cstart && chunk >= NBUF &&
              !tc::mbar_wait_bounded(tc::smem_u32(&tempty[buf]), ((chunk / NBUF) & 1) ^ 1,
                                     status, kStatusTimeoutMma, wc.limit_ns)) {
            live = false;
            break;
          }
          if (!tc::mbar_wait_bounded(tc::smem_u32(&full[s]), (g / STAGES) & 1, status,
                                     kStatusTimeoutMma, wc.limit_ns)) {
            live = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t st = tc::smem_u32(smem + s * C_::STAGE_BYTES);
          const uint32_t a0 = st, a1 = st + C_::A_BYTES;
          const uint32_t b0 = st + kPlanes * C_::A_BYTES, b1 = b0 + C_::B_BYTES;
          // x1 y0, then x0 y1, then x0 y0 over the whole slab: the large
          // terms enter the truncating tensor-core accumulator last.
          const uint32_t d = tmem + buf * BN;
#pragma unroll
          for (int kk = 0; kk < kBK / 16; kk++)
            tc::mma_bf16(d, tc::sdesc_k128(a1 + kk * 32), tc::sdesc_k128(b0 + kk * 32), idesc,
                         (!cstart || kk > 0) ? 1u : 0u);
#pragma unroll
          for (int kk = 0; kk < kBK / 16; kk++)
            tc::mma_bf16(d, tc::sdesc_k128(a0 + kk * 32), tc::sdesc_k128(b1 + kk * 32), idesc, 1u);
#pragma unroll
          for (int kk = 0; kk < kBK / 16; kk++)
            tc::mma_bf16(d, tc::sdesc_k128(a0 + kk * 32), tc::sdesc_k128(b0 + kk * 32), idesc, 1u);
          tc::mma_commit(tc::smem_u32(&empty[s]));
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
    constexpr int CW = C_::CW;
    const int quad = warp & 3, half = (warp - 2) >> 2;
    const int cbase = half * CW;
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    int chunk = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      const Tile tl = tiles[t];
      const Prob &P = probs[tl.prob];
      const int row = tl.m0 + quad * 32 + lane;
      float acc[CW];
#pragma unroll
      for (int j = 0; j < CW; j++) acc[j] = 0.0f;
      int kb0, kb1;
      slice_range(P, tl.ks, kb0, kb1);
      const int nchunks = (kb1 - kb0 + FLUSH - 1) / FLUSH;
      for (int c = 0; c < nchunks; c++, chunk++) {
        const int buf = chunk % NBUF;
        ok = tc::mbar_wait_bounded(tc::smem_u32(&tfull[buf]), (chunk / NBUF) & 1, status,
                                   kStatusTimeoutEpilogue, wc.limit_ns);
        ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld below is warp-collective
        if (!ok) break;
        tc::tc_fence_after();
        uint32_t r[CW];
#pragma unroll
        for (int c0 = 0; c0 < CW; c0 += 32)
          tc::tmem_ld_32x32b_x32(tmem + lane_off + buf * BN + cbase + c0,
                                 *reinterpret_cast<uint32_t(*)[32]>(&r[c0]));
        tc::tmem_ld_wait();
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(tc::smem_u32(&tempty[buf]));
#pragma unroll
        for (int j = 0; j < CW; j++) acc[j] = __fadd_rn(acc[j], __uint_as_float(r[j]));
      }
      if (!ok) break;
      if (P.splits > 1) {
        // split-K: this slice's unscaled partial sums; the ordered
        // reduction adds the slices, rescales and checks the flags
        float *stage =
            (float *)(smem + STAGES * C_::STAGE_BYTES + 256) + (warp - 2) * kEpiStageFloats;
        store_rows_coalesced<CW>(acc, stage, P.part + (int64_t)tl.ks * P.M * P.N, P.N,
                                 tl.m0 + quad * 32, tl.n0 + cbase, P.M, P.N, lane);
        __syncwarp();
        continue;
      }
      bool nonfinite = P.flags_a[tl.m0 / kBM] == gen;
      for (int c = tl.n0 / 64; c < (tl.n0 + BN) / 64 && c * 64 < P.N; c++)
        nonfinite |= P.flags_b[c] == gen;
      if (F16 && !nonfinite) {
        // acc * 2^-(s_row + s_col), correctly rounded (see gemm_tc.cu); the
        // warp's column exponents are loaded once and broadcast (every lane
        // runs this, rows past M included: nonfinite is the warp's tile's)
        const int lc = tl.n0 + cbase + lane;
        const int eb_lo = lc < P.N ? f16_scale_exp(P.max_b[lc]) : 0;
        const int eb_hi = (CW > 32 && lc + 32 < P.N) ? f16_scale_exp(P.max_b[lc + 32]) : 0;
        const int sa = row < P.M ? f16_scale_exp(P.max_a[row]) : 0;
#pragma unroll
        for (int j = 0; j < CW; j++) {
          const int e = -(sa + __shfl_sync(0xffffffffu, j < 32 ? eb_lo : eb_hi, j & 31));
          acc[j] = (e >= -126 && e <= 127) ? acc[j] * exp2_int(e) : ldexpf(acc[j], e);
        }
      }
      if (row >= P.M) {
        // rows past M: nothing to store
      } else if (nonfinite) {
#pragma unroll 1
        for (int j = 0; j < CW; j++) {
          const int col = tl.n0 + cbase + j;
          if (col >= P.N) break;
          float f = 0.0f;
#pragma unroll 1
          for (int k = 0; k < P.K; k++)
            f = __fmaf_rn(P.A[(int64_t)row * P.rsa + (int64_t)k * P.csa],
                          P.B[(int64_t)k * P.rsb + (int64_t)col * P.csb], f);
          P.C[(int64_t)row * P.rso + (int64_t)col * P.cso] = f;
        }
      } else if (P.cso != 1) {
        float *crow = P.C + (int64_t)row * P.rso;
#pragma unroll
        for (int j = 0; j < CW; j++) {
          const int col = tl.n0 + cbase + j;
          if (col < P.N) crow[(int64_t)col * P.cso] = acc[j];
        }
      }
      __syncwarp();
      if (!nonfinite && P.cso == 1) {   // warp-uniform: every lane stores
        float *stage =
            (float *)(smem + STAGES * C_::STAGE_BYTES + 256) + (warp - 2) * kEpiStageFloats;
        store_rows_coalesced<CW>(acc, stage, P.C, P.rso, tl.m0 + quad * 32, tl.n0 + cbase, P.M,
                                 P.N, lane);
      }
      __syncwarp();   // reconverge before the next tile's tcgen05.ld
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 512);
  }
}

// ---- split-K: ordered reduction of the slices ---------------------------------
//
// Block b: 256 consecutive outputs (row-major) of split problem
// probs_idx[jobs[b].x], block jobs[b].y.  Each output is the FP32 sum of its
// slices' partial sums in slice (K) order — deterministic — then, as in the
// GEMM's own epilogue, rescaled (float16 planes) or, in a tile with a
// non-finite input, recomputed as numc's FMA chain.
template <bool F16>
__global__ void __launch_bounds__(256)
grouped_splitk_reduce(const Prob *__restrict__ probs, const int *__restrict__ probs_idx,
                      const int2 *__restrict__ jobs, unsigned long long gen) {
  const int2 job = jobs[blockIdx.x];
  const Prob &P = probs[probs_idx[job.x]];
  const int64_t e = (int64_t)job.y * 256 + threadIdx.x;
  const int64_t MN = (int64_t)P.M * P.N;
  if (e >= MN) return;
  const int i = (int)(e / P.N), j = (int)(e % P.N);
  float *dst = P.C + (int64_t)i * P.rso + (int64_t)j * P.cso;
  if (P.flags_a[i / kBM] == gen || P.flags_b[j / 64] == gen) {
    float f = 0.0f;
    for (int k = 0; k < P.K; k++)
      f = __fmaf_rn(P.A[(int64_t)i * P.rsa + (int64_t)k * P.csa],
                    P.B[(int64_t)k * P.rsb + (int64_t)j * P.csb], f);
    *dst = f;
    return;
  }
  float acc = P.part[e];
  for (int ks = 1; ks < P.splits; ks++) acc = __fadd_rn(acc, P.part[ks * MN + e]);
  if (F16) {
    const int ex = -(f16_scale_exp(P.max_a[i]) + f16_scale_exp(P.max_b[j]));
    acc = (ex >= -126 && ex <= 127) ? acc * exp2_int(ex) : (float)((double)acc * exp2_dbl(ex));
  }
  *dst = acc;
}

// ---- grouped CUDA-core kernel ---------------------------------------------------

constexpr int kSimtBM = 128, kSimtBN = 128;

// numc_matmul's gemmsup threshold for float32 (src/matmul/matmul.c:241-256).
__host__ __device__ inline bool numc_packed(const Prob &P) {
  return (double)P.M * P.K * P.N > 96.0 * 96 * 96;
}

// One instantiation per kernel (the packed and the unpacked arithmetic in
// one kernel needed 255 registers, half the occupancy of either alone).
template <int KIND>
__global__ void __launch_bounds__(simt::kThreads, 2)
grouped_simt(const Prob *__restrict__ probs, const Tile *__restrict__ tiles) {
  const Tile tl = tiles[blockIdx.x];
  const Prob &P = probs[tl.prob];
  Gemm g;
  g.a = P.A; g.b = P.B; g.c = P.C;
  g.M = P.M; g.K = P.K; g.N = P.N;
  g.rsa = P.rsa; g.csa = P.csa; g.rsb = P.rsb; g.csb = P.csb; g.rso = P.rso; g.cso = P.cso;
  g.isa = P.isa;
  simt::simt_tile<float, kSimtBM, kSimtBN, 8, 8, 8, KIND>(g, 0, tl.m0, tl.n0);
}

// numc's packed-path remainder tiles of the CUDA-core problems listed in
// `probs_idx`: 16 remainder groups per block (one a half-warp), block b
// being block jobs[b].y of problem probs_idx[jobs[b].x].
__global__ void __launch_bounds__(256)
grouped_float_edges(const Prob *__restrict__ probs, const int *__restrict__ probs_idx,
                    const int2 *__restrict__ jobs) {
  const int2 job = jobs[blockIdx.x];
  const Prob &P = probs[probs_idx[job.x]];
  Gemm g;
  g.a = P.A; g.b = P.B; g.c = P.C;
  g.M = P.M; g.K = P.K; g.N = P.N;
  g.rsa = P.rsa; g.csa = P.csa; g.rsb = P.rsb; g.csb = P.csb; g.rso = P.rso; g.cso = P.cso;
  g.isa = P.isa;
  const int64_t r0 = simt::edge_row<float>(g.M, g.isa), c0 = simt::edge_col<float>(g.N, g.isa);
  const int64_t n = simt::float_edge_groups<float>(g.M, g.N, g.isa);
  const int64_t gi = (int64_t)job.y * 16 + threadIdx.x / 16;
  if (gi < n) simt::float_edge_output<float>(g, gi, threadIdx.x % 16, r0, c0);
}

}  // namespace grouped
}  // namespace numc_k

// ---- plans ------------------------------------------------------------------------

using namespace numc_k;
using namespace numc_k::grouped;

enum Variant : int { kVarTc128 = 0, kVarTc64 = 1, kVarSimt = 2, kNumVar = 3 };

struct NumcCudaGemmPlan {
  int device;
  int algo;
  size_t count;
  std::vector<Prob> probs;        // host copy
  std::vector<int> variant;       // per problem
  char *dev;                      // owned device block
  size_t dev_bytes;
  CUtensorMap *d_tmaps;
  Prob *d_probs;
  int2 *d_split_jobs;             // (problem, job) of each split block
  long long split_jobs;
  bool f16;                       // scaled float16 planes (else bfloat16)
  int2 *d_max_jobs;               // (problem, job) of each scale block (float16 planes)
  int2 *d_fused_jobs;             // (problem, block) of the fused scale + split pass
  long long fused_jobs;
  long long max_jobs;
  int n_split_probs;
  Prob *d_split_probs;
  Tile *d_tiles[kNumVar];
  int ntiles[kNumVar];
  int nsimt_packed;               // CUDA-core tiles of numc's packed path (listed first)
  int *d_sk_probs;                // split-K problems (indices into probs)
  int2 *d_sk_jobs;                // (split-K problem, block) of each reduction block
  int n_sk_probs;
  long long sk_jobs;
  int *d_edge_probs;              // CUDA-core problems with packed-path remainders
  int2 *d_edge_jobs;              // (edge problem, block) of each remainder block
  int n_edge_probs;
  long long edge_jobs;
  unsigned long long *flags;      // all flag words and maxima (memset per run)
  size_t flags_bytes;
  unsigned long long gen;
  cudaGraphExec_t graph;
  unsigned graph_kernels;         // kernels per graph replay
  int sms;
};

namespace {

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

int size_class(size_t x) {
  int c = 0;
  while (x > 32 && c < 6) {   // <=32, <=64, ..., <=1024, >1024
    x = (x + 1) / 2;
    c++;
  }
  return c;
}

// The autotune table: "mclass nclass kclass variant [splits]" per line (#
// comments), classes as size_class(); written by numc_gb300/autotune.py on a
// GB300.  splits: K slices of the tensor-core variants (1 when absent).
struct TuneTable {
  bool loaded = false;
  int v[7][7][7];
  int splits[7][7][7];
};
TuneTable g_tune;
std::once_flag g_tune_once;

std::string library_dir() {
  Dl_info info;
  if (dladdr((void *)&library_dir, &info) && info.dli_fname) {
    std::string p(info.dli_fname);
    size_t s = p.rfind('/');
    if (s != std::string::npos) return p.substr(0, s);
  }
  return ".";
}

void load_tune_table() {
  for (auto &a : g_tune.v)
    for (auto &b : a)
      for (int &c : b) c = -1;
  for (auto &a : g_tune.splits)
    for (auto &b : a)
      for (int &c : b) c = 1;
  const char *env = getenv("NUMC_CUDA_AUTOTUNE_TABLE");
  std::string path = env ? env : library_dir() + "/autotune_table.txt";
  FILE *f = fopen(path.c_str(), "r");
  if (!f) return;
  char line[256];
  while (fgets(line, sizeof line, f)) {
    if (line[0] == '#') continue;
    int a, b, c, v, sp = 1;
    const int n = sscanf(line, "%d %d %d %d %d", &a, &b, &c, &v, &sp);
    if (n >= 4 && a >= 0 && a < 7 && b >= 0 && b < 7 && c >= 0 && c < 7 && v >= 0 &&
        v < kNumVar) {
      g_tune.v[a][b][c] = v;
      g_tune.splits[a][b][c] = (n == 5 && (sp == 1 || sp == 2 || sp == 4)) ? sp : 1;
      g_tune.loaded = true;
    }
  }
  fclose(f);
}

// Variant for one split-BF16 problem: the tuned choice, else a size rule.
int pick_variant(size_t M, size_t N, size_t K) {
  std::call_once(g_tune_once, load_tune_table);
  if (K == 0) return kVarSimt;
  const int v = g_tune.v[size_class(M)][size_class(N)][size_class(K)];
  if (v >= 0) return v;
  if ((double)M * N * K < (double)(1 << 18)) return kVarSimt;
  return N <= 64 ? kVarTc64 : kVarTc128;
}

// K slices for a tensor-core problem: the tuned choice (at most one slice
// per 64-deep slab).
int pick_splits(size_t M, size_t N, size_t K, int num_kb) {
  std::call_once(g_tune_once, load_tune_table);
  const int sp = g_tune.splits[size_class(M)][size_class(N)][size_class(K)];
  return std::max(1, std::min(sp, num_kb));
}

int fail(cudaError_t e, const char *what) {
  cudaGetLastError();
  return NUMC_SET_ERROR(e == cudaErrorMemoryAllocation ? NUMC_ERR_MALLOC : NUMC_ERR_INTERNAL,
                        "%s: %s", what, cudaGetErrorString(e));
}

std::atomic<unsigned long long> g_plan_gen{0x9a0c000000000001ull};

// K slabs per TMEM chain: bfloat16 planes 8 (their 2^-16 split error
// dominates), float16 planes 1.  Grouped problems are mostly short in K,
// where the tensor core's truncating accumulation dominates the float16
// split's error: on 30 problems with M, N, K log-uniform in [64, 1024]
// (max / mean error relative to |A||B| against float64; FP32 FMA chain
// 3.0e-7 / 1.7e-8) flush 4 gave 4.1e-7 / 3.4e-8 and flush 1 1.5e-7 / 8.0e-9,
// at 2.74 against 2.21 ms for 2048 problems.
constexpr int kFlushBf16 = 8, kFlushF16 = 1;

template <int BN, int STAGES, int FLUSH, bool F16>
cudaError_t prepare_tc() {
  return cudaFuncSetAttribute(grouped_split_gemm<BN, STAGES, FLUSH, F16>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              Cfg<BN, STAGES, FLUSH>::SMEM);
}

template <int BN, int STAGES, int FLUSH, bool F16>
cudaError_t launch_tc(const NumcCudaGemmPlan *p, int var, unsigned *status, cudaStream_t s) {
  using C_ = Cfg<BN, STAGES, FLUSH>;
  auto kern = grouped_split_gemm<BN, STAGES, FLUSH, F16>;
  const int grid = std::min(p->ntiles[var], p->sms);
  kern<<<grid, C_::THREADS, C_::SMEM, s>>>(p->d_tmaps, p->d_probs, p->d_tiles[var],
                                          p->ntiles[var], status, p->gen, wait_cfg());
  return cudaGetLastError();
}

// Enqueue one run; `kernels` receives the number of kernels launched.
int plan_enqueue(NumcCudaGemmPlan *p, cudaStream_t s, unsigned *kernels) {
  *kernels = 0;
  unsigned *status = status_word();
  if (!status) return NUMC_SET_ERROR(NUMC_ERR_MALLOC, "status word allocation failed");
  cudaError_t e;
  if (p->flags_bytes && (e = cudaMemsetAsync(p->flags, 0, p->flags_bytes, s)))
    return fail(e, "plan flags");
  if (p->f16 && p->max_jobs > 0) {
    grouped_absmax<<<(unsigned)p->max_jobs, 256, 0, s>>>(p->d_split_probs, p->d_max_jobs);
    if ((e = cudaGetLastError())) return fail(e, "grouped scale pass");
    ++*kernels;
  }
  if (p->fused_jobs > 0) {
    grouped_scale_split<<<(unsigned)p->fused_jobs, 256, 0, s>>>(
        p->d_split_probs, p->d_fused_jobs, p->gen);
    if ((e = cudaGetLastError())) return fail(e, "grouped scale and split");
    ++*kernels;
  }
  if (p->split_jobs > 0) {
    if (p->f16)
      grouped_split<true><<<(unsigned)p->split_jobs, 256, 0, s>>>(p->d_split_probs,
                                                                  p->d_split_jobs, p->gen);
    else
      grouped_split<false><<<(unsigned)p->split_jobs, 256, 0, s>>>(p->d_split_probs,
                                                                   p->d_split_jobs, p->gen);
    if ((e = cudaGetLastError())) return fail(e, "grouped split");
    ++*kernels;
  }
  if (p->ntiles[kVarTc128]) {
    e = p->f16 ? launch_tc<128, 3, kFlushF16, true>(p, kVarTc128, status, s)
               : launch_tc<128, 3, kFlushBf16, false>(p, kVarTc128, status, s);
    if (e) return fail(e, "grouped split GEMM (128)");
    ++*kernels;
  }
  if (p->ntiles[kVarTc64]) {
    e = p->f16 ? launch_tc<64, 4, kFlushF16, true>(p, kVarTc64, status, s)
               : launch_tc<64, 4, kFlushBf16, false>(p, kVarTc64, status, s);
    if (e) return fail(e, "grouped split GEMM (64)");
    ++*kernels;
  }
  if (p->sk_jobs > 0) {
    if (p->f16)
      grouped_splitk_reduce<true><<<(unsigned)p->sk_jobs, 256, 0, s>>>(p->d_probs, p->d_sk_probs,
                                                                      p->d_sk_jobs, p->gen);
    else
      grouped_splitk_reduce<false><<<(unsigned)p->sk_jobs, 256, 0, s>>>(
          p->d_probs, p->d_sk_probs, p->d_sk_jobs, p->gen);
    if ((e = cudaGetLastError())) return fail(e, "grouped split-K reduction");
    ++*kernels;
  }
  if (p->nsimt_packed) {
    grouped_simt<simt::kFloat><<<p->nsimt_packed, simt::kThreads, 0, s>>>(
        p->d_probs, p->d_tiles[kVarSimt]);
    if ((e = cudaGetLastError())) return fail(e, "grouped SIMT");
    ++*kernels;
  }
  if (p->ntiles[kVarSimt] > p->nsimt_packed) {
    grouped_simt<simt::kFloatSmall><<<p->ntiles[kVarSimt] - p->nsimt_packed, simt::kThreads, 0,
                                      s>>>(p->d_probs, p->d_tiles[kVarSimt] + p->nsimt_packed);
    if ((e = cudaGetLastError())) return fail(e, "grouped SIMT (unpacked path)");
    ++*kernels;
  }
  if (p->n_edge_probs) {
    grouped_float_edges<<<(unsigned)p->edge_jobs, 256, 0, s>>>(p->d_probs, p->d_edge_probs,
                                                               p->d_edge_jobs);
    if ((e = cudaGetLastError())) return fail(e, "grouped SIMT remainder tiles");
    ++*kernels;
  }
  return 0;
}

}  // namespace

extern "C" NumcCudaGemmPlan *numc_cuda_gemm_plan_create(NumcDType dtype, int algo, int param,
                                                        const NumcCudaGemmDesc *descs,
                                                        size_t count) {
  if (dtype != NUMC_DTYPE_FLOAT32) {
    NUMC_SET_ERROR(NUMC_ERR_TYPE, "grouped GEMM plans are float32");
    return nullptr;
  }
  if (algo == NUMC_CUDA_ALGO_DEFAULT || algo == NUMC_CUDA_ALGO_AUTO) algo = NUMC_CUDA_ALGO_SPLIT_FP16;
  if (algo != NUMC_CUDA_ALGO_SPLIT_FP16 && algo != NUMC_CUDA_ALGO_SPLIT_BF16 &&
      algo != NUMC_CUDA_ALGO_SIMT) {
    NUMC_SET_ERROR(NUMC_ERR_VALUE, "grouped GEMM algorithm %d (SIMT, SPLIT_BF16 or SPLIT_FP16)",
                   algo);
    return nullptr;
  }
  // Split param: 0 (or 3 for SPLIT_BF16) = per-problem choice from the
  // autotune table; 128 / 64 = every problem on that tile width, plus
  // 1000 x s for s K slices (2 or 4; e.g. 2128 = 128 columns, 2 slices).
  const int force_width = param > 0 ? param % 1000 : 0, force_splits = param > 0 ? param / 1000 : 0;
  if (algo != NUMC_CUDA_ALGO_SIMT && param != 0 && param != 3 && param != -1 &&
      !((force_width == 128 || force_width == 64) &&
        (force_splits == 0 || force_splits == 1 || force_splits == 2 || force_splits == 4))) {
    NUMC_SET_ERROR(NUMC_ERR_VALUE,
                   "grouped split param %d (0, 3, or 64 / 128 plus 1000 x 1, 2 or 4)", param);
    return nullptr;
  }
  if (count > 0 && !descs) {
    NUMC_SET_ERROR(NUMC_ERR_NULL, "plan_create: descs is NULL");
    return nullptr;
  }
  NumcCudaGemmPlan *p = new (std::nothrow) NumcCudaGemmPlan();
  if (!p) {
    NUMC_SET_ERROR(NUMC_ERR_MALLOC, "plan allocation failed");
    return nullptr;
  }
  p->algo = algo;
  p->f16 = algo == NUMC_CUDA_ALGO_SPLIT_FP16;
  p->count = count;
  p->dev = nullptr;
  p->graph = nullptr;
  p->graph_kernels = 0;
  p->gen = ++g_plan_gen;
  if (cudaGetDevice(&p->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess) {
    cudaGetLastError();
    delete p;
    NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "plan_create: no CUDA device");
    return nullptr;
  }

  // Problems, variants and the device layout.
  std::vector<size_t> plane_off(count, 0), flag_off(count, 0);
  size_t planes_bytes = 0, flags_bytes = 0;
  p->probs.resize(count);
  const int isa = float_isa();   // numc build whose CUDA-core arithmetic to follow
  p->variant.resize(count);
  for (size_t i = 0; i < count; i++) {
    const NumcCudaGemmDesc &d = descs[i];
    if (d.M >= (1u << 30) || d.N >= (1u << 30) || d.K >= (1u << 30) ||
        (d.M && d.N && (!d.out || (d.K && (!d.a || !d.b)))) || d.rsa < 0 || d.csa < 0 ||
        d.rsb < 0 || d.csb < 0 || d.rso < 0 || d.cso < 0) {
      delete p;
      NUMC_SET_ERROR(NUMC_ERR_VALUE, "plan_create: invalid problem %zu", i);
      return nullptr;
    }
    Prob &P = p->probs[i];
    memset(&P, 0, sizeof P);
    P.A = (const float *)d.a; P.B = (const float *)d.b; P.C = (float *)d.out;
    P.rsa = d.rsa; P.csa = d.csa; P.rsb = d.rsb; P.csb = d.csb; P.rso = d.rso; P.cso = d.cso;
    P.M = (int)d.M; P.N = (int)d.N; P.K = (int)d.K;
    P.isa = isa;
    P.Kp = (int)align_up(d.K ? d.K : 1, kBK);
    P.num_kb = P.Kp / kBK;
    int v = algo == NUMC_CUDA_ALGO_SIMT ? kVarSimt
            : force_width == 128        ? (d.K ? kVarTc128 : kVarSimt)
            : force_width == 64         ? (d.K ? kVarTc64 : kVarSimt)
                                        : pick_variant(d.M, d.N, d.K);
    if (d.M == 0 || d.N == 0) v = -1;
    p->variant[i] = v;
    P.splits = 1;
    if (v == kVarTc128 || v == kVarTc64)
      P.splits = force_width ? std::max(1, std::min(force_splits ? force_splits : 1, P.num_kb))
                             : pick_splits(d.M, d.N, d.K, P.num_kb);
    if (v == kVarTc128 || v == kVarTc64) {
      plane_off[i] = planes_bytes;
      planes_bytes += align_up((size_t)kPlanes * P.Kp * (d.M + d.N) * 2, 256);
      flag_off[i] = flags_bytes;
      flags_bytes += align_up(((d.M + kBM - 1) / kBM + (d.N + 63) / 64) * 8, 256);
      if (p->f16) flags_bytes += align_up((d.M + d.N) * 4, 256);   // row / column maxima
      P.split_mode_a = split_mode(P.A, P.rsa, P.csa);
      P.split_mode_b = split_mode(P.B, P.csb, P.rsb);
    }
  }
  // Tile lists, problems sorted by K (largest first) within each variant.
  std::vector<size_t> order(count);
  for (size_t i = 0; i < count; i++) order[i] = i;
  // (split problems by their slices' depth)
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
    return p->probs[x].num_kb / p->probs[x].splits > p->probs[y].num_kb / p->probs[y].splits;
  });
  std::vector<Tile> tiles[kNumVar], simt_small;
  std::vector<size_t> split_idx;
  std::vector<int> edge_idx;
  for (size_t i : order) {
    const int v = p->variant[i];
    if (v < 0) continue;
    if (v == kVarSimt && simt::float_edges_needed<float>(p->probs[i].K) && numc_packed(p->probs[i]) &&
        simt::float_edge_count<float>(p->probs[i].M, p->probs[i].N, p->probs[i].isa) > 0)
      edge_idx.push_back((int)i);
    const int bn = v == kVarTc128 ? 128 : v == kVarTc64 ? 64 : kSimtBN;
    const int bm = v == kVarSimt ? kSimtBM : kBM;
    // CUDA-core problems on numc's unpacked path go to a list of their own
    std::vector<Tile> &tl = (v == kVarSimt && !numc_packed(p->probs[i])) ? simt_small : tiles[v];
    for (int m0 = 0; m0 < p->probs[i].M; m0 += bm)
      for (int n0 = 0; n0 < p->probs[i].N; n0 += bn)
        for (int ks = 0; ks < p->probs[i].splits; ks++) tl.push_back(Tile{(int)i, m0, n0, ks});
    if (v != kVarSimt) split_idx.push_back(i);
  }
  // the CUDA-core list: numc's packed-path problems, then the unpacked ones
  p->nsimt_packed = (int)tiles[kVarSimt].size();
  tiles[kVarSimt].insert(tiles[kVarSimt].end(), simt_small.begin(), simt_small.end());
  // Job tables: (problem, job within it) for every block of the scale,
  // split and remainder passes, so a block finds its problem in one load.
  std::vector<int2> split_jobs, max_jobs, edge_jobs, fused_jobs;
  for (size_t q = 0; q < split_idx.size(); q++) {
    const Prob &P = p->probs[split_idx[q]];
    if (p->f16) {   // float16 planes: one fused scale + split pass
      const long long n = (P.M + kFusedRows - 1) / kFusedRows + (P.N + kFusedRows - 1) / kFusedRows;
      for (long long j = 0; j < n; j++) fused_jobs.push_back(make_int2((int)q, (int)j));
      continue;
    }
    const long long kt = (P.Kp + kSplitK - 1) / kSplitK;
    const long long n = ((P.M + kSplitRows - 1) / kSplitRows) * kt +
                        ((P.N + kSplitRows - 1) / kSplitRows) * kt;
    for (long long j = 0; j < n; j++) split_jobs.push_back(make_int2((int)q, (int)j));
    if (p->f16) {
      const dim3 ga = absmax_grid(P.M, P.K, absmax_mode(P.split_mode_a, P.csa));
      const dim3 gb = absmax_grid(P.N, P.K, absmax_mode(P.split_mode_b, P.rsb));
      const long long nm = (long long)ga.x * ga.y + (long long)gb.x * gb.y;
      for (long long j = 0; j < nm; j++) max_jobs.push_back(make_int2((int)q, (int)j));
    }
  }
  // split-K problems: partial sums (splits x M x N floats each) and the
  // reduction's blocks
  std::vector<int> sk_idx;
  std::vector<int2> sk_jobs;
  std::vector<size_t> part_off(count, 0);
  size_t part_bytes = 0;
  for (size_t i = 0; i < count; i++) {
    const Prob &P = p->probs[i];
    if (p->variant[i] < 0 || P.splits <= 1) continue;
    part_off[i] = part_bytes;
    part_bytes += align_up((size_t)P.splits * P.M * P.N * 4, 256);
    const long long n = ((long long)P.M * P.N + 255) / 256;
    for (long long j = 0; j < n; j++) sk_jobs.push_back(make_int2((int)sk_idx.size(), (int)j));
    sk_idx.push_back((int)i);
  }
  for (size_t q = 0; q < edge_idx.size(); q++) {
    const Prob &P = p->probs[edge_idx[q]];
    const long long n = (simt::float_edge_groups<float>(P.M, P.N, P.isa) + 15) / 16;
    for (long long j = 0; j < n; j++) edge_jobs.push_back(make_int2((int)q, (int)j));
  }
  p->split_jobs = (long long)split_jobs.size();
  p->n_split_probs = (int)split_idx.size();
  p->max_jobs = (long long)max_jobs.size();
  p->edge_jobs = (long long)edge_jobs.size();
  p->fused_jobs = (long long)fused_jobs.size();
  p->sk_jobs = (long long)sk_jobs.size();
  p->n_sk_probs = (int)sk_idx.size();
  if (p->split_jobs > 0x7FFFFFFFll || p->max_jobs > 0x7FFFFFFFll || p->edge_jobs > 0x7FFFFFFFll ||
      p->fused_jobs > 0x7FFFFFFFll || p->sk_jobs > 0x7FFFFFFFll) {
    delete p;
    NUMC_SET_ERROR(NUMC_ERR_VALUE, "plan_create: too many split blocks");
    return nullptr;
  }

  // One device block: tmaps | probs | split probs | job tables | tiles | flags | planes.
  size_t off = 0;
  const size_t o_tmaps = off; off = align_up(off + count * 2 * sizeof(CUtensorMap), 256);
  const size_t o_probs = off; off = align_up(off + count * sizeof(Prob), 256);
  const size_t o_sprobs = off; off = align_up(off + split_idx.size() * sizeof(Prob), 256);
  const size_t o_split_jobs = off; off = align_up(off + split_jobs.size() * sizeof(int2), 256);
  const size_t o_max_jobs = off; off = align_up(off + max_jobs.size() * sizeof(int2), 256);
  const size_t o_fused_jobs = off; off = align_up(off + fused_jobs.size() * sizeof(int2), 256);
  const size_t o_sk = off; off = align_up(off + sk_idx.size() * sizeof(int), 256);
  const size_t o_sk_jobs = off; off = align_up(off + sk_jobs.size() * sizeof(int2), 256);
  const size_t o_edges = off; off = align_up(off + edge_idx.size() * sizeof(int), 256);
  const size_t o_edge_jobs = off; off = align_up(off + edge_jobs.size() * sizeof(int2), 256);
  size_t o_tiles[kNumVar];
  for (int v = 0; v < kNumVar; v++) {
    o_tiles[v] = off;
    off = align_up(off + tiles[v].size() * sizeof(Tile), 256);
  }
  const size_t o_flags = off; off = align_up(off + flags_bytes, 256);
  const size_t o_planes = off; off = align_up(off + planes_bytes, 256);
  const size_t o_part = off; off += part_bytes;
  p->dev_bytes = off;
  cudaError_t e = dev_malloc((void **)&p->dev, off ? off : 256);
  if (e) {
    delete p;
    fail(e, "plan workspace");
    return nullptr;
  }
  p->d_tmaps = (CUtensorMap *)(p->dev + o_tmaps);
  p->d_probs = (Prob *)(p->dev + o_probs);
  p->d_split_probs = (Prob *)(p->dev + o_sprobs);
  p->d_split_jobs = (int2 *)(p->dev + o_split_jobs);
  p->d_max_jobs = (int2 *)(p->dev + o_max_jobs);
  p->d_fused_jobs = (int2 *)(p->dev + o_fused_jobs);
  p->d_sk_probs = (int *)(p->dev + o_sk);
  p->d_sk_jobs = (int2 *)(p->dev + o_sk_jobs);
  p->d_edge_probs = (int *)(p->dev + o_edges);
  p->d_edge_jobs = (int2 *)(p->dev + o_edge_jobs);
  p->n_edge_probs = (int)edge_idx.size();
  for (int v = 0; v < kNumVar; v++) {
    p->d_tiles[v] = (Tile *)(p->dev + o_tiles[v]);
    p->ntiles[v] = (int)tiles[v].size();
  }
  p->flags = (unsigned long long *)(p->dev + o_flags);
  p->flags_bytes = flags_bytes;

  std::vector<CUtensorMap> tm(count * 2);
  memset(tm.data(), 0, tm.size() * sizeof(CUtensorMap));
  for (size_t i = 0; i < count; i++) {
    Prob &P = p->probs[i];
    const int v = p->variant[i];
    if (v != kVarTc128 && v != kVarTc64) continue;
    P.pa = (uint16_t *)(p->dev + o_planes + plane_off[i]);
    P.pb = P.pa + (size_t)kPlanes * P.M * P.Kp;
    P.flags_a = (unsigned long long *)(p->dev + o_flags + flag_off[i]);
    P.flags_b = P.flags_a + (P.M + kBM - 1) / kBM;
    if (p->f16) {
      P.max_a = (unsigned *)(p->dev + o_flags + flag_off[i] +
                             align_up(((P.M + kBM - 1) / kBM + (P.N + 63) / 64) * 8, 256));
      P.max_b = P.max_a + P.M;
    }
    if (P.splits > 1) P.part = (float *)(p->dev + o_part + part_off[i]);
    const uint32_t bn = v == kVarTc128 ? 128 : 64;
    const auto dt = p->f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    if ((e = make_tmap_3d(&tm[2 * i], P.pa, dt, 2, kPlanes, P.M, P.Kp, P.Kp, kBM, kBK)) ||
        (e = make_tmap_3d(&tm[2 * i + 1], P.pb, dt, 2, kPlanes, P.N, P.Kp, P.Kp, bn, kBK))) {
      numc_cuda_gemm_plan_free(p);
      fail(e, "plan tensor maps");
      return nullptr;
    }
  }
  // Kernel attributes are set here, not per run, so runs can be captured.
  if ((e = prepare_tc<128, 3, kFlushBf16, false>()) || (e = prepare_tc<64, 4, kFlushBf16, false>()) ||
      (e = prepare_tc<128, 3, kFlushF16, true>()) || (e = prepare_tc<64, 4, kFlushF16, true>()) ||
      !status_word()) {
    numc_cuda_gemm_plan_free(p);
    fail(e ? e : cudaErrorMemoryAllocation, "plan kernel setup");
    return nullptr;
  }
  std::vector<Prob> sp(split_idx.size());
  for (size_t q = 0; q < split_idx.size(); q++) sp[q] = p->probs[split_idx[q]];
  if ((e = cudaMemcpy(p->d_tmaps, tm.data(), tm.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(p->d_probs, p->probs.data(), count * sizeof(Prob), cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(p->d_split_probs, sp.data(), sp.size() * sizeof(Prob), cudaMemcpyHostToDevice)) ||
      (!split_jobs.empty() &&
       (e = cudaMemcpy(p->d_split_jobs, split_jobs.data(), split_jobs.size() * sizeof(int2),
                       cudaMemcpyHostToDevice))) ||
      (!max_jobs.empty() &&
       (e = cudaMemcpy(p->d_max_jobs, max_jobs.data(), max_jobs.size() * sizeof(int2),
                       cudaMemcpyHostToDevice))) ||
      (!fused_jobs.empty() &&
       (e = cudaMemcpy(p->d_fused_jobs, fused_jobs.data(), fused_jobs.size() * sizeof(int2),
                       cudaMemcpyHostToDevice))) ||
      (!sk_idx.empty() &&
       ((e = cudaMemcpy(p->d_sk_probs, sk_idx.data(), sk_idx.size() * sizeof(int),
                        cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(p->d_sk_jobs, sk_jobs.data(), sk_jobs.size() * sizeof(int2),
                        cudaMemcpyHostToDevice)))) ||
      (!edge_idx.empty() &&
       ((e = cudaMemcpy(p->d_edge_probs, edge_idx.data(), edge_idx.size() * sizeof(int),
                        cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(p->d_edge_jobs, edge_jobs.data(), edge_jobs.size() * sizeof(int2),
                        cudaMemcpyHostToDevice))))) {
    numc_cuda_gemm_plan_free(p);
    fail(e, "plan upload");
    return nullptr;
  }
  for (int v = 0; v < kNumVar; v++)
    if (!tiles[v].empty() &&
        (e = cudaMemcpy(p->d_tiles[v], tiles[v].data(), tiles[v].size() * sizeof(Tile),
                        cudaMemcpyHostToDevice))) {
      numc_cuda_gemm_plan_free(p);
      fail(e, "plan upload");
      return nullptr;
    }
  return p;
}

extern "C" int numc_cuda_gemm_plan_run(NumcCudaGemmPlan *p, void *stream) {
  if (!p) return NUMC_SET_ERROR(NUMC_ERR_NULL, "plan_run: plan is NULL");
  unsigned k = 0;
  const int err = plan_enqueue(p, (cudaStream_t)stream, &k);
  count_launch(k);
  return err;
}

extern "C" int numc_cuda_gemm_plan_run_graph(NumcCudaGemmPlan *p, void *stream) {
  if (!p) return NUMC_SET_ERROR(NUMC_ERR_NULL, "plan_run_graph: plan is NULL");
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  if (!p->graph) {
    // Capture on a private stream so that the caller's stream may be the
    // legacy default stream.
    cudaStream_t cs;
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking))) return fail(e, "capture stream");
    status_word();   // allocate before capture
    cudaGraph_t graph = nullptr;
    int err = 0;
    if ((e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal))) {
      cudaStreamDestroy(cs);
      return fail(e, "begin capture");
    }
    err = plan_enqueue(p, cs, &p->graph_kernels);
    e = cudaStreamEndCapture(cs, &graph);
    cudaStreamDestroy(cs);
    if (err) {
      if (graph) cudaGraphDestroy(graph);
      return err;
    }
    if (e) return fail(e, "end capture");
    e = cudaGraphInstantiate(&p->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e) {
      p->graph = nullptr;
      return fail(e, "graph instantiate");
    }
  }
  if ((e = cudaGraphLaunch(p->graph, s))) return fail(e, "graph launch");
  count_launch(p->graph_kernels);
  return 0;
}

extern "C" int numc_cuda_gemm_plan_info(const NumcCudaGemmPlan *p, int *tc128, int *tc64,
                                        int *simt, size_t *workspace_bytes) {
  if (!p) return NUMC_SET_ERROR(NUMC_ERR_NULL, "plan_info: plan is NULL");
  int c[kNumVar] = {0, 0, 0};
  for (int v : p->variant)
    if (v >= 0) c[v]++;
  if (tc128) *tc128 = c[kVarTc128];
  if (tc64) *tc64 = c[kVarTc64];
  if (simt) *simt = c[kVarSimt];
  if (workspace_bytes) *workspace_bytes = p->dev_bytes;
  return 0;
}

extern "C" void numc_cuda_gemm_plan_free(NumcCudaGemmPlan *p) {
  if (!p) return;
  if (p->graph) cudaGraphExecDestroy(p->graph);
  if (p->dev) {
    cudaDeviceSynchronize();   // work queued from this plan may still read it
    cudaFree(p->dev);
  }
  delete p;
}

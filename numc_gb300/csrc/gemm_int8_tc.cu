// int8 / uint8 GEMM on the tcgen05 tensor cores with numc's store rules —
// the tensor path for numc's gemm_i8_avx2 / gemm_u8_avx2
// (src/intrinsics/gemm_avx2.h:2741-2880, 2983-3125), gemm_i8_neon and
// gemm_i8_avx512.
//
// 8-bit integers are exact in bfloat16 (|x| <= 255 needs 8 significant
// bits), products are exact in FP32, and so is every partial sum below
// 2^24: a 512-deep K block of int8 products stays below 512 * 128^2 = 2^23,
// a 256-deep block of uint8 products below 256 * 255^2 < 2^24.  The MMA
// warp accumulates numc's K blocks in TMEM chunks, and the accumulator
// warps turn the chunk sums into numc's stored bytes with the rule the
// CUDA-core kernel uses (x86 packed saturation per block and tile class,
// NEON / AVX-512 clamp-once, or truncation).  Results are bit-exact.
//
// Passes: one convert launch writes A as bf16 (M x Kp, K-major) and B^T as
// bf16 (N x Kp), K padded to 512 with zeros.  Then either the persistent
// CTA-pair kernel (int8_pair_gemm: 256 x 256 tiles, from about 2048^3) or
// one output tile per CTA (int8_tc_gemm): 128 x 64 (24 KiB TMA ring
// stages, 8 of them, 320 threads) or, once the 128 x 128 tiles give every
// SM one, 128 x 128 (32 KiB stages, 6 of them, 576 threads): a TMA warp, an
// MMA warp and accumulator warps of 32 columns each.  Both store their
// output bytes through a per-warp staging buffer, whole rows a store.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#include "kernels.h"
#include "phase_timing.h"
#include "simt_common.cuh"
#include "status.h"
#include "tc_common.cuh"

namespace numc_k {
namespace {

constexpr int kBM = 128, kBK = 64;
constexpr int kBlockK = 512;                 // numc's int8 K block (KC)
constexpr uint32_t kBarBytes = 512;          // 2*(kStages + kNumBuf) + 1 mbarriers + TMEM slot

// Output tile 128 x BN: BN = 64 (8 accumulator warps, 8 TMEM buffers, 8
// ring stages of 24 KiB) for problems with few tiles, BN = 128 (16 warps,
// 4 buffers, 6 stages of 32 KiB: half the operand traffic per MMA) when
// the 128-column tiles still give every SM one.
template <int BN> struct I8Cfg {
  static constexpr int kNumBuf = 512 / BN, kStages = BN == 64 ? 8 : 6;
  static constexpr int kAccWarps = BN / 8, kThreads = 64 + 32 * kAccWarps;
};

inline int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

// Coalesced stores of a warp's 32 rows x CW output bytes (d[j] of row
// row0 + lane, column col0 + j; CW = 32 or 64) to row-major uint8 C (unit
// column stride, 4-byte aligned rows), through the warp's 32 * CW byte
// `stage`: each lane writes its row's 16-byte chunks (chunk c of row r at
// position c ^ ((r / (8 / chunks)) % chunks), so the 8 lanes of a store
// phase hit 32 distinct banks), then each store instruction writes
// 128 / CW whole rows, 4 bytes a lane.  A direct store instruction touched
// 32 rows.  Rows >= M and columns >= N are not written.  All 32 lanes must
// call it.
// The low bytes of four values, first in the low byte.
__device__ __forceinline__ uint32_t pack4(int32_t a, int32_t b, int32_t c, int32_t d) {
  return __byte_perm(__byte_perm((uint32_t)a, (uint32_t)b, 0x0040),
                     __byte_perm((uint32_t)c, (uint32_t)d, 0x0040), 0x5410);
}

template <int CW>
__device__ __forceinline__ void pack_bytes(const int32_t (&d)[CW], uint32_t (&w)[CW / 4]) {
#pragma unroll
  for (int q = 0; q < CW / 4; q++) w[q] = pack4(d[4 * q], d[4 * q + 1], d[4 * q + 2], d[4 * q + 3]);
}

// w: the row's CW bytes packed four a word, column col0 first.
template <int CW>
__device__ __forceinline__ void store_bytes_coalesced(const uint32_t (&w)[CW / 4], uint8_t *stage,
                                                      uint8_t *C, int64_t rso, int row0,
                                                      int col0, int M, int N, int lane) {
  constexpr int CH = CW / 16, LPR = CW / 4, RPI = 32 / LPR;
  static_assert(CW == 32 || CW == 64, "row width");
  auto swz = [](int r) { return (r / (8 / CH)) % CH; };
#pragma unroll
  for (int h = 0; h < CH; h++)
    *reinterpret_cast<uint4 *>(stage + lane * CW + (h ^ swz(lane)) * 16) =
        make_uint4(w[4 * h], w[4 * h + 1], w[4 * h + 2], w[4 * h + 3]);
  __syncwarp();
  const int sub = lane % LPR, c = col0 + 4 * sub;
#pragma unroll
  for (int rr = 0; rr < 32; rr += RPI) {
    const int r = rr + lane / LPR;
    const uint32_t v = *reinterpret_cast<const uint32_t *>(
        stage + r * CW + (((sub >> 2) ^ swz(r)) * 16) + (sub & 3) * 4);
    if (row0 + r < M) {
      uint8_t *dst = C + (int64_t)(row0 + r) * rso + c;
      if (c + 4 <= N) {
        *reinterpret_cast<uint32_t *>(dst) = v;
      } else {
#pragma unroll
        for (int b = 0; b < 4; b++)
          if (c + b < N) dst[b] = (uint8_t)(v >> (8 * b));
      }
    }
  }
  __syncwarp();
}

// One operand of the conversion pass: dst(row, k) = bf16(src[row * rs_row +
// k * rs_k]) for row < R, k < K, zero for K <= k < Kp.
struct I8Operand {
  const uint8_t *src;
  int64_t rs_row, rs_k, R;
  __nv_bfloat16 *dst;
};

constexpr int kCvtRows = 64;

// Four 8-bit integers (bytes of w, low first) as four bfloat16, packed two
// a word.  Integers of 8 bits are exact in bfloat16: the value's float32
// bits with the low 16 (zero) dropped.
template <bool SIGNED>
__device__ __forceinline__ uint2 bytes_to_bf16x4(uint32_t w) {
  // Without an int-to-float conversion (a quarter of the FP32 rate): the
  // float with bits 0x4B0000xx is 2^23 + xx, so subtracting 2^23 (int8:
  // offset binary, 2^23 + 128) leaves the byte's value exactly.
  if (SIGNED) w ^= 0x80808080u;
  constexpr float kBias = SIGNED ? 8388736.0f : 8388608.0f;
  uint32_t f[4];
#pragma unroll
  for (int i = 0; i < 4; i++)
    f[i] = __float_as_uint(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + i)) - kBias);
  return make_uint2(__byte_perm(f[0], f[1], 0x7632), __byte_perm(f[2], f[3], 0x7632));
}

// Both operands in one launch (A's tiles first, then B^T's), 64 rows x
// kCvtK (128 or 256) k a block.  Each source layout gets its own mapping, all of them writing
// whole 32-byte sectors of the destination:
//   * k contiguous (row-major A): 16 bytes a thread along k, converted in
//     registers, two 16-byte stores;
//   * rows contiguous (row-major B, read as B^T): a 4 x 4 byte block a
//     thread (four 4-byte loads, one per k, each warp load covering four
//     whole 32-byte sectors), transposed with byte permutes, four 8-byte
//     stores of 4 bfloat16 along k (8 rows x 32 bytes a warp store);
//   * any other strides: byte gathers staged in shared memory.
template <bool SIGNED, int kCvtK>
__global__ void __launch_bounds__(256)
int8_pair_to_bf16(I8Operand a, I8Operand b, int64_t K, int64_t Kp, int64_t blocks_a) {
  static_assert(kCvtK == 128 || kCvtK == 256, "conversion block depth");
  __shared__ __align__(16) uint8_t tile[kCvtRows][kCvtK + 16];
  tc::griddep_launch_dependents();   // the GEMM may launch and set up meanwhile
  int64_t blk = blockIdx.x;
  const I8Operand &op = blk < blocks_a ? a : b;
  if (blk >= blocks_a) blk -= blocks_a;
  const int64_t kblocks = Kp / kCvtK;
  const int64_t r0 = (blk / kblocks) * kCvtRows, k0 = (blk % kblocks) * kCvtK;
  const int tid = threadIdx.x;
  const uint8_t *src = op.src;
  // Every load of a thread is issued before its first store (the
  // destination may alias nothing it reads, but the compiler cannot know).
  if (op.rs_k == 1) {
    uint4 v[kCvtK / 64];
#pragma unroll
    for (int it = 0; it < kCvtK / 64; it++) {   // 8 threads a row, 16 k each, 128-k halves
      const int r = (tid >> 3) + 32 * (it & 1), kk = (tid & 7) * 16 + 128 * (it >> 1);
      const int64_t gr = r0 + r, gk = k0 + kk;
      v[it] = make_uint4(0, 0, 0, 0);
      if (gr < op.R && gk < K) {
        const uint8_t *p = src + gr * op.rs_row + gk;
        if (gk + 16 <= K && (reinterpret_cast<uintptr_t>(p) & 15) == 0) {
          v[it] = __ldg(reinterpret_cast<const uint4 *>(p));
        } else {
          uint32_t w[4] = {0, 0, 0, 0};
#pragma unroll
          for (int i = 0; i < 16; i++)
            if (gk + i < K) w[i >> 2] |= (uint32_t)p[i] << (8 * (i & 3));
          v[it] = make_uint4(w[0], w[1], w[2], w[3]);
        }
      }
    }
#pragma unroll
    for (int it = 0; it < kCvtK / 64; it++) {
      const int r = (tid >> 3) + 32 * (it & 1), kk = (tid & 7) * 16 + 128 * (it >> 1);
      const int64_t gr = r0 + r, gk = k0 + kk;
      if (gr >= op.R) continue;
      const uint2 c0 = bytes_to_bf16x4<SIGNED>(v[it].x), c1 = bytes_to_bf16x4<SIGNED>(v[it].y);
      const uint2 c2 = bytes_to_bf16x4<SIGNED>(v[it].z), c3 = bytes_to_bf16x4<SIGNED>(v[it].w);
      uint4 *d = reinterpret_cast<uint4 *>(op.dst + gr * Kp + gk);
      d[0] = make_uint4(c0.x, c0.y, c1.x, c1.y);
      d[1] = make_uint4(c2.x, c2.y, c3.x, c3.y);
    }
    return;
  }
  if (op.rs_row == 1) {
    const int warp = tid >> 5, lane = tid & 31;
    uint32_t w[kCvtK / 64][4];
#pragma unroll
    for (int it = 0; it < kCvtK / 64; it++) {   // a warp: 8 row quads x 4 k quads
      const int grp = warp + 8 * it;
      const int rq = (grp & 1) * 8 + (lane & 7), kq = (grp >> 1) * 4 + (lane >> 3);
      const int64_t gr = r0 + 4 * rq, gk = k0 + 4 * kq;
#pragma unroll
      for (int i = 0; i < 4; i++) {
        w[it][i] = 0;
        if (gr < op.R && gk + i < K) {
          const uint8_t *p = src + (gk + i) * op.rs_k + gr;
          if (gr + 4 <= op.R && (reinterpret_cast<uintptr_t>(p) & 3) == 0) {
            w[it][i] = __ldg(reinterpret_cast<const uint32_t *>(p));
          } else {
#pragma unroll
            for (int j = 0; j < 4; j++)
              if (gr + j < op.R) w[it][i] |= (uint32_t)p[j] << (8 * j);
          }
        }
      }
    }
#pragma unroll
    for (int it = 0; it < kCvtK / 64; it++) {
      const int grp = warp + 8 * it;
      const int rq = (grp & 1) * 8 + (lane & 7), kq = (grp >> 1) * 4 + (lane >> 3);
      const int64_t gr = r0 + 4 * rq, gk = k0 + 4 * kq;
      if (gr >= op.R) continue;
      // w[it][i] holds rows gr..gr+3 at k = gk + i; o[j] holds k = gk..gk+3 of row gr + j
      const uint32_t *x = w[it];
      const uint32_t lo01 = __byte_perm(x[0], x[1], 0x5140), hi01 = __byte_perm(x[0], x[1], 0x7362);
      const uint32_t lo23 = __byte_perm(x[2], x[3], 0x5140), hi23 = __byte_perm(x[2], x[3], 0x7362);
      const uint32_t o[4] = {__byte_perm(lo01, lo23, 0x5410), __byte_perm(lo01, lo23, 0x7632),
                             __byte_perm(hi01, hi23, 0x5410), __byte_perm(hi01, hi23, 0x7632)};
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (gr + j < op.R)
          *reinterpret_cast<uint2 *>(op.dst + (gr + j) * Kp + gk) = bytes_to_bf16x4<SIGNED>(o[j]);
    }
    return;
  }
#pragma unroll 4
  for (int q = 0; q < kCvtRows * kCvtK / 256; q++) {
    const int e = tid + 256 * q, r = e / kCvtK, kk = e % kCvtK;
    const int64_t gr = r0 + r, gk = k0 + kk;
    tile[r][kk] = (gr < op.R && gk < K) ? src[gr * op.rs_row + gk * op.rs_k] : 0;
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < kCvtRows * kCvtK / 8 / 256; it++) {   // 8 k a thread
    const int e = tid + 256 * it, r = e / (kCvtK / 8), kk = (e % (kCvtK / 8)) * 8;
    const int64_t gr = r0 + r;
    if (gr >= op.R) continue;
    const uint2 raw = *reinterpret_cast<const uint2 *>(&tile[r][kk]);
    const uint2 c0 = bytes_to_bf16x4<SIGNED>(raw.x), c1 = bytes_to_bf16x4<SIGNED>(raw.y);
    *reinterpret_cast<uint4 *>(op.dst + gr * Kp + k0 + kk) = make_uint4(c0.x, c0.y, c1.x, c1.y);
  }
}

template <bool SIGNED, int kBN>
__global__ void __launch_bounds__(I8Cfg<kBN>::kThreads, 1)
int8_tc_gemm(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB,
             uint8_t *__restrict__ C, int64_t rso, int64_t cso, int M, int N, int num_kb,
             int tiles_m, int tiles_n, int rule, unsigned *status, WaitCfg wc) {
  constexpr int kNumBuf = I8Cfg<kBN>::kNumBuf, kStages = I8Cfg<kBN>::kStages;
  constexpr int kAccWarps = I8Cfg<kBN>::kAccWarps;
  // slabs per TMEM chunk: a whole 512-deep block, except for uint8 under
  // the rules that need its exact sum (two 256-deep halves; the x86 rule
  // decides every byte from a rounded sum past 2^24 as from the exact one,
  // see int8_pair_gemm)
  const int chunk_log2 = (SIGNED || rule == kRuleX86Packed) ? 3 : 2;
  const int CHUNK = 1 << chunk_log2, CHUNKS_PER_BLOCK = (kBlockK / kBK) >> chunk_log2;
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

  const int tile = blockIdx.x;
  constexpr int GM = 16;
  const int group = tile / (GM * tiles_n);
  const int first_m = group * GM;
  const int gm = min(tiles_m - first_m, GM);
  const int local = tile - group * GM * tiles_n;
  const int m0 = (first_m + local % gm) * kBM;
  const int n0 = (local / gm) * kBN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; s++) {
      tc::mbar_init(tc::smem_u32(&full[s]), 1);
      tc::mbar_init(tc::smem_u32(&empty[s]), 1);
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
  tc::griddep_wait();   // the conversion pass has completed

  if (warp == 0) {
    if (lane == 0) {
      for (int kb = 0; kb < num_kb; kb++) {
        const int s = kb % kStages;
        if (kb >= kStages &&
            !tc::mbar_wait_bounded(tc::smem_u32(&empty[s]), ((kb / kStages) & 1) ^ 1, status,
                                   kStatusTimeoutProducer, wc.limit_ns))
          break;
        if (wc.starve) continue;   // give-up test: no load, no barrier completes
        const uint32_t fbar = tc::smem_u32(&full[s]);
        const uint32_t st = tc::smem_u32(smem + s * STAGE_BYTES);
        tc::mbar_arrive_expect_tx(fbar, STAGE_BYTES);
        tc::tma_load_2d(st, &tA, fbar, kb * kBK, m0);
        tc::tma_load_2d(st + A_BYTES, &tB, fbar, kb * kBK, n0);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_bf16_f32(kBM, kBN);
      for (int kb = 0; kb < num_kb; kb++) {
        const int s = kb % kStages, chunk = kb >> chunk_log2, buf = chunk % kNumBuf;
        const bool cstart = (kb & (CHUNK - 1)) == 0, cend = (kb & (CHUNK - 1)) == CHUNK - 1;
        if (cstart && chunk >= kNumBuf &&
            !tc::mbar_wait_bounded(tc::smem_u32(&tempty[buf]), ((chunk / kNumBuf) & 1) ^ 1,
                                   status, kStatusTimeoutMma, wc.limit_ns))
          break;
        if (!tc::mbar_wait_bounded(tc::smem_u32(&full[s]), (kb / kStages) & 1, status,
                                   kStatusTimeoutMma, wc.limit_ns))
          break;
        tc::tc_fence_after();
        const uint32_t sa = tc::smem_u32(smem + s * STAGE_BYTES), sb = sa + A_BYTES;
#pragma unroll
        for (int kk = 0; kk < kBK / 16; kk++)
          tc::mma_bf16(tmem + buf * kBN, tc::sdesc_k128(sa + kk * 32),
                       tc::sdesc_k128(sb + kk * 32), idesc, (!cstart || kk > 0) ? 1u : 0u);
        tc::mma_commit(tc::smem_u32(&empty[s]));
        if (cend) tc::mma_commit(tc::smem_u32(&tfull[buf]));
      }
      // Every MMA issued above completes before TMEM is released, also when
      // the loop gave up (a commit with none outstanding arrives at once).
      tc::mma_commit(tc::smem_u32(drain));
      tc::mbar_wait_bounded(tc::smem_u32(drain), 0, status, kStatusTimeoutDrain, wc.limit_ns);
    }
    __syncwarp();
  } else {
    constexpr int CW = 32;   // columns per accumulator thread
    const int quad = warp & 3, group = (warp - 2) >> 2;
    const int row = m0 + quad * 32 + lane;
    const int cbase = group * CW;
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    int32_t d[CW], part[CW];
    // x86 rule: columns inside numc's full 6x16 tiles
    const uint32_t fullmask = rule == kRuleX86Packed && simt::x86_row_full(row, M)
                                  ? (uint32_t)simt::x86_col_mask(n0 + cbase, N, CW)
                                  : 0u;
#pragma unroll
    for (int j = 0; j < CW; j++) d[j] = 0;
    const int nchunks = num_kb >> chunk_log2;   // num_kb is a multiple of the block size
    bool ok = true;
    for (int chunk = 0; chunk < nchunks; chunk++) {
      const int buf = chunk % kNumBuf;
      ok = tc::mbar_wait_bounded(tc::smem_u32(&tfull[buf]), (chunk / kNumBuf) & 1, status,
                                 kStatusTimeoutEpilogue, wc.limit_ns);
      ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld below is warp-collective
      if (!ok) break;
      tc::tc_fence_after();
      const bool block_start = chunk % CHUNKS_PER_BLOCK == 0;
#pragma unroll
      for (int c0 = 0; c0 < CW; c0 += 16) {   // 16 columns a load: fewer live registers
        uint32_t r[16];
        tc::tmem_ld_32x32b_x16(tmem + lane_off + buf * kBN + cbase + c0, r);
        tc::tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const int32_t v = __float2int_rn(__uint_as_float(r[j]));   // exact
          part[c0 + j] = block_start ? v : part[c0 + j] + v;
        }
      }
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(tc::smem_u32(&tempty[buf]));
      if (chunk % CHUNKS_PER_BLOCK == CHUNKS_PER_BLOCK - 1) {
        const int b = chunk / CHUNKS_PER_BLOCK;
        if (rule != kRuleX86Packed) {
          // one block over all K: accumulate the wrapped int32 sum
#pragma unroll
          for (int j = 0; j < CW; j++) d[j] = (int32_t)((uint32_t)d[j] + (uint32_t)part[j]);
        } else {
#pragma unroll
          for (int j = 0; j < CW; j++)
            d[j] = simt::fold8_x86(d[j], part[j], b == 0, (fullmask >> j) & 1u, SIGNED);
        }
      }
    }
    const bool staged = cso == 1 && (rso & 3) == 0 && (reinterpret_cast<uintptr_t>(C) & 3) == 0;
    if (ok && row < M && rule != kRuleX86Packed) {
      const bool rf = simt::clamp_row_full(row, M, rule);
      const int ncut = simt::clamp_col_limit(N, rule);
#pragma unroll
      for (int j = 0; j < CW; j++)
        d[j] = simt::narrow_once(d[j], rf && n0 + cbase + j < ncut, SIGNED);
    }
    if (ok && staged) {   // warp-uniform
      uint8_t *stage = smem + kStages * STAGE_BYTES + kBarBytes + (warp - 2) * 1024;
      uint32_t w[CW / 4];
      pack_bytes<CW>(d, w);
      store_bytes_coalesced<CW>(w, stage, C, rso, m0 + quad * 32, n0 + cbase, M, N, lane);
    } else if (ok && row < M) {
      const int col0 = n0 + cbase;
      uint8_t *dst = C + (int64_t)row * rso + (int64_t)col0 * cso;
      if (cso == 1 && ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) && col0 + CW <= N) {
        // the thread's 32 bytes of its row: two 16-byte stores, one sector
        // (byte stores would cost a sector write each)
#pragma unroll
        for (int h = 0; h < CW / 16; h++) {
          uint32_t w[4];
#pragma unroll
          for (int q = 0; q < 4; q++)
            w[q] = (uint32_t)(uint8_t)d[16 * h + 4 * q] |
                   ((uint32_t)(uint8_t)d[16 * h + 4 * q + 1] << 8) |
                   ((uint32_t)(uint8_t)d[16 * h + 4 * q + 2] << 16) |
                   ((uint32_t)(uint8_t)d[16 * h + 4 * q + 3] << 24);
          *reinterpret_cast<uint4 *>(dst + 16 * h) = make_uint4(w[0], w[1], w[2], w[3]);
        }
      } else {
#pragma unroll
        for (int j = 0; j < CW; j++)
          if (col0 + j < N) dst[(int64_t)j * cso] = (uint8_t)d[j];
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

// ---- CTA pairs for large problems -------------------------------------------
//
// Clusters of two CTAs on neighbouring SMs walk 256 x BN output tiles
// persistently (tiles rasterised in groups of 2048 rows).  Each CTA loads
// its own 128 rows of A and BN/2 rows of B^T per 64-deep slab; the even
// CTA's MMA thread multiplies both halves with cta_group::2 MMAs into TMEM
// of both CTAs, so an SM fetches (128 + BN/2) x 64 operand elements per
// 128 x BN x 64 multiply-adds: at BN = 256 half the bytes per MMA of the
// single-CTA 128 x 128 tiles.  TMEM holds two (BN = 256) or four (BN = 128)
// chunk buffers of 128 lanes x BN FP32 columns; 16 accumulator warps per CTA
// (4 per TMEM lane quarter, BN / 4 columns each) fold every finished chunk
// into numc's stored bytes while the next chunk is multiplied.
//
// X86 selects numc's x86 packed rule at compile time: a fold per 512-deep
// block, done in FP32 on the block's sum (fold8_x86_f).  For uint8 that sum
// may exceed 2^24, where FP32 accumulation rounds; but uint8 products are
// non-negative, so the partial sums only grow, the accumulation is exact as
// long as the true sum is at most 2^24, and past that the rounded sum stays
// far above the rule's largest threshold (32767): every stored byte is
// decided exactly, and the block needs one TMEM chunk.  The other rules
// add the chunks' exact sums (uint8: two 256-deep halves) into a wrapped
// int32 and narrow once at the end.

// numc's x86 packed int8/uint8 fold (simt::fold8_x86) in FP32 on the block
// sums read from TMEM, without a float-to-int conversion per block.  d: the
// byte stored so far as a float; P: the block's sum.
template <bool SIGNED>
__device__ __forceinline__ float sat8_f(float x) {
  if constexpr (SIGNED) return fminf(fmaxf(x, -128.0f), 127.0f);
  // packusdw then packuswb: [0,255] kept, (255, 32767] -> 255, else 0
  return x <= 255.0f ? fmaxf(x, 0.0f) : (x <= 32767.0f ? 255.0f : 0.0f);
}
template <bool SIGNED>
__device__ __forceinline__ float fold8_x86_f(float d, float P, bool first, bool full) {
  if (full) return sat8_f<SIGNED>(d + P);
  const float t = sat8_f<SIGNED>(P);
  if (first) return t;
  const float x = d + t;   // wrap to 8 bits
  if constexpr (SIGNED) return x > 127.0f ? x - 256.0f : (x < -128.0f ? x + 256.0f : x);
  return x > 255.0f ? x - 256.0f : x;
}
// s0 = low bfloat16 of `pair` + p0, s1 = high + p1, in FP32 (one
// mixed-precision add each: the bfloat16 operand is widened exactly).
__device__ __forceinline__ void add_bf16_pair(uint32_t pair, float p0, float p1, float &s0,
                                              float &s1) {
  asm("{\n .reg .b16 lo, hi;\n mov.b32 {lo, hi}, %2;\n"
      " add.rn.f32.bf16 %0, lo, %3;\n add.rn.f32.bf16 %1, hi, %4;\n}"
      : "=f"(s0), "=f"(s1)
      : "r"(pair), "f"(p0), "f"(p1));
}

// f integral in [-128, 255]: 1.5 x 2^23 + f has f mod 256 as its low
// mantissa byte.
__device__ __forceinline__ uint32_t f_to_bits(float f) { return __float_as_uint(f + 12582912.0f); }

template <int BN> struct I8PairCfg {
  static constexpr int BN_CTA = BN / 2;
  static constexpr uint32_t A_BYTES = kBM * kBK * 2, B_BYTES = BN_CTA * kBK * 2;
  static constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int STAGES = BN == 256 ? 6 : 8;
  static constexpr int NBUF = 512 / BN;
  static constexpr uint32_t TMEM_COLS = 512;
  static constexpr int CW = BN / 4;            // columns per accumulator thread
  static constexpr int ACC_WARPS = 16, THREADS = 64 + 32 * ACC_WARPS;
  static constexpr uint32_t BAR_BYTES = 256;
  static constexpr uint32_t EPI_BYTES = ACC_WARPS * 32 * CW;   // byte staging per warp
  static constexpr uint32_t SMEM = STAGES * STAGE_BYTES + 1024 + BAR_BYTES + EPI_BYTES;
  static_assert(SMEM <= 232448, "shared memory");
  static_assert((2 * STAGES + 2 * NBUF + 1) * 8 + 4 <= BAR_BYTES, "barrier space");
};

template <bool SIGNED, int BN, bool X86>
__global__ void __launch_bounds__(I8PairCfg<BN>::THREADS, 1)
int8_pair_gemm(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB,
               uint8_t *__restrict__ C, int64_t rso, int64_t cso, int M, int N, int num_kb,
               int tiles_m, int tiles_n, int rule, unsigned *status, WaitCfg wc) {
  using Cfg = I8PairCfg<BN>;
  constexpr int STAGES = Cfg::STAGES, NBUF = Cfg::NBUF, CW = Cfg::CW;
  // slabs per TMEM chunk: the x86 rule folds every 512-deep block; the
  // other rules need exact sums only, which FP32 keeps up to 2^24 (int8:
  // 1024-deep chunks, |sum| <= 1024 * 128^2 = 2^24; uint8: 256-deep ones)
  constexpr int CHUNK = X86 ? kBlockK / kBK : SIGNED ? 2 * kBlockK / kBK : kBlockK / kBK / 2;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *bars = (uint64_t *)(smem + STAGES * Cfg::STAGE_BYTES);
  uint64_t *full = bars, *empty = bars + STAGES;
  uint64_t *tfull = bars + 2 * STAGES, *tempty = tfull + NBUF;
  uint64_t *drain = tempty + NBUF;   // all issued MMAs complete
  uint32_t *tmem_slot = (uint32_t *)(drain + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
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
    n0 = (local / gm) * BN;
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      tc::mbar_init(tc::smem_u32(&full[s]), 1);
      tc::mbar_init(tc::smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < NBUF; b++) {
      tc::mbar_init(tc::smem_u32(&tfull[b]), 1);
      tc::mbar_init(tc::smem_u32(&tempty[b]), Cfg::ACC_WARPS * 2);   // both CTAs' warps
    }
    tc::mbar_init(tc::smem_u32(drain), 1);
    tc::fence_barrier_init();
    tc::tma_prefetch_desc(&tA);
    tc::tma_prefetch_desc(&tB);
  }
  if (warp == 1) tc::tmem_alloc_pair(tc::smem_u32(tmem_slot), Cfg::TMEM_COLS);
  tc::tc_fence_before();
  __syncthreads();
  tc::cluster_sync();   // peer barriers initialised
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  tc::griddep_wait();   // the conversion pass has completed
  // per tile; num_kb is a multiple of the 512-deep block (8 slabs), and a
  // 1024-deep chunk may end early at the last slab
  const int nchunks = (num_kb + CHUNK - 1) / CHUNK;

  if (warp == 0) {
    if (lane == 0) {
      int g = 0;   // stage counter across tiles
      bool live = true;
      for (int t = first_tile; t < ntiles && live; t += tile_step) {
        int m0, n0;
        tile_origin(t, m0, n0);
        const int ma = m0 + (int)rank * kBM, nb = n0 + (int)rank * Cfg::BN_CTA;
        for (int kb = 0; kb < num_kb; kb++, g++) {
          const int s = g % STAGES;
          if (g >= STAGES &&
              !tc::mbar_wait_bounded(tc::smem_u32(&empty[s]), ((g / STAGES) & 1) ^ 1, status,
                                     kStatusTimeoutProducer, wc.limit_ns)) {
            live = false;
            break;
          }
          if (wc.starve) continue;   // give-up test: no load, no barrier ever completes
          const uint32_t fbar = tc::smem_u32(&full[s]);
          const uint32_t st = tc::smem_u32(smem + s * Cfg::STAGE_BYTES);
          // the even CTA's full barrier counts the bytes of both CTAs
          if (leader) tc::mbar_arrive_expect_tx(fbar, 2 * Cfg::STAGE_BYTES);
          const uint32_t fbar_leader = tc::mapa_shared(fbar, 0);
          tc::tma_load_3d_pair(st, &tA, fbar_leader, kb * kBK, ma, 0);
          tc::tma_load_3d_pair(st + Cfg::A_BYTES, &tB, fbar_leader, kb * kBK, nb, 0);
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0 && leader) {
      constexpr uint32_t idesc = tc::idesc_bf16_f32(2 * kBM, BN);
      int g = 0, chunk = 0;   // stage and chunk counters across tiles
      bool live = true;
      for (int t = first_tile; t < ntiles && live; t += tile_step) {
        for (int kb = 0; kb < num_kb; kb++, g++) {
          const int s = g % STAGES, buf = chunk % NBUF;
          const bool cstart = kb % CHUNK == 0;
          const bool cend = kb % CHUNK == CHUNK - 1 || kb == num_kb - 1;
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
          const uint32_t sa = tc::smem_u32(smem + s * Cfg::STAGE_BYTES), sb = sa + Cfg::A_BYTES;
#pragma unroll
          for (int kk = 0; kk < kBK / 16; kk++)
            tc::mma_f16_pair(tmem + buf * BN, tc::sdesc_k128(sa + kk * 32),
                             tc::sdesc_k128(sb + kk * 32), idesc, (!cstart || kk > 0) ? 1u : 0u);
          tc::mma_commit_pair(tc::smem_u32(&empty[s]), 0x3);
          if (cend) {
            tc::mma_commit_pair(tc::smem_u32(&tfull[buf]), 0x3);
            chunk++;
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
    // warp w reads TMEM lanes 32 * (w % 4); the four warps of a lane quarter
    // split the tile's columns CW apiece
    const int quad = warp & 3, grp = (warp - 2) >> 2;
    const int cbase = grp * CW;
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    uint8_t *stage = smem + STAGES * Cfg::STAGE_BYTES + Cfg::BAR_BYTES + (warp - 2) * (32 * CW);
    const bool staged = cso == 1 && (rso & 3) == 0 && (reinterpret_cast<uintptr_t>(C) & 3) == 0;
    int chunk = 0;   // across tiles
    bool ok = true;
    for (int t = first_tile; t < ntiles && ok; t += tile_step) {
      int m0, n0;
      tile_origin(t, m0, n0);
      const int mr = m0 + (int)rank * kBM;   // this CTA's 128 rows
      const int row = mr + quad * 32 + lane;
      // x86 rule: the stored values so far as bfloat16 pairs (every fold
      // leaves an integer in [-128, 255], exact in bfloat16); other rules:
      // the wrapped int32 sums
      int32_t d[X86 ? 1 : CW];
      uint32_t d16[X86 ? CW / 2 : 1];
      // x86 rule: columns inside numc's full 6x16 tiles
      const uint64_t fullmask =
          X86 && simt::x86_row_full(row, M) ? simt::x86_col_mask(n0 + cbase, N, CW) : 0ull;
      if constexpr (!X86) {
#pragma unroll
        for (int j = 0; j < CW; j++) d[j] = 0;
      }
#pragma unroll
      for (int q = 0; q < (X86 ? CW / 2 : 1); q++) d16[q] = 0;
      // warp-uniform: every column of every lane inside numc's full tiles
      const bool all_full = X86 && __all_sync(0xffffffffu, fullmask == ~0ull >> (64 - CW));
      for (int c = 0; c < nchunks; c++, chunk++) {
        const int buf = chunk % NBUF;
        ok = tc::mbar_wait_bounded(tc::smem_u32(&tfull[buf]), (chunk / NBUF) & 1, status,
                                   kStatusTimeoutEpilogue, wc.limit_ns);
        ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld below is warp-collective
        if (!ok) break;
        tc::tc_fence_after();
        const bool first = c == 0;
        const uint32_t taddr = tmem + lane_off + buf * BN + cbase;
        if constexpr (X86) {
          // 32 columns per TMEM wait; the tile class decided outside the loop
          auto drain = [&](auto full_tag) {
            constexpr bool ALL_FULL = decltype(full_tag)::value;
#pragma unroll
            for (int c0 = 0; c0 < CW; c0 += 32) {
              uint32_t r[32];
              tc::tmem_ld_32x32b_x16(taddr + c0, *reinterpret_cast<uint32_t(*)[16]>(&r[0]));
              tc::tmem_ld_32x32b_x16(taddr + c0 + 16, *reinterpret_cast<uint32_t(*)[16]>(&r[16]));
              tc::tmem_ld_wait();
#pragma unroll
              for (int h = 0; h < 16; h++) {
                const int q = (c0 >> 1) + h;   // bfloat16 pair: columns 2q, 2q + 1
                const float p0 = __uint_as_float(r[2 * h]), p1 = __uint_as_float(r[2 * h + 1]);
                const float v0 = __uint_as_float(d16[q] << 16);
                const float v1 = __uint_as_float(d16[q] & 0xffff0000u);
                float f0, f1;
                if constexpr (ALL_FULL && SIGNED) {
                  // d = clamp(d + P, -128, 127) on the pair in bfloat16: the
                  // FP32 sums are exact integers, bfloat16 keeps those up to
                  // 256 in magnitude exactly and rounds larger ones to values
                  // past the same bound
                  float s0, s1;
                  add_bf16_pair(d16[q], p0, p1, s0, s1);
                  const __nv_bfloat162 c = __hmin2(
                      __hmax2(__floats2bfloat162_rn(s0, s1), __float2bfloat162_rn(-128.0f)),
                      __float2bfloat162_rn(127.0f));
                  d16[q] = *reinterpret_cast<const uint32_t *>(&c);
                  continue;
                } else if constexpr (ALL_FULL) {   // d = sat(d + P)
                  f0 = sat8_f<SIGNED>(v0 + p0);
                  f1 = sat8_f<SIGNED>(v1 + p1);
                } else {
                  f0 = fold8_x86_f<SIGNED>(v0, p0, first, (fullmask >> (2 * q)) & 1ull);
                  f1 = fold8_x86_f<SIGNED>(v1, p1, first, (fullmask >> (2 * q + 1)) & 1ull);
                }
                d16[q] = __byte_perm(__float_as_uint(f0), __float_as_uint(f1), 0x7632);
              }
            }
          };
          if (all_full) drain(std::true_type{});   // warp-uniform
          else drain(std::false_type{});
        } else {
#pragma unroll
          for (int c0 = 0; c0 < CW; c0 += 16) {
            uint32_t r[16];
            tc::tmem_ld_32x32b_x16(taddr + c0, r);
            tc::tmem_ld_wait();
#pragma unroll
            for (int j = 0; j < 16; j++)
              d[c0 + j] = (int32_t)((uint32_t)d[c0 + j] +
                                    (uint32_t)__float2int_rn(__uint_as_float(r[j])));   // exact
          }
        }
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0)   // the buffer's loads completed at tcgen05.wait::ld
          tc::mbar_arrive_cluster_relaxed(tc::mapa_shared(tc::smem_u32(&tempty[buf]), 0));
      }
      if (!ok) break;
      uint32_t w[CW / 4];
      if constexpr (X86) {
#pragma unroll
        for (int q = 0; q < CW / 4; q++) {
          const uint32_t a = d16[2 * q], b = d16[2 * q + 1];
          w[q] = pack4((int32_t)f_to_bits(__uint_as_float(a << 16)),
                       (int32_t)f_to_bits(__uint_as_float(a & 0xffff0000u)),
                       (int32_t)f_to_bits(__uint_as_float(b << 16)),
                       (int32_t)f_to_bits(__uint_as_float(b & 0xffff0000u)));
        }
      } else {
        if (row < M) {
          const bool rf = simt::clamp_row_full(row, M, rule);
          const int ncut = simt::clamp_col_limit(N, rule);
#pragma unroll
          for (int j = 0; j < CW; j++)
            d[j] = simt::narrow_once(d[j], rf && n0 + cbase + j < ncut, SIGNED);
        }
        pack_bytes<CW>(d, w);
      }
      if (staged) {   // warp-uniform
        store_bytes_coalesced<CW>(w, stage, C, rso, mr + quad * 32, n0 + cbase, M, N, lane);
      } else if (row < M) {
#pragma unroll
        for (int j = 0; j < CW; j++)
          if (n0 + cbase + j < N)
            C[(int64_t)row * rso + (int64_t)(n0 + cbase + j) * cso] = (uint8_t)(w[j >> 2] >> (8 * (j & 3)));
      }
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
    tc::tmem_dealloc_pair(tmem, Cfg::TMEM_COLS);
  }
}

struct I8Layout {
  int64_t Kp;
  size_t a, b, total;
};

I8Layout i8_layout(int64_t M, int64_t K, int64_t N) {
  I8Layout L;
  L.Kp = round_up(K > 0 ? K : 1, kBlockK);
  L.a = 0;
  L.b = (size_t)round_up(M * L.Kp * 2, 256);
  L.total = L.b + (size_t)round_up(N * L.Kp * 2, 256);
  return L;
}

template <bool SIGNED, int kBN>
cudaError_t launch_i8_gemm(const Gemm &g, int rule, const I8Layout &L, __nv_bfloat16 *pa,
                           __nv_bfloat16 *pb, unsigned *status, cudaStream_t s) {
  using Cfg = I8Cfg<kBN>;
  CUtensorMap ta, tb;
  cudaError_t e;
  if ((e = make_tmap_2d(&ta, pa, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, g.M, L.Kp, L.Kp, kBM, kBK)))
    return e;
  if ((e = make_tmap_2d(&tb, pb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, g.N, L.Kp, L.Kp, kBN, kBK)))
    return e;
  static_assert((2 * Cfg::kStages + 2 * Cfg::kNumBuf + 1) * 8 + 4 <= kBarBytes, "barrier space");
  // ring, alignment, barriers, and 1 KiB of store staging per accumulator warp
  constexpr uint32_t SMEM =
      Cfg::kStages * (kBM + kBN) * kBK * 2 + 1024 + kBarBytes + Cfg::kAccWarps * 1024;
  static_assert(SMEM <= 232448, "shared memory");
  static LaunchCache lc;
  if ((e = smem_attr_once(lc, (const void *)int8_tc_gemm<SIGNED, kBN>, SMEM))) return e;
  const int tiles_m = (int)((g.M + kBM - 1) / kBM), tiles_n = (int)((g.N + kBN - 1) / kBN);
  // programmatic dependent launch: set up while the conversion pass ends
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
  cfg.gridDim = dim3((unsigned)(tiles_m * tiles_n));
  cfg.blockDim = dim3(Cfg::kThreads);
  cfg.dynamicSmemBytes = SMEM;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if ((e = cudaLaunchKernelEx(&cfg, int8_tc_gemm<SIGNED, kBN>, ta, tb, (uint8_t *)g.c, g.rso,
                              g.cso, (int)g.M, (int)g.N, (int)(L.Kp / kBK), tiles_m, tiles_n,
                              rule, status, wait_cfg())))
    return e;
  count_launch();
  return cudaGetLastError();
}

template <bool SIGNED, int BN, bool X86>
cudaError_t launch_i8_pair(const Gemm &g, int rule, const I8Layout &L, const __nv_bfloat16 *pa,
                           const __nv_bfloat16 *pb, unsigned *status, cudaStream_t s) {
  using Cfg = I8PairCfg<BN>;
  CUtensorMap ta, tb;
  cudaError_t e;
  if ((e = make_tmap_3d(&ta, pa, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, 1, g.M, L.Kp, L.Kp, kBM,
                        kBK)))
    return e;
  if ((e = make_tmap_3d(&tb, pb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, 1, g.N, L.Kp, L.Kp,
                        Cfg::BN_CTA, kBK)))
    return e;
  auto kern = int8_pair_gemm<SIGNED, BN, X86>;
  static LaunchCache lc;
  if ((e = smem_attr_once(lc, (const void *)kern, Cfg::SMEM))) return e;
  const int tiles_m = (int)((g.M + 2 * kBM - 1) / (2 * kBM));
  const int tiles_n = (int)((g.N + BN - 1) / BN);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  // programmatic dependent launch: set up while the conversion pass ends
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
  cfg.blockDim = dim3(Cfg::THREADS);
  cfg.dynamicSmemBytes = Cfg::SMEM;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3((unsigned)(2 * std::max(1, sm_count() / 2)));
  int pairs = clusters_once(lc, (const void *)kern, cfg);
  if (pairs <= 0) pairs = std::max(1, sm_count() / 2);
  pairs = std::min(pairs, tiles_m * tiles_n);
  cfg.gridDim = dim3((unsigned)(2 * pairs));
  cfg.numAttrs = 2;
  e = cudaLaunchKernelEx(&cfg, kern, ta, tb, (uint8_t *)g.c, (int64_t)g.rso, (int64_t)g.cso,
                         (int)g.M, (int)g.N, (int)(L.Kp / kBK), tiles_m, tiles_n, rule, status,
                         wait_cfg());
  if (e != cudaSuccess) return e;
  count_launch();
  return cudaGetLastError();
}

// Tile schedule when the caller names none: CTA pairs with 256 x 256
// tiles once those give three pairs in four a tile (measured on GB300: at
// 2048^3 and above they beat the single-CTA tiles by 1.2-1.4x), else
// single-CTA tiles (128 x 128 while they cover the SMs, else 128 x 64).
int pick_tile(const Gemm &g) {
  const int64_t pairs = std::max(1, sm_count() / 2);
  const int64_t tiles = (g.M + 2 * kBM - 1) / (2 * kBM) * ((g.N + 255) / 256);
  return 4 * tiles >= 3 * pairs ? kI8TilePair256 : kI8TileSingle;
}

template <bool SIGNED>
cudaError_t launch_i8(const Gemm &g, int rule, int tile, char *ws, const I8Layout &L,
                      cudaStream_t s) {
  unsigned *status = status_word();
  if (!status) return cudaErrorMemoryAllocation;
  PhaseMark mark(s);
  auto *pa = (__nv_bfloat16 *)(ws + L.a), *pb = (__nv_bfloat16 *)(ws + L.b);
  const I8Operand oa{(const uint8_t *)g.a, g.rsa, g.csa, g.M, pa};
  const I8Operand ob{(const uint8_t *)g.b, g.csb, g.rsb, g.N, pb};   // B^T
  // 64 x 256 blocks, or 64 x 128 while the deeper blocks would not give
  // every SM two
  const int64_t rows = (g.M + kCvtRows - 1) / kCvtRows + (g.N + kCvtRows - 1) / kCvtRows;
  const int kc = rows * (L.Kp / 256) >= 2 * sm_count() ? 256 : 128;
  const int64_t kblocks = L.Kp / kc;
  const int64_t blocks_a = (g.M + kCvtRows - 1) / kCvtRows * kblocks;
  const int64_t blocks_b = (g.N + kCvtRows - 1) / kCvtRows * kblocks;
  if (blocks_a + blocks_b >= (1ll << 31)) return cudaErrorInvalidConfiguration;
  if (kc == 256)
    int8_pair_to_bf16<SIGNED, 256><<<(unsigned)(blocks_a + blocks_b), 256, 0, s>>>(
        oa, ob, g.K, L.Kp, blocks_a);
  else
    int8_pair_to_bf16<SIGNED, 128><<<(unsigned)(blocks_a + blocks_b), 256, 0, s>>>(
        oa, ob, g.K, L.Kp, blocks_a);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e) return e;
  mark.split_done();
  const bool x86 = rule == kRuleX86Packed;
  if (tile == kI8TileAuto) tile = pick_tile(g);
  if (tile == kI8TilePair256)
    e = x86 ? launch_i8_pair<SIGNED, 256, true>(g, rule, L, pa, pb, status, s)
            : launch_i8_pair<SIGNED, 256, false>(g, rule, L, pa, pb, status, s);
  else if (tile == kI8TilePair128)
    e = x86 ? launch_i8_pair<SIGNED, 128, true>(g, rule, L, pa, pb, status, s)
            : launch_i8_pair<SIGNED, 128, false>(g, rule, L, pa, pb, status, s);
  else if (((g.M + kBM - 1) / kBM) * ((g.N + 127) / 128) >= sm_count())
    e = launch_i8_gemm<SIGNED, 128>(g, rule, L, pa, pb, status, s);
  else
    e = launch_i8_gemm<SIGNED, 64>(g, rule, L, pa, pb, status, s);
  mark.gemm_done();
  return e;
}

}  // namespace

size_t int8_tc_workspace(int64_t M, int64_t K, int64_t N) { return i8_layout(M, K, N).total; }

cudaError_t launch_int8_tc(NumcDType dt, const Gemm &g, int param, void *ws, size_t ws_bytes,
                           cudaStream_t s) {
  if (g.M == 0 || g.N == 0) return cudaSuccess;
  if (g.K == 0) return launch_simt(dt, g, param & 0xff, s);   // C = 0
  if (g.M >= (1ll << 31) || g.N >= (1ll << 31) || g.K >= (1ll << 31)) return cudaErrorInvalidValue;
  const I8Layout L = i8_layout(g.M, g.K, g.N);
  if (ws_bytes < L.total || ((uintptr_t)ws & 255)) return cudaErrorInvalidValue;
  const int rule = param & 0xff, tile = param >> 8;
  if (tile < kI8TileAuto || tile > kI8TilePair256) return cudaErrorInvalidValue;
  if (dt == NUMC_DTYPE_INT8) return launch_i8<true>(g, rule, tile, (char *)ws, L, s);
  if (dt == NUMC_DTYPE_UINT8) return launch_i8<false>(g, rule, tile, (char *)ws, L, s);
  return cudaErrorInvalidValue;
}

}  // namespace numc_k

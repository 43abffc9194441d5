// float32 GEMM as a 3-pass split-BF16 product on the 5th-generation tensor
// cores (tcgen05), the fast alternative to numc's FP32 FMA GEMM
// (src/intrinsics/gemm_avx2.h:852 gemm_f32_avx2).
//
// Every float32 x is split as x = hi + lo + r with hi = bf16(x) and
// lo = bf16(x - hi) (|r| <= 2^-17 |x|).  C = A_hi B_hi + A_hi B_lo + A_lo B_hi
// accumulated in FP32 in tensor memory; the dropped A_lo B_lo term is below
// 2^-16 of each product.
//
// Pass 1 (split kernel, HBM-bound): reads A and B once with any strides and
// writes hi/lo planes, K-major with K padded to 64 (B is transposed on the
// way), so both operands suit a 128-byte-swizzled TMA box.
// Pass 2 (GEMM kernel): one 128 x BN output tile per CTA.  Warp 0 lane 0
// streams (A_hi, A_lo, B_hi, B_lo) 64-deep K slabs into a STAGES-deep
// shared-memory ring with TMA; warp 1 lane 0 issues three
// tcgen05.mma.kind::f16 per 16-deep K step into one FP32 TMEM accumulator
// and releases ring slots with tcgen05.commit; then all four warps drain
// TMEM (tcgen05.ld 32x32b) and store the tile.  Tiles are rasterised in
// groups of 16 row-tiles so the live operand panels stay in L2.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <mutex>

#include "numc/cuda.h"
#include "numc/error.h"

#include "kernels.h"
#include "phase_timing.h"
#include "status.h"
#include "tc_common.cuh"

namespace numc_k {
namespace {

constexpr int kBM = 128, kBK = 64;

__host__ __device__ inline int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

// ---- pass 1: split float32 into bf16 hi/lo planes -------------------------
//
// dst(row, k) = src[row * rs_row + k * rs_k] for row < R, k < K; zero for
// K <= k < Kp.  hi and lo are R x Kp row-major.  A 32 x 64 tile per block is
// staged through shared memory so both the read (along whichever source
// dimension is contiguous) and the write (along k) are coalesced.
//
// Non-finite inputs cannot go through the split (inf * lo with lo = 0 gives
// NaN where the true product is infinite), so the block records them: the
// flag word of the row group (row / flag_rows) is set to `gen`, the call's
// generation number, and the GEMM recomputes the affected output tiles with
// plain FMA chains.  Stale flags from earlier calls hold other numbers.
__global__ void __launch_bounds__(256) split_f32_bf16(const float *__restrict__ src,
                                                      int64_t rs_row, int64_t rs_k, int64_t R,
                                                      int64_t K, int64_t Kp,
                                                      __nv_bfloat16 *__restrict__ hi,
                                                      __nv_bfloat16 *__restrict__ lo,
                                                      unsigned long long *flags, int flag_rows,
                                                      unsigned long long gen) {
  __shared__ float tile[32][65];
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 64;
  const int tid = threadIdx.x;
  const bool kfast = rs_k == 1 || rs_row != 1;
#pragma unroll
  for (int q = 0; q < 8; q++) {
    int e = tid + 256 * q;
    int r = kfast ? e / 64 : e % 32;
    int k = kfast ? e % 64 : e / 32;
    int64_t gr = r0 + r, gk = k0 + k;
    float x = (gr < R && gk < K) ? src[gr * rs_row + gk * rs_k] : 0.0f;
    if (!isfinite(x)) flags[gr / flag_rows] = gen;
    tile[r][k] = x;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 4; q++) {
    int e = tid + 256 * q;
    int r = e / 32, kp = e % 32;
    int64_t gr = r0 + r;
    if (gr >= R) continue;
    __nv_bfloat16 h[2], l[2];
#pragma unroll
    for (int t = 0; t < 2; t++) {
      float x = tile[r][2 * kp + t];
      __nv_bfloat16 hb = __float2bfloat16_rn(x);
      float hf = __bfloat162float(hb);
      if (isinf(hf) && !isinf(x)) {            // rounding overflowed: truncate
        hb = __float2bfloat16_rz(x);
        hf = __bfloat162float(hb);
      }
      h[t] = hb;
      l[t] = isfinite(x) ? __float2bfloat16_rn(x - hf) : __float2bfloat16_rn(0.0f);
    }
    int64_t off = gr * Kp + k0 + 2 * kp;
    *reinterpret_cast<__nv_bfloat162 *>(hi + off) = __halves2bfloat162(h[0], h[1]);
    *reinterpret_cast<__nv_bfloat162 *>(lo + off) = __halves2bfloat162(l[0], l[1]);
  }
}

// ---- pass 2: the tcgen05 GEMM ------------------------------------------------

// Original operands and the non-finite flags, for tiles that must be
// recomputed with plain FMA chains.
struct Fallback {
  const float *A, *B;
  int64_t rsa, csa, rsb, csb, K;
  const unsigned long long *flags_a, *flags_b;   // per 128 rows of A, per 64 columns of B
  unsigned long long gen;
};

template <int BN, int STAGES>
struct SplitCfg {
  static constexpr uint32_t A_BYTES = kBM * kBK * 2;
  static constexpr uint32_t B_BYTES = BN * kBK * 2;
  static constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
  static constexpr uint32_t SMEM = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
  static constexpr uint32_t TMEM_COLS = BN;   // FP32 accumulator columns
};

template <int BN, int STAGES>
__global__ void __launch_bounds__(128, 1)
split_bf16_gemm(const __grid_constant__ CUtensorMap tAhi, const __grid_constant__ CUtensorMap tAlo,
                const __grid_constant__ CUtensorMap tBhi, const __grid_constant__ CUtensorMap tBlo,
                float *__restrict__ C, int64_t rso, int64_t cso, int M, int N, int num_kb,
                int tiles_m, int tiles_n, int vec4, unsigned *status, Fallback fb) {
  using Cfg = SplitCfg<BN, STAGES>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *bars = (uint64_t *)(smem + STAGES * Cfg::STAGE_BYTES);
  uint64_t *full = bars, *empty = bars + STAGES, *accum = bars + 2 * STAGES;
  uint32_t *tmem_slot = (uint32_t *)(bars + 2 * STAGES + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // Grouped rasterisation: 16 row-tiles per group sweep all column tiles.
  const int tile = blockIdx.x;
  constexpr int GM = 16;
  const int group = tile / (GM * tiles_n);
  const int first_m = group * GM;
  const int gm = min(tiles_m - first_m, GM);
  const int local = tile - group * GM * tiles_n;
  const int m0 = (first_m + local % gm) * kBM;
  const int n0 = (local / gm) * BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      tc::mbar_init(tc::smem_u32(&full[s]), 1);
      tc::mbar_init(tc::smem_u32(&empty[s]), 1);
    }
    tc::mbar_init(tc::smem_u32(accum), 1);
    tc::fence_barrier_init();
    tc::tma_prefetch_desc(&tAhi);
    tc::tma_prefetch_desc(&tAlo);
    tc::tma_prefetch_desc(&tBhi);
    tc::tma_prefetch_desc(&tBlo);
  }
  if (warp == 1) tc::tmem_alloc(tc::smem_u32(tmem_slot), Cfg::TMEM_COLS);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // TMA producer
    for (int kb = 0; kb < num_kb; kb++) {
      const int s = kb % STAGES;
      if (kb >= STAGES &&
          !tc::mbar_wait_bounded(tc::smem_u32(&empty[s]), ((kb / STAGES) & 1) ^ 1, status,
                                 kStatusTimeoutProducer))
        break;
      const uint32_t fbar = tc::smem_u32(&full[s]);
      uint8_t *st = smem + s * Cfg::STAGE_BYTES;
      tc::mbar_arrive_expect_tx(fbar, Cfg::STAGE_BYTES);
      const int k = kb * kBK;
      tc::tma_load_2d(tc::smem_u32(st), &tAhi, fbar, k, m0);
      tc::tma_load_2d(tc::smem_u32(st + Cfg::A_BYTES), &tAlo, fbar, k, m0);
      tc::tma_load_2d(tc::smem_u32(st + 2 * Cfg::A_BYTES), &tBhi, fbar, k, n0);
      tc::tma_load_2d(tc::smem_u32(st + 2 * Cfg::A_BYTES + Cfg::B_BYTES), &tBlo, fbar, k, n0);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: 3 products per 16-deep K step into one accumulator.
    constexpr uint32_t idesc = tc::idesc_bf16_f32(kBM, BN);
    for (int kb = 0; kb < num_kb; kb++) {
      const int s = kb % STAGES;
      if (!tc::mbar_wait_bounded(tc::smem_u32(&full[s]), (kb / STAGES) & 1, status,
                                 kStatusTimeoutMma))
        break;
      tc::tc_fence_after();
      const uint32_t st = tc::smem_u32(smem + s * Cfg::STAGE_BYTES);
      const uint32_t a_hi = st, a_lo = st + Cfg::A_BYTES;
      const uint32_t b_hi = st + 2 * Cfg::A_BYTES, b_lo = b_hi + Cfg::B_BYTES;
#pragma unroll
      for (int kk = 0; kk < kBK / 16; kk++) {
        const uint32_t koff = kk * 32;   // 16 bf16 = 32 bytes inside the swizzle atom
        const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
        tc::mma_bf16(tmem, tc::sdesc_k128(a_lo + koff), tc::sdesc_k128(b_hi + koff), idesc, acc);
        tc::mma_bf16(tmem, tc::sdesc_k128(a_hi + koff), tc::sdesc_k128(b_lo + koff), idesc, 1u);
        tc::mma_bf16(tmem, tc::sdesc_k128(a_hi + koff), tc::sdesc_k128(b_hi + koff), idesc, 1u);
      }
      tc::mma_commit(tc::smem_u32(&empty[s]));
    }
    tc::mma_commit(tc::smem_u32(accum));
  }
  __syncwarp();

  // Epilogue: TMEM -> registers -> global.  Warp w owns TMEM lanes
  // [32w, 32w + 32), i.e. tile rows m0 + 32w + lane.
  const uint64_t limit = 2000000000ull + (uint64_t)num_kb * 20000ull;
  const bool ok = tc::mbar_wait_bounded(tc::smem_u32(accum), 0, status, kStatusTimeoutEpilogue, limit);
  tc::tc_fence_after();
  bool nonfinite = fb.flags_a[m0 / kBM] == fb.gen;
#pragma unroll 1
  for (int c = n0 / 64; c < (n0 + BN) / 64 && c * 64 < N; c++)
    nonfinite |= fb.flags_b[c] == fb.gen;
  if (ok && nonfinite) {
    // numc's arithmetic: one FMA chain per output in k order (slow path).
    const int row = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < BN && row < M; c0 += 32) {
      float acc[32];
#pragma unroll
      for (int j = 0; j < 32; j++) acc[j] = 0.0f;
#pragma unroll 1
      for (int64_t k = 0; k < fb.K; k++) {
        const float av = fb.A[(int64_t)row * fb.rsa + k * fb.csa];
        const float *brow = fb.B + k * fb.rsb;
#pragma unroll
        for (int j = 0; j < 32; j++) {
          const int col = n0 + c0 + j;
          const float bv = col < N ? brow[(int64_t)col * fb.csb] : 0.0f;
          acc[j] = __fmaf_rn(av, bv, acc[j]);
        }
      }
#pragma unroll
      for (int j = 0; j < 32; j++)
        if (n0 + c0 + j < N) C[(int64_t)row * rso + (int64_t)(n0 + c0 + j) * cso] = acc[j];
    }
  } else if (ok) {
    const int row = m0 + warp * 32 + lane;
    float *crow = C + (int64_t)row * rso;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
      uint32_t r[32];
      tc::tmem_ld_32x32b_x32(tmem + ((uint32_t)(warp * 32) << 16) + c0, r);
      tc::tmem_ld_wait();
      if (row < M) {
        const int nb = n0 + c0;
        if (vec4 && nb + 32 <= N) {
          float4 *p = reinterpret_cast<float4 *>(crow + nb);
#pragma unroll
          for (int j = 0; j < 8; j++)
            p[j] = make_float4(__uint_as_float(r[4 * j]), __uint_as_float(r[4 * j + 1]),
                               __uint_as_float(r[4 * j + 2]), __uint_as_float(r[4 * j + 3]));
        } else {
#pragma unroll
          for (int j = 0; j < 32; j++)
            if (nb + j < N) crow[(int64_t)(nb + j) * cso] = __uint_as_float(r[j]);
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, Cfg::TMEM_COLS);
  }
}

struct SplitLayout {
  int64_t Kp;
  size_t a_hi, a_lo, b_hi, b_lo, flags_a, flags_b, total;
};

SplitLayout split_layout(int64_t M, int64_t K, int64_t N) {
  SplitLayout L;
  L.Kp = round_up(K > 0 ? K : 1, kBK);
  size_t a = (size_t)round_up(M * L.Kp * 2, 256), b = (size_t)round_up(N * L.Kp * 2, 256);
  L.a_hi = 0;
  L.a_lo = a;
  L.b_hi = 2 * a;
  L.b_lo = 2 * a + b;
  L.flags_a = 2 * a + 2 * b;
  L.flags_b = L.flags_a + (size_t)round_up(((M + kBM - 1) / kBM) * 8, 256);
  L.total = L.flags_b + (size_t)round_up(((N + 63) / 64) * 8, 256);
  return L;
}

// Generation numbers of split calls (never 0; flags hold the last writer's).
std::atomic<unsigned long long> g_split_gen{0x5eed000000000000ull};

template <int BN, int STAGES>
cudaError_t launch_gemm_status(const SplitLayout &L, char *ws, const Gemm &g,
                               unsigned long long gen, unsigned *status, cudaStream_t s) {
  using Cfg = SplitCfg<BN, STAGES>;
  CUtensorMap ta_hi, ta_lo, tb_hi, tb_lo;
  cudaError_t e;
  if ((e = make_tmap_2d(&ta_hi, ws + L.a_hi, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, g.M, L.Kp, L.Kp, kBM, kBK))) return e;
  if ((e = make_tmap_2d(&ta_lo, ws + L.a_lo, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, g.M, L.Kp, L.Kp, kBM, kBK))) return e;
  if ((e = make_tmap_2d(&tb_hi, ws + L.b_hi, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, g.N, L.Kp, L.Kp, BN, kBK))) return e;
  if ((e = make_tmap_2d(&tb_lo, ws + L.b_lo, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, g.N, L.Kp, L.Kp, BN, kBK))) return e;
  auto kern = split_bf16_gemm<BN, STAGES>;
  if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM)))
    return e;
  const int tiles_m = (int)((g.M + kBM - 1) / kBM), tiles_n = (int)((g.N + BN - 1) / BN);
  const int vec4 = g.cso == 1 && (g.rso % 4) == 0 && ((uintptr_t)g.c % 16) == 0;
  Fallback fb;
  fb.A = (const float *)g.a;
  fb.B = (const float *)g.b;
  fb.rsa = g.rsa; fb.csa = g.csa; fb.rsb = g.rsb; fb.csb = g.csb; fb.K = g.K;
  fb.flags_a = (const unsigned long long *)(ws + L.flags_a);
  fb.flags_b = (const unsigned long long *)(ws + L.flags_b);
  fb.gen = gen;
  kern<<<tiles_m * tiles_n, 128, Cfg::SMEM, s>>>(ta_hi, ta_lo, tb_hi, tb_lo, (float *)g.c, g.rso,
                                                 g.cso, (int)g.M, (int)g.N, (int)(L.Kp / kBK),
                                                 tiles_m, tiles_n, vec4, status, fb);
  count_launch();
  return cudaGetLastError();
}

template <int BN, int STAGES>
cudaError_t launch_gemm(const SplitLayout &L, char *ws, const Gemm &g, unsigned long long gen,
                        cudaStream_t s) {
  unsigned *status = status_word();
  if (!status) return cudaErrorMemoryAllocation;
  return launch_gemm_status<BN, STAGES>(L, ws, g, gen, status, s);
}

}  // namespace

size_t split_bf16_workspace(int64_t M, int64_t K, int64_t N) {
  return split_layout(M, K, N).total;
}

cudaError_t launch_split_bf16(const Gemm &g, void *ws_v, size_t ws_bytes, cudaStream_t s) {
  if (g.M == 0 || g.N == 0) return cudaSuccess;
  if (g.K == 0) return launch_simt(NUMC_DTYPE_FLOAT32, g, 0, s);   // C = 0
  if (g.M >= (1ll << 31) || g.N >= (1ll << 31) || g.K >= (1ll << 31))
    return cudaErrorInvalidValue;
  const SplitLayout L = split_layout(g.M, g.K, g.N);
  if (ws_bytes < L.total || ((uintptr_t)ws_v & 255)) return cudaErrorInvalidValue;
  char *ws = (char *)ws_v;
  auto *ahi = (__nv_bfloat16 *)(ws + L.a_hi), *alo = (__nv_bfloat16 *)(ws + L.a_lo);
  auto *bhi = (__nv_bfloat16 *)(ws + L.b_hi), *blo = (__nv_bfloat16 *)(ws + L.b_lo);
  dim3 ga((unsigned)(L.Kp / 64), (unsigned)((g.M + 31) / 32));
  dim3 gb((unsigned)(L.Kp / 64), (unsigned)((g.N + 31) / 32));
  if (ga.y > 65535 || gb.y > 65535) return cudaErrorInvalidConfiguration;
  PhaseMark mark(s);
  const unsigned long long gen = ++g_split_gen;
  auto *fa = (unsigned long long *)(ws + L.flags_a), *fbw = (unsigned long long *)(ws + L.flags_b);
  split_f32_bf16<<<ga, 256, 0, s>>>((const float *)g.a, g.rsa, g.csa, g.M, g.K, L.Kp, ahi, alo,
                                    fa, kBM, gen);
  split_f32_bf16<<<gb, 256, 0, s>>>((const float *)g.b, g.csb, g.rsb, g.N, g.K, L.Kp, bhi, blo,
                                    fbw, 64, gen);
  count_launch(2);
  cudaError_t e = cudaGetLastError();
  if (e) return e;
  mark.split_done();
  e = launch_gemm<128, 3>(L, ws, g, gen, s);
  mark.gemm_done();
  return e;
}

size_t ozaki_workspace(int64_t, int64_t, int64_t, int) { return 0; }
cudaError_t launch_ozaki(const Gemm &, int, void *, size_t, cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace numc_k

// ---- allocation-free entry point ---------------------------------------------
//
// Some callers of a GEMM may not allocate device memory at call time: code
// that records work into a CUDA graph or runs from a stream callback (where
// cudaMalloc is not allowed), real-time services that forbid allocation
// after start-up, and hosts whose device memory is owned by another
// framework's allocator.  numc_cuda_sgemm_split_static runs the split-BF16
// GEMM on a fixed scratch array compiled into this library instead of
// asking for workspace: the caller passes only inputs and outputs.
//
// The scratch array below is part of this module's device image: every GPU
// on which the library's kernels are loaded holds its 64 MiB until the
// process exits.  All calls share it, so calls that overlap on the GPU
// (two streams, or two host threads) race on it and must be serialised by
// the caller.  Its contents persist between calls; nothing in it needs to
// start at zero (the split planes are rewritten in full, the non-finite
// flags are tagged with the call's generation number) except the
// caller's status word, which each call clears.

namespace numc_k {
namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_static_mu;
void *g_static_addr[64] = {nullptr};

// Device address of g_static_scratch on the current device.  Host code may
// not use the array's name as an address (it names a host-side shadow), so
// the address is looked up once per device, with that device current.
cudaError_t static_scratch_address(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    g_static_addr[dev] = p;
  }
  *out = g_static_addr[dev];
  return cudaSuccess;
}

}  // namespace
}  // namespace numc_k

extern "C" int numc_cuda_sgemm_split_static(const float *a, const float *b, float *out,
                                            size_t M, size_t K, size_t N, intptr_t rsa,
                                            intptr_t csa, intptr_t rsb, intptr_t csb,
                                            intptr_t rso, intptr_t cso, unsigned *status,
                                            void *stream) {
  using namespace numc_k;
  if (M == 0 || N == 0) return 0;
  if (!out || (K > 0 && (!a || !b)))
    return NUMC_SET_ERROR(NUMC_ERR_NULL, "sgemm_split_static: NULL operand (a=%p b=%p out=%p)",
                          (const void *)a, (const void *)b, (void *)out);
  if (rsa < 0 || csa < 0 || rsb < 0 || csb < 0 || rso < 0 || cso < 0)
    return NUMC_SET_ERROR(NUMC_ERR_VALUE, "sgemm_split_static: negative stride");
  if (M >= (1ull << 31) || N >= (1ull << 31) || K >= (1ull << 31))
    return NUMC_SET_ERROR(NUMC_ERR_VALUE, "sgemm_split_static: dimension above 2^31");
  const SplitLayout L = split_layout((int64_t)M, (int64_t)K, (int64_t)N);
  if (L.total > kStaticScratchBytes)
    return NUMC_SET_ERROR(NUMC_ERR_VALUE,
                          "sgemm_split_static: %zux%zux%zu needs %zu bytes of scratch; the "
                          "static scratch holds %zu (4*(M+N)*roundup(K,64) bytes plus flags "
                          "must fit); use numc_cuda_gemm with a workspace instead",
                          M, K, N, L.total, kStaticScratchBytes);
  void *base = nullptr;
  cudaError_t e = static_scratch_address(&base);
  if (e != cudaSuccess)
    return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "sgemm_split_static: scratch address: %s",
                          cudaGetErrorString(e));
  cudaStream_t s = (cudaStream_t)stream;
  if (status && (e = cudaMemsetAsync(status, 0, sizeof(unsigned), s)) != cudaSuccess)
    return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "sgemm_split_static: %s", cudaGetErrorString(e));
  Gemm g;
  g.a = a; g.b = b; g.c = out;
  g.M = (int64_t)M; g.K = (int64_t)K; g.N = (int64_t)N;
  g.rsa = rsa; g.csa = csa; g.rsb = rsb; g.csb = csb; g.rso = rso; g.cso = cso;
  if (K == 0) {
    e = launch_simt(NUMC_DTYPE_FLOAT32, g, 0, s);   // out = 0, no scratch
  } else {
    char *ws = (char *)base;
    auto *ahi = (__nv_bfloat16 *)(ws + L.a_hi), *alo = (__nv_bfloat16 *)(ws + L.a_lo);
    auto *bhi = (__nv_bfloat16 *)(ws + L.b_hi), *blo = (__nv_bfloat16 *)(ws + L.b_lo);
    dim3 ga((unsigned)(L.Kp / 64), (unsigned)((M + 31) / 32));
    dim3 gb((unsigned)(L.Kp / 64), (unsigned)((N + 31) / 32));
    if (ga.y > 65535 || gb.y > 65535)
      return NUMC_SET_ERROR(NUMC_ERR_VALUE, "sgemm_split_static: too many rows for the split grid");
    const unsigned long long gen = ++g_split_gen;
    split_f32_bf16<<<ga, 256, 0, s>>>(a, rsa, csa, (int64_t)M, (int64_t)K, L.Kp, ahi, alo,
                                      (unsigned long long *)(ws + L.flags_a), kBM, gen);
    split_f32_bf16<<<gb, 256, 0, s>>>(b, csb, rsb, (int64_t)N, (int64_t)K, L.Kp, bhi, blo,
                                      (unsigned long long *)(ws + L.flags_b), 64, gen);
    count_launch(2);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = launch_gemm_status<128, 3>(L, ws, g, gen, status, s);
  }
  if (e != cudaSuccess)
    return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "sgemm_split_static: launch failed: %s",
                          cudaGetErrorString(e));
  return 0;
}

// float32 GEMM as a split product on the 5th-generation tensor cores
// (tcgen05), the fast alternative to numc's FP32 FMA GEMM
// (src/intrinsics/gemm_avx2.h:852 gemm_f32_avx2).
//
// Every float32 x is cut into 16-bit planes by repeated rounding.
// bfloat16 planes:
//   x0 = bf16(x), x1 = bf16(x - x0), x2 = bf16(x - x0 - x1).
// Each remainder is exact in float32, and x0 + x1 + x2 == x exactly for
// normal numbers (8 + 8 + 8 significant bits).
//   2 planes, 3 products:  A0B0 + A0B1 + A1B0           (error ~2^-16 |ab|)
//   3 planes, 6 products:  ... + A0B2 + A1B1 + A2B0     (error ~2^-24 |ab|)
// Scaled float16 planes (split_common.cuh): rows of A and columns of B are
// scaled by powers of two into [2^14, 2^15), x 2^s = h0 + h1 (11 + 11
// bits); 3 products h1h0 + h0h1 + h0h0 give float32-level error, and the
// epilogue multiplies by 2^-(s_row + s_col).
// Products of 16-bit values are exact in FP32.  Within a chunk of K slabs the
// products are summed in a tensor-memory FP32 accumulator (smallest terms
// first); the chunks' partial sums are added in FP32 registers with
// round-to-nearest, because the tensor core's accumulation truncates at
// every MMA step and loses hundreds of ulps over a K = 8192 chain.
//
// Pass 1 (split kernels, HBM-bound): for float16 planes a scale pass finds
// the row / column maxima; the split pass reads A and B once with any
// strides and writes the planes K-major with K padded to 64 (B is
// transposed on the way), so every plane suits a 128-byte-swizzled TMA box.
// Pass 2 (GEMM kernel): persistent; by default clusters of two CTAs on
// neighbouring SMs walk 256 x 256 output tiles (each CTA 128 rows, 18
// warps).  Warp 0 streams 64-deep K slabs of every plane of A and of its
// half of B into a STAGES-deep shared-memory ring with TMA (one 3-D tensor
// map per operand, the plane is the third coordinate); warp 1 of the even
// CTA issues the tcgen05.mma.cta_group::2.kind::f16 products of each chunk
// into one of two TMEM buffers of both CTAs and releases ring slots with
// tcgen05.commit; 16 accumulator warps per CTA drain each finished buffer
// (tcgen05.ld 32x32b) into register accumulators while the next chunk is
// multiplied, then store the tile.  Tiles are rasterised in groups of 2048
// rows so the live operand panels stay in L2.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <mutex>

#include "kernels.h"
#include "numc/cuda.h"
#include "numc/error.h"
#include "phase_timing.h"
#include "split_common.cuh"
#include "status.h"
#include "tc_common.cuh"

namespace numc_k {

// Streaming multiprocessors of the current device (persistent grid size).
int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (!cached[dev]) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = n > 0 ? n : 148;
  }
  return cached[dev];
}

// Programmatic dependent launch of the GEMM kernels after their operand
// passes (on unless NUMC_CUDA_PDL=0; read once).
bool pdl_enabled() {
  static const bool on = [] {
    const char *v = getenv("NUMC_CUDA_PDL");
    return !(v && v[0] == '0');
  }();
  return on;
}

// Co-resident clusters of `kern` launched with `cfg` (0 if the query fails).
int max_active_clusters(const void *kern, const cudaLaunchConfig_t &cfg) {
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

cudaError_t smem_attr_once(LaunchCache &lc, const void *kern, int bytes) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
  const bool cacheable = dev >= 0 && dev < 64;
  if (cacheable && ((lc.attr_done.load(std::memory_order_acquire) >> dev) & 1)) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && cacheable) lc.attr_done.fetch_or(1ull << dev, std::memory_order_release);
  return e;
}

int clusters_once(LaunchCache &lc, const void *kern, const cudaLaunchConfig_t &cfg) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return max_active_clusters(kern, cfg);
  int n = lc.clusters[dev].load(std::memory_order_relaxed);
  if (!n) {
    n = max_active_clusters(kern, cfg);
    if (n > 0) lc.clusters[dev].store(n, std::memory_order_relaxed);
  }
  return n;
}

namespace {

constexpr int kBM = 128, kBK = 64;
constexpr int kFusedMaxKp = 1024;   // single problems: fused scale + split up to this K

__host__ __device__ inline int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

// ---- pass 1: split float32 into bf16 planes (split_common.cuh) -------------

template <int PLANES, bool F16, int MODE>
__global__ void __launch_bounds__(256)
split_planes(const float *__restrict__ src, int64_t rs_row, int64_t rs_k, int64_t R,
               int64_t K, int64_t Kp, uint16_t *__restrict__ planes,
               unsigned long long *flags, int flag_rows, unsigned long long gen,
               const unsigned *maxbits) {
  __shared__ __align__(16) float tile[kSplitRows][kSplitK + 4];
  tc::griddep_launch_dependents();   // the GEMM may launch and set up meanwhile
  split_tile<PLANES, F16, MODE>(src, rs_row, rs_k, R, K, Kp, planes, flags, flag_rows, gen,
                                MODE, (int64_t)blockIdx.y * kSplitRows,
                                (int64_t)blockIdx.x * kSplitK, tile, maxbits);
}

// split_planes with the read mode as a template argument.
template <int PLANES, bool F16>
void launch_split_planes(dim3 grid, cudaStream_t s, int mode, const float *src, int64_t rs_row,
                         int64_t rs_k, int64_t R, int64_t K, int64_t Kp, uint16_t *planes,
                         unsigned long long *flags, int flag_rows, unsigned long long gen,
                         const unsigned *maxbits) {
  if (mode == 1)
    split_planes<PLANES, F16, 1><<<grid, 256, 0, s>>>(src, rs_row, rs_k, R, K, Kp, planes,
                                                      flags, flag_rows, gen, maxbits);
  else if (mode == 2)
    split_planes<PLANES, F16, 2><<<grid, 256, 0, s>>>(src, rs_row, rs_k, R, K, Kp, planes,
                                                      flags, flag_rows, gen, maxbits);
  else
    split_planes<PLANES, F16, 0><<<grid, 256, 0, s>>>(src, rs_row, rs_k, R, K, Kp, planes,
                                                      flags, flag_rows, gen, maxbits);
}

// Which one-launch float16 scale-and-split kernels run (NUMC_CUDA_SPLIT_PASS,
// a bit mask read once; default 3): bit 0 scale_split_rows for k-contiguous
// operands (A), bit 1 scale_split_cols for rows-contiguous ones (B^T of a
// row-major B); a clear bit runs the scale pass and the split pass instead.
// Every setting writes the same planes, maxima and flags.
int split_pass_kernels() {
  static const int v = [] {
    const char *e = getenv("NUMC_CUDA_SPLIT_PASS");
    return e && e[0] >= '0' && e[0] <= '3' && !e[1] ? e[0] - '0' : 3;
  }();
  return v;
}

// Scale and split of k-contiguous, 16-byte aligned rows (read mode 1) with
// Kp <= 1024 V: one row a block, each value read once (scale_split_row_regs).
constexpr int kRowRegsMaxKp = 16384;

template <int V>
__global__ void __launch_bounds__(256)
scale_split_rows(const float *__restrict__ src, int64_t rs_row, int64_t R, int K, int Kp,
                 uint16_t *__restrict__ planes, unsigned long long *flags, int flag_rows,
                 unsigned *__restrict__ maxbits, unsigned long long gen) {
  tc::griddep_launch_dependents();   // the GEMM may launch and set up meanwhile
  scale_split_row_regs<V>(src, rs_row, R, K, Kp, (int64_t)blockIdx.x, planes, flags, flag_rows,
                          maxbits, gen);
}

// Scale and split of rows-contiguous operands (read mode 2: the columns of a
// row-major B, as B^T's rows), each value read once and held in registers
// while the row maxima are found.  A row's maximum needs all of K, more
// than one CTA's registers hold, so a cluster of 8 CTAs takes 16 rows: CTA q
// of the cluster holds k in [q Kc, (q + 1) Kc), Kc = Kp / 8, and the CTAs'
// partial maxima are combined through distributed shared memory.  Thread t
// holds rows 4 (t % 4) .. + 3 at NQ k-quads, k = 4 (t / 4 + 128 p) + 0..3:
// a warp load covers 8 k x 64 contiguous bytes, a warp store 4 rows x 64
// contiguous bytes of a plane.  Same arithmetic as split_tile<2, true>
// after absmax_rows_f32.
constexpr int kColCluster = 8, kColRows = 16, kColThreads = 512;

template <int NQ>
__global__ void __cluster_dims__(kColCluster, 1, 1) __launch_bounds__(kColThreads, 2)
scale_split_cols(const float *__restrict__ src, int64_t rs_k, int64_t R, int64_t K, int Kp,
                 uint16_t *__restrict__ planes, unsigned long long *flags, int flag_rows,
                 unsigned *__restrict__ maxbits, unsigned long long gen) {
  __shared__ unsigned red[kColThreads / 32][kColRows];
  __shared__ unsigned pmax[kColRows], fmax[kColRows];
  tc::griddep_launch_dependents();   // the GEMM may launch and set up meanwhile
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t q = tc::cluster_ctarank();
  const int Kc = Kp / kColCluster;   // a multiple of 8: a k-quad is all in or all out
  const int64_t r0 = (int64_t)(blockIdx.x / kColCluster) * kColRows;
  const int cg = tid & 3;
  const int64_t rr = r0 + 4 * cg, klo = (int64_t)q * Kc;
  // v[p][t]: rows rr .. rr + 3 at k = klo + 4 (tid / 4 + 128 p) + t
  float4 v[NQ][4];
#pragma unroll
  for (int p = 0; p < NQ; p++) {
    const int kl = 4 * ((tid >> 2) + 128 * p);
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const int64_t k = klo + kl + t;
      v[p][t] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (kl < Kc && k < K) {
        const float *ptr = src + k * rs_k + rr;
        if (rr + 3 < R) {
          v[p][t] = __ldcs(reinterpret_cast<const float4 *>(ptr));
        } else {
          if (rr < R) v[p][t].x = ptr[0];
          if (rr + 1 < R) v[p][t].y = ptr[1];
          if (rr + 2 < R) v[p][t].z = ptr[2];
        }
      }
    }
  }
  unsigned m[4] = {0, 0, 0, 0};
  bool bad = false;
#pragma unroll
  for (int p = 0; p < NQ; p++)
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const float x[4] = {v[p][t].x, v[p][t].y, v[p][t].z, v[p][t].w};
#pragma unroll
      for (int j = 0; j < 4; j++) {
        bad |= !isfinite(x[j]);
        m[j] = max(m[j], absbits(x[j]));
      }
    }
#pragma unroll
  for (int j = 0; j < 4; j++) {   // lanes of one row group: lane % 4 equal
    m[j] = max(m[j], __shfl_xor_sync(0xffffffffu, m[j], 4));
    m[j] = max(m[j], __shfl_xor_sync(0xffffffffu, m[j], 8));
    m[j] = max(m[j], __shfl_xor_sync(0xffffffffu, m[j], 16));
  }
  if (lane < 4)
#pragma unroll
    for (int j = 0; j < 4; j++) red[warp][4 * lane + j] = m[j];
  const int anybad = __syncthreads_or(bad);
  if (tid < kColRows) {
    unsigned mm = 0;
#pragma unroll
    for (int w = 0; w < kColThreads / 32; w++) mm = max(mm, red[w][tid]);
    pmax[tid] = mm;
  }
  if (tid == 0 && anybad) flags[r0 / flag_rows] = gen;
  __syncwarp();
  tc::cluster_sync();   // every CTA's partial maxima written
  if (tid < kColRows) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(&pmax[tid]);
    unsigned mm = 0;
#pragma unroll
    for (uint32_t c = 0; c < kColCluster; c++)
      mm = max(mm, tc::ld_shared_cluster_u32(tc::mapa_shared(a, c)));
    fmax[tid] = mm;
    if (q == 0 && r0 + tid < R) maxbits[r0 + tid] = mm;
  }
  __syncwarp();
  tc::cluster_arrive();   // done reading the peers' partial maxima
  __syncthreads();
  const int64_t plane_elems = R * Kp;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int64_t r = rr + j;
    if (r >= R) break;
    const int sexp = f16_scale_exp(fmax[4 * cg + j]);
    uint16_t *dst = planes + r * Kp + klo;
#pragma unroll
    for (int p = 0; p < NQ; p++) {
      const int kl = 4 * ((tid >> 2) + 128 * p);
      if (kl >= Kc) continue;
      const float rem[4] = {(&v[p][0].x)[j], (&v[p][1].x)[j], (&v[p][2].x)[j], (&v[p][3].x)[j]};
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
        *reinterpret_cast<uint2 *>(dst + pl * plane_elems + kl) = w;
      }
    }
  }
  __syncwarp();
  tc::cluster_wait();   // no CTA leaves while a peer may read its maxima
}

// Largest Kp scale_split_cols takes: NQ = 2 (32 values a thread; more
// would not fit the 64 registers of two 512-thread CTAs an SM).
constexpr int kColMaxKp = kColCluster * 512 * 2;

// Launch scale_split_cols on R rows (false if its clusters cannot be
// resident on this device: the caller runs the two passes instead).
bool launch_split_cols(const float *src, int64_t rs_k, int64_t R, int64_t K, int64_t Kp,
                       uint16_t *planes, unsigned long long *flags, int flag_rows,
                       unsigned *maxbits, unsigned long long gen, cudaStream_t s,
                       cudaError_t *err) {
  const int64_t clusters = (R + kColRows - 1) / kColRows;
  if (clusters * kColCluster >= (1ll << 31)) return false;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(clusters * kColCluster));
  cfg.blockDim = dim3(kColThreads);
  cfg.stream = s;
  auto go = [&](auto kern, LaunchCache &lc) {
    if (clusters_once(lc, (const void *)kern, cfg) <= 0) return false;
    *err = cudaLaunchKernelEx(&cfg, kern, src, rs_k, R, K, (int)Kp, planes, flags, flag_rows,
                              maxbits, gen);
    return true;
  };
  static LaunchCache lc1, lc2;
  if (Kp <= kColCluster * 512) return go(scale_split_cols<1>, lc1);
  return go(scale_split_cols<2>, lc2);
}

// Both operands of one float16-plane split through fused_scale_split_rows:
// blocks [0, a_blocks) take 16 rows of A each, the
// rest 16 columns of B.  One launch replaces two zeroings of the maxima,
// two absmax passes and two split passes.
__global__ void __launch_bounds__(256)
scale_split_pair(const float *A, int64_t rsa, int64_t csa, int M, const float *B,
                 int64_t rsb, int64_t csb, int N, int K, int Kp, uint16_t *pa, uint16_t *pb,
                 unsigned long long *fa, unsigned long long *fbl, unsigned *max_a,
                 unsigned *max_b, unsigned long long gen) {
  tc::griddep_launch_dependents();   // the GEMM may launch and set up meanwhile
  const int a_blocks = (M + kFusedRows - 1) / kFusedRows;
  const bool is_a = (int)blockIdx.x < a_blocks;
  fused_scale_split_rows<true>(is_a ? A : B, is_a ? rsa : csb, is_a ? csa : rsb, is_a ? M : N, K, Kp,
                         (is_a ? (int)blockIdx.x : (int)blockIdx.x - a_blocks) * kFusedRows,
                         is_a ? pa : pb, is_a ? fa : fbl, is_a ? kBM : 64, is_a ? max_a : max_b,
                         gen);
}

// ---- pass 2: the tcgen05 GEMM ------------------------------------------------

// Original operands and the non-finite flags, for tiles that must be
// recomputed with plain FMA chains.
struct Fallback {
  const float *A, *B;
  int64_t rsa, csa, rsb, csb, K;
  const unsigned long long *flags_a, *flags_b;   // per 128 rows of A, per 64 columns of B
  unsigned long long gen;
  const unsigned *max_a, *max_b;   // scaled float16 planes: row / column maxima
  const float *bias;                // numc_linear: added to each column, or null
  int64_t bias_stride;
};

template <int BN, int STAGES, int PLANES, int FLUSH, int CTAS>
struct SplitCfg {
  static constexpr int BN_CTA = BN / CTAS;            // B rows (output columns) held per CTA
  static constexpr uint32_t A_BYTES = kBM * kBK * 2;   // one plane of a K slab of A
  static constexpr uint32_t B_BYTES = BN_CTA * kBK * 2;
  static constexpr uint32_t STAGE_BYTES = PLANES * (A_BYTES + B_BYTES);   // per CTA
  static constexpr int NBUF = 512 / BN;           // FP32 accumulator buffers in TMEM
  static constexpr uint32_t TMEM_COLS = NBUF * BN;
  static constexpr int COLS_PER_WARP = 64;
  static constexpr int ACC_WARPS = 4 * BN / COLS_PER_WARP;   // BN / 64 per TMEM lane quadrant
  // per accumulator warp, a staging buffer for coalesced stores, where the
  // ring leaves room for it
  static constexpr uint32_t RING = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
  static constexpr uint32_t EPI_BYTES = ACC_WARPS * kEpiStageFloats * 4;
  static constexpr bool EPI_STAGE = RING + EPI_BYTES <= 232448;
  static constexpr uint32_t SMEM = RING + (EPI_STAGE ? EPI_BYTES : 0);
  static constexpr int THREADS = 64 + 32 * ACC_WARPS;   // producer, MMA, accumulators
  static_assert(BN == 64 || BN == 128 || BN == 256, "tile width");
  static_assert(CTAS == 1 || CTAS == 2, "one CTA or a CTA pair");
  static_assert(SMEM <= 232448, "shared memory");
  static_assert((2 * STAGES + 2 * NBUF + 1) * 8 + 4 <= 256, "barrier space");
  static_assert(TMEM_COLS <= 512, "tensor memory");
};

// The (A plane, B plane) products summed per K step, smallest first.
template <int PLANES> struct Products;
template <> struct Products<2> {
  static constexpr int n = 3;
  __device__ static constexpr int a(int t) { return t == 0 ? 1 : 0; }
  __device__ static constexpr int b(int t) { return t == 1 ? 1 : 0; }
};
template <> struct Products<3> {
  static constexpr int n = 6;
  // (2,0) (1,1) (0,2) (1,0) (0,1) (0,0)
  __device__ static constexpr int a(int t) { return t == 0 ? 2 : (t == 1 || t == 3) ? 1 : 0; }
  __device__ static constexpr int b(int t) { return t == 2 ? 2 : (t == 1 || t == 4) ? 1 : 0; }
};

// Warp roles (64 + 32 * BN / 16 threads per CTA):
//   warp 0, lane 0   TMA producer: fills the STAGES-deep ring of K slabs.
//   warp 1, lane 0   MMA issuer: for chunk c (FLUSH consecutive K slabs),
//                    accumulates all products into TMEM buffer c % NBUF
//                    (starting from zero) and commits it to the
//                    accumulator warps.
//   warps 2..        accumulator warps, BN / 64 per TMEM lane quadrant,
//                    each owning 64 of the tile's columns: drain each
//                    chunk's partial sums from TMEM and add them into FP32
//                    registers (round to nearest), then release the
//                    buffer; finally store.
// BN = 256 halves the MMA instructions, waits and commits per flop against
// BN = 128; measured on GB300 with the operand loads and TMEM drains
// switched off, the bare MMA loop reached 1478 TFLOP/s at BN = 128 and
// 1807 at BN = 256 (flush 4).
// The tensor core's own FP32 accumulation truncates at every MMA step; a
// chain of K/16 x passes steps loses hundreds of ulps at K = 8192, so the
// chain in TMEM is restarted every FLUSH K slabs and the chunks are summed
// with correctly rounded FP32 adds.
//
// CTAS = 2 runs the kernel as clusters of two CTAs on neighbouring SMs
// sharing 256 x BN output tiles: each CTA loads its own 128 rows of A and
// BN/2 rows of B^T, the even CTA's MMA thread multiplies both halves with
// cta_group::2 MMAs (each SM reads half of B from its own shared memory,
// so per-SM operand traffic per flop drops by a quarter), its commits
// arrive on the barriers of both CTAs, both producers count their bytes on
// the even CTA's full barrier, and both CTAs' accumulator warps release
// TMEM buffers on the even CTA's empty barrier.
template <int BN, int STAGES, int PLANES, int FLUSH, bool F16, int CTAS>
__global__ void __launch_bounds__(SplitCfg<BN, STAGES, PLANES, FLUSH, CTAS>::THREADS, 1)
split_gemm(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB,
           float *__restrict__ C, int64_t rso, int64_t cso, int M, int N, int num_kb,
           int tiles_m, int tiles_n, int vec4, unsigned *status, Fallback fb, WaitCfg wc) {
  using Cfg = SplitCfg<BN, STAGES, PLANES, FLUSH, CTAS>;
  using P = Products<PLANES>;
  constexpr bool PAIR = CTAS == 2;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *bars = (uint64_t *)(smem + STAGES * Cfg::STAGE_BYTES);
  uint64_t *full = bars, *empty = bars + STAGES;
  constexpr int NBUF = Cfg::NBUF;
  uint64_t *tfull = bars + 2 * STAGES, *tempty = bars + 2 * STAGES + NBUF;
  uint64_t *drain = bars + 2 * STAGES + 2 * NBUF;   // all issued MMAs complete
  uint32_t *tmem_slot = (uint32_t *)(bars + 2 * STAGES + 2 * NBUF + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = tiles_m * tiles_n;   // tiles of CTAS * 128 rows
  const uint32_t rank = PAIR ? tc::cluster_ctarank() : 0;
  const bool leader = rank == 0;
  const int first_tile = blockIdx.x / CTAS, tile_step = gridDim.x / CTAS;

  // Persistent: CTA (pair) b handles tiles b, b + grid, ...  Tiles are
  // rasterised in groups of 2048 rows that sweep all column tiles, so the
  // CTAs in flight share A and B panels in L2.
  auto tile_origin = [&](int t, int &m0, int &n0) {
    constexpr int GM = 16 / CTAS;
    const int group = t / (GM * tiles_n);
    const int first_m = group * GM;
    const int gm = min(tiles_m - first_m, GM);
    const int local = t - group * GM * tiles_n;
    m0 = (first_m + local % gm) * (kBM * CTAS);
    n0 = (local / gm) * BN;
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      tc::mbar_init(tc::smem_u32(&full[s]), 1);
      tc::mbar_init(tc::smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < NBUF; b++) {
      tc::mbar_init(tc::smem_u32(&tfull[b]), 1);
      // one arrive per accumulator warp of every CTA
      tc::mbar_init(tc::smem_u32(&tempty[b]), Cfg::ACC_WARPS * CTAS);
    }
    tc::mbar_init(tc::smem_u32(drain), 1);
    tc::fence_barrier_init();
    tc::tma_prefetch_desc(&tA);
    tc::tma_prefetch_desc(&tB);
  }
  if (warp == 1) {
    if constexpr (PAIR) tc::tmem_alloc_pair(tc::smem_u32(tmem_slot), Cfg::TMEM_COLS);
    else tc::tmem_alloc(tc::smem_u32(tmem_slot), Cfg::TMEM_COLS);
  }
  tc::tc_fence_before();
  __syncthreads();
  if constexpr (PAIR) tc::cluster_sync();   // peer barriers initialised
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  tc::griddep_wait();   // the split pass has completed
  const int num_chunks = (num_kb + FLUSH - 1) / FLUSH;   // per tile

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
          // The even CTA's full barrier counts the bytes of both CTAs.
          if (leader) tc::mbar_arrive_expect_tx(fbar, CTAS * Cfg::STAGE_BYTES);
          const int k = kb * kBK;
          if constexpr (PAIR) {
            const uint32_t fbar_leader = tc::mapa_shared(fbar, 0);
#pragma unroll
            for (int p = 0; p < PLANES; p++) {
              tc::tma_load_3d_pair(st + p * Cfg::A_BYTES, &tA, fbar_leader, k, ma, p);
              tc::tma_load_3d_pair(st + PLANES * Cfg::A_BYTES + p * Cfg::B_BYTES, &tB,
                                   fbar_leader, k, nb, p);
            }
          } else {
#pragma unroll
            for (int p = 0; p < PLANES; p++) {
              tc::tma_load_3d(st + p * Cfg::A_BYTES, &tA, fbar, k, ma, p);
              tc::tma_load_3d(st + PLANES * Cfg::A_BYTES + p * Cfg::B_BYTES, &tB, fbar, k, nb, p);
            }
          }
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0 && leader) {
      constexpr uint32_t idesc =
          F16 ? tc::idesc_f16_f32(kBM * CTAS, BN) : tc::idesc_bf16_f32(kBM * CTAS, BN);
      int g = 0, chunk = 0;   // stage and chunk counters across tiles
      bool live = true;
      for (int t = first_tile; t < ntiles && live; t += tile_step) {
        for (int kb = 0; kb < num_kb; kb++, g++) {
          const int s = g % STAGES, buf = chunk % NBUF;
          const bool chunk_start = kb % FLUSH == 0;
          const bool chunk_end = kb % FLUSH == FLUSH - 1 || kb == num_kb - 1;
          if (chunk_start && chunk >= NBUF &&
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
          const uint32_t st = tc::smem_u32(smem + s * Cfg::STAGE_BYTES);
          const uint32_t bbase = st + PLANES * Cfg::A_BYTES;
          const uint32_t acc_tmem = tmem + buf * BN;
          // Product by product over the slab, smallest first: the tensor
          // core truncates the accumulator at every MMA, so the large
          // x0 y0 terms enter last and are truncated only kBK / 16 times
          // at full magnitude per chunk start.
#pragma unroll
          for (int p = 0; p < P::n; p++) {
#pragma unroll
            for (int kk = 0; kk < kBK / 16; kk++) {
              const uint32_t koff = kk * 32;   // 16 elements = 32 bytes inside the swizzle atom
              const uint32_t acc = (!chunk_start || kk > 0 || p > 0) ? 1u : 0u;
              const uint64_t ad = tc::sdesc_k128(st + P::a(p) * Cfg::A_BYTES + koff);
              const uint64_t bd = tc::sdesc_k128(bbase + P::b(p) * Cfg::B_BYTES + koff);
              if constexpr (PAIR) tc::mma_f16_pair(acc_tmem, ad, bd, idesc, acc);
              else tc::mma_bf16(acc_tmem, ad, bd, idesc, acc);
            }
          }
          if constexpr (PAIR) {
            tc::mma_commit_pair(tc::smem_u32(&empty[s]), 0x3);
            if (chunk_end) tc::mma_commit_pair(tc::smem_u32(&tfull[buf]), 0x3);
          } else {
            tc::mma_commit(tc::smem_u32(&empty[s]));
            if (chunk_end) tc::mma_commit(tc::smem_u32(&tfull[buf]));
          }
          if (chunk_end) chunk++;
        }
      }
      // Whether the loop ran to the end or gave up, every MMA issued above
      // completes before TMEM is released (a commit with none outstanding
      // arrives at once).
      if constexpr (PAIR) tc::mma_commit_pair(tc::smem_u32(drain), 0x1);
      else tc::mma_commit(tc::smem_u32(drain));
      tc::mbar_wait_bounded(tc::smem_u32(drain), 0, status, kStatusTimeoutDrain, wc.limit_ns);
    }
    __syncwarp();
  } else {
    // Accumulator warps: warp w may read TMEM lanes 32 * (w % 4); the
    // warps of a quadrant split the columns 64 apiece.
    constexpr int CW = Cfg::COLS_PER_WARP;
    const int quad = warp & 3, part = (warp - 2) >> 2;
    const int cbase = part * CW;
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    int chunk = 0;   // across tiles
    bool ok = true;
    for (int t = first_tile; t < ntiles && ok; t += tile_step) {
      int m0, n0;
      tile_origin(t, m0, n0);
      const int mr = m0 + (int)rank * kBM;   // this CTA's 128 rows
      const int row = mr + quad * 32 + lane;
      float acc[CW];
#pragma unroll
      for (int j = 0; j < CW; j++) acc[j] = 0.0f;
      for (int c = 0; c < num_chunks; c++, chunk++) {
        const int buf = chunk % NBUF;
        ok = tc::mbar_wait_bounded(tc::smem_u32(&tfull[buf]), (chunk / NBUF) & 1, status,
                                   kStatusTimeoutEpilogue, wc.limit_ns);
        ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld below is warp-collective
        if (!ok) break;
        tc::tc_fence_after();
        if constexpr (BN <= 128) {
          uint32_t r[CW];
#pragma unroll
          for (int c0 = 0; c0 < CW; c0 += 32)
            tc::tmem_ld_32x32b_x32(tmem + lane_off + buf * BN + cbase + c0,
                                   *reinterpret_cast<uint32_t(*)[32]>(&r[c0]));
          tc::tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < CW; j++) acc[j] = __fadd_rn(acc[j], __uint_as_float(r[j]));
        } else {
          // 18 warps leave 112 registers a thread: drain 16 columns at a time.
#pragma unroll
          for (int c0 = 0; c0 < CW; c0 += 16) {
            uint32_t r[16];
            tc::tmem_ld_32x32b_x16(tmem + lane_off + buf * BN + cbase + c0, r);
            tc::tmem_ld_wait();
#pragma unroll
            for (int j = 0; j < 16; j++) acc[c0 + j] = __fadd_rn(acc[c0 + j], __uint_as_float(r[j]));
          }
        }
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          if constexpr (PAIR) tc::mbar_arrive_cluster(tc::mapa_shared(tc::smem_u32(&tempty[buf]), 0));
          else tc::mbar_arrive(tc::smem_u32(&tempty[buf]));
        }
      }
      if (!ok) break;

      // (a pair's odd CTA may lie wholly below the last row: no flag there)
      bool nonfinite = mr < M && fb.flags_a[mr / kBM] == fb.gen;
#pragma unroll 1
      for (int c = n0 / 64; c < (n0 + BN) / 64 && c * 64 < N; c++)
        nonfinite |= fb.flags_b[c] == fb.gen;
      // The warp's staging buffer: first its 64 column scale exponents
      // (float16 planes; one load per lane and half, read back as
      // broadcasts), then the coalesced stores.
      float *stage = (float *)(smem + STAGES * Cfg::STAGE_BYTES + 256) +
                     (warp - 2) * kEpiStageFloats;
      const int *colexp = (const int *)stage;
      if constexpr (F16) {
        static_assert(Cfg::EPI_STAGE, "float16 planes stage their epilogue");
        if (!nonfinite) {
          const int lc = n0 + cbase + lane;
          ((int *)stage)[lane] = lc < N ? f16_scale_exp(fb.max_b[lc]) : 0;
          ((int *)stage)[lane + 32] = lc + 32 < N ? f16_scale_exp(fb.max_b[lc + 32]) : 0;
          __syncwarp();
        }
      }
      if (nonfinite) {
        // numc's arithmetic: one FMA chain per output in k order (slow path).
#pragma unroll 1
        for (int c0 = cbase; c0 < cbase + CW && row < M; c0 += 32) {
          float f[32];
#pragma unroll
          for (int j = 0; j < 32; j++) f[j] = 0.0f;
#pragma unroll 1
          for (int64_t k = 0; k < fb.K; k++) {
            const float av = fb.A[(int64_t)row * fb.rsa + k * fb.csa];
            const float *brow = fb.B + k * fb.rsb;
#pragma unroll
            for (int j = 0; j < 32; j++) {
              const int col = n0 + c0 + j;
              const float bv = col < N ? brow[(int64_t)col * fb.csb] : 0.0f;
              f[j] = __fmaf_rn(av, bv, f[j]);
            }
          }
#pragma unroll
          for (int j = 0; j < 32; j++)
            if (n0 + c0 + j < N)
              C[(int64_t)row * rso + (int64_t)(n0 + c0 + j) * cso] =
                  fb.bias ? __fadd_rn(f[j], fb.bias[(int64_t)(n0 + c0 + j) * fb.bias_stride]) : f[j];
        }
      } else {   // warp-uniform branch (nonfinite is per tile)
        if (row < M) {
          if constexpr (F16) {
            // Undo the row and column scaling, acc * 2^-(sa + sb) correctly
            // rounded: float multiplies by powers of two when every exponent
            // is a normal float32's (the product then rounds once, if at
            // all), else the product in double (exact: acc has 24 bits)
            // rounded once to float.  Column exponents come from the warp's
            // table.
            const int sa = f16_scale_exp(fb.max_a[row]);
            bool in_range = true;
#pragma unroll 8
            for (int j = 0; j < CW; j++) {
              const int e = -(sa + colexp[j]);
              in_range &= e >= -126 && e <= 127;
            }
            if (in_range) {
#pragma unroll
              for (int j = 0; j < CW; j++) acc[j] *= exp2_int(-(sa + colexp[j]));
            } else {
#pragma unroll
              for (int j = 0; j < CW; j++)
                acc[j] = (float)((double)acc[j] * exp2_dbl(-(sa + colexp[j])));
            }
          }
          if (fb.bias) {
#pragma unroll
            for (int j = 0; j < CW; j++) {
              const int col = n0 + cbase + j;
              if (col < N) acc[j] = __fadd_rn(acc[j], fb.bias[(int64_t)col * fb.bias_stride]);
            }
          }
        }
        if (Cfg::EPI_STAGE && cso == 1) {   // warp-uniform: every lane stores
          __syncwarp();
          store_rows_coalesced<CW>(acc, stage, C, rso, mr + quad * 32, n0 + cbase, M, N, lane);
        } else if (row < M) {
          float *crow = C + (int64_t)row * rso;
#pragma unroll
          for (int c0 = 0; c0 < CW; c0 += 32) {
            const int nb = n0 + cbase + c0;
            if (vec4 && nb + 32 <= N) {
              float4 *p = reinterpret_cast<float4 *>(crow + nb);
#pragma unroll
              for (int j = 0; j < 8; j++)
                p[j] = make_float4(acc[c0 + 4 * j], acc[c0 + 4 * j + 1], acc[c0 + 4 * j + 2],
                                   acc[c0 + 4 * j + 3]);
            } else {
#pragma unroll
              for (int j = 0; j < 32; j++)
                if (nb + j < N) crow[(int64_t)(nb + j) * cso] = acc[c0 + j];
            }
          }
        }
      }
      __syncwarp();   // reconverge before the next tile's tcgen05.ld
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  // Neither CTA of a pair leaves while the other may still signal its
  // barriers or read its shared memory.
  if constexpr (PAIR) tc::cluster_sync();
  if (warp == 1) {
    tc::tc_fence_after();
    if constexpr (PAIR) tc::tmem_dealloc_pair(tmem, Cfg::TMEM_COLS);
    else tc::tmem_dealloc(tmem, Cfg::TMEM_COLS);
  }
}

// Workspace: PLANES planes of A (M x Kp), PLANES planes of B^T (N x Kp),
// the non-finite flags, and for scaled float16 planes the row maxima of A
// and column maxima of B (float32 bits, M + N words).
struct SplitLayout {
  int planes;
  bool f16;
  int flush;   // K slabs per TMEM accumulation chain
  int64_t Kp;
  size_t a, b, flags_a, flags_b, max_a, max_b, total;
};

SplitLayout split_layout(int64_t M, int64_t K, int64_t N, int planes, bool f16 = false,
                         int flush = 0) {
  SplitLayout L;
  L.planes = planes;
  L.f16 = f16;
  L.flush = flush;
  L.Kp = round_up(K > 0 ? K : 1, kBK);
  L.a = 0;
  L.b = (size_t)round_up(planes * M * L.Kp * 2, 256);
  L.flags_a = L.b + (size_t)round_up(planes * N * L.Kp * 2, 256);
  L.flags_b = L.flags_a + (size_t)round_up(((M + kBM - 1) / kBM) * 8, 256);
  L.max_a = L.flags_b + (size_t)round_up(((N + 63) / 64) * 8, 256);
  L.max_b = L.max_a + (f16 ? (size_t)round_up(M * 4, 256) : 0);
  L.total = L.max_b + (f16 ? (size_t)round_up(N * 4, 256) : 0);
  return L;
}

// Device addresses of one GEMM's split operands.
struct SplitBufs {
  uint16_t *pa, *pb;                      // planes
  unsigned long long *flags_a, *flags_b;  // per 128 rows of A, per 64 columns of B
  unsigned *max_a, *max_b;                // float16 planes: row / column maxima
};

SplitBufs bufs_of(const SplitLayout &L, char *ws) {
  SplitBufs b;
  b.pa = (uint16_t *)(ws + L.a);
  b.pb = (uint16_t *)(ws + L.b);
  b.flags_a = (unsigned long long *)(ws + L.flags_a);
  b.flags_b = (unsigned long long *)(ws + L.flags_b);
  b.max_a = L.f16 ? (unsigned *)(ws + L.max_a) : nullptr;
  b.max_b = L.f16 ? (unsigned *)(ws + L.max_b) : nullptr;
  return b;
}

// Generation numbers of split calls (never 0; flags hold the last writer's).
std::atomic<unsigned long long> g_split_gen{0x5eed000000000000ull};

// Split one operand (R rows of src[r * rs_row + k * rs_k], k < K) into
// planes; for float16 planes first its row maxima.
cudaError_t split_operand(const SplitLayout &L, const float *src, int64_t rs_row, int64_t rs_k,
                          int64_t R, int64_t K, uint16_t *planes, unsigned long long *flags,
                          int flag_rows, unsigned *maxbits, unsigned long long gen,
                          cudaStream_t s) {
  const int mode = split_mode(src, rs_row, rs_k);
  cudaError_t e = cudaSuccess;
  if (L.f16 && mode == 2 && L.Kp <= kColMaxKp && (split_pass_kernels() & 2) &&
      launch_split_cols(src, rs_k, R, K, L.Kp, planes, flags, flag_rows, maxbits, gen, s, &e)) {
    if (e == cudaSuccess) {
      count_launch(1);
      return cudaGetLastError();
    }
    // a cluster launch refused at run time (a launch-configuration error,
    // which does not stick to the context): the two passes below instead
    cudaGetLastError();
    e = cudaSuccess;
  }
  const dim3 grid((unsigned)((L.Kp + kSplitK - 1) / kSplitK),
                  (unsigned)((R + kSplitRows - 1) / kSplitRows));
  if (grid.y > 65535) return cudaErrorInvalidConfiguration;
  if (L.f16 && mode == 1 && L.Kp <= kRowRegsMaxKp && R < (1ll << 31) &&
      (split_pass_kernels() & 1)) {
    const unsigned blocks = (unsigned)R;
    const int k = (int)K, kp = (int)L.Kp;
    if (L.Kp <= 1024)
      scale_split_rows<1><<<blocks, 256, 0, s>>>(src, rs_row, R, k, kp, planes, flags, flag_rows,
                                                 maxbits, gen);
    else if (L.Kp <= 2048)
      scale_split_rows<2><<<blocks, 256, 0, s>>>(src, rs_row, R, k, kp, planes, flags, flag_rows,
                                                 maxbits, gen);
    else if (L.Kp <= 4096)
      scale_split_rows<4><<<blocks, 256, 0, s>>>(src, rs_row, R, k, kp, planes, flags, flag_rows,
                                                 maxbits, gen);
    else if (L.Kp <= 8192)
      scale_split_rows<8><<<blocks, 256, 0, s>>>(src, rs_row, R, k, kp, planes, flags, flag_rows,
                                                 maxbits, gen);
    else
      scale_split_rows<16><<<blocks, 256, 0, s>>>(src, rs_row, R, k, kp, planes, flags,
                                                  flag_rows, maxbits, gen);
    count_launch(1);
  } else if (L.f16) {
    const int amode = absmax_mode(mode, rs_k);
    const dim3 rg = absmax_grid(R, K, amode);
    if (rg.y > 65535) return cudaErrorInvalidConfiguration;
    if ((e = cudaMemsetAsync(maxbits, 0, (size_t)R * 4, s))) return e;
    absmax_rows_f32<<<rg, 256, 0, s>>>(src, rs_row, rs_k, R, K, amode, maxbits);
    launch_split_planes<2, true>(grid, s, mode, src, rs_row, rs_k, R, K, L.Kp, planes, flags,
                                 flag_rows, gen, maxbits);
    count_launch(2);
  } else if (L.planes == 3) {
    launch_split_planes<3, false>(grid, s, mode, src, rs_row, rs_k, R, K, L.Kp, planes, flags,
                                  flag_rows, gen, nullptr);
    count_launch(1);
  } else {
    launch_split_planes<2, false>(grid, s, mode, src, rs_row, rs_k, R, K, L.Kp, planes, flags,
                                  flag_rows, gen, nullptr);
    count_launch(1);
  }
  return cudaGetLastError();
}

cudaError_t split_a(const SplitLayout &L, const SplitBufs &b, const Gemm &g,
                    unsigned long long gen, cudaStream_t s) {
  return split_operand(L, (const float *)g.a, g.rsa, g.csa, g.M, g.K, b.pa, b.flags_a, kBM,
                       b.max_a, gen, s);
}

// B is split as B^T: its rows are B's columns.
cudaError_t split_b(const SplitLayout &L, const SplitBufs &b, const Gemm &g,
                    unsigned long long gen, cudaStream_t s) {
  return split_operand(L, (const float *)g.b, g.csb, g.rsb, g.N, g.K, b.pb, b.flags_b, 64,
                       b.max_b, gen, s);
}

// Launch the split pass of both operands: for float16 planes with K up to
// kFusedMaxKp one fused scale + split launch over both, else a scale pass
// and a split pass per operand (large operands: the fused pass's second read
// would miss L2 like the split pass's does, and the two-pass kernels move
// 16-byte vectors).
cudaError_t launch_split_pass(const SplitLayout &L, const SplitBufs &b, const Gemm &g,
                              unsigned long long gen, cudaStream_t s) {
  if (L.f16 && L.Kp <= kFusedMaxKp && g.M < (1ll << 30) && g.N < (1ll << 30)) {
    const int64_t blocks = (g.M + kFusedRows - 1) / kFusedRows + (g.N + kFusedRows - 1) / kFusedRows;
    scale_split_pair<<<(unsigned)blocks, 256, 0, s>>>(
        (const float *)g.a, g.rsa, g.csa, (int)g.M, (const float *)g.b, g.rsb, g.csb, (int)g.N,
        (int)g.K, (int)L.Kp, b.pa, b.pb, b.flags_a, b.flags_b, b.max_a, b.max_b, gen);
    count_launch();
    return cudaGetLastError();
  }
  cudaError_t e = split_a(L, b, g, gen, s);
  return e != cudaSuccess ? e : split_b(L, b, g, gen, s);
}

template <int BN, int STAGES, int PLANES, int FLUSH, bool F16, int CTAS>
cudaError_t launch_gemm_status(const SplitLayout &L, const SplitBufs &bufs, const Gemm &g,
                               unsigned long long gen, unsigned *status, cudaStream_t s,
                               bool pdl) {
  using Cfg = SplitCfg<BN, STAGES, PLANES, FLUSH, CTAS>;
  CUtensorMap ta, tb;
  cudaError_t e;
  const auto dtype = F16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  if ((e = make_tmap_3d(&ta, bufs.pa, dtype, 2, PLANES, g.M, L.Kp, L.Kp, kBM, kBK))) return e;
  if ((e = make_tmap_3d(&tb, bufs.pb, dtype, 2, PLANES, g.N, L.Kp, L.Kp, Cfg::BN_CTA, kBK)))
    return e;
  auto kern = split_gemm<BN, STAGES, PLANES, FLUSH, F16, CTAS>;
  static LaunchCache lc;
  if ((e = smem_attr_once(lc, (const void *)kern, Cfg::SMEM))) return e;
  const int tiles_m = (int)((g.M + kBM * CTAS - 1) / (kBM * CTAS));
  const int tiles_n = (int)((g.N + BN - 1) / BN);
  const int vec4 = g.cso == 1 && (g.rso % 4) == 0 && ((uintptr_t)g.c % 16) == 0;
  Fallback fb;
  fb.A = (const float *)g.a;
  fb.B = (const float *)g.b;
  fb.rsa = g.rsa; fb.csa = g.csa; fb.rsb = g.rsb; fb.csb = g.csb; fb.K = g.K;
  fb.flags_a = bufs.flags_a;
  fb.flags_b = bufs.flags_b;
  fb.gen = gen;
  fb.max_a = bufs.max_a;
  fb.max_b = bufs.max_b;
  fb.bias = (const float *)g.bias;
  fb.bias_stride = g.bias_stride;
  const int num_kb = (int)(L.Kp / kBK);
  // programmatic dependent launch: the GEMM sets up while the split pass
  // ends (only when that pass is the previous work in the stream)
  cudaLaunchAttribute pdl_attr;
  pdl_attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
  pdl_attr.val.programmaticStreamSerializationAllowed = pdl && pdl_enabled() ? 1 : 0;
  if (CTAS == 1) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)std::min(tiles_m * tiles_n, sm_count()));
    cfg.blockDim = dim3(Cfg::THREADS);
    cfg.dynamicSmemBytes = Cfg::SMEM;
    cfg.stream = s;
    cfg.attrs = &pdl_attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, kern, ta, tb, (float *)g.c, (int64_t)g.rso, (int64_t)g.cso,
                           (int)g.M, (int)g.N, num_kb, tiles_m, tiles_n, vec4, status, fb,
                           wait_cfg());
    if (e != cudaSuccess) return e;
  } else {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CTAS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1] = pdl_attr;
    cfg.blockDim = dim3(Cfg::THREADS);
    cfg.dynamicSmemBytes = Cfg::SMEM;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // One pair per two SMs, capped by how many pairs fit at once.
    cfg.gridDim = dim3((unsigned)(CTAS * std::max(1, sm_count() / CTAS)));
    int pairs = clusters_once(lc, (const void *)kern, cfg);
    if (pairs <= 0) pairs = std::max(1, sm_count() / CTAS);
    pairs = std::min(pairs, tiles_m * tiles_n);
    cfg.gridDim = dim3((unsigned)(CTAS * pairs));
    cfg.numAttrs = 2;
    e = cudaLaunchKernelEx(&cfg, kern, ta, tb, (float *)g.c, (int64_t)g.rso, (int64_t)g.cso,
                           (int)g.M, (int)g.N, num_kb, tiles_m, tiles_n, vec4, status, fb,
                           wait_cfg());
    if (e != cudaSuccess) return e;
  }
  count_launch();
  return cudaGetLastError();
}

// Flush interval (K slabs per TMEM accumulation chain) of the bfloat16
// planes, measured at 8192^3 on GB300 with 128 x 128 single-CTA tiles
// against a float64 reference (K = 4096 errors):
//   3 passes: 1 slab 65 % of bf16 peak, 8 slabs 79 %, same error (the
//             2^-16 split residual dominates) -> 8.
//   6 passes: 1 slab 82 %, max error 6e-8 |A||B|; 2 slabs 87 %, 1e-7;
//             plain FP32 FMA 2.3e-7 -> 1, the margin is the point of 6.
//   scaled float16, 3 passes: see kF16DefaultFlush.
// Two-plane products run on 256-column tiles: as CTA pairs (256 x 256,
// each CTA holding 128 rows of B^T, 3 stages of 64 KiB) or single CTAs
// (128 x 256, 2 stages of 96 KiB).  Three planes need 128-column tiles to
// fit a ring of at least two stages.
// K slabs per TMEM chain for scaled float16 planes.  Measured at 8192^3 on
// GB300 with CTA pairs and 256 x 256 tiles (N(0,1) and row/column-scaled
// 10^U(-4,4) inputs, 512 outputs against a float64 reference; max / mean
// relative error; plain FP32 FMA 1.3e-3 / 5.6e-6, ill-scaled 7.5e-4 /
// 5.6e-6; TFLOP/s of the whole call):
//   1 slab  346 TFLOP/s   2.1e-5 / 8.2e-7
//   2 slabs 485           1.2e-4 / 1.5e-6
//   4 slabs 519           4.2e-4 / 3.5e-6   (ill-scaled 5.0e-4 / 3.0e-6)
//   8 slabs 537           6.9e-4 / 5.7e-6   (ill-scaled 1.0e-3 / 6.5e-6)
// 4 is the fastest that stays at or below the FP32 FMA chain's error on
// both inputs.
constexpr int kF16DefaultFlush = 4;

// Output tile width of the float16-plane GEMM: 256 columns; 128 when the
// 256-column tiles would leave more than half of the CTA pairs idle, and 64
// when even single-CTA 128 x 128 tiles would leave more than half of the
// SMs idle (small problems: more SMs share the multiply).  Every output is
// the same for every width.  NUMC_CUDA_SPLIT_TILE=64, 128 or 256 pins it
// (read once).
int split_tile_width(const Gemm &g, int ctas) {
  static const int forced = [] {
    const char *e = getenv("NUMC_CUDA_SPLIT_TILE");
    return e ? atoi(e) : 0;
  }();
  if (forced == 64 || forced == 128 || forced == 256) return forced;
  const int64_t rows = 128 * ctas;
  const int64_t wide = (g.M + rows - 1) / rows * ((g.N + 255) / 256);
  if (2 * wide >= sm_count() / ctas) return 256;
  const int64_t narrow = (g.M + 127) / 128 * ((g.N + 127) / 128);   // single-CTA tiles
  return 2 * narrow < sm_count() ? 64 : 128;
}

template <int CTAS>
cudaError_t launch_gemm_ctas(const SplitLayout &L, const SplitBufs &ws, const Gemm &g,
                             unsigned long long gen, unsigned *status, cudaStream_t s,
                             int narrow, bool pdl) {
  constexpr int S2 = CTAS == 2 ? 3 : 2;   // stages of the 2-plane ring
  if (L.f16 && L.flush == kF16DefaultFlush && narrow == 64)
    // 64-column single-CTA tiles: 48 KiB stages
    return launch_gemm_status<64, 4, 2, kF16DefaultFlush, true, 1>(L, ws, g, gen, status, s, pdl);
  if (L.f16 && L.flush == kF16DefaultFlush && narrow == 128)
    // 128-column tiles: 48 KiB (pair) or 64 KiB (single CTA) stages
    return launch_gemm_status<128, CTAS == 2 ? 4 : 3, 2, kF16DefaultFlush, true, CTAS>(
        L, ws, g, gen, status, s, pdl);
  if (L.f16) {
    switch (L.flush) {
    case 1: return launch_gemm_status<256, S2, 2, 1, true, CTAS>(L, ws, g, gen, status, s, pdl);
    case 2: return launch_gemm_status<256, S2, 2, 2, true, CTAS>(L, ws, g, gen, status, s, pdl);
    case 4: return launch_gemm_status<256, S2, 2, 4, true, CTAS>(L, ws, g, gen, status, s, pdl);
    default: return launch_gemm_status<256, S2, 2, 8, true, CTAS>(L, ws, g, gen, status, s, pdl);
    }
  }
  if (L.planes == 3)
    return launch_gemm_status<128, CTAS == 2 ? 3 : 2, 3, 1, false, CTAS>(L, ws, g, gen, status, s, pdl);
  return launch_gemm_status<256, S2, 2, 8, false, CTAS>(L, ws, g, gen, status, s, pdl);
}

// CTA pairs unless NUMC_CUDA_SPLIT_CTAS=1 asks for single CTAs (for hosts
// where clusters cannot be launched).  At 8192^3 the pairs measured 519
// against 461 TFLOP/s (float16 planes, flush 4) and 600 against 500
// (bfloat16, 3 passes).
int split_ctas() {
  static const int v = [] {
    const char *e = getenv("NUMC_CUDA_SPLIT_CTAS");
    return (e && atoi(e) == 1) ? 1 : 2;
  }();
  return v;
}

// Small problems that take 128-column tiles run them on single CTAs
// (measured on GB300 at 512^3 - 1536^3: 0.5-0.7 us faster than pairs).
cudaError_t launch_gemm(const SplitLayout &L, const SplitBufs &ws, const Gemm &g, unsigned long long gen,
                        unsigned *status, cudaStream_t s, bool pdl = true) {
  const int ctas = split_ctas();
  const int width = split_tile_width(g, ctas);
  const int narrow = width < 256 ? width : 0;   // 0: the wide tiles
  if (ctas == 2 && !(narrow && L.f16 && L.flush == kF16DefaultFlush))
    return launch_gemm_ctas<2>(L, ws, g, gen, status, s, narrow, pdl);
  return launch_gemm_ctas<1>(L, ws, g, gen, status, s, narrow, pdl);
}

int planes_for(int passes) { return passes == 6 ? 3 : 2; }


}  // namespace

size_t split_bf16_workspace(int64_t M, int64_t K, int64_t N, int passes) {
  return split_layout(M, K, N, planes_for(passes)).total;
}

size_t split_f16_workspace(int64_t M, int64_t K, int64_t N) {
  return split_layout(M, K, N, 2, true).total;
}

namespace {
cudaError_t run_split(const Gemm &g, const SplitLayout &L, void *ws_v, size_t ws_bytes,
                      cudaStream_t s);
}

cudaError_t launch_split_bf16(const Gemm &g, int passes, void *ws_v, size_t ws_bytes,
                              cudaStream_t s) {
  return run_split(g, split_layout(g.M, g.K, g.N, planes_for(passes)), ws_v, ws_bytes, s);
}

cudaError_t launch_split_f16(const Gemm &g, int flush, void *ws_v, size_t ws_bytes,
                             cudaStream_t s) {
  if (flush == 0) flush = kF16DefaultFlush;
  if (flush != 1 && flush != 2 && flush != 4 && flush != 8) return cudaErrorInvalidValue;
  return run_split(g, split_layout(g.M, g.K, g.N, 2, true, flush), ws_v, ws_bytes, s);
}

// ---- row-panel pipeline ---------------------------------------------------------

SplitPipe split_pipe_layout(int algo, int param, int64_t M, int64_t K, int64_t N,
                            int64_t panel_rows, int64_t bpanel_cols) {
  SplitPipe p;
  p.f16 = algo == NUMC_CUDA_ALGO_SPLIT_FP16;
  p.planes = p.f16 ? 2 : planes_for(param);
  p.flush = p.f16 ? (param ? param : kF16DefaultFlush) : 0;
  p.M = M; p.K = K; p.N = N;
  p.Kp = round_up(K > 0 ? K : 1, kBK);
  p.panel_rows = panel_rows;
  p.npanels = (int)((M + panel_rows - 1) / panel_rows);
  p.bpanel_cols = bpanel_cols;
  p.nbpanels = (int)((N + bpanel_cols - 1) / bpanel_cols);
  // one region per column panel of B: planes, flags, maxima
  p.bregion_bytes = (size_t)round_up(p.planes * bpanel_cols * p.Kp * 2, 256) +
                    (size_t)round_up(((bpanel_cols + 63) / 64) * 8, 256) +
                    (p.f16 ? (size_t)round_up(bpanel_cols * 4, 256) : 0);
  p.panel_off = p.nbpanels * p.bregion_bytes;
  p.panel_bytes = (size_t)round_up(p.planes * panel_rows * p.Kp * 2, 256) +
                  (size_t)round_up(((panel_rows + kBM - 1) / kBM) * 8, 256) +
                  (p.f16 ? (size_t)round_up(panel_rows * 4, 256) : 0);
  p.total = p.panel_off + p.npanels * p.panel_bytes;
  return p;
}

unsigned long long split_pipe_gen() { return ++g_split_gen; }

namespace {
SplitLayout pipe_params(const SplitPipe &p) {
  SplitLayout L = split_layout(1, p.K, 1, p.planes, p.f16, p.flush);   // offsets unused
  return L;
}

SplitBufs pipe_bufs(const SplitPipe &p, int panel, int bpanel, char *ws) {
  SplitBufs b;
  char *q = ws + (size_t)(bpanel < 0 ? 0 : bpanel) * p.bregion_bytes;
  b.pb = (uint16_t *)q;
  q += round_up(p.planes * p.bpanel_cols * p.Kp * 2, 256);
  b.flags_b = (unsigned long long *)q;
  q += round_up(((p.bpanel_cols + 63) / 64) * 8, 256);
  b.max_b = p.f16 ? (unsigned *)q : nullptr;
  q = ws + p.panel_off + (size_t)(panel < 0 ? 0 : panel) * p.panel_bytes;
  b.pa = (uint16_t *)q;
  q += round_up(p.planes * p.panel_rows * p.Kp * 2, 256);
  b.flags_a = (unsigned long long *)q;
  q += round_up(((p.panel_rows + kBM - 1) / kBM) * 8, 256);
  b.max_a = p.f16 ? (unsigned *)q : nullptr;
  return b;
}
}  // namespace

cudaError_t split_pipe_b(const SplitPipe &p, int bpanel, const Gemm &g, void *ws,
                         unsigned long long gen, cudaStream_t s) {
  if (bpanel < 0 || bpanel >= p.nbpanels || g.N > p.bpanel_cols || g.N <= 0 || g.K <= 0)
    return cudaErrorInvalidValue;
  return split_b(pipe_params(p), pipe_bufs(p, -1, bpanel, (char *)ws), g, gen, s);
}

cudaError_t split_pipe_a(const SplitPipe &p, int panel, const Gemm &g, void *ws,
                         unsigned long long gen, cudaStream_t s) {
  if (panel < 0 || panel >= p.npanels || g.M > p.panel_rows || g.M <= 0 || g.K <= 0)
    return cudaErrorInvalidValue;
  return split_a(pipe_params(p), pipe_bufs(p, panel, -1, (char *)ws), g, gen, s);
}

cudaError_t split_pipe_gemm(const SplitPipe &p, int panel, int bpanel, const Gemm &g, void *ws,
                            unsigned long long gen, cudaStream_t s) {
  if (panel < 0 || panel >= p.npanels || g.M > p.panel_rows || g.M <= 0 || bpanel < 0 ||
      bpanel >= p.nbpanels || g.N > p.bpanel_cols || g.N <= 0 || g.K <= 0)
    return cudaErrorInvalidValue;
  unsigned *status = status_word();
  if (!status) return cudaErrorMemoryAllocation;
  // the pipeline orders this GEMM after its panels' splits with events on
  // other streams: no programmatic launch
  return launch_gemm(pipe_params(p), pipe_bufs(p, panel, bpanel, (char *)ws), g, gen, status, s,
                     false);
}

namespace {
cudaError_t run_split(const Gemm &g, const SplitLayout &L, void *ws_v, size_t ws_bytes,
                      cudaStream_t s) {
  if (g.M == 0 || g.N == 0) return cudaSuccess;
  if (g.K == 0) return launch_simt(NUMC_DTYPE_FLOAT32, g, 0, s);   // C = 0
  if (g.M >= (1ll << 31) || g.N >= (1ll << 31) || g.K >= (1ll << 31))
    return cudaErrorInvalidValue;
  if (ws_bytes < L.total || ((uintptr_t)ws_v & 255)) return cudaErrorInvalidValue;
  const SplitBufs bufs = bufs_of(L, (char *)ws_v);
  unsigned *status = status_word();
  if (!status) return cudaErrorMemoryAllocation;
  PhaseMark mark(s);
  const unsigned long long gen = ++g_split_gen;
  cudaError_t e = launch_split_pass(L, bufs, g, gen, s);
  if (e) return e;
  mark.split_done();
  e = launch_gemm(L, bufs, g, gen, status, s);
  mark.gemm_done();
  return e;
}
}  // namespace

}  // namespace numc_k

// ---- allocation-free entry point ---------------------------------------------
//
// Some callers of a GEMM may not allocate device memory at call time:
// real-time services that forbid allocation after start-up, work issued
// from stream callbacks (where CUDA calls that allocate are not allowed),
// and hosts whose device memory is owned by another framework's allocator.
// numc_cuda_sgemm_split_static runs the split-BF16 GEMM on a fixed scratch
// array compiled into this library instead of asking for workspace: the
// caller passes only inputs and outputs.
//
// The scratch array below is part of this module's device image: every GPU
// on which the library's kernels are loaded holds its 64 MiB until the
// process exits.  All calls share it, so calls that overlap on the GPU
// (two streams, or two host threads) race on it and must be serialised by
// the caller.  Its contents persist between calls; nothing in it needs to
// start at zero (the split planes are rewritten in full, the non-finite
// flags are tagged with the call's generation number) except the status
// word: the caller's, which each call clears, or, when the caller passes
// none, the library's own word g_static_status, which numc_cuda_check_status
// reads and clears.

namespace numc_k {
namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];
static __device__ unsigned g_static_status;

// Devices on which a call ran with the library's own status word.
std::atomic<uint64_t> g_static_status_used{0};

// Device addresses of g_static_scratch and g_static_status on the current
// device.  Host code may not use the arrays' names as addresses (they name
// host-side shadows), so the addresses are looked up with the device
// current, on every call: the lookup is a host-side table read once the
// module is loaded, and a cached pointer would outlive a context that
// cudaDeviceReset replaced.
cudaError_t static_addresses(void **scratch, unsigned **status) {
  cudaError_t e = cudaGetSymbolAddress(scratch, g_static_scratch);
  if (e != cudaSuccess) return e;
  return cudaGetSymbolAddress((void **)status, g_static_status);
}

}  // namespace

int static_status_read_and_clear(unsigned *status, void *stream) {
  *status = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  if (dev < 0 || dev >= 64 || !(g_static_status_used.load() >> dev & 1)) return 0;
  void *scratch = nullptr;
  unsigned *word = nullptr;
  cudaStream_t s = (cudaStream_t)stream;
  if ((e = static_addresses(&scratch, &word)) != cudaSuccess) return (int)e;
  if ((e = cudaMemcpyAsync(status, word, sizeof(unsigned), cudaMemcpyDeviceToHost, s)))
    return (int)e;
  if ((e = cudaMemsetAsync(word, 0, sizeof(unsigned), s))) return (int)e;
  return (int)cudaStreamSynchronize(s);
}

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
  const SplitLayout L = split_layout((int64_t)M, (int64_t)K, (int64_t)N, 2);
  if (L.total > kStaticScratchBytes)
    return NUMC_SET_ERROR(NUMC_ERR_VALUE,
                          "sgemm_split_static: %zux%zux%zu needs %zu bytes of scratch; the "
                          "static scratch holds %zu (4*(M+N)*roundup(K,64) bytes plus flags "
                          "must fit); use numc_cuda_gemm with a workspace instead",
                          M, K, N, L.total, kStaticScratchBytes);
  void *base = nullptr;
  unsigned *own_status = nullptr;
  cudaError_t e = static_addresses(&base, &own_status);
  if (e != cudaSuccess)
    return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "sgemm_split_static: scratch address: %s",
                          cudaGetErrorString(e));
  cudaStream_t s = (cudaStream_t)stream;
  if (!status) {
    // The library's word keeps the first failure until numc_cuda_check_status
    // reads and clears it, so one check covers a run of calls.
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess || dev < 0 || dev >= 64)
      return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "sgemm_split_static: device %d", dev);
    g_static_status_used.fetch_or(1ull << dev);
    status = own_status;
  } else if ((e = cudaMemsetAsync(status, 0, sizeof(unsigned), s)) != cudaSuccess) {
    return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "sgemm_split_static: %s", cudaGetErrorString(e));
  }
  Gemm g;
  g.a = a; g.b = b; g.c = out;
  g.M = (int64_t)M; g.K = (int64_t)K; g.N = (int64_t)N;
  g.rsa = rsa; g.csa = csa; g.rsb = rsb; g.csb = csb; g.rso = rso; g.cso = cso;
  if (K == 0) {
    e = launch_simt(NUMC_DTYPE_FLOAT32, g, 0, s);   // out = 0, no scratch
  } else {
    const SplitBufs bufs = bufs_of(L, (char *)base);
    const unsigned long long gen = ++g_split_gen;
    e = launch_split_pass(L, bufs, g, gen, s);
    if (e == cudaSuccess) e = launch_gemm(L, bufs, g, gen, status, s);
  }
  if (e != cudaSuccess)
    return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "sgemm_split_static: launch failed: %s",
                          cudaGetErrorString(e));
  return 0;
}

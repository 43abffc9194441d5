// numc_array_rand on the GPU: numc's four-lane xoshiro256** uniform fill
// (numc's src/random/kernel.h:18-400 and src/random/random.c:28-180),
// bit-identical to numc for every dtype and both of numc's fill paths.
//
// numc's generator state is per host thread (kernel.h:40-41): four
// xoshiro256** streams ("lanes").  A fill of n elements of `size` bytes:
//  * n * size <= 1 MiB: element 4j + l is lane l's j-th output (j < n/4),
//    the n % 4 tail continues lane 0; the lanes end n/4 steps further on
//    and lane 0 n % 4 more;
//  * otherwise numc splits it over T = min(n * size / 512 KiB, its OpenMP
//    maximum) threads with chunks of ceil(n / T) elements: element
//    start + 4j + l of the chunk at `start` is X(start + l + j) and its
//    tail element start + 4J + r is X(start + J + r), X(m) being lane 0's
//    output m steps on (J = chunk length / 4); every lane ends n steps on.
// Both index maps need the state m steps ahead for arbitrary m.  A
// xoshiro256 step is linear over GF(2)^256, so m steps are the matrix T^m:
// tables of T^(2^k), k < 64, are built once on the host (columns, for the
// host's own jumps) and kept on each device (rows).  Every warp is an
// independent unit owning 32 runs of kSteps consecutive steps of one chunk:
// it jumps its start state with the row tables (lane L computes rows
// L + 32 kk of each product, ballots assemble the words), spreads it to its
// lanes in five doubling stages (stage s: lanes [2^s, 2^(s+1)) get
// T^(kSteps 2^s) of lanes [0, 2^s)), and each lane steps its run.  In the
// large fill the four outputs of step j are X(m..m+3) of one stream, so a
// lane generates each value once and slides a window of four.  Outputs go
// through a per-warp shared-memory stage so that the warp writes whole
// 128-byte rows.  The host advances its copy of the state with the same
// tables.
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <unistd.h>

#include "kernels.h"

namespace numc_k {
namespace {

__host__ __device__ __forceinline__ uint64_t rotl64(uint64_t x, int k) {
  return (x << k) | (x >> (64 - k));
}
// xoshiro256**: output of state s, then the state update (kernel.h:177-189)
__host__ __device__ __forceinline__ uint64_t xo_output(const uint64_t s[4]) {
  return rotl64(s[1] * 5, 7) * 9;
}
__host__ __device__ __forceinline__ void xo_advance(uint64_t s[4]) {
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl64(s[3], 45);
}

// ---- T^(2^k) as 256 x 256 bit matrices ------------------------------------
// Vector bit 64 w + i is bit i of state word w.  col[k][b] = T^(2^k) e_b;
// bit b of row[k][r] = bit r of col[k][b].
constexpr int kPowers = 64;
constexpr size_t kTableWords = (size_t)kPowers * 256 * 4;   // one table kind

struct Tables {
  uint64_t col[kPowers][256][4];
  uint64_t row[kPowers][256][4];
};
Tables *g_tables = nullptr;
std::once_flag g_tables_once;

void apply_cols_host(const uint64_t (*col)[4], uint64_t v[4]) {
  uint64_t r[4] = {0, 0, 0, 0};
  for (int b = 0; b < 256; b++)
    if ((v[b >> 6] >> (b & 63)) & 1)
      for (int w = 0; w < 4; w++) r[w] ^= col[b][w];
  memcpy(v, r, sizeof r);
}

void build_tables() {
  Tables *t = new Tables;
  for (int b = 0; b < 256; b++) {
    uint64_t s[4] = {0, 0, 0, 0};
    s[b >> 6] = 1ull << (b & 63);
    xo_advance(s);
    memcpy(t->col[0][b], s, sizeof s);
  }
  for (int k = 1; k < kPowers; k++)
    for (int b = 0; b < 256; b++) {     // T^(2^k) e_b = T^(2^(k-1)) (T^(2^(k-1)) e_b)
      uint64_t v[4];
      memcpy(v, t->col[k - 1][b], sizeof v);
      apply_cols_host(t->col[k - 1], v);
      memcpy(t->col[k][b], v, sizeof v);
    }
  for (int k = 0; k < kPowers; k++)
    for (int r = 0; r < 256; r++) {
      uint64_t row[4] = {0, 0, 0, 0};
      for (int b = 0; b < 256; b++)
        if ((t->col[k][b][r >> 6] >> (r & 63)) & 1) row[b >> 6] |= 1ull << (b & 63);
      memcpy(t->row[k][r], row, sizeof row);
    }
  g_tables = t;
}

const Tables &tables() {
  std::call_once(g_tables_once, build_tables);
  return *g_tables;
}

// v = T^m v
void jump_host(uint64_t v[4], uint64_t m) {
  const Tables &t = tables();
  for (int k = 0; k < kPowers; k++)
    if ((m >> k) & 1) apply_cols_host(t.col[k], v);
}

// Device copies of the row tables (512 KiB), one per device, made on the
// first fill on that device and kept until exit.
std::mutex g_dev_mu;
uint64_t *g_dev_tables[64] = {nullptr};

cudaError_t device_tables(uint64_t **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_dev_mu);
  if (!g_dev_tables[dev]) {
    const Tables &t = tables();
    uint64_t *p = nullptr;
    if ((e = dev_malloc((void **)&p, kTableWords * sizeof(uint64_t))) != cudaSuccess) return e;
    if ((e = cudaMemcpy(p, t.row, kTableWords * sizeof(uint64_t), cudaMemcpyHostToDevice)) !=
        cudaSuccess) {
      cudaFree(p);
      return e;
    }
    g_dev_tables[dev] = p;
  }
  *out = g_dev_tables[dev];
  return cudaSuccess;
}

// ---- numc's per-thread state -----------------------------------------------

// [word][lane], numc's layout
thread_local uint64_t t_state[4][4];
thread_local bool t_seeded = false;

uint64_t splitmix64(uint64_t *x) {
  uint64_t z = (*x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// 2^128 steps by xoshiro256's published jump polynomial (kernel.h:60-96).
void jump128(uint64_t s[4]) {
  static const uint64_t kJump[4] = {0x180ec6d33cfd0abaull, 0xd5a61266f0c9392cull,
                                    0xa9582618e03fc9aaull, 0x39abdc4529b1661cull};
  uint64_t acc[4] = {0, 0, 0, 0};
  for (int i = 0; i < 4; i++)
    for (int b = 0; b < 64; b++) {
      if ((kJump[i] >> b) & 1)
        for (int w = 0; w < 4; w++) acc[w] ^= s[w];
      xo_advance(s);
    }
  memcpy(s, acc, sizeof acc);
}

// prng_seed (kernel.h:100-121): lane 0 from splitmix64, lanes 1-3 jumped.
void seed_state(uint64_t seed) {
  uint64_t base[4];
  for (int w = 0; w < 4; w++) base[w] = splitmix64(&seed);
  for (int w = 0; w < 4; w++) t_state[w][0] = base[w];
  for (int l = 1; l < 4; l++) {
    jump128(base);
    for (int w = 0; w < 4; w++) t_state[w][l] = base[w];
  }
  t_seeded = true;
}

void ensure_seeded() {
  if (!t_seeded) seed_state(0xdeadbeefcafe1234ull);   // numc's default (kernel.h:123-126)
}

// numc's OpenMP maximum thread count (omp_get_max_threads()): 0 = not set,
// taken from OMP_NUM_THREADS or the online CPU count on first use.
std::atomic<int> g_threads{0};

int default_threads() {
  if (const char *e = getenv("OMP_NUM_THREADS")) {
    const int v = atoi(e);   // first entry of a nesting list
    if (v > 0) return v;
  }
  const long c = sysconf(_SC_NPROCESSORS_ONLN);
  return c > 0 ? (int)c : 1;
}

// ---- the fill kernel -------------------------------------------------------

constexpr int kWarps = 4;                       // independent warps per block
// steps per lane: 32 in the small fill (at most 1 MiB: many short runs),
// 256 in large fills (64 measured 1.8x slower at 64 Mi float32: the jump
// and doubling products per lane then outweigh the generation)
constexpr int kLogStepsSmall = 5, kLogStepsLarge = 8;

struct RandArgs {
  uint64_t base[4][4];   // [stream][word]: the four lanes (small fill), lane 0 (large)
  int64_t n;             // elements
  int64_t chunk;         // elements per numc thread (large fill)
  int64_t warps_per_seg; // warps per numc thread's chunk (or the whole fill)
  void *out;
};

// Raw 64-bit output to the stored bits: integers keep the low bits;
// float32 (raw >> 41 | 0x3F800000) - 1, float64 (raw >> 11 | 0x3FF0...) - 1
// (random.c:28-39, kernel.h:200-212), both exact.
template <typename U, int KIND>
__device__ __forceinline__ U convert(uint64_t raw) {
  if constexpr (KIND == 1) {
    const float v = __fsub_rn(__uint_as_float((uint32_t)(raw >> 41) | 0x3F800000u), 1.0f);
    return (U)__float_as_uint(v);
  } else if constexpr (KIND == 2) {
    const double v =
        __dsub_rn(__longlong_as_double((long long)((raw >> 11) | 0x3FF0000000000000ull)), 1.0);
    return (U)__double_as_longlong(v);
  } else {
    return (U)raw;
  }
}

// Bit r = L + 32 kk (kk < 8) of R x, R a row-form table, for every lane L;
// returns the product assembled from the warp's ballots (all lanes).
__device__ __forceinline__ void row_product(const uint64_t *__restrict__ R, const uint64_t (&x)[4],
                                            uint64_t (&y)[4], int lane) {
  uint32_t word[8];
#pragma unroll
  for (int kk = 0; kk < 8; kk++) {
    const ulonglong2 *rp = reinterpret_cast<const ulonglong2 *>(R + (kk * 32 + lane) * 4);
    const ulonglong2 r01 = rp[0], r23 = rp[1];
    const uint64_t t = (r01.x & x[0]) ^ (r01.y & x[1]) ^ (r23.x & x[2]) ^ (r23.y & x[3]);
    word[kk] = __ballot_sync(0xffffffffu, __popcll(t) & 1);
  }
#pragma unroll
  for (int w = 0; w < 4; w++) y[w] = (uint64_t)word[2 * w] | ((uint64_t)word[2 * w + 1] << 32);
}

__device__ __forceinline__ uint64_t shfl64(uint64_t v, int src) {
  const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)v, src);
  const uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(v >> 32), src);
  return (uint64_t)lo | ((uint64_t)hi << 32);
}

// Staging row of one lane: 4 outputs a step packed into sizeof(U) words.
template <typename U>
__device__ __forceinline__ void stage_step(uint32_t *wp, const U (&o)[4]) {
  if constexpr (sizeof(U) == 1) {
    wp[0] = (uint32_t)o[0] | ((uint32_t)o[1] << 8) | ((uint32_t)o[2] << 16) | ((uint32_t)o[3] << 24);
  } else if constexpr (sizeof(U) == 2) {
    *reinterpret_cast<uint2 *>(wp) =
        make_uint2((uint32_t)o[0] | ((uint32_t)o[1] << 16), (uint32_t)o[2] | ((uint32_t)o[3] << 16));
  } else if constexpr (sizeof(U) == 4) {
    *reinterpret_cast<uint4 *>(wp) = make_uint4(o[0], o[1], o[2], o[3]);
  } else {
    reinterpret_cast<uint4 *>(wp)[0] = make_uint4((uint32_t)o[0], (uint32_t)((uint64_t)o[0] >> 32),
                                                  (uint32_t)o[1], (uint32_t)((uint64_t)o[1] >> 32));
    reinterpret_cast<uint4 *>(wp)[1] = make_uint4((uint32_t)o[2], (uint32_t)((uint64_t)o[2] >> 32),
                                                  (uint32_t)o[3], (uint32_t)((uint64_t)o[3] >> 32));
  }
}

// NV = 4: the four lanes of a small fill (runs of 2^LOGS steps of each);
// NV = 1: lane 0 of a large fill.  One unit of work per warp.
template <typename U, int KIND, int NV, int LOGS>
__global__ void __launch_bounds__(32 * kWarps)
rand_fill_kernel(const __grid_constant__ RandArgs a, const uint64_t *__restrict__ rows) {
  constexpr int kSteps = 1 << LOGS;
  constexpr int kStepsPerChunk = 32 / (int)sizeof(U);   // 4 outputs a step: 128 B a chunk row
  constexpr int kRowWords = 36;                         // 32 + pad, 16-byte aligned rows
  __shared__ __align__(16) uint32_t stage[kWarps][32][kRowWords];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t gw = (int64_t)blockIdx.x * kWarps + warp;
  const int64_t seg = gw / a.warps_per_seg, lw = gw % a.warps_per_seg;
  const int64_t start = NV == 1 ? seg * a.chunk : 0;
  const int64_t len = NV == 1 ? min(a.chunk, a.n - start) : a.n;
  if (len <= 0) return;
  const int64_t J = len / 4;
  const int tail = (int)(len % 4);
  const int64_t jw = lw * 32 * kSteps;
  if (lw > 0 && jw >= J) return;   // warp 0 of a chunk always runs (it may own only the tail)

  // Warp start T^(start + jw) on each stream, then lane L = T^(kSteps L) of it.
  uint64_t v[NV][4];
#pragma unroll
  for (int q = 0; q < NV; q++)
#pragma unroll
    for (int w = 0; w < 4; w++) v[q][w] = a.base[q][w];
  const uint64_t m = (uint64_t)(start + jw);
  for (int k = 0; k < kPowers; k++) {
    if (!((m >> k) & 1)) continue;
#pragma unroll
    for (int q = 0; q < NV; q++) row_product(rows + (size_t)k * 1024, v[q], v[q], lane);
  }
#pragma unroll 1
  for (int st = 0; st < 5; st++) {
    const int lo = 1 << st;
    const uint64_t *R = rows + (size_t)(LOGS + st) * 1024;
#pragma unroll 1
    for (int t = 0; t < lo; t++) {
#pragma unroll
      for (int q = 0; q < NV; q++) {
        uint64_t x[4], y[4];
#pragma unroll
        for (int w = 0; w < 4; w++) x[w] = shfl64(v[q][w], t);
        row_product(R, x, y, lane);
        if (lane == lo + t)
#pragma unroll
          for (int w = 0; w < 4; w++) v[q][w] = y[w];
      }
    }
  }

  const int64_t j0 = jw + (int64_t)lane * kSteps;
  const int64_t j1 = min(j0 + (int64_t)kSteps, J);
  const int mysteps = (int)max((int64_t)0, j1 - j0);
  U *out = (U *)a.out + start;
  const bool vec16 = ((uintptr_t)out & 15) == 0;
  uint32_t *row = stage[warp][lane];
  // fast write path: the warp's 32 runs all lie within the chunk
  const bool full = jw + 32 * (int64_t)kSteps <= J;
  constexpr size_t kPassBytes = (size_t)4 * kSteps * 4 * sizeof(U);   // 4 runs of output
  char *dfast = reinterpret_cast<char *>(out + 4 * (jw + (int64_t)(lane >> 3) * kSteps)) +
                16 * (lane & 7);
  const uint32_t *sfast = &stage[warp][lane >> 3][4 * (lane & 7)];

  // streams: four lanes, or a window X(m), X(m+1), X(m+2) of one stream
  uint64_t s[NV][4];
#pragma unroll
  for (int q = 0; q < NV; q++)
#pragma unroll
    for (int w = 0; w < 4; w++) s[q][w] = v[q][w];
  U win[3];
  if (NV == 1) {
#pragma unroll
    for (int l = 0; l < 3; l++) {
      win[l] = convert<U, KIND>(xo_output(s[0]));
      xo_advance(s[0]);
    }
  }

  for (int c = 0; c < kSteps / kStepsPerChunk; c++) {
    const int nv = min(kStepsPerChunk, mysteps - c * kStepsPerChunk);
#pragma unroll
    for (int i = 0; i < kStepsPerChunk; i++) {
      if (i < nv) {
        U o[4];
        if (NV == 1) {
          o[0] = win[0];
          o[1] = win[1];
          o[2] = win[2];
          o[3] = convert<U, KIND>(xo_output(s[0]));
          xo_advance(s[0]);
          win[0] = o[1];
          win[1] = o[2];
          win[2] = o[3];
        } else {
#pragma unroll
          for (int l = 0; l < 4; l++) {
            o[l] = convert<U, KIND>(xo_output(s[NV == 1 ? 0 : l]));
            xo_advance(s[NV == 1 ? 0 : l]);
          }
        }
        stage_step<U>(row + i * (int)sizeof(U), o);
      }
    }
    __syncwarp();
    // Write rows: row q holds steps jw + q kSteps + c C .. of lane q.
    if (vec16 && full) {
      // every row complete: 8 lanes a row (16 bytes each), 4 rows a pass
#pragma unroll
      for (int p = 0; p < 8; p++)
        *reinterpret_cast<uint4 *>(dfast + (size_t)p * kPassBytes + (size_t)c * 128) =
            *reinterpret_cast<const uint4 *>(sfast + p * 4 * kRowWords);
    } else if (vec16) {
      // 8 lanes a row (16 bytes each), 4 rows a pass
#pragma unroll 2
      for (int p = 0; p < 8; p++) {
        const int q = 4 * p + (lane >> 3), seg16 = lane & 7;
        const int64_t jq = jw + (int64_t)q * kSteps + (int64_t)c * kStepsPerChunk;
        const int64_t nq = min((int64_t)kStepsPerChunk, J - jq);
        const int vbytes = nq > 0 ? (int)nq * 4 * (int)sizeof(U) : 0;
        char *dst = reinterpret_cast<char *>(out + 4 * jq) + 16 * seg16;
        const uint32_t *src = &stage[warp][q][4 * seg16];
        if (16 * seg16 + 16 <= vbytes) {
          *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(src);
        } else if (16 * seg16 < vbytes) {
          const char *sb = reinterpret_cast<const char *>(src);
          for (int bb = 0; bb < vbytes - 16 * seg16; bb++) dst[bb] = sb[bb];
        }
      }
    } else {
      for (int q = 0; q < 32; q++) {
        const int64_t jq = jw + (int64_t)q * kSteps + (int64_t)c * kStepsPerChunk;
        const int64_t nq = min((int64_t)kStepsPerChunk, J - jq);
        const U *src = reinterpret_cast<const U *>(stage[warp][q]);
        for (int e = lane; e < 4 * nq; e += 32) out[4 * jq + e] = src[e];
      }
    }
    __syncwarp();
  }
  // The chunk's tail continues stream 0 from step J (in the large fill the
  // window then holds X(start + J .. start + J + 2)).
  if (tail && ((J == 0 && lw == 0 && lane == 0) || (j0 < J && j1 == J))) {
    for (int r = 0; r < tail; r++) {
      if (NV == 1) {
        out[4 * J + r] = win[r];
      } else {
        out[4 * J + r] = convert<U, KIND>(xo_output(s[0]));
        xo_advance(s[0]);
      }
    }
  }
}

template <typename U, int KIND>
cudaError_t launch_fill(const RandArgs &a, bool large, unsigned blocks, const uint64_t *rows,
                        cudaStream_t s) {
  if (large)
    rand_fill_kernel<U, KIND, 1, kLogStepsLarge><<<blocks, 32 * kWarps, 0, s>>>(a, rows);
  else
    rand_fill_kernel<U, KIND, 4, kLogStepsSmall><<<blocks, 32 * kWarps, 0, s>>>(a, rows);
  count_launch();
  return cudaGetLastError();
}

}  // namespace

void rand_seed(uint64_t seed) { seed_state(seed); }

int rand_threads() {
  int t = g_threads.load();
  if (t <= 0) {
    t = default_threads();
    int expect = 0;
    g_threads.compare_exchange_strong(expect, t);
    t = g_threads.load();
  }
  return t;
}

void rand_set_threads(int threads) { g_threads.store(threads > 0 ? threads : 0); }

cudaError_t rand_fill(NumcDType dt, void *out, size_t n, cudaStream_t s) {
  ensure_seeded();
  if (n == 0) return cudaSuccess;
  uint64_t *tabs = nullptr;
  cudaError_t e = device_tables(&tabs);
  if (e != cudaSuccess) return e;
  const size_t size = numc_dtype_size(dt);
  const size_t bytes = n * size;
  RandArgs a;
  memset(&a, 0, sizeof a);
  a.n = (int64_t)n;
  a.out = out;
  bool large;
  int logs;
  int64_t per_seg_steps, nseg;
  if (bytes <= (1u << 20)) {        // NUMC_OMP_BYTE_THRESHOLD
    large = false;
    for (int q = 0; q < 4; q++)
      for (int w = 0; w < 4; w++) a.base[q][w] = t_state[w][q];
    nseg = 1;
    per_seg_steps = (int64_t)n / 4;
    logs = kLogStepsSmall;
  } else {
    int64_t T = (int64_t)(bytes / (1u << 19));   // NUMC_OMP_BYTES_PER_THREAD
    T = std::min<int64_t>(T, rand_threads());
    if (T < 1) T = 1;
    large = true;
    for (int w = 0; w < 4; w++) a.base[0][w] = t_state[w][0];
    a.chunk = ((int64_t)n + T - 1) / T;
    nseg = T;
    per_seg_steps = a.chunk / 4;
    logs = kLogStepsLarge;
  }
  const int64_t steps_per_warp = (int64_t)32 << logs;
  a.warps_per_seg = std::max<int64_t>(1, (per_seg_steps + steps_per_warp - 1) / steps_per_warp);
  const int64_t blocks = (nseg * a.warps_per_seg + kWarps - 1) / kWarps;
  if (blocks > 0x7FFFFFFFll) return cudaErrorInvalidConfiguration;
  switch (dt) {
  case NUMC_DTYPE_INT8: case NUMC_DTYPE_UINT8: e = launch_fill<uint8_t, 0>(a, large, (unsigned)blocks, tabs, s); break;
  case NUMC_DTYPE_INT16: case NUMC_DTYPE_UINT16: e = launch_fill<uint16_t, 0>(a, large, (unsigned)blocks, tabs, s); break;
  case NUMC_DTYPE_INT32: case NUMC_DTYPE_UINT32: e = launch_fill<uint32_t, 0>(a, large, (unsigned)blocks, tabs, s); break;
  case NUMC_DTYPE_INT64: case NUMC_DTYPE_UINT64: e = launch_fill<uint64_t, 0>(a, large, (unsigned)blocks, tabs, s); break;
  case NUMC_DTYPE_FLOAT32: e = launch_fill<uint32_t, 1>(a, large, (unsigned)blocks, tabs, s); break;
  case NUMC_DTYPE_FLOAT64: e = launch_fill<uint64_t, 2>(a, large, (unsigned)blocks, tabs, s); break;
  default: return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  // numc's state after the fill: the small path moves every lane n/4 steps
  // and lane 0 n%4 more; the large path moves every lane n steps.
  for (int l = 0; l < 4; l++) {
    uint64_t v[4];
    for (int w = 0; w < 4; w++) v[w] = t_state[w][l];
    if (large) {
      jump_host(v, n);
    } else {
      jump_host(v, n / 4);
      if (l == 0)
        for (size_t r = 0; r < n % 4; r++) xo_advance(v);
    }
    for (int w = 0; w < 4; w++) t_state[w][l] = v[w];
  }
  return cudaSuccess;
}

}  // namespace numc_k

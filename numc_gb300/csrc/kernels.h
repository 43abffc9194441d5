// Launchers of the CUDA kernels (internal C++ interface of the backend).
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <atomic>
#include <cstdint>

#include "numc/cuda.h"
#include "numc/dtype.h"

namespace numc_k {

// One GEMM: c[i*rso + j*cso] = sum_k a[i*rsa + k*csa] * b[k*rsb + j*csb].
// Element strides; device pointers.
struct Gemm {
  const void *a, *b;
  void *c;
  int64_t M, K, N;
  int64_t rsa, csa, rsb, csb, rso, cso;
  // numc_linear: bias[j * bias_stride] added to column j of the product as
  // numc's elementwise add would (floats: one rounding; integers: modulo
  // 2^bits), folded into the store of the kernels that support it.
  const void *bias = nullptr;
  int64_t bias_stride = 1;
  // CUDA-core float kernels: which numc build's register-tile geometry to
  // follow (kIsaX86: x86-64 AVX2, kIsaNeon: aarch64 NEON).
  int isa = 0;
};
enum NumcIsa : int { kIsaX86 = 0, kIsaNeon = 1 };

// Whether `algo` adds Gemm::bias in its own epilogue (else the caller runs
// launch_bias_add after the GEMM).
bool fuses_bias(int algo);
// out[i, j] += bias[j] for an M x N output (the unfused form).
cudaError_t launch_bias_add(NumcDType dt, const Gemm &g, cudaStream_t s);

// int8/uint8 store rule applied by the SIMT integer kernel.
enum Rule8 : int {
  kRuleWrap = 0,      // truncate the full sum to 8 bits
  kRuleX86Packed = 1, // numc x86 AVX2 packed path (K blocks of 512)
  kRuleNeon = 2,      // numc aarch64 NEON path (one block over all K, 6x8 tiles)
  kRuleAvx512 = 3,    // numc x86-64 AVX-512 path (one block over all K, 12x16 tiles)
};

// float32/float64 SIMT variant (numc's x86 AVX2 arithmetic, bit-exact):
//   kFloatNumc       numc_matmul: the packed path above numc's gemmsup
//                    threshold (M K N > 96^3 float32, 48^3 float64), else
//                    the unpacked one;
//   kFloatNaive      numc's naive kernels (product and sum each rounded);
//   kFloatNumcPacked the packed path at every size (numc_dot's GEMM branch);
//   kFloatNumcSmall  the unpacked (gemmsup) path at every size.
// Full register tiles are one FMA chain per output in k order on both
// paths; remainder tiles differ (see simt_common.cuh).
// kFloatIsaNeon, or'ed in, follows numc's aarch64 NEON tile geometry
// instead of x86 AVX2's.
enum FloatSimt : int {
  kFloatNumc = 0, kFloatNaive = 1, kFloatNumcPacked = 2, kFloatNumcSmall = 3,
  kFloatKindMask = 15, kFloatIsaNeon = 16
};

// CUDA-core kernels for every dtype.  `rule8` is the Rule8 for int8/uint8,
// the FloatSimt variant for float32/float64, unused otherwise.
cudaError_t launch_simt(NumcDType dt, const Gemm &g, int rule8, cudaStream_t s);
// The float variant kFloatNumc resolves to for problem g.
int float_rule(NumcDType dt, const Gemm &g, int rule);
// The float tile geometry (NumcIsa) of the process-wide ISA profile.
int float_isa();

// numc_dot's non-GEMM cases (dot_kernels.cu), all on device pointers:
// out[i] = x[i] * scalar over an N-D strided array (scalar read from
// device memory, converted through double as numc does)...
constexpr int kDotMaxDims = 16;
struct DotNd {
  int dim;
  int64_t shape[kDotMaxDims], xs[kDotMaxDims], os[kDotMaxDims];   // element strides
};
cudaError_t launch_dot_scalar(NumcDType dt, const void *x, const void *scalar, void *out,
                              const DotNd &ix, cudaStream_t s);
// ...and the 1-D inner product a . b -> out[0].  `contiguous` selects numc's
// SIMD arithmetic (else its strided reduction); `scratch` holds at least
// dot1d_scratch_bytes() bytes.
size_t dot1d_scratch_bytes();
// dst[e] = src at the e-th multi-index of ix (row-major order) for
// elements of elem_size bytes (1, 2, 4 or 8): strided -> contiguous.
cudaError_t launch_gather(const void *src, void *dst, size_t elem_size, const DotNd &ix,
                          cudaStream_t s);
cudaError_t launch_dot_1d(NumcDType dt, const void *a, int64_t sa, const void *b, int64_t sb,
                          int64_t n, bool contiguous, void *out, void *scratch,
                          cudaStream_t s);
// float64 on the mma.sync f64 tensor path.
cudaError_t launch_dmma(const Gemm &g, cudaStream_t s);

// float32 split-BF16 on tcgen05 with `passes` = 3 (two bf16 planes) or 6
// (three planes): workspace bytes and launcher.
size_t split_bf16_workspace(int64_t M, int64_t K, int64_t N, int passes);
size_t split_f16_workspace(int64_t M, int64_t K, int64_t N);

// Row-panel pipeline of the split GEMMs (numc_matmul with host operands
// overlaps the panels with its host copies): B is split once, then each
// panel of `panel_rows` rows of A is split and multiplied into the same
// rows of C.  Workspace: B's planes, flags and maxima, then one region per
// panel.
struct SplitPipe {
  bool f16;
  int planes, flush;
  int64_t M, K, N, Kp, panel_rows, bpanel_cols;
  int npanels, nbpanels;
  size_t bregion_bytes, panel_off, panel_bytes, total;
};
// algo / param as resolved for numc_cuda_gemm (SPLIT_BF16 or SPLIT_FP16);
// A in row panels of panel_rows, B in column panels of bpanel_cols (a
// multiple of 256, or N for one panel).
SplitPipe split_pipe_layout(int algo, int param, int64_t M, int64_t K, int64_t N,
                            int64_t panel_rows, int64_t bpanel_cols);
unsigned long long split_pipe_gen();
// g: B's column panel `bpanel` as its own K x g.N matrix (g.b, g.rsb, g.csb).
cudaError_t split_pipe_b(const SplitPipe &p, int bpanel, const Gemm &g, void *ws,
                         unsigned long long gen, cudaStream_t s);
// g: A's row panel `panel` (g.a, g.M rows).
cudaError_t split_pipe_a(const SplitPipe &p, int panel, const Gemm &g, void *ws,
                         unsigned long long gen, cudaStream_t s);
// The product of A's row panel `panel` and B's column panel `bpanel`, both
// split: g.a / g.M the panel's rows, g.b / g.N the column panel as given to
// split_pipe_b, g.c its block of C.
cudaError_t split_pipe_gemm(const SplitPipe &p, int panel, int bpanel, const Gemm &g, void *ws,
                            unsigned long long gen, cudaStream_t s);
// float32 from scaled float16 planes (3 products); `flush` = K slabs per
// TMEM accumulation chain (1, 2, 4, 8; 0 = default).
cudaError_t launch_split_f16(const Gemm &g, int flush, void *ws, size_t ws_bytes,
                             cudaStream_t s);
cudaError_t launch_split_bf16(const Gemm &g, int passes, void *ws, size_t ws_bytes,
                              cudaStream_t s);

// int8/uint8 on tcgen05: `param` = numc's store rule (kRule*) + 256 x the
// tile schedule (kI8Tile*; auto picks by problem size).
enum I8Tile { kI8TileAuto = 0, kI8TileSingle = 1, kI8TilePair128 = 2, kI8TilePair256 = 3 };
size_t int8_tc_workspace(int64_t M, int64_t K, int64_t N);
cudaError_t launch_int8_tc(NumcDType dt, const Gemm &g, int param, void *ws, size_t ws_bytes,
                           cudaStream_t s);

// float64 Ozaki slicing on tcgen05.
size_t ozaki_workspace(int64_t M, int64_t K, int64_t N, int slices);
cudaError_t launch_ozaki(const Gemm &g, int slices, void *ws, size_t ws_bytes,
                         cudaStream_t s);

// numc_array_rand's generator (rand.cu): numc's four-lane xoshiro256**
// state of the calling host thread, and numc's OpenMP maximum thread count
// (its large-array fill splits the stream by thread count).
void rand_seed(uint64_t seed);
int rand_threads();
void rand_set_threads(int threads);
// Fill n elements of dtype at device pointer `out` as numc_array_rand
// would, and advance the calling thread's state as numc does.
cudaError_t rand_fill(NumcDType dt, void *out, size_t n, cudaStream_t s);

// Device-side status word set by kernels that give up on a bounded wait.
cudaError_t read_and_clear_status(unsigned *status, cudaStream_t s);

// Every device allocation of the library goes through here (cudaMalloc,
// or a simulated out-of-memory failure set by numc_cuda_debug_fail_malloc).
cudaError_t dev_malloc(void **p, size_t bytes);

// Streaming multiprocessors of the current device (cached per device).
int sm_count();
// Programmatic dependent launch of GEMM kernels after their operand passes
// (on unless the environment sets NUMC_CUDA_PDL=0).
bool pdl_enabled();
// Co-resident clusters of `kern` launched with `cfg` (0 if the query fails).
int max_active_clusters(const void *kern, const cudaLaunchConfig_t &cfg);

// Launch setup of one kernel, done once per device: its dynamic shared
// memory limit and its co-resident cluster count (host calls that cost
// microseconds, against launches of a few microseconds for small problems).
struct LaunchCache {
  std::atomic<uint64_t> attr_done{0};   // bit d: attribute set on device d
  std::atomic<int> clusters[64] = {};   // per device, 0 = not queried yet
};
cudaError_t smem_attr_once(LaunchCache &lc, const void *kern, int bytes);
int clusters_once(LaunchCache &lc, const void *kern, const cudaLaunchConfig_t &cfg);

// Count of kernel launches issued by this library.
void count_launch(unsigned n = 1);
uint64_t launches();

}  // namespace numc_k

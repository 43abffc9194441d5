// CUDA backend: numc_matmul dispatch, device residency, the device-pointer
// C-ABI (numc_cuda_gemm) and algorithm selection.
//
// numc_matmul keeps numc's contract (src/matmul/matmul.c:347-389,
// src/matmul/dispatch.h:20-59): validation order and error codes are the
// same, inputs are const, out is caller-allocated, and the call returns when
// the result is in `out`.  Where numc picks an ISA kernel from a dtype
// table, this backend picks a CUDA kernel; there is no CPU fallback: without
// a usable GPU the call fails with NUMC_ERR_INTERNAL.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.h"
#include "runtime.h"
#include "status.h"

using namespace numc_rt;

namespace {

// ---- process-wide algorithm choice ----------------------------------------

struct AlgoChoice {
  std::atomic<int> algo;
  std::atomic<int> param;
};
AlgoChoice g_algo[NUMC_DTYPE_COUNT];
std::once_flag g_algo_once;

// Which numc build's results to reproduce where numc's arithmetic depends
// on the ISA it was compiled for (int8/uint8 store rules, float register
// tiles): numc_cuda_set_isa_profile.  numc picks its kernels at compile
// time for the host it is built on (src/arch_dispatch.h), so the default is
// this host's: the NEON build on aarch64, the AVX2 build on x86-64.
std::atomic<int> g_isa_profile{
#if defined(__aarch64__)
    NUMC_INT8_ARM_NEON
#else
    NUMC_INT8_X86_AVX2
#endif
};

int parse_profile(const std::string &v) {
  if (v == "neon") return NUMC_INT8_ARM_NEON;
  if (v == "avx512") return NUMC_INT8_X86_AVX512;
  if (v == "wrap") return NUMC_INT8_WRAP;
  if (v == "x86" || v == "avx2") return NUMC_INT8_X86_AVX2;
  return -1;
}

void init_algos_from_env() {
  for (int d = 0; d < NUMC_DTYPE_COUNT; d++) {
    g_algo[d].algo = NUMC_CUDA_ALGO_SIMT;
    g_algo[d].param = 0;
  }
  // int8/uint8 and the CUDA-core float kernels follow the ISA profile
  for (NumcDType d : {NUMC_DTYPE_INT8, NUMC_DTYPE_UINT8, NUMC_DTYPE_FLOAT32, NUMC_DTYPE_FLOAT64})
    g_algo[d].param = -1;
  if (const char *e = getenv("NUMC_CUDA_ISA_PROFILE")) {
    const int p = parse_profile(e);
    if (p == NUMC_INT8_X86_AVX2 || p == NUMC_INT8_ARM_NEON || p == NUMC_INT8_X86_AVX512)
      g_isa_profile = p;
  }
  // int8/uint8: the tensor path is bit-exact and faster beyond tiny sizes.
  g_algo[NUMC_DTYPE_INT8].algo = NUMC_CUDA_ALGO_AUTO;
  g_algo[NUMC_DTYPE_UINT8].algo = NUMC_CUDA_ALGO_AUTO;
  if (const char *e = getenv("NUMC_CUDA_F32_ALGO")) {
    std::string v(e);
    if (v == "split" || v == "split3") g_algo[NUMC_DTYPE_FLOAT32].algo = NUMC_CUDA_ALGO_SPLIT_BF16;
    if (v == "split6") {
      g_algo[NUMC_DTYPE_FLOAT32].algo = NUMC_CUDA_ALGO_SPLIT_BF16;
      g_algo[NUMC_DTYPE_FLOAT32].param = 6;
    }
    else if (v == "split16") g_algo[NUMC_DTYPE_FLOAT32].algo = NUMC_CUDA_ALGO_SPLIT_FP16;
    else if (v == "auto") g_algo[NUMC_DTYPE_FLOAT32].algo = NUMC_CUDA_ALGO_AUTO;
  }
  if (const char *e = getenv("NUMC_CUDA_F64_ALGO")) {
    std::string v(e);
    if (v == "dmma") g_algo[NUMC_DTYPE_FLOAT64].algo = NUMC_CUDA_ALGO_DMMA;
    if (v.rfind("ozaki", 0) == 0) {
      g_algo[NUMC_DTYPE_FLOAT64].algo = NUMC_CUDA_ALGO_OZAKI;
      int s = v.size() > 6 ? atoi(v.c_str() + 6) : 8;
      g_algo[NUMC_DTYPE_FLOAT64].param = s;
    }
  }
  if (const char *e = getenv("NUMC_CUDA_INT8_PROFILE")) {
    const int p = parse_profile(e);
    if (p >= 0) {
      g_algo[NUMC_DTYPE_INT8].param = p;
      g_algo[NUMC_DTYPE_UINT8].param = p;
    }
  }
}

void ensure_algos() { std::call_once(g_algo_once, init_algos_from_env); }

// ---- device discovery -----------------------------------------------------

int g_device_count = -1;
std::once_flag g_dev_once;

int device_count() {
  std::call_once(g_dev_once, [] {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
      n = 0;
      cudaGetLastError();
    }
    g_device_count = n;
  });
  return g_device_count;
}

// Bytes of array data copied between host and device by this library
// (numc_cuda_transfer_bytes): staging of host operands and results,
// numc_cuda_array_to_device / _to_host.
std::atomic<uint64_t> g_transfer_bytes{0};

cudaError_t xfer_async(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind,
                       cudaStream_t s) {
  g_transfer_bytes += bytes;
  return cudaMemcpyAsync(dst, src, bytes, kind, s);
}

int cuda_fail(cudaError_t e, const char *what) {
  int code = (e == cudaErrorMemoryAllocation) ? NUMC_ERR_MALLOC : NUMC_ERR_INTERNAL;
  cudaGetLastError();
  return NUMC_SET_ERROR(code, "%s: %s", what, cudaGetErrorString(e));
}

#define CU(call, what)                         \
  do {                                         \
    cudaError_t e_ = (call);                   \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

// ---- library-managed per-device workspace for numc_cuda_gemm(NULL ws) -----

std::mutex g_ws_mu;
void *g_ws[64] = {nullptr};
size_t g_ws_bytes[64] = {0};

int library_workspace(size_t bytes, cudaStream_t s, void **out) {
  int dev = 0;
  CU(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev < 0 || dev >= 64) return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "device index %d", dev);
  std::lock_guard<std::mutex> lock(g_ws_mu);
  if (g_ws_bytes[dev] < bytes) {
    if (g_ws[dev]) {
      // Work queued on any stream may still use the old buffer.
      CU(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
      cudaFree(g_ws[dev]);
      g_ws[dev] = nullptr;
      g_ws_bytes[dev] = 0;
    }
    size_t grow = bytes + bytes / 4;
    CU(numc_k::dev_malloc(&g_ws[dev], grow), "cudaMalloc(workspace)");
    g_ws_bytes[dev] = grow;
  }
  (void)s;
  *out = g_ws[dev];
  return 0;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// ---- algorithm resolution -------------------------------------------------

struct Plan {
  int algo;     // concrete algorithm
  int param;    // Rule8 for int8/uint8, FloatSimt for SIMT floats, slices for Ozaki
};

// numc_matmul_naive's arithmetic, passed as `param` by the library itself.
constexpr int kParamNaive = -1000;

// `packed_only`: numc_dot's GEMM branch (src/reduction/dot.c:386-400), which
// calls numc's x86 AVX2 packed kernels directly — no small-size unpacked
// branch — and on NEON builds, whose dot has no GEMM table (dot.c:275-288),
// numc's naive kernels.
int resolve(NumcDType dt, int algo, int param, size_t M, size_t K, size_t N, Plan *p,
            bool packed_only = false) {
  ensure_algos();
  if (algo == NUMC_CUDA_ALGO_DEFAULT) {
    algo = g_algo[dt].algo.load();
    if (param == -1) param = g_algo[dt].param.load();
  }
  const bool is8 = dt == NUMC_DTYPE_INT8 || dt == NUMC_DTYPE_UINT8;
  const bool isf = dt == NUMC_DTYPE_FLOAT32 || dt == NUMC_DTYPE_FLOAT64;
  if (algo == NUMC_CUDA_ALGO_AUTO && is8) {
    algo = ((double)M * K * N >= (double)(1 << 21)) ? NUMC_CUDA_ALGO_TC_INT8 : NUMC_CUDA_ALGO_SIMT;
  } else if (algo == NUMC_CUDA_ALGO_AUTO) {
    if (dt != NUMC_DTYPE_FLOAT32)
      return NUMC_SET_ERROR(NUMC_ERR_VALUE, "AUTO algorithm is float32, int8 or uint8 only");
    // The scaled float16 split (float32-level error) pays for its scale
    // and split passes once each output sums enough terms and the grid
    // fills the GPU.
    const bool split = (uint64_t)M * N >= (1u << 16) && K >= 128;
    algo = split ? NUMC_CUDA_ALGO_SPLIT_FP16 : NUMC_CUDA_ALGO_SIMT;
    param = split ? 0 : -1;
  }
  // int8 tensor path: 16 x the tile schedule on top of the profile
  int i8_tile = 0;
  if (is8 && algo == NUMC_CUDA_ALGO_TC_INT8 && param >= 16) {
    i8_tile = param >> 4;
    param &= 15;
    if (i8_tile > NUMC_INT8_TILE_PAIR256)
      return NUMC_SET_ERROR(NUMC_ERR_VALUE, "int8 tile schedule %d outside 0..3", i8_tile);
  }
  // int8/uint8 and CUDA-core floats: `param` names the numc build (profile)
  const bool profiled = is8 || (isf && algo == NUMC_CUDA_ALGO_SIMT);
  if (profiled && param == -1) param = g_isa_profile.load();
  if (!profiled && param < 0) param = 0;   // default slices / passes / flush
  switch (algo) {
  case NUMC_CUDA_ALGO_SIMT: break;
  case NUMC_CUDA_ALGO_SPLIT_BF16:
    if (dt != NUMC_DTYPE_FLOAT32)
      return NUMC_SET_ERROR(NUMC_ERR_TYPE, "split-BF16 GEMM is float32 only");
    if (param == 0) param = 3;
    if (param != 3 && param != 6)
      return NUMC_SET_ERROR(NUMC_ERR_VALUE, "split-BF16 pass count %d is not 3 or 6", param);
    break;
  case NUMC_CUDA_ALGO_SPLIT_FP16:
    if (dt != NUMC_DTYPE_FLOAT32)
      return NUMC_SET_ERROR(NUMC_ERR_TYPE, "split-FP16 GEMM is float32 only");
    if (param != 0 && param != 1 && param != 2 && param != 4 && param != 8)
      return NUMC_SET_ERROR(NUMC_ERR_VALUE, "split-FP16 flush interval %d is not 1, 2, 4 or 8",
                            param);
    break;
  case NUMC_CUDA_ALGO_DMMA:
    if (dt != NUMC_DTYPE_FLOAT64)
      return NUMC_SET_ERROR(NUMC_ERR_TYPE, "DMMA GEMM is float64 only");
    break;
  case NUMC_CUDA_ALGO_TC_INT8:
    if (!is8)
      return NUMC_SET_ERROR(NUMC_ERR_TYPE, "the int8 tensor path is int8/uint8 only");
    break;
  case NUMC_CUDA_ALGO_OZAKI:
    if (dt != NUMC_DTYPE_FLOAT64)
      return NUMC_SET_ERROR(NUMC_ERR_TYPE, "Ozaki GEMM is float64 only");
    if (param == 0) param = 8;
    if (param < 1 || param > 8)
      return NUMC_SET_ERROR(NUMC_ERR_VALUE, "Ozaki slice count %d outside 1..8", param);
    break;
  default:
    return NUMC_SET_ERROR(NUMC_ERR_VALUE, "unknown algorithm %d", algo);
  }
  p->algo = algo;
  p->param = param;
  if (isf && algo == NUMC_CUDA_ALGO_SIMT) {
    // numc's AVX-512 float kernels are not reproduced (their float64 packed
    // path overflows its stack buffer, gemm_avx512.h:278,797): the AVX-512
    // profile keeps the AVX2 tiles for floats, as numc_dot does there.
    const bool naive = param == kParamNaive || param == NUMC_INT8_WRAP ||
                       (packed_only && param == NUMC_INT8_ARM_NEON);
    if (naive) p->param = numc_k::kFloatNaive;
    else if (param == NUMC_INT8_X86_AVX2 || param == NUMC_INT8_X86_AVX512)
      p->param = packed_only ? numc_k::kFloatNumcPacked : numc_k::kFloatNumc;
    else if (param == NUMC_INT8_ARM_NEON)
      p->param = numc_k::kFloatNumc | numc_k::kFloatIsaNeon;
    else return NUMC_SET_ERROR(NUMC_ERR_VALUE, "unknown float profile %d", param);
  }
  if (is8) {
    const bool sup = !packed_only && (uint64_t)M * K * N <= 192ull * 192 * 192;
    if (param == kParamNaive || param == NUMC_INT8_WRAP) p->param = numc_k::kRuleWrap;
    else if (param == NUMC_INT8_ARM_NEON)
      // NEON builds have no integer gemmsup (matmul.c:187-205) and numc_dot
      // falls to its naive kernels there
      p->param = packed_only ? numc_k::kRuleWrap : numc_k::kRuleNeon;
    else if (param == NUMC_INT8_X86_AVX2)
      // numc's x86 build sends M*K*N <= 192^3 to its unpacked kernels, which
      // truncate (src/matmul/matmul.c:241-256, gemmsup_avx2.h:744-756).
      p->param = sup ? numc_k::kRuleWrap : numc_k::kRuleX86Packed;
    else if (param == NUMC_INT8_X86_AVX512)
      // the AVX-512 build keeps AVX2's integer gemmsup and numc_dot's AVX2
      // GEMM table; numc_matmul's packed int8 is gemm_i8_avx512
      p->param = sup ? numc_k::kRuleWrap
                     : packed_only ? numc_k::kRuleX86Packed : numc_k::kRuleAvx512;
    else return NUMC_SET_ERROR(NUMC_ERR_VALUE, "unknown int8 profile %d", param);
    if (algo == NUMC_CUDA_ALGO_TC_INT8) p->param |= i8_tile << 8;
  }
  return 0;
}

size_t plan_workspace(const Plan &p, size_t M, size_t K, size_t N) {
  if (p.algo == NUMC_CUDA_ALGO_SPLIT_BF16) return numc_k::split_bf16_workspace(M, K, N, p.param);
  if (p.algo == NUMC_CUDA_ALGO_SPLIT_FP16) return numc_k::split_f16_workspace(M, K, N);
  if (p.algo == NUMC_CUDA_ALGO_OZAKI) return numc_k::ozaki_workspace(M, K, N, p.param);
  if (p.algo == NUMC_CUDA_ALGO_TC_INT8) return numc_k::int8_tc_workspace(M, K, N);
  return 0;
}

int run_plan(NumcDType dt, const Plan &p, const numc_k::Gemm &g, void *ws,
             size_t ws_bytes, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  switch (p.algo) {
  case NUMC_CUDA_ALGO_SIMT: e = numc_k::launch_simt(dt, g, p.param, s); break;
  case NUMC_CUDA_ALGO_DMMA: e = numc_k::launch_dmma(g, s); break;
  case NUMC_CUDA_ALGO_SPLIT_BF16: e = numc_k::launch_split_bf16(g, p.param, ws, ws_bytes, s); break;
  case NUMC_CUDA_ALGO_SPLIT_FP16: e = numc_k::launch_split_f16(g, p.param, ws, ws_bytes, s); break;
  case NUMC_CUDA_ALGO_OZAKI: e = numc_k::launch_ozaki(g, p.param, ws, ws_bytes, s); break;
  case NUMC_CUDA_ALGO_TC_INT8: e = numc_k::launch_int8_tc(dt, g, p.param, ws, ws_bytes, s); break;
  }
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
  return 0;
}

// ---- context stream and scratch ------------------------------------------

int ctx_stream(NumcCtx *ctx, cudaStream_t *s) {
  if (device_count() <= 0)
    return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "no CUDA device available (the GB300 backend has no CPU fallback)");
  if (!ctx->stream) {
    int dev = 0;
    CU(cudaGetDevice(&dev), "cudaGetDevice");
    cudaStream_t st;
    CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    ctx->stream = st;
    ctx->device = dev;
  }
  *s = (cudaStream_t)ctx->stream;
  return 0;
}

int ctx_scratch(NumcCtx *ctx, size_t bytes, cudaStream_t s, char **out) {
  if (ctx->scratch_bytes < bytes) {
    if (ctx->scratch) {
      CU(cudaStreamSynchronize(s), "cudaStreamSynchronize");
      cudaFree(ctx->scratch);
      ctx->scratch = nullptr;
      ctx->scratch_bytes = 0;
    }
    size_t grow = align_up(bytes + bytes / 4, 1 << 20);
    CU(numc_k::dev_malloc(&ctx->scratch, grow), "cudaMalloc(scratch)");
    ctx->scratch_bytes = grow;
  }
  *out = (char *)ctx->scratch;
  return 0;
}

bool is_resident(const NumcArray *a) {
  return a->dev_base && a->residency != kHostOnly;
}

int check_matmul(const NumcArray *a, const NumcArray *b, const NumcArray *out) {
  if (!a || !b || !out)
    return NUMC_SET_ERROR(NUMC_ERR_NULL, "matmul: NULL pointer (a=%p b=%p out=%p)",
                          (const void *)a, (const void *)b, (const void *)out);
  if (a->dtype != b->dtype || a->dtype != out->dtype)
    return NUMC_SET_ERROR(NUMC_ERR_TYPE, "matmul: dtype mismatch (a=%d b=%d out=%d)",
                          a->dtype, b->dtype, out->dtype);
  if (a->dim != 2 || b->dim != 2 || out->dim != 2)
    return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "matmul: ndim mismatch (a.dim=%zu b.dim=%zu out.dim=%zu)",
                          a->dim, b->dim, out->dim);
  if (a->shape[1] != b->shape[0])
    return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "matmul: shape mismatch (a.shape[1]=%zu b.shape[0]=%zu)",
                          a->shape[1], b->shape[0]);
  if (out->shape[0] != a->shape[0] || out->shape[1] != b->shape[1])
    return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "matmul: out shape (%zu, %zu) != (%zu, %zu)",
                          out->shape[0], out->shape[1], a->shape[0], b->shape[1]);
  return 0;
}

// A lazily created non-blocking stream kept in the context.
int ctx_aux_stream(NumcCtx *ctx, void **slot, cudaStream_t *s) {
  if (!*slot) {
    cudaStream_t st;
    CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    *slot = st;
  }
  *s = (cudaStream_t)*slot;
  return 0;
}

bool rows_contiguous(const NumcArray *x) {
  return x->strides[1] == x->elem_size && x->strides[0] == x->shape[1] * x->elem_size;
}

// Whether a split GEMM with host operands runs as a row-panel pipeline.
bool use_pipeline(const Plan &plan, const NumcArray *a, const NumcArray *b, const NumcArray *out,
                  size_t M, size_t K, size_t N) {
  if (plan.algo != NUMC_CUDA_ALGO_SPLIT_FP16 && plan.algo != NUMC_CUDA_ALGO_SPLIT_BF16) return false;
  if (is_resident(a) || is_resident(b) || is_resident(out)) return false;
  if (!rows_contiguous(a) || !rows_contiguous(out)) return false;
  return M >= 1024 && K >= 64 && (double)M * K * N >= 4294967296.0;
}

cudaError_t xfer2d_async(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width,
                         size_t height, cudaMemcpyKind kind, cudaStream_t s) {
  g_transfer_bytes += width * height;
  return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, kind, s);
}

// Host operands of a large split GEMM: the host copies overlap the work.
// A moves in row panels and B in column panels, interleaved on the copy-in
// stream (A0, B0, A1, B1, ...); the compute stream splits each panel once it
// has arrived and multiplies every (row panel, column panel) pair as soon as
// both are split; the copy-out stream returns each block of C as soon as its
// GEMM is done.  The GEMMs thus start after two panels instead of after all
// of B.  The splits run on the compute stream and the block GEMMs alternate
// between two more streams, so a split never queues behind a GEMM and a
// block's kernel starts on the SMs its predecessor leaves idle (a 2048 x
// 2048 block is 64 tiles for 76 CTA pairs).  Every output's arithmetic is that of one device-resident call (the
// float16 planes' scales are per row of A and per column of B), so the
// results are identical.  B whose rows and columns are both strided moves
// whole, as one column panel.
int matmul_pipelined(const NumcArray *a, const NumcArray *b, NumcArray *out, const Plan &plan,
                     cudaStream_t s) {
  NumcCtx *ctx = out->ctx;
  const size_t M = a->shape[0], K = a->shape[1], N = b->shape[1], es = 4;
  // panels of A (rows) and of B (columns): NUMC_CUDA_PIPE_PANELS, else 4
  // from 4096 rows, 2 below
  size_t want = M >= 4096 ? 4 : 2;
  if (const char *pe = getenv("NUMC_CUDA_PIPE_PANELS")) {
    const long v = strtol(pe, nullptr, 10);
    if (v >= 1 && v <= 64) want = (size_t)v;
  }
  const size_t rows = align_up((M + want - 1) / want, 256);
  const size_t sb0 = b->strides[0], sb1 = b->strides[1];
  // 1: B's rows contiguous, 2: its columns contiguous, 0: neither
  const int bmode = (sb1 == es && sb0 % es == 0 && sb0 >= N * es) ? 1
                    : (sb0 == es && sb1 % es == 0 && sb1 >= K * es) ? 2 : 0;
  const size_t bcols = (bmode && N >= 1024) ? align_up((N + want - 1) / want, 256) : N;
  const numc_k::SplitPipe pp =
      numc_k::split_pipe_layout(plan.algo, plan.param, M, K, N, rows, bcols);
  const int na = pp.npanels, nb = pp.nbpanels;
  const size_t sa = array_span_bytes(a), so = array_span_bytes(out);
  const size_t sbytes = bmode ? K * N * es : array_span_bytes(b);
  const size_t off_b = align_up(sa, 256), off_c = off_b + align_up(sbytes, 256);
  const size_t off_w = off_c + align_up(so, 256);
  char *scratch = nullptr;
  int err;
  if ((err = ctx_scratch(ctx, off_w + pp.total + 256, s, &scratch))) return err;
  cudaStream_t cin, cout, s2, s3;
  if ((err = ctx_aux_stream(ctx, &ctx->copy_in, &cin))) return err;
  if ((err = ctx_aux_stream(ctx, &ctx->copy_out, &cout))) return err;
  if ((err = ctx_aux_stream(ctx, &ctx->gemm2, &s2))) return err;
  if ((err = ctx_aux_stream(ctx, &ctx->gemm3, &s3))) return err;
  char *dA = scratch, *dB = scratch + off_b, *dC = scratch + off_c, *ws = scratch + off_w;

  std::vector<cudaEvent_t> ev;
  auto cleanup = [&] {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
  };
  auto fail_cu = [&](cudaError_t e, const char *what) {
    cudaStreamSynchronize(cin);
    cudaStreamSynchronize(s);
    cudaStreamSynchronize(s2);
    cudaStreamSynchronize(s3);
    cudaStreamSynchronize(cout);
    cleanup();
    return cuda_fail(e, what);
  };
  // ev[0]: scratch free; ev[1 + p]: A panel p copied; ev[1 + na + q]: B
  // panel q copied; ev[1 + na + nb + p nb + q]: block (p, q) of C computed;
  // then A panel p split, then B panel q split.
  for (int i = 0; i < 1 + 2 * (na + nb) + na * nb; i++) {
    cudaEvent_t e;
    cudaError_t ce = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (ce != cudaSuccess) return fail_cu(ce, "cudaEventCreate");
    ev.push_back(e);
  }
  auto ev_a = [&](int p) { return ev[1 + p]; };
  auto ev_b = [&](int q) { return ev[1 + na + q]; };
  auto ev_c = [&](int p, int q) { return ev[1 + na + nb + p * nb + q]; };
  auto ev_sa = [&](int p) { return ev[1 + na + nb + na * nb + p]; };
  auto ev_sb = [&](int q) { return ev[1 + 2 * na + nb + na * nb + q]; };
  int nblock = 0;   // blocks issued so far: even ones on s2, odd ones on s3
  auto arows = [&](int p) { return std::min(rows, M - (size_t)p * rows); };
  auto bcount = [&](int q) { return std::min(bcols, N - (size_t)q * bcols); };
  // B column panel q on the device: compact K x nq (bmode 1 row-major,
  // bmode 2 column-major), or all of B with its own strides (bmode 0).
  auto b_panel = [&](int q, numc_k::Gemm *g) {
    const size_t n0 = (size_t)q * bcols, nq = bcount(q);
    if (bmode == 1) {
      g->b = dB + K * n0 * es; g->rsb = (int64_t)nq; g->csb = 1;
    } else if (bmode == 2) {
      g->b = dB + K * n0 * es; g->rsb = 1; g->csb = (int64_t)K;
    } else {
      g->b = dB; g->rsb = (int64_t)(sb0 / es); g->csb = (int64_t)(sb1 / es);
    }
    g->N = (int64_t)nq;
  };
  cudaError_t e;
  // The previous user of the scratch (the compute stream) must be done
  // before the copy-in stream overwrites it.
  if ((e = cudaEventRecord(ev[0], s)) || (e = cudaStreamWaitEvent(cin, ev[0], 0)))
    return fail_cu(e, "stream order");
  for (int i = 0; i < std::max(na, nb); i++) {
    if (i < na) {
      const size_t r0 = (size_t)i * rows;
      if ((e = xfer_async(dA + r0 * K * es, (const char *)a->data + r0 * K * es,
                          arows(i) * K * es, cudaMemcpyHostToDevice, cin)) ||
          (e = cudaEventRecord(ev_a(i), cin)))
        return fail_cu(e, "copy an A panel to device");
    }
    if (i < nb) {
      const size_t n0 = (size_t)i * bcols, nq = bcount(i);
      if (bmode == 1)
        e = xfer2d_async(dB + K * n0 * es, nq * es, (const char *)b->data + n0 * sb1, sb0,
                         nq * es, K, cudaMemcpyHostToDevice, cin);
      else if (bmode == 2)
        e = xfer2d_async(dB + K * n0 * es, K * es, (const char *)b->data + n0 * sb1, sb1,
                         K * es, nq, cudaMemcpyHostToDevice, cin);
      else
        e = xfer_async(dB, b->data, sbytes, cudaMemcpyHostToDevice, cin);
      if (e || (e = cudaEventRecord(ev_b(i), cin))) return fail_cu(e, "copy a B panel to device");
    }
  }
  numc_k::Gemm g;
  g.a = dA; g.b = dB; g.c = dC;
  g.M = M; g.K = K; g.N = N;
  g.rsa = K; g.csa = 1;
  g.rsb = 0; g.csb = 0;
  g.rso = N; g.cso = 1;
  const unsigned long long gen = numc_k::split_pipe_gen();
  auto gemm_block = [&](int p, int q) -> cudaError_t {
    const size_t r0 = (size_t)p * rows, n0 = (size_t)q * bcols;
    numc_k::Gemm gp = g;
    gp.a = dA + r0 * K * es;
    gp.M = (int64_t)arows(p);
    b_panel(q, &gp);
    gp.c = dC + (r0 * N + n0) * es;
    cudaStream_t gs = (nblock++ % 2) ? s3 : s2;
    cudaError_t ce;
    if ((ce = cudaStreamWaitEvent(gs, ev_sa(p), 0)) || (ce = cudaStreamWaitEvent(gs, ev_sb(q), 0)) ||
        (ce = numc_k::split_pipe_gemm(pp, p, q, gp, ws, gen, gs)) ||
        (ce = cudaEventRecord(ev_c(p, q), gs)) || (ce = cudaStreamWaitEvent(cout, ev_c(p, q), 0)))
      return ce;
    char *hc = (char *)out->data + (r0 * N + n0) * es;
    if (nb == 1)
      return xfer_async(hc, gp.c, arows(p) * N * es, cudaMemcpyDeviceToHost, cout);
    return xfer2d_async(hc, N * es, gp.c, N * es, bcount(q) * es, arows(p),
                        cudaMemcpyDeviceToHost, cout);
  };
  for (int i = 0; i < std::max(na, nb); i++) {
    if (i < na) {       // A panel i: split, then its blocks with the B panels before it
      numc_k::Gemm gp = g;
      gp.a = dA + (size_t)i * rows * K * es;
      gp.M = (int64_t)arows(i);
      if ((e = cudaStreamWaitEvent(s, ev_a(i), 0)) ||
          (e = numc_k::split_pipe_a(pp, i, gp, ws, gen, s)) || (e = cudaEventRecord(ev_sa(i), s)))
        return fail_cu(e, "split of an A panel");
      for (int q = 0; q < std::min(i, nb); q++)
        if ((e = gemm_block(i, q))) return fail_cu(e, "panel GEMM");
    }
    if (i < nb) {       // B panel i: split, then its blocks with the A panels so far
      numc_k::Gemm gp = g;
      b_panel(i, &gp);
      if ((e = cudaStreamWaitEvent(s, ev_b(i), 0)) ||
          (e = numc_k::split_pipe_b(pp, i, gp, ws, gen, s)) || (e = cudaEventRecord(ev_sb(i), s)))
        return fail_cu(e, "split of a B panel");
      for (int p = 0; p < std::min(i + 1, na); p++)
        if ((e = gemm_block(p, i))) return fail_cu(e, "panel GEMM");
    }
  }
  if ((e = cudaStreamSynchronize(cout)) || (e = cudaStreamSynchronize(s)) ||
      (e = cudaStreamSynchronize(s2)) || (e = cudaStreamSynchronize(s3)))
    return fail_cu(e, "cudaStreamSynchronize");
  cleanup();
  unsigned st = 0;
  CU(numc_k::read_and_clear_status(&st, s), "status read");
  if (st) return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "matmul kernel abandoned a bounded wait (code %u)", st);
  return 0;
}

// `bias` (numc_linear): a 1-D array of N elements added to every row of the
// product, or null.
int matmul_impl(const NumcArray *a, const NumcArray *b, NumcArray *out, int algo, int param,
                const NumcArray *bias = nullptr) {
  int err = check_matmul(a, b, out);
  if (err) return err;
  const size_t M = a->shape[0], K = a->shape[1], N = b->shape[1];
  if (M == 0 || N == 0) return 0;
  NumcDType dt = a->dtype;
  Plan plan;
  if ((err = resolve(dt, algo, param, M, K, N, &plan))) return err;
  NumcCtx *ctx = out->ctx;
  cudaStream_t s;
  if ((err = ctx_stream(ctx, &s))) return err;
  if (!bias && use_pipeline(plan, a, b, out, M, K, N)) return matmul_pipelined(a, b, out, plan, s);

  const size_t es = a->elem_size;
  const bool ra = is_resident(a), rb = is_resident(b), ro = is_resident(out);
  const bool rbias = bias && is_resident(bias);
  const size_t sa = array_span_bytes(a), sb = array_span_bytes(b), so = array_span_bytes(out);
  const size_t sbias = bias ? array_span_bytes(bias) : 0;
  size_t off_a = 0, off_b = align_up(ra ? 0 : sa, 256);
  size_t off_o = off_b + align_up(rb ? 0 : sb, 256);
  size_t off_bias = off_o + align_up(ro ? 0 : so, 256);
  size_t off_w = off_bias + align_up(rbias ? 0 : sbias, 256);
  size_t ws_bytes = plan_workspace(plan, M, K, N);
  char *scratch = nullptr;
  if ((err = ctx_scratch(ctx, off_w + ws_bytes + 256, s, &scratch))) return err;

  const char *da = ra ? a->dev_base : scratch + off_a;
  const char *db = rb ? b->dev_base : scratch + off_b;
  char *dout = ro ? out->dev_base : scratch + off_o;
  if (!ra) CU(xfer_async((void *)da, a->data, sa, cudaMemcpyHostToDevice, s), "copy a to device");
  if (!rb) CU(xfer_async((void *)db, b->data, sb, cudaMemcpyHostToDevice, s), "copy b to device");
  // A strided `out` with gaps between rows keeps the gap bytes: stage them.
  if (!ro && so > out->capacity)
    CU(xfer_async(dout, out->data, so, cudaMemcpyHostToDevice, s), "copy out to device");

  numc_k::Gemm g;
  g.a = da; g.b = db; g.c = dout;
  g.M = M; g.K = K; g.N = N;
  g.rsa = a->strides[0] / es; g.csa = a->strides[1] / es;
  g.rsb = b->strides[0] / es; g.csb = b->strides[1] / es;
  g.rso = out->strides[0] / es; g.cso = out->strides[1] / es;
  if (bias) {
    const char *dbias = rbias ? bias->dev_base : scratch + off_bias;
    if (!rbias && sbias)
      CU(xfer_async((void *)dbias, bias->data, sbias, cudaMemcpyHostToDevice, s), "copy bias to device");
    g.bias = dbias;
    g.bias_stride = (int64_t)(bias->strides[0] / es);
  }
  // The fused epilogues add the bias themselves; the others get one pass.
  numc_k::Gemm gk = g;
  if (!numc_k::fuses_bias(plan.algo)) gk.bias = nullptr;
  if ((err = run_plan(dt, plan, gk, scratch + off_w, ws_bytes, s))) return err;
  if (g.bias && !gk.bias) {
    cudaError_t be = numc_k::launch_bias_add(dt, g, s);
    if (be != cudaSuccess) return cuda_fail(be, "bias add");
  }

  if (ro) {
    out->residency = kDeviceOnly;
    // Host operands were read by asynchronous copies: finish them before
    // the caller may modify the host buffers.
    if (!ra || !rb) CU(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  } else {
    CU(xfer_async(out->data, dout, so, cudaMemcpyDeviceToHost, s), "copy out to host");
    CU(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  }
  if (plan.algo == NUMC_CUDA_ALGO_SPLIT_BF16 || plan.algo == NUMC_CUDA_ALGO_SPLIT_FP16 ||
      plan.algo == NUMC_CUDA_ALGO_OZAKI || plan.algo == NUMC_CUDA_ALGO_TC_INT8) {
    unsigned st = 0;
    CU(numc_k::read_and_clear_status(&st, s), "status read");
    if (st) return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "matmul kernel abandoned a bounded wait (code %u)", st);
  }
  return 0;
}

}  // namespace

// ---- hooks used by the core ------------------------------------------------

namespace numc_rt {

bool cuda_present() { return device_count() > 0; }

void *host_alloc_pinned(size_t bytes) {
  void *p = nullptr;
  if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}

void host_free_pinned(void *p) { cudaFreeHost(p); }

// Device memory for an array of `bytes` owned by the header at `owner`:
// bump allocation from the context's slabs, continuing in slab dev_cur and
// moving on to a later slab with room, or a new one (kDeviceSlab bytes, or
// the array's size if larger).
cudaError_t dev_arena_alloc(NumcCtx *ctx, size_t bytes, const ArenaPos &owner, char **out) {
  const size_t need = align_up(bytes ? bytes : 1, 256);
  auto &slabs = *ctx->dev_slabs;
  size_t i = ctx->dev_cur;
  while (i < slabs.size() && slabs[i].cap - slabs[i].used < need) i++;
  if (i == slabs.size()) {
    void *p = nullptr;
    const size_t cap = need > kDeviceSlab ? need : kDeviceSlab;
    cudaError_t e = numc_k::dev_malloc(&p, cap);
    if (e != cudaSuccess) return e;
    slabs.push_back(DeviceSlab{(char *)p, cap, 0});
  }
  DeviceSlab &sl = slabs[i];
  ctx->dev_cur = i;
  *out = sl.base + sl.used;
  ctx->dev_allocs->push_back(DeviceAlloc{*out, bytes, owner, sl.base});
  sl.used += need;
  return cudaSuccess;
}

int device_copy_contiguous(const NumcArray *src, NumcArray *dst) {
  if (src->dim > (size_t)numc_k::kDotMaxDims)
    return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "device copy: %zu dimensions (at most %d)", src->dim,
                          numc_k::kDotMaxDims);
  cudaStream_t s;
  int err = ctx_stream(dst->ctx, &s);
  if (err) return err;
  if (!dst->dev_base)
    CU(dev_arena_alloc(dst->ctx, dst->capacity, dst->pos, &dst->dev_base), "cudaMalloc(array)");
  numc_k::DotNd ix;
  ix.dim = (int)src->dim;
  for (size_t d = 0; d < src->dim; d++) {
    ix.shape[d] = (int64_t)src->shape[d];
    ix.xs[d] = (int64_t)(src->strides[d] / src->elem_size);
    ix.os[d] = 0;
  }
  cudaError_t e = numc_k::launch_gather(src->dev_base, dst->dev_base, src->elem_size, ix, s);
  if (e != cudaSuccess) return cuda_fail(e, "device gather");
  // The source may be released by the caller right after: finish here.
  CU(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  dst->residency = kDeviceOnly;
  return 0;
}

void ctx_release_device(NumcCtx *ctx, const ArenaPos *keep_upto) {
  if (!ctx->dev_allocs) return;
  if (ctx->stream && !ctx->dev_allocs->empty())
    cudaStreamSynchronize((cudaStream_t)ctx->stream);
  auto &v = *ctx->dev_allocs;
  auto &slabs = *ctx->dev_slabs;
  size_t w = 0;
  for (size_t r = 0; r < v.size(); r++)
    if (keep_upto && v[r].owner.before(*keep_upto)) v[w++] = v[r];
  v.resize(w);
  // Each slab rewinds to the end of its last surviving array.
  for (auto &sl : slabs) sl.used = 0;
  for (const auto &a : v)
    for (auto &sl : slabs)
      if (sl.base == a.slab) {
        const size_t end = (size_t)((char *)a.ptr - sl.base) + align_up(a.bytes ? a.bytes : 1, 256);
        if (end > sl.used) sl.used = end;
      }
  ctx->dev_cur = 0;
  for (size_t i = 0; i < slabs.size(); i++)
    if (slabs[i].used) ctx->dev_cur = i;
  if (!keep_upto) {
    for (auto &sl : slabs) cudaFree(sl.base);
    slabs.clear();
  }
  if (!keep_upto) {
    if (ctx->scratch) {
      if (ctx->stream) cudaStreamSynchronize((cudaStream_t)ctx->stream);
      cudaFree(ctx->scratch);
    }
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
    if (ctx->stream) cudaStreamDestroy((cudaStream_t)ctx->stream);
    ctx->stream = nullptr;
    for (void **cs : {&ctx->copy_in, &ctx->copy_out, &ctx->gemm2, &ctx->gemm3}) {
      if (*cs) {
        cudaStreamSynchronize((cudaStream_t)*cs);
        cudaStreamDestroy((cudaStream_t)*cs);
      }
      *cs = nullptr;
    }
  }
}

}  // namespace numc_rt

// ---- public API ------------------------------------------------------------

extern "C" int numc_matmul(const NumcArray *a, const NumcArray *b, NumcArray *out) {
  return matmul_impl(a, b, out, NUMC_CUDA_ALGO_DEFAULT, -1);
}

// numc's GemmSimdKernel on host memory: views of the caller's buffers on a
// per-thread context, run through numc_matmul's host-operand path.
namespace {
struct ThreadCtx {
  NumcCtx *ctx = nullptr;
  ~ThreadCtx() {
    if (ctx) numc_ctx_free(ctx);
  }
};
thread_local ThreadCtx t_host_ctx;

void host_view(NumcArray *v, NumcCtx *ctx, NumcDType dt, const void *data, size_t rows,
               size_t cols, intptr_t rs, intptr_t cs) {
  memset(v, 0, sizeof *v);
  const size_t es = numc_dtype_size(dt);
  v->ctx = ctx;
  v->data = const_cast<void *>(data);
  v->dim = 2;
  v->shape = v->shape_buf;
  v->strides = v->strides_buf;
  v->shape[0] = rows;
  v->shape[1] = cols;
  v->strides[0] = (size_t)rs * es;
  v->strides[1] = (size_t)cs * es;
  v->elem_size = es;
  v->size = rows * cols;
  v->capacity = rows && cols ? ((rows - 1) * (size_t)rs + (cols - 1) * (size_t)cs + 1) * es : 0;
  v->is_contiguous = cs == 1 && (size_t)rs == cols;
  v->dtype = dt;
  v->residency = kHostOnly;
}
}  // namespace

extern "C" int numc_cuda_gemm_host(NumcDType dt, const void *a, const void *b, void *out,
                                   size_t M, size_t K, size_t N, intptr_t rsa, intptr_t csa,
                                   intptr_t rsb, intptr_t rso) {
  if ((int)dt < 0 || (int)dt >= NUMC_DTYPE_COUNT)
    return NUMC_SET_ERROR(NUMC_ERR_TYPE, "gemm_host: unknown dtype %d", (int)dt);
  if (M == 0 || N == 0) return 0;
  if (!out || (K > 0 && (!a || !b)))
    return NUMC_SET_ERROR(NUMC_ERR_NULL, "gemm_host: NULL operand (a=%p b=%p out=%p)", a, b, out);
  if (rsa < 0 || csa < 0 || rsb < 0 || rso < 0)
    return NUMC_SET_ERROR(NUMC_ERR_VALUE, "gemm_host: negative stride");
  if (!t_host_ctx.ctx && !(t_host_ctx.ctx = numc_ctx_create()))
    return NUMC_SET_ERROR(NUMC_ERR_MALLOC, "gemm_host: context creation failed");
  NumcArray va, vb, vo;
  host_view(&va, t_host_ctx.ctx, dt, a, M, K, rsa, csa);
  host_view(&vb, t_host_ctx.ctx, dt, b, K, N, rsb, 1);   // numc: unit column strides
  host_view(&vo, t_host_ctx.ctx, dt, out, M, N, rso, 1);
  return matmul_impl(&va, &vb, &vo, NUMC_CUDA_ALGO_DEFAULT, -1);
}

extern "C" int numc_matmul_naive(const NumcArray *a, const NumcArray *b, NumcArray *out) {
  // numc's naive kernels (kernel.h:18-62): integers accumulate in the
  // storage type (8-bit through 32 bits, truncated), floats `acc += a * b`
  // without contraction.
  return matmul_impl(a, b, out, NUMC_CUDA_ALGO_SIMT, kParamNaive);
}

// ---- numc_linear / numc_bmm (numc's ROADMAP.md, "Linear algebra") -------------

extern "C" int numc_linear(const NumcArray *x, const NumcArray *w, const NumcArray *bias,
                           NumcArray *out) {
  if (bias) {
    if (!x || !w || !out)
      return NUMC_SET_ERROR(NUMC_ERR_NULL, "linear: NULL pointer (x=%p w=%p out=%p)",
                            (const void *)x, (const void *)w, (const void *)out);
    if (bias->dtype != x->dtype)
      return NUMC_SET_ERROR(NUMC_ERR_TYPE, "linear: bias dtype %d differs from x dtype %d",
                            bias->dtype, x->dtype);
    if (bias->dim != 1 || w->dim != 2 || bias->shape[0] != w->shape[1])
      return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "linear: bias must be 1-D of length N = %zu",
                            w->dim == 2 ? w->shape[1] : (size_t)0);
  }
  return matmul_impl(x, w, out, NUMC_CUDA_ALGO_DEFAULT, -1, bias);
}

namespace {

int check_bmm(const NumcArray *a, const NumcArray *b, const NumcArray *out) {
  if (!a || !b || !out)
    return NUMC_SET_ERROR(NUMC_ERR_NULL, "bmm: NULL pointer (a=%p b=%p out=%p)",
                          (const void *)a, (const void *)b, (const void *)out);
  if (a->dtype != b->dtype || a->dtype != out->dtype)
    return NUMC_SET_ERROR(NUMC_ERR_TYPE, "bmm: dtype mismatch (a=%d b=%d out=%d)", a->dtype,
                          b->dtype, out->dtype);
  if (a->dim < 2 || a->dim != b->dim || a->dim != out->dim)
    return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "bmm: ndim mismatch (a.dim=%zu b.dim=%zu out.dim=%zu)",
                          a->dim, b->dim, out->dim);
  const size_t d = a->dim;
  for (size_t i = 0; i + 2 < d; i++)
    if (a->shape[i] != b->shape[i] || a->shape[i] != out->shape[i])
      return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "bmm: batch axis %zu differs", i);
  if (a->shape[d - 1] != b->shape[d - 2])
    return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "bmm: shape mismatch (a.shape[-1]=%zu b.shape[-2]=%zu)",
                          a->shape[d - 1], b->shape[d - 2]);
  if (out->shape[d - 2] != a->shape[d - 2] || out->shape[d - 1] != b->shape[d - 1])
    return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "bmm: out shape (%zu, %zu) != (%zu, %zu)",
                          out->shape[d - 2], out->shape[d - 1], a->shape[d - 2], b->shape[d - 1]);
  return 0;
}

// numc_bmm: numc_matmul of every batch (the leading axes), one plan reused.
int bmm_impl(const NumcArray *a, const NumcArray *b, NumcArray *out) {
  int err = check_bmm(a, b, out);
  if (err) return err;
  const size_t d = a->dim;
  const size_t M = a->shape[d - 2], K = a->shape[d - 1], N = b->shape[d - 1];
  size_t P = 1;
  for (size_t i = 0; i + 2 < d; i++) P *= a->shape[i];
  if (P == 0 || M == 0 || N == 0) return 0;
  const NumcDType dt = a->dtype;
  Plan plan;
  if ((err = resolve(dt, NUMC_CUDA_ALGO_DEFAULT, -1, M, K, N, &plan))) return err;
  NumcCtx *ctx = out->ctx;
  cudaStream_t s;
  if ((err = ctx_stream(ctx, &s))) return err;
  const size_t es = a->elem_size;
  const bool ra = is_resident(a), rb = is_resident(b), ro = is_resident(out);
  const size_t sa = array_span_bytes(a), sb = array_span_bytes(b), so = array_span_bytes(out);
  const size_t off_b = align_up(ra ? 0 : sa, 256);
  const size_t off_o = off_b + align_up(rb ? 0 : sb, 256);
  const size_t off_w = off_o + align_up(ro ? 0 : so, 256);
  const size_t ws_bytes = plan_workspace(plan, M, K, N);
  char *scratch = nullptr;
  if ((err = ctx_scratch(ctx, off_w + ws_bytes + 256, s, &scratch))) return err;
  const char *da = ra ? a->dev_base : scratch;
  const char *db = rb ? b->dev_base : scratch + off_b;
  char *dout = ro ? out->dev_base : scratch + off_o;
  if (!ra && sa) CU(xfer_async((void *)da, a->data, sa, cudaMemcpyHostToDevice, s), "copy a to device");
  if (!rb && sb) CU(xfer_async((void *)db, b->data, sb, cudaMemcpyHostToDevice, s), "copy b to device");
  if (!ro && so > out->capacity)
    CU(xfer_async(dout, out->data, so, cudaMemcpyHostToDevice, s), "copy out to device");
  for (size_t p = 0; p < P; p++) {
    size_t rem = p, oa = 0, ob = 0, oo = 0;   // byte offsets of batch p
    for (size_t i = d - 2; i-- > 0;) {
      const size_t q = rem % a->shape[i];
      rem /= a->shape[i];
      oa += q * a->strides[i];
      ob += q * b->strides[i];
      oo += q * out->strides[i];
    }
    numc_k::Gemm g;
    g.a = da + oa; g.b = db + ob; g.c = dout + oo;
    g.M = M; g.K = K; g.N = N;
    g.rsa = a->strides[d - 2] / es; g.csa = a->strides[d - 1] / es;
    g.rsb = b->strides[d - 2] / es; g.csb = b->strides[d - 1] / es;
    g.rso = out->strides[d - 2] / es; g.cso = out->strides[d - 1] / es;
    if ((err = run_plan(dt, plan, g, scratch + off_w, ws_bytes, s))) return err;
  }
  if (ro) {
    out->residency = kDeviceOnly;
    if (!ra || !rb) CU(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  } else {
    CU(xfer_async(out->data, dout, so, cudaMemcpyDeviceToHost, s), "copy out to host");
    CU(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  }
  if (plan.algo != NUMC_CUDA_ALGO_SIMT && plan.algo != NUMC_CUDA_ALGO_DMMA) {
    unsigned st = 0;
    CU(numc_k::read_and_clear_status(&st, s), "status read");
    if (st) return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "bmm kernel abandoned a bounded wait (code %u)", st);
  }
  return 0;
}

}  // namespace

extern "C" int numc_bmm(const NumcArray *a, const NumcArray *b, NumcArray *out) {
  return bmm_impl(a, b, out);
}

namespace {

// ---- numc_dot (src/reduction/dot.c of numc) -----------------------------------

// numc's validation (src/reduction/dispatch.h:199-281): same checks, codes
// and messages.
int check_dot(const NumcArray *a, const NumcArray *b, const NumcArray *out) {
  if (!a || !b || !out)
    return NUMC_SET_ERROR(NUMC_ERR_NULL, "dot: NULL pointer (a=%p b=%p out=%p)",
                          (const void *)a, (const void *)b, (const void *)out);
  if (a->dtype != b->dtype || a->dtype != out->dtype)
    return NUMC_SET_ERROR(NUMC_ERR_TYPE, "dot: dtype mismatch (a=%d b=%d out=%d)", a->dtype,
                          b->dtype, out->dtype);
  if (a->dim == 0 || b->dim == 0) {
    const NumcArray *other = a->dim == 0 ? b : a;
    if (out->dim != other->dim)
      return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "dot: output ndim mismatch (out.dim=%zu other.dim=%zu)",
                            out->dim, other->dim);
    for (size_t i = 0; i < out->dim; i++)
      if (out->shape[i] != other->shape[i])
        return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "dot: shape mismatch at axis %zu", i);
    return 0;
  }
  const size_t a_last = a->dim - 1, b_red = b->dim == 1 ? 0 : b->dim - 2;
  if (a->shape[a_last] != b->shape[b_red])
    return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "dot: axis mismatch (a.shape[%zu]=%zu b.shape[%zu]=%zu)",
                          a_last, a->shape[a_last], b_red, b->shape[b_red]);
  const size_t expected = (a->dim - 1) + (b->dim > 1 ? b->dim - 1 : 0);
  const bool scalar_out =
      (expected == 0 && out->dim == 1 && out->size == 1) || (expected == 0 && out->dim == 0);
  if (!scalar_out && out->dim != expected)
    return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "dot: output ndim mismatch (out.dim=%zu expected=%zu)",
                          out->dim, expected);
  if (!scalar_out) {
    size_t o = 0;
    bool ok = true;
    for (size_t i = 0; i + 1 < a->dim; i++) ok &= out->shape[o++] == a->shape[i];
    if (b->dim > 1) {
      for (size_t i = 0; i + 2 < b->dim; i++) ok &= out->shape[o++] == b->shape[i];
      ok &= out->shape[o++] == b->shape[b->dim - 1];
    }
    if (!ok) return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "dot: output shape mismatch");
  }
  return 0;
}

// Axes [0, upto) of x collapse into one row axis (unit axes ignored).
bool flattenable(const NumcArray *x, size_t upto) {
  for (size_t d = 0; d + 1 < upto; d++)
    if (x->shape[d + 1] != 1 && x->strides[d] != x->strides[d + 1] * x->shape[d + 1]) return false;
  return true;
}

int dot_impl(const NumcArray *a, const NumcArray *b, NumcArray *out) {
  int err = check_dot(a, b, out);
  if (err) return err;
  if (out->size == 0) return 0;
  const NumcDType dt = a->dtype;
  const int64_t es = (int64_t)a->elem_size;
  enum { kScalar, kVector, kMatrix } kind =
      (a->dim == 0 || b->dim == 0) ? kScalar : (a->dim == 1 && b->dim == 1) ? kVector : kMatrix;

  // numc's N-D case (dot.c:367-420), element strides.
  int64_t M = 0, K = 0, N = 0, P = 1, rsa = 0, csa = 0, rsb = 0, csb = 0, rso = 0, cso = 0;
  bool gemm_branch = false;
  Plan plan{NUMC_CUDA_ALGO_SIMT, 0};
  size_t ws_bytes = 0;
  if (kind == kMatrix) {
    if (a->dim >= 3 && b->dim >= 3)
      return NUMC_SET_ERROR(NUMC_ERR_SHAPE,
                            "dot: a (%zu-D) and b (%zu-D) both above 2-D are not supported",
                            a->dim, b->dim);
    if (a->dim >= 3 && (!flattenable(a, a->dim - 1) || !flattenable(out, a->dim - 1)))
      return NUMC_SET_ERROR(NUMC_ERR_SHAPE,
                            "dot: the leading axes of a (and of out) must collapse into rows");
    K = (int64_t)a->shape[a->dim - 1];
    N = b->dim == 1 ? 1 : (int64_t)b->shape[b->dim - 1];
    M = 1;
    for (size_t d = 0; d + 1 < a->dim; d++) M *= (int64_t)a->shape[d];
    for (size_t d = 0; d + 2 < b->dim; d++) P *= (int64_t)b->shape[d];
    // numc's row stride is strides[0]; for a of 3+ dims that walks past
    // the array, so rows step by the second-to-last axis there.
    rsa = (int64_t)a->strides[a->dim >= 3 ? a->dim - 2 : 0] / es;
    csa = (int64_t)a->strides[a->dim - 1] / es;
    rsb = (int64_t)(b->dim > 1 ? b->strides[b->dim - 2] : b->strides[0]) / es;
    csb = (int64_t)b->strides[b->dim - 1] / es;
    rso = (int64_t)out->strides[a->dim >= 3 ? a->dim - 2 : 0] / es;
    cso = (int64_t)out->strides[out->dim - 1] / es;
    gemm_branch = P == 1 && csb == 1 && cso == 1;
    if (gemm_branch) {
      if ((err = resolve(dt, NUMC_CUDA_ALGO_DEFAULT, -1, M, K, N, &plan, true))) return err;
      ws_bytes = plan_workspace(plan, M, K, N);
    }
  } else if (kind == kVector) {
    ws_bytes = numc_k::dot1d_scratch_bytes();
  }

  NumcCtx *ctx = out->ctx;
  cudaStream_t s;
  if ((err = ctx_stream(ctx, &s))) return err;
  const bool ra = is_resident(a), rb = is_resident(b), ro = is_resident(out);
  const size_t sa = array_span_bytes(a), sb = array_span_bytes(b), so = array_span_bytes(out);
  const size_t off_b = align_up(ra ? 0 : sa, 256);
  const size_t off_o = off_b + align_up(rb ? 0 : sb, 256);
  const size_t off_w = off_o + align_up(ro ? 0 : so, 256);
  char *scratch = nullptr;
  if ((err = ctx_scratch(ctx, off_w + ws_bytes + 256, s, &scratch))) return err;
  const char *da = ra ? a->dev_base : scratch;
  const char *db = rb ? b->dev_base : scratch + off_b;
  char *dout = ro ? out->dev_base : scratch + off_o;
  char *ws = scratch + off_w;
  if (!ra && sa) CU(xfer_async((void *)da, a->data, sa, cudaMemcpyHostToDevice, s), "copy a to device");
  if (!rb && sb) CU(xfer_async((void *)db, b->data, sb, cudaMemcpyHostToDevice, s), "copy b to device");
  if (!ro && so > out->capacity)
    CU(xfer_async(dout, out->data, so, cudaMemcpyHostToDevice, s), "copy out to device");

  cudaError_t e = cudaSuccess;
  if (kind == kScalar) {
    const NumcArray *other = a->dim == 0 ? b : a;
    const char *dx = a->dim == 0 ? db : da, *dsc = a->dim == 0 ? da : db;
    if (other->dim > (size_t)numc_k::kDotMaxDims)
      return NUMC_SET_ERROR(NUMC_ERR_SHAPE, "dot: %zu dimensions (at most %d)", other->dim,
                            numc_k::kDotMaxDims);
    numc_k::DotNd ix;
    ix.dim = (int)other->dim;
    for (size_t d = 0; d < other->dim; d++) {
      ix.shape[d] = (int64_t)other->shape[d];
      ix.xs[d] = (int64_t)other->strides[d] / es;
      ix.os[d] = (int64_t)out->strides[d] / es;
    }
    e = numc_k::launch_dot_scalar(dt, dx, dsc, dout, ix, s);
  } else if (kind == kVector) {
    e = numc_k::launch_dot_1d(dt, da, (int64_t)a->strides[0] / es, db,
                              (int64_t)b->strides[0] / es, (int64_t)a->shape[0],
                              a->is_contiguous && b->is_contiguous, dout, ws, s);
  } else {
    numc_k::Gemm g;
    g.a = da; g.b = db; g.c = dout;
    g.M = M; g.K = K; g.N = N;
    g.rsa = rsa; g.csa = csa; g.rsb = rsb; g.csb = csb; g.rso = rso; g.cso = cso;
    // numc's naive kernels (dot.c:42-72): integers truncated (int8/uint8
    // sums wrap), floats unfused.
    const int naive = (dt == NUMC_DTYPE_INT8 || dt == NUMC_DTYPE_UINT8) ? numc_k::kRuleWrap
                      : (dt == NUMC_DTYPE_FLOAT32 || dt == NUMC_DTYPE_FLOAT64) ? numc_k::kFloatNaive
                                                                                : 0;
    if (gemm_branch) {
      if ((err = run_plan(dt, plan, g, ws, ws_bytes, s))) return err;
    } else if (P == 1) {
      e = numc_k::launch_simt(dt, g, naive, s);
    } else {
      for (int64_t p = 0; p < P && e == cudaSuccess; p++) {
        numc_k::Gemm gp = g;
        gp.b = db + (b->dim == 3 ? p * (int64_t)b->strides[0] : p * K * N * es);
        gp.c = dout + (out->dim == 3 ? p * (int64_t)out->strides[1] : p * N * es);
        e = numc_k::launch_simt(dt, gp, naive, s);
      }
    }
  }
  if (e != cudaSuccess) return cuda_fail(e, "dot kernel launch");

  if (ro) {
    out->residency = kDeviceOnly;
    if (!ra || !rb) CU(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  } else {
    CU(xfer_async(out->data, dout, so, cudaMemcpyDeviceToHost, s), "copy out to host");
    CU(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  }
  if (gemm_branch && plan.algo != NUMC_CUDA_ALGO_SIMT && plan.algo != NUMC_CUDA_ALGO_DMMA) {
    unsigned st = 0;
    CU(numc_k::read_and_clear_status(&st, s), "status read");
    if (st) return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "dot kernel abandoned a bounded wait (code %u)", st);
  }
  return 0;
}

}  // namespace

extern "C" int numc_dot(const NumcArray *a, const NumcArray *b, NumcArray *out) {
  return dot_impl(a, b, out);
}

extern "C" int numc_matmul_grouped(const NumcArray *const *a, const NumcArray *const *b,
                                   NumcArray *const *out, size_t n) {
  if (n == 0) return 0;
  if (!a || !b || !out) return NUMC_SET_ERROR(NUMC_ERR_NULL, "matmul_grouped: NULL array list");
  for (size_t i = 0; i < n; i++) {
    int err = check_matmul(a[i], b[i], out[i]);
    if (err) return err;
    if (a[i]->dtype != a[0]->dtype)
      return NUMC_SET_ERROR(NUMC_ERR_TYPE, "matmul_grouped: problem %zu dtype differs", i);
  }
  if (a[0]->dtype != NUMC_DTYPE_FLOAT32) {
    for (size_t i = 0; i < n; i++) {
      int err = numc_matmul(a[i], b[i], out[i]);
      if (err) return err;
    }
    return 0;
  }
  ensure_algos();
  // The process-wide float32 choice: SIMT stays numc's FMA chains,
  // SPLIT_BF16 keeps bfloat16 planes, AUTO and SPLIT_FP16 use scaled
  // float16 planes.
  int algo = g_algo[NUMC_DTYPE_FLOAT32].algo.load();
  if (algo != NUMC_CUDA_ALGO_SIMT && algo != NUMC_CUDA_ALGO_SPLIT_BF16)
    algo = NUMC_CUDA_ALGO_SPLIT_FP16;
  NumcCtx *ctx = out[0]->ctx;
  cudaStream_t s;
  int err = ctx_stream(ctx, &s);
  if (err) return err;

  // Stage every non-resident operand in the context scratch.
  const size_t es = 4;
  std::vector<size_t> off(3 * n, 0);
  size_t total = 0;
  bool staged_input = false;
  for (size_t i = 0; i < n; i++) {
    const NumcArray *arrs[3] = {a[i], b[i], out[i]};
    for (int t = 0; t < 3; t++) {
      if (is_resident(arrs[t])) continue;
      off[3 * i + t] = total;
      total += align_up(array_span_bytes(arrs[t]) + 1, 256);
      if (t < 2) staged_input = true;
    }
  }
  char *scratch = nullptr;
  if ((err = ctx_scratch(ctx, total + 256, s, &scratch))) return err;
  std::vector<NumcCudaGemmDesc> descs(n);
  for (size_t i = 0; i < n; i++) {
    const NumcArray *arrs[3] = {a[i], b[i], out[i]};
    char *dev[3];
    for (int t = 0; t < 3; t++) {
      if (is_resident(arrs[t])) {
        dev[t] = arrs[t]->dev_base;
      } else {
        dev[t] = scratch + off[3 * i + t];
        const size_t span = array_span_bytes(arrs[t]);
        if (span && (t < 2 || span > arrs[t]->capacity))
          CU(xfer_async(dev[t], arrs[t]->data, span, cudaMemcpyHostToDevice, s), "stage operand");
      }
    }
    NumcCudaGemmDesc &d = descs[i];
    d.a = dev[0]; d.b = dev[1]; d.out = dev[2];
    d.M = a[i]->shape[0]; d.K = a[i]->shape[1]; d.N = b[i]->shape[1];
    d.rsa = a[i]->strides[0] / es; d.csa = a[i]->strides[1] / es;
    d.rsb = b[i]->strides[0] / es; d.csb = b[i]->strides[1] / es;
    d.rso = out[i]->strides[0] / es; d.cso = out[i]->strides[1] / es;
  }
  NumcCudaGemmPlan *plan = numc_cuda_gemm_plan_create(NUMC_DTYPE_FLOAT32, algo, 0, descs.data(), n);
  if (!plan) return numc_get_error().code ? numc_get_error().code : NUMC_ERR_INTERNAL;
  err = numc_cuda_gemm_plan_run(plan, s);
  for (size_t i = 0; i < n && !err; i++) {
    if (is_resident(out[i])) {
      out[i]->residency = kDeviceOnly;
      continue;
    }
    const size_t span = array_span_bytes(out[i]);
    if (span) {
      cudaError_t e = xfer_async(out[i]->data, descs[i].out, span, cudaMemcpyDeviceToHost, s);
      if (e) err = cuda_fail(e, "copy out to host");
    }
  }
  cudaError_t e = cudaStreamSynchronize(s);
  (void)staged_input;
  numc_cuda_gemm_plan_free(plan);
  if (err) return err;
  if (e) return cuda_fail(e, "cudaStreamSynchronize");
  unsigned st = 0;
  CU(numc_k::read_and_clear_status(&st, s), "status read");
  if (st) return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "grouped kernel abandoned a bounded wait (code %u)", st);
  return 0;
}

extern "C" int numc_cuda_device_count(void) { return device_count(); }

extern "C" int numc_cuda_set_algo(NumcDType dt, int algo, int param) {
  ensure_algos();
  if ((int)dt < 0 || (int)dt >= NUMC_DTYPE_COUNT)
    return NUMC_SET_ERROR(NUMC_ERR_TYPE, "unknown dtype %d", (int)dt);
  Plan p;
  int err = resolve(dt, algo == NUMC_CUDA_ALGO_DEFAULT ? NUMC_CUDA_ALGO_SIMT : algo,
                    param, 1024, 1024, 1024, &p);
  if (err) return err;
  g_algo[dt].algo = algo == NUMC_CUDA_ALGO_DEFAULT ? NUMC_CUDA_ALGO_SIMT : algo;
  g_algo[dt].param = param;
  return 0;
}

extern "C" int numc_cuda_set_isa_profile(int profile) {
  ensure_algos();
  if (profile != NUMC_INT8_X86_AVX2 && profile != NUMC_INT8_ARM_NEON &&
      profile != NUMC_INT8_X86_AVX512)
    return NUMC_SET_ERROR(NUMC_ERR_VALUE, "unknown ISA profile %d", profile);
  g_isa_profile = profile;
  return 0;
}

extern "C" int numc_cuda_get_isa_profile(void) {
  ensure_algos();
  return g_isa_profile.load();
}

namespace numc_k {
int float_isa() { return numc_cuda_get_isa_profile() == NUMC_INT8_ARM_NEON ? kIsaNeon : kIsaX86; }
}  // namespace numc_k

extern "C" int numc_cuda_get_algo(NumcDType dt, int *algo, int *param) {
  ensure_algos();
  if ((int)dt < 0 || (int)dt >= NUMC_DTYPE_COUNT)
    return NUMC_SET_ERROR(NUMC_ERR_TYPE, "unknown dtype %d", (int)dt);
  if (algo) *algo = g_algo[dt].algo.load();
  if (param) *param = g_algo[dt].param.load();
  return 0;
}

extern "C" int numc_cuda_array_to_device(NumcArray *arr) {
  if (!arr) return NUMC_SET_ERROR(NUMC_ERR_NULL, "to_device: arr is NULL");
  if (is_resident(arr)) return 0;
  cudaStream_t s;
  int err = ctx_stream(arr->ctx, &s);
  if (err) return err;
  size_t span = array_span_bytes(arr);
  if (!arr->dev_base)
    CU(dev_arena_alloc(arr->ctx, span, arr->pos, &arr->dev_base), "cudaMalloc(array)");
  if (span) CU(xfer_async(arr->dev_base, arr->data, span, cudaMemcpyHostToDevice, s), "copy to device");
  CU(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  arr->residency = kBoth;
  return 0;
}

extern "C" int numc_cuda_array_to_host(NumcArray *arr) {
  if (!arr) return NUMC_SET_ERROR(NUMC_ERR_NULL, "to_host: arr is NULL");
  if (arr->residency != kDeviceOnly) return 0;
  cudaStream_t s;
  int err = ctx_stream(arr->ctx, &s);
  if (err) return err;
  size_t span = array_span_bytes(arr);
  if (span) CU(xfer_async(arr->data, arr->dev_base, span, cudaMemcpyDeviceToHost, s), "copy to host");
  CU(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  arr->residency = kBoth;
  return 0;
}

extern "C" uint64_t numc_cuda_transfer_bytes(void) { return g_transfer_bytes.load(); }

extern "C" int numc_cuda_ctx_device_usage(const NumcCtx *ctx, size_t *slabs,
                                          size_t *reserved_bytes, size_t *used_bytes) {
  if (!ctx) return NUMC_SET_ERROR(NUMC_ERR_NULL, "device usage: ctx is NULL");
  size_t n = 0, res = 0, used = 0;
  if (ctx->dev_slabs)
    for (const auto &sl : *ctx->dev_slabs) {
      n++;
      res += sl.cap;
      used += sl.used;
    }
  if (slabs) *slabs = n;
  if (reserved_bytes) *reserved_bytes = res;
  if (used_bytes) *used_bytes = used;
  return 0;
}

// ---- numc_manual_seed / numc_array_rand (numc's src/random/random.c) --------

extern "C" void numc_manual_seed(uint64_t seed) { numc_k::rand_seed(seed); }

namespace {

// A new array filled on the GPU, in its own device buffer, as numc's
// numc_array_rand fills it (_rand_impl, random.c:279-296); `to_host` copies
// it into the host buffer as well.
NumcArray *rand_array(NumcCtx *ctx, const size_t *shape, size_t dim, NumcDType dtype,
                      bool to_host) {
  if (!ctx || !shape || dim == 0) {
    NUMC_SET_ERROR(NUMC_ERR_NULL, "rand: NULL or invalid args (ctx=%p shape=%p dim=%zu)",
                   (void *)ctx, (const void *)shape, dim);
    return nullptr;
  }
  NumcArray *arr = numc_array_create(ctx, shape, dim, dtype);
  if (!arr) return nullptr;
  cudaStream_t s;
  if (ctx_stream(ctx, &s)) return nullptr;
  const size_t bytes = arr->capacity;
  if (!arr->dev_base) {
    cudaError_t e = dev_arena_alloc(ctx, bytes, arr->pos, &arr->dev_base);
    if (e != cudaSuccess) {
      cuda_fail(e, "cudaMalloc(array)");
      return nullptr;
    }
  }
  cudaError_t e = numc_k::rand_fill(dtype, arr->dev_base, arr->size, s);
  if (e != cudaSuccess) {
    cuda_fail(e, "rand fill");
    return nullptr;
  }
  if (to_host) {
    if (bytes && (e = xfer_async(arr->data, arr->dev_base, bytes, cudaMemcpyDeviceToHost, s)) !=
                     cudaSuccess) {
      cuda_fail(e, "copy to host");
      return nullptr;
    }
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) {
      cuda_fail(e, "cudaStreamSynchronize");
      return nullptr;
    }
    arr->residency = kBoth;
  } else {
    arr->residency = kDeviceOnly;
  }
  return arr;
}

}  // namespace

extern "C" NumcArray *numc_array_rand(NumcCtx *ctx, const size_t *shape, size_t dim,
                                      NumcDType dtype) {
  return rand_array(ctx, shape, dim, dtype, true);
}

extern "C" NumcArray *numc_cuda_array_rand(NumcCtx *ctx, const size_t *shape, size_t dim,
                                           NumcDType dtype) {
  return rand_array(ctx, shape, dim, dtype, false);
}

extern "C" int numc_cuda_rand_fill(NumcDType dtype, void *out, size_t n, void *stream) {
  if ((int)dtype < 0 || (int)dtype >= NUMC_DTYPE_COUNT)
    return NUMC_SET_ERROR(NUMC_ERR_TYPE, "rand_fill: unknown dtype %d", (int)dtype);
  if (!out && n) return NUMC_SET_ERROR(NUMC_ERR_NULL, "rand_fill: out is NULL");
  if (device_count() <= 0)
    return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "no CUDA device available (the GB300 backend has no CPU fallback)");
  CU(numc_k::rand_fill(dtype, out, n, (cudaStream_t)stream), "rand fill");
  return 0;
}

extern "C" int numc_cuda_rand_set_threads(int threads) {
  if (threads < 0) return NUMC_SET_ERROR(NUMC_ERR_VALUE, "rand_set_threads: %d < 0", threads);
  numc_k::rand_set_threads(threads);
  return 0;
}

extern "C" int numc_cuda_rand_threads(void) { return numc_k::rand_threads(); }


extern "C" void *numc_cuda_array_device_data(const NumcArray *arr) {
  return (arr && is_resident(arr)) ? arr->dev_base : nullptr;
}

extern "C" int numc_cuda_array_is_resident(const NumcArray *arr) {
  return arr && is_resident(arr);
}

extern "C" void *numc_cuda_ctx_stream(NumcCtx *ctx) {
  if (!ctx) return nullptr;
  cudaStream_t s;
  return ctx_stream(ctx, &s) ? nullptr : (void *)s;
}

extern "C" int numc_cuda_ctx_synchronize(NumcCtx *ctx) {
  if (!ctx) return NUMC_SET_ERROR(NUMC_ERR_NULL, "synchronize: ctx is NULL");
  if (!ctx->stream) return 0;
  CU(cudaStreamSynchronize((cudaStream_t)ctx->stream), "cudaStreamSynchronize");
  return 0;
}

extern "C" size_t numc_cuda_gemm_workspace_size(NumcDType dt, int algo, int param,
                                                size_t M, size_t K, size_t N) {
  if ((int)dt < 0 || (int)dt >= NUMC_DTYPE_COUNT) return 0;
  Plan p;
  if (resolve(dt, algo, param, M, K, N, &p)) return 0;
  return plan_workspace(p, M, K, N);
}

extern "C" int numc_cuda_gemm(NumcDType dt, int algo, int param, const void *a,
                              const void *b, void *out, size_t M, size_t K, size_t N,
                              intptr_t rsa, intptr_t csa, intptr_t rsb, intptr_t csb,
                              intptr_t rso, intptr_t cso, void *workspace,
                              size_t workspace_bytes, void *stream) {
  if ((int)dt < 0 || (int)dt >= NUMC_DTYPE_COUNT)
    return NUMC_SET_ERROR(NUMC_ERR_TYPE, "unknown dtype %d", (int)dt);
  if (M == 0 || N == 0) return 0;
  if (!out || (K > 0 && (!a || !b)))
    return NUMC_SET_ERROR(NUMC_ERR_NULL, "gemm: NULL operand (a=%p b=%p out=%p)", a, b, out);
  if (rsa < 0 || csa < 0 || rsb < 0 || csb < 0 || rso < 0 || cso < 0)
    return NUMC_SET_ERROR(NUMC_ERR_VALUE, "gemm: negative stride");
  if (device_count() <= 0)
    return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "no CUDA device available (the GB300 backend has no CPU fallback)");
  Plan p;
  int err = resolve(dt, algo, param, M, K, N, &p);
  if (err) return err;
  cudaStream_t s = (cudaStream_t)stream;
  size_t need = plan_workspace(p, M, K, N);
  void *ws = workspace;
  size_t ws_bytes = workspace_bytes;
  if (need) {
    if (!ws) {
      if ((err = library_workspace(need, s, &ws))) return err;
      ws_bytes = need;
    } else if (ws_bytes < need || ((uintptr_t)ws & 255)) {
      return NUMC_SET_ERROR(NUMC_ERR_VALUE, "gemm: workspace needs %zu bytes aligned to 256 (got %zu at %p)",
                            need, ws_bytes, ws);
    }
  }
  numc_k::Gemm g;
  g.a = a; g.b = b; g.c = out;
  g.M = M; g.K = K; g.N = N;
  g.rsa = rsa; g.csa = csa; g.rsb = rsb; g.csb = csb; g.rso = rso; g.cso = cso;
  return run_plan(dt, p, g, ws, ws_bytes, s);
}

extern "C" int numc_cuda_check_status(void *stream) {
  unsigned st = 0, st_static = 0;
  CU(numc_k::read_and_clear_status(&st, (cudaStream_t)stream), "status read");
  // numc_cuda_sgemm_split_static calls made without a status word of their
  // own report through the library's static word.
  CU((cudaError_t)numc_k::static_status_read_and_clear(&st_static, stream), "status read");
  if (!st) st = st_static;
  if (st) return NUMC_SET_ERROR(NUMC_ERR_INTERNAL, "a kernel abandoned a bounded wait (code %u)", st);
  return 0;
}

extern "C" uint64_t numc_cuda_launch_count(void) { return numc_k::launches(); }

/* CUDA backend extensions (GB300, sm_103a).  numc itself has no GPU API;
 * these entry points are additions.  They keep numc's conventions: return 0
 * or a negative NumcErrorCode, message via numc_get_error().
 *
 * Two layers:
 *   1. Device residency for NumcArray, so chains of numc_matmul calls keep
 *      their operands in HBM.
 *   2. The C-ABI GEMM below numc_matmul: plain device pointers, sizes and
 *      element strides.  It mirrors numc's per-dtype kernel table entry
 *        void (*GemmSimdKernel)(const void *a, const void *b, void *out,
 *                               size_t M, size_t K, size_t N, intptr_t rsa,
 *                               intptr_t csa, intptr_t rsb, intptr_t rso)
 *      (src/matmul/matmul.c:84-86), adding the column strides numc assumes
 *      to be 1, an algorithm choice, scratch memory and a CUDA stream.
 */
#ifndef NUMC_CUDA_H
#define NUMC_CUDA_H

#include "numc/array.h"
#include "numc/export.h"
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  NUMC_CUDA_ALGO_DEFAULT = 0,    /* process-wide choice for the dtype */
  NUMC_CUDA_ALGO_SIMT = 1,       /* CUDA cores; every dtype.  float32/64 are
                                    per-output FMA chains in k order */
  NUMC_CUDA_ALGO_SPLIT_BF16 = 2, /* float32 on tcgen05 from bfloat16 planes
                                    x = x0 + x1 (+ x2), float32 accumulation
                                    in TMEM.  `param` = passes: 3 (x0x0 +
                                    x0x1 + x1x0, default) or 6 (all
                                    products of order <= 2, float32-level
                                    error) */
  NUMC_CUDA_ALGO_DMMA = 3,       /* float64: mma.sync f64 tensor path */
  NUMC_CUDA_ALGO_OZAKI = 4,      /* float64: Ozaki slicing into 8-bit
                                    integer slices, exact slice products on
                                    tcgen05, integer recombination; `param`
                                    = slice count 1..8 (default 8) */
  NUMC_CUDA_ALGO_AUTO = 5,       /* float32: SPLIT_FP16 when the problem is
                                    large enough to pay for it, else SIMT;
                                    int8/uint8 (their default): TC_INT8 when
                                    M*K*N >= 2^21, else SIMT */
  NUMC_CUDA_ALGO_TC_INT8 = 6,    /* int8/uint8 on tcgen05 (values exact in
                                    bfloat16, exact FP32 sums per numc K
                                    block) with numc's store rules; `param`
                                    is a NumcInt8Profile, plus 16 x a
                                    NumcInt8Tile to pin the tile schedule */
  NUMC_CUDA_ALGO_SPLIT_FP16 = 7  /* float32 on tcgen05 from float16 planes:
                                    each row of A and column of B scaled by
                                    a power of two, x 2^s = h0 + h1 (22
                                    significant bits), h0h0 + h0h1 + h1h0
                                    with float32 accumulation, result
                                    scaled back exactly.  float32-level
                                    error at the cost of 3 products.
                                    `param` = K slabs of 64 per tensor-
                                    memory accumulation chain: 1, 2, 4 or 8
                                    (0 = default) */
} NumcCudaAlgo;

/* Which numc build's results to reproduce where numc's arithmetic depends
 * on the ISA it was compiled for: the store rules of its packed int8/uint8
 * kernels, and the register-tile geometry of its float32/float64 kernels
 * (which outputs are one FMA chain and which sum per-256 K-block chains, or
 * mix vector and scalar columns).  Used as `param` of int8/uint8 (every
 * algorithm) and of float32/float64 with NUMC_CUDA_ALGO_SIMT; -1 there
 * means the process-wide profile (numc_cuda_set_isa_profile). */
typedef enum {
  NUMC_INT8_X86_AVX2 = 0,  /* numc built for x86-64 AVX2 */
  NUMC_INT8_ARM_NEON = 1,  /* numc built for aarch64 NEON (-march=armv8-a) */
  NUMC_INT8_WRAP = 2,      /* numc_matmul_naive: int8 sums truncated to 8
                              bits, floats `acc += a * b` unfused */
  NUMC_INT8_X86_AVX512 = 3 /* numc built for x86-64 with AVX-512 (its
                              -march=native on such hosts): int8/uint8 only;
                              floats keep the AVX2 tiles */
} NumcInt8Profile;

/* Tile schedules of NUMC_CUDA_ALGO_TC_INT8 (16 x the schedule is added to
 * the profile in `param`).  Every schedule stores the same bytes. */
typedef enum {
  NUMC_INT8_TILE_AUTO = 0,    /* by problem size (the default) */
  NUMC_INT8_TILE_SINGLE = 1,  /* one CTA per 128 x 128 or 128 x 64 tile */
  NUMC_INT8_TILE_PAIR128 = 2, /* CTA pairs, persistent, 256 x 128 tiles */
  NUMC_INT8_TILE_PAIR256 = 3  /* CTA pairs, persistent, 256 x 256 tiles */
} NumcInt8Tile;

/* Number of usable CUDA devices (0 when none). */
NUMC_API int numc_cuda_device_count(void);

/* Process-wide algorithm per dtype used by numc_matmul and by
 * NUMC_CUDA_ALGO_DEFAULT.  For float64 OZAKI, `param` is the slice count;
 * for int8/uint8 and for SIMT float32/float64, `param` is a NumcInt8Profile
 * or -1 (the process-wide ISA profile, the default).  Environment
 * defaults: NUMC_CUDA_F32_ALGO (simt|split|split6|split16|auto),
 * NUMC_CUDA_F64_ALGO (simt|dmma|ozaki[:slices]), NUMC_CUDA_INT8_PROFILE
 * (x86|neon|avx512|wrap: int8/uint8 only). */
NUMC_API int numc_cuda_set_algo(NumcDType dtype, int algo, int param);
NUMC_API int numc_cuda_get_algo(NumcDType dtype, int *algo, int *param);

/* The process-wide ISA profile: NUMC_INT8_X86_AVX2, NUMC_INT8_ARM_NEON or
 * NUMC_INT8_X86_AVX512.  numc selects its kernels when it is compiled, for
 * the host it is compiled on, so the default is this host's build: NEON on
 * aarch64 (numc's -march=armv8-a build; no SVE), AVX2 on x86-64.
 * Environment: NUMC_CUDA_ISA_PROFILE (x86|neon|avx512).  numc_dot follows
 * it too: its GEMM branch calls numc's AVX2 kernels on x86 builds and its
 * naive kernels on NEON builds. */
NUMC_API int numc_cuda_set_isa_profile(int profile);
NUMC_API int numc_cuda_get_isa_profile(void);

/* --- device residency --------------------------------------------------- */

/* Copy the array to HBM and make the device copy authoritative: later
 * numc_matmul calls read/write it there without host transfers. */
NUMC_API int numc_cuda_array_to_device(NumcArray *arr);
/* Copy a device-resident array back into its host buffer (it stays
 * resident; both copies are valid until the next device write). */
NUMC_API int numc_cuda_array_to_host(NumcArray *arr);
/* Device address of the element at index 0, or NULL if not resident. */
NUMC_API void *numc_cuda_array_device_data(const NumcArray *arr);
NUMC_API int numc_cuda_array_is_resident(const NumcArray *arr);
/* The context's CUDA stream (cudaStream_t) and a wait for its work. */
NUMC_API void *numc_cuda_ctx_stream(NumcCtx *ctx);
NUMC_API int numc_cuda_ctx_synchronize(NumcCtx *ctx);

/* --- random inputs generated in HBM (no numc counterpart) --------------- */

/* numc_array_rand into a device-resident array: the same values and state
 * advance as numc_array_rand, but the data stays in HBM (the host buffer is
 * not written; numc_cuda_array_to_host copies it).  Asynchronous on the
 * context's stream. */
NUMC_API NumcArray *numc_cuda_array_rand(NumcCtx *ctx, const size_t *shape,
                                         size_t dim, NumcDType dtype);
/* numc_array_rand's fill of n elements of `dtype` at device pointer `out`,
 * enqueued on `stream` (a cudaStream_t); advances the calling thread's
 * state.  The first fill on a device uploads the generator's 1 MiB jump
 * tables there (cudaMalloc, kept until exit). */
NUMC_API int numc_cuda_rand_fill(NumcDType dtype, void *out, size_t n,
                                 void *stream);
/* numc's OpenMP maximum thread count that the large-array layout follows
 * (numc's omp_get_max_threads()); 0 restores the default: OMP_NUM_THREADS,
 * else the number of online CPUs. */
NUMC_API int numc_cuda_rand_set_threads(int threads);
NUMC_API int numc_cuda_rand_threads(void);

/* --- C-ABI GEMM on device pointers -------------------------------------- */

/* Scratch bytes numc_cuda_gemm needs for this problem (0 for SIMT/DMMA). */
NUMC_API size_t numc_cuda_gemm_workspace_size(NumcDType dtype, int algo,
                                              int param, size_t M, size_t K,
                                              size_t N);

/* out[i*rso + j*cso] = sum_k a[i*rsa + k*csa] * b[k*rsb + j*csb] with numc's
 * arithmetic for `dtype`.  a, b, out are device pointers; strides are in
 * elements.  `workspace` may be NULL (the library then keeps a per-device
 * scratch buffer, grown with cudaMalloc) or caller memory of at least
 * numc_cuda_gemm_workspace_size() bytes, aligned to 256 bytes.  `stream` is
 * a cudaStream_t (NULL = legacy default stream).  Asynchronous: returns
 * after enqueueing; launch errors are returned, kernel-side timeouts are
 * reported by numc_cuda_check_status(). */
NUMC_API int numc_cuda_gemm(NumcDType dtype, int algo, int param,
                            const void *a, const void *b, void *out,
                            size_t M, size_t K, size_t N, intptr_t rsa,
                            intptr_t csa, intptr_t rsb, intptr_t csb,
                            intptr_t rso, intptr_t cso, void *workspace,
                            size_t workspace_bytes, void *stream);

/* numc's per-dtype kernel-table entry (GemmSimdKernel, src/matmul/
 * matmul.c:84-86) with the dtype as first argument, on HOST memory: what
 * numc's own numc_matmul would call in place of gemm_simd_table[dtype]
 * (the in-tree binding).  out[i*rso + j] = sum_k a[i*rsa + k*csa] *
 * b[k*rsb + j] with the default algorithm of `dtype` (numc_cuda_set_algo);
 * b and out have unit column stride, as numc assumes.  Stages the operands
 * to the GPU, runs, copies the result back and returns when `out` holds it
 * (0, or a negative NumcErrorCode).  Device scratch comes from a context
 * kept per calling thread. */
NUMC_API int numc_cuda_gemm_host(NumcDType dtype, const void *a, const void *b,
                                 void *out, size_t M, size_t K, size_t N,
                                 intptr_t rsa, intptr_t csa, intptr_t rsb,
                                 intptr_t rso);

/* Waits for `stream` and reports any kernel that gave up on a bounded
 * wait (NUMC_ERR_INTERNAL); clears the flag. */
NUMC_API int numc_cuda_check_status(void *stream);

/* Testing aids for the failure paths (no counterpart in numc).
 * numc_cuda_debug_fail_malloc: the next `count` device allocations this
 * library makes fail as if the device were out of memory, so the calls
 * that needed them return NUMC_ERR_MALLOC (0 cancels).
 * numc_cuda_debug_wait_timeout: the tensor-core kernels launched from now
 * on give up a bounded wait after `limit_ns` nanoseconds (0 restores the
 * default, 2 s); with `starve` nonzero their TMA producers also issue no
 * loads, so every wait runs out, no copy or MMA is in flight when the
 * kernel leaves, and numc_cuda_check_status() reports NUMC_ERR_INTERNAL. */
NUMC_API int numc_cuda_debug_fail_malloc(int count);
NUMC_API int numc_cuda_debug_wait_timeout(unsigned long long limit_ns, int starve);

/* Number of kernels this library has launched since load (diagnostics). */
NUMC_API uint64_t numc_cuda_launch_count(void);
/* Bytes of array data this library has copied between host and device
 * (operand staging, results, numc_cuda_array_to_device/_to_host); lets a
 * caller check that a chain of device-resident calls makes no round trip. */
NUMC_API uint64_t numc_cuda_transfer_bytes(void);

/* Device memory of a context's arrays: bump-allocated from slabs of 64 MiB
 * (an array larger than that gets a slab of its own) in the order arrays
 * first need device memory.  numc_ctx_restore rewinds each slab to the end
 * of its last surviving array and keeps the slabs for reuse; numc_ctx_free
 * releases them.  Reports the slab count, their total size and the bytes
 * in use (any pointer may be NULL). */
NUMC_API int numc_cuda_ctx_device_usage(const NumcCtx *ctx, size_t *slabs,
                                        size_t *reserved_bytes, size_t *used_bytes);

/* Per-phase timing of the tensor-core GEMMs (split-BF16, Ozaki): when
 * enabled, each call records CUDA events on its stream around the operand
 * preparation kernels and around the GEMM kernel.  Enabling resets the
 * totals.  Do not enable while capturing a CUDA graph. */
NUMC_API int numc_cuda_phase_timing(int enable);
/* Sums since enabling, in milliseconds, over `calls` completed calls
 * (waits for the last recorded call). */
NUMC_API int numc_cuda_phase_times(double *prep_ms, double *gemm_ms,
                                   uint64_t *calls);

/* --- grouped GEMM (many uneven problems, one plan) ------------------------ */

/* One problem of a grouped GEMM: out = a @ b on device pointers with
 * element strides, as in numc_cuda_gemm. */
typedef struct {
  const void *a, *b;
  void *out;
  size_t M, K, N;
  intptr_t rsa, csa, rsb, csb, rso, cso;
} NumcCudaGemmDesc;

typedef struct NumcCudaGemmPlan NumcCudaGemmPlan;

/* Plan `count` float32 problems once: each problem gets a kernel from the
 * committed autotune table (the split GEMM with 128- or 64-column tiles and
 * 1, 2 or 4 K slices, or the CUDA-core kernel for small problems; `algo`
 * SIMT sends all to the CUDA cores), the plan allocates its workspace and
 * uploads TMA descriptors and tile lists.  With the split algorithms,
 * `param` 128 or 64 forces that tile width on every problem, plus 1000 x s
 * for s K slices (2 or 4; 0 = table).  K slices add their partial sums in K
 * order in a reduction pass: results are deterministic.  Pointers in `descs` are fixed from here on.  numc has no
 * counterpart: its callers loop numc_matmul (src/matmul/matmul.c:347). */
NUMC_API NumcCudaGemmPlan *numc_cuda_gemm_plan_create(NumcDType dtype, int algo,
                                                      int param,
                                                      const NumcCudaGemmDesc *descs,
                                                      size_t count);
/* Enqueue every problem of the plan on `stream` (a few launches, no host
 * synchronisation, no allocation; can be captured in a CUDA graph). */
NUMC_API int numc_cuda_gemm_plan_run(NumcCudaGemmPlan *plan, void *stream);
/* The same as one CUDA graph, captured on first use and replayed. */
NUMC_API int numc_cuda_gemm_plan_run_graph(NumcCudaGemmPlan *plan, void *stream);
/* Problems per kernel variant and the plan's device bytes. */
NUMC_API int numc_cuda_gemm_plan_info(const NumcCudaGemmPlan *plan, int *tc128,
                                      int *tc64, int *simt,
                                      size_t *workspace_bytes);
NUMC_API void numc_cuda_gemm_plan_free(NumcCudaGemmPlan *plan);

/* numc_matmul over n independent (a[i], b[i], out[i]) triples in one
 * grouped launch (float32; other dtypes run one numc_matmul per triple).
 * Same validation and host/device semantics as numc_matmul. */
NUMC_API int numc_matmul_grouped(const NumcArray *const *a,
                                 const NumcArray *const *b,
                                 NumcArray *const *out, size_t n);

/* float32 split-BF16 GEMM that allocates nothing.  No counterpart in the
 * reference (numc has no GPU API).  It is for callers that cannot call
 * cudaMalloc when they run a product: services that forbid device
 * allocation after start-up (an allocation can synchronise the device and
 * take milliseconds), and plugins inside a host program whose device memory
 * belongs to that program's own allocator.
 * Scratch is a 64 MiB array compiled into the library (held by every GPU
 * that loads it until exit), so 4*(M+N)*roundup(K,64) bytes plus a few
 * flag words must fit; larger problems are rejected with NUMC_ERR_VALUE.
 * The caller passes device pointers for a, b and out and, optionally, a
 * device word `status` that the call clears and a kernel sets nonzero if
 * it abandoned a bounded wait.  With status == NULL the library's own
 * status word is used instead: it keeps the first failure until
 * numc_cuda_check_status() reads it.  Either way `out` is valid only if
 * the status word reads 0 after the call's work has finished.  The first
 * call on each device looks up the scratch address, which loads the
 * library's device code there if it is not loaded yet; make that first call
 * before any stream capture.  Calls share the scratch: calls that overlap
 * on the GPU race and must be serialised.  Asynchronous on `stream`, like
 * numc_cuda_gemm. */
NUMC_API int numc_cuda_sgemm_split_static(const float *a, const float *b,
                                          float *out, size_t M, size_t K,
                                          size_t N, intptr_t rsa, intptr_t csa,
                                          intptr_t rsb, intptr_t csb,
                                          intptr_t rso, intptr_t cso,
                                          unsigned *status, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* NUMC_CUDA_H */

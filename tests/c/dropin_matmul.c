/*
 * A C program written against numc's public headers (include/numc/), built
 * with a plain C compiler and linked to libnumc_gb300.so: the drop-in check
 * at the C level.  It uses numc's API the way numc programs and numc's own
 * tests do (tests/matmul/test_matmul.c, test_matmul_naive.c): contexts,
 * arrays written through numc_array_data(), numc_matmul,
 * numc_matmul_naive, transposed views and error codes, and numc's
 * kernel-table call (GemmSimdKernel, src/matmul/matmul.c:84-86) on plain
 * host buffers through numc_cuda_gemm_host, as numc's matmul.c would make
 * it with a CUDA backend in its table.
 *
 * Every result is checked against a triple loop in C: integers exactly
 * (wrapping in the storage width, inputs small enough that numc's int8
 * saturation never applies), floats within a bound relative to |A||B|.
 * Prints one summary line; exit status 0 when every check passed.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "numc/numc.h"

static int g_checks = 0, g_fails = 0;

#define CHECK(cond, ...)                                     \
  do {                                                       \
    g_checks++;                                              \
    if (!(cond)) {                                           \
      g_fails++;                                             \
      fprintf(stderr, "FAIL %s:%d: ", __FILE__, __LINE__);   \
      fprintf(stderr, __VA_ARGS__);                          \
      fprintf(stderr, "\n");                                 \
    }                                                        \
  } while (0)

static const char *dt_name(NumcDType dt) {
  static const char *names[] = {"int8", "int16", "int32", "int64", "uint8",
                                "uint16", "uint32", "uint64", "float32", "float64"};
  return names[dt];
}

/* Element i of a buffer of dtype dt, widened (integers exactly). */
static double get_f(const void *p, NumcDType dt, size_t i) {
  switch (dt) {
  case NUMC_DTYPE_FLOAT32: return ((const float *)p)[i];
  case NUMC_DTYPE_FLOAT64: return ((const double *)p)[i];
  default: return 0.0;
  }
}

static int64_t get_i(const void *p, NumcDType dt, size_t i) {
  switch (dt) {
  case NUMC_DTYPE_INT8: return ((const int8_t *)p)[i];
  case NUMC_DTYPE_INT16: return ((const int16_t *)p)[i];
  case NUMC_DTYPE_INT32: return ((const int32_t *)p)[i];
  case NUMC_DTYPE_INT64: return ((const int64_t *)p)[i];
  case NUMC_DTYPE_UINT8: return ((const uint8_t *)p)[i];
  case NUMC_DTYPE_UINT16: return ((const uint16_t *)p)[i];
  case NUMC_DTYPE_UINT32: return ((const uint32_t *)p)[i];
  case NUMC_DTYPE_UINT64: return (int64_t)((const uint64_t *)p)[i];
  default: return 0;
  }
}

static void put(void *p, NumcDType dt, size_t i, int64_t v) {
  switch (dt) {
  case NUMC_DTYPE_INT8: ((int8_t *)p)[i] = (int8_t)v; break;
  case NUMC_DTYPE_INT16: ((int16_t *)p)[i] = (int16_t)v; break;
  case NUMC_DTYPE_INT32: ((int32_t *)p)[i] = (int32_t)v; break;
  case NUMC_DTYPE_INT64: ((int64_t *)p)[i] = v; break;
  case NUMC_DTYPE_UINT8: ((uint8_t *)p)[i] = (uint8_t)v; break;
  case NUMC_DTYPE_UINT16: ((uint16_t *)p)[i] = (uint16_t)v; break;
  case NUMC_DTYPE_UINT32: ((uint32_t *)p)[i] = (uint32_t)v; break;
  case NUMC_DTYPE_UINT64: ((uint64_t *)p)[i] = (uint64_t)v; break;
  case NUMC_DTYPE_FLOAT32: ((float *)p)[i] = (float)v; break;
  case NUMC_DTYPE_FLOAT64: ((double *)p)[i] = (double)v; break;
  }
}

static int is_float(NumcDType dt) {
  return dt == NUMC_DTYPE_FLOAT32 || dt == NUMC_DTYPE_FLOAT64;
}

/* Fill value for operand element i: small integers whose products and sums
 * stay inside every dtype's range for the shapes below (8-bit dtypes get
 * values in {-1, 0, 1} / {0, 1}, so K <= 127 keeps every sum exact). */
static int64_t fill_value(NumcDType dt, size_t i, int which) {
  if (dt == NUMC_DTYPE_INT8) return (int64_t)((i * (which ? 5 : 3) + 1) % 3) - 1;
  if (dt == NUMC_DTYPE_UINT8) return (int64_t)((i * (which ? 5 : 3) + 1) % 2);
  return which ? (int64_t)(i % 5) + 1 : (int64_t)(i % 7) + 1;
}

/* c[i*rsc + j] compared with sum_k a[i*rsa + k*csa] b[k*N + j]. */
static void check_product(const char *what, NumcDType dt, const void *a, const void *b,
                          const void *c, size_t M, size_t K, size_t N, size_t rsa, size_t csa,
                          size_t rsc) {
  int bad = 0;
  double worst = 0.0;
  for (size_t i = 0; i < M && bad < 3; i++)
    for (size_t j = 0; j < N && bad < 3; j++) {
      if (is_float(dt)) {
        double s = 0.0, sa = 0.0;
        for (size_t k = 0; k < K; k++) {
          double p = get_f(a, dt, i * rsa + k * csa) * get_f(b, dt, k * N + j);
          s += p;
          sa += fabs(p);
        }
        const double tol = (dt == NUMC_DTYPE_FLOAT32 ? 1e-6 : 1e-14) * (sa + 1.0);
        const double d = fabs(get_f(c, dt, i * rsc + j) - s);
        if (d > worst) worst = d;
        if (d > tol) bad++;
      } else {
        uint64_t s = 0;
        for (size_t k = 0; k < K; k++)
          s += (uint64_t)get_i(a, dt, i * rsa + k * csa) * (uint64_t)get_i(b, dt, k * N + j);
        int64_t want;
        unsigned char tmp[8];
        put(tmp, dt, 0, (int64_t)s);   /* wrap into the storage width */
        want = get_i(tmp, dt, 0);
        if (get_i(c, dt, i * rsc + j) != want) bad++;
      }
    }
  CHECK(bad == 0, "%s %s %zux%zux%zu: %d wrong outputs (worst float diff %g)", what,
        dt_name(dt), M, K, N, bad, worst);
}

/* numc_matmul and numc_matmul_naive on numc arrays, A optionally a
 * transposed view (numc_array_transpose of a K x M array). */
static void test_api(NumcDType dt, size_t M, size_t K, size_t N, int transposed_a) {
  NumcCtx *ctx = numc_ctx_create();
  CHECK(ctx != NULL, "numc_ctx_create");
  if (!ctx) return;
  size_t sha[2] = {transposed_a ? K : M, transposed_a ? M : K};
  size_t shb[2] = {K, N}, sho[2] = {M, N};
  NumcArray *a = numc_array_zeros(ctx, sha, 2, dt);
  NumcArray *b = numc_array_create(ctx, shb, 2, dt);
  NumcArray *c = numc_array_zeros(ctx, sho, 2, dt);
  NumcArray *cn = numc_array_zeros(ctx, sho, 2, dt);
  CHECK(a && b && c && cn, "array creation %s", dt_name(dt));
  if (!(a && b && c && cn)) {
    numc_ctx_free(ctx);
    return;
  }
  void *da = numc_array_data(a);
  for (size_t i = 0; i < M * K; i++) put(da, dt, i, fill_value(dt, i, 0));
  /* B through numc_array_write from a caller buffer */
  void *hb = malloc(K * N * numc_dtype_size(dt));
  for (size_t i = 0; i < K * N; i++) put(hb, dt, i, fill_value(dt, i, 1));
  numc_array_write(b, hb);
  size_t rsa = K, csa = 1;
  if (transposed_a) {
    size_t axes[2] = {1, 0};
    CHECK(numc_array_transpose(a, axes) == 0, "numc_array_transpose");
    CHECK(!numc_array_is_contiguous(a), "transposed view is not contiguous");
    rsa = 1;
    csa = M;
  }
  int rc = numc_matmul(a, b, c);
  CHECK(rc == 0, "numc_matmul %s returned %d", dt_name(dt), rc);
  check_product(transposed_a ? "numc_matmul(A^T view)" : "numc_matmul", dt, da, hb,
                numc_array_data(c), M, K, N, rsa, csa, N);
  rc = numc_matmul_naive(a, b, cn);
  CHECK(rc == 0, "numc_matmul_naive %s returned %d", dt_name(dt), rc);
  check_product("numc_matmul_naive", dt, da, hb, numc_array_data(cn), M, K, N, rsa, csa, N);
  free(hb);
  numc_ctx_free(ctx);
}

/* A (sequential values) times the identity gives A exactly. */
static void test_identity(NumcDType dt, size_t n) {
  NumcCtx *ctx = numc_ctx_create();
  size_t sh[2] = {n, n};
  NumcArray *a = numc_array_zeros(ctx, sh, 2, dt);
  NumcArray *e = numc_array_zeros(ctx, sh, 2, dt);
  NumcArray *c = numc_array_zeros(ctx, sh, 2, dt);
  void *da = numc_array_data(a), *de = numc_array_data(e);
  const int64_t mod = (dt == NUMC_DTYPE_INT8 || dt == NUMC_DTYPE_UINT8) ? 100 : 100000;
  for (size_t i = 0; i < n * n; i++) put(da, dt, i, (int64_t)(i % mod) + 1);
  for (size_t i = 0; i < n; i++) put(de, dt, i * n + i, 1);
  CHECK(numc_matmul(a, e, c) == 0, "identity numc_matmul %s", dt_name(dt));
  CHECK(memcmp(numc_array_data(c), da, n * n * numc_dtype_size(dt)) == 0,
        "A @ I != A for %s %zux%zu", dt_name(dt), n, n);
  numc_ctx_free(ctx);
}

/* numc's argument checks: the same codes for the same bad calls. */
static void test_errors(void) {
  NumcCtx *ctx = numc_ctx_create();
  size_t s23[2] = {2, 3}, s34[2] = {3, 4}, s24[2] = {2, 4}, s44[2] = {4, 4}, s3[1] = {3};
  NumcArray *a = numc_array_zeros(ctx, s23, 2, NUMC_DTYPE_FLOAT32);
  NumcArray *b = numc_array_zeros(ctx, s34, 2, NUMC_DTYPE_FLOAT32);
  NumcArray *c = numc_array_zeros(ctx, s24, 2, NUMC_DTYPE_FLOAT32);
  NumcArray *bi = numc_array_zeros(ctx, s34, 2, NUMC_DTYPE_INT32);
  NumcArray *wrong = numc_array_zeros(ctx, s44, 2, NUMC_DTYPE_FLOAT32);
  NumcArray *vec = numc_array_zeros(ctx, s3, 1, NUMC_DTYPE_FLOAT32);
  CHECK(numc_matmul(NULL, b, c) == NUMC_ERR_NULL, "NULL a");
  CHECK(numc_matmul(a, b, NULL) == NUMC_ERR_NULL, "NULL out");
  CHECK(numc_matmul(a, bi, c) == NUMC_ERR_TYPE, "dtype mismatch");
  CHECK(numc_matmul(a, wrong, c) == NUMC_ERR_SHAPE, "inner dimension mismatch");
  CHECK(numc_matmul(a, b, wrong) == NUMC_ERR_SHAPE, "output shape mismatch");
  CHECK(numc_matmul(vec, b, c) == NUMC_ERR_SHAPE, "1-D operand");
  CHECK(numc_matmul_naive(a, bi, c) == NUMC_ERR_TYPE, "naive dtype mismatch");
  NumcError err = numc_get_error();
  CHECK(err.code == NUMC_ERR_TYPE, "numc_get_error keeps the last code");
  CHECK(numc_matmul(a, b, c) == 0, "a valid call after errors");
  numc_ctx_free(ctx);
}

/* numc's kernel table with this library in it: one GemmSimdKernel-shaped
 * function per dtype forwarding to numc_cuda_gemm_host, called on malloc'd
 * host buffers with numc's element strides (A read column-major here). */
typedef int (*KernelEntry)(const void *a, const void *b, void *out, size_t M, size_t K,
                           size_t N, intptr_t rsa, intptr_t csa, intptr_t rsb, intptr_t rso);
#define CUDA_ENTRY(NAME, DT)                                                                 \
  static int NAME(const void *a, const void *b, void *out, size_t M, size_t K, size_t N,  \
                  intptr_t rsa, intptr_t csa, intptr_t rsb, intptr_t rso) {               \
    return numc_cuda_gemm_host(DT, a, b, out, M, K, N, rsa, csa, rsb, rso);               \
  }
CUDA_ENTRY(gemm_cuda_i8, NUMC_DTYPE_INT8)
CUDA_ENTRY(gemm_cuda_i16, NUMC_DTYPE_INT16)
CUDA_ENTRY(gemm_cuda_i32, NUMC_DTYPE_INT32)
CUDA_ENTRY(gemm_cuda_i64, NUMC_DTYPE_INT64)
CUDA_ENTRY(gemm_cuda_u8, NUMC_DTYPE_UINT8)
CUDA_ENTRY(gemm_cuda_u16, NUMC_DTYPE_UINT16)
CUDA_ENTRY(gemm_cuda_u32, NUMC_DTYPE_UINT32)
CUDA_ENTRY(gemm_cuda_u64, NUMC_DTYPE_UINT64)
CUDA_ENTRY(gemm_cuda_f32, NUMC_DTYPE_FLOAT32)
CUDA_ENTRY(gemm_cuda_f64, NUMC_DTYPE_FLOAT64)
static const KernelEntry kernel_table[NUMC_DTYPE_COUNT] = {
    gemm_cuda_i8,  gemm_cuda_i16, gemm_cuda_i32, gemm_cuda_i64, gemm_cuda_u8,
    gemm_cuda_u16, gemm_cuda_u32, gemm_cuda_u64, gemm_cuda_f32, gemm_cuda_f64};

static void test_kernel_table(NumcDType dt, size_t M, size_t K, size_t N) {
  const size_t es = numc_dtype_size(dt);
  void *a = malloc(M * K * es), *b = malloc(K * N * es), *c = calloc(M * N + 1, es);
  for (size_t i = 0; i < M * K; i++) put(a, dt, i, fill_value(dt, i, 0));
  for (size_t i = 0; i < K * N; i++) put(b, dt, i, fill_value(dt, i, 1));
  /* A stored K x M, read as M x K: rsa = 1, csa = M */
  int rc = kernel_table[dt](a, b, c, M, K, N, 1, (intptr_t)M, (intptr_t)N, (intptr_t)N);
  CHECK(rc == 0, "numc_cuda_gemm_host %s returned %d", dt_name(dt), rc);
  check_product("numc_cuda_gemm_host", dt, a, b, c, M, K, N, 1, M, N);
  free(a);
  free(b);
  free(c);
}

int main(void) {
  static const size_t shapes[][3] = {{1, 64, 32},   {32, 64, 1},   {7, 7, 7},
                                     {37, 41, 43},  {97, 101, 103}, {144, 127, 64},
                                     {128, 96, 300}, {260, 120, 270}};
  const size_t nshapes = sizeof shapes / sizeof shapes[0];
  for (int dt = 0; dt < NUMC_DTYPE_COUNT; dt++) {
    for (size_t s = 0; s < nshapes; s++)
      test_api((NumcDType)dt, shapes[s][0], shapes[s][1], shapes[s][2], 0);
    test_api((NumcDType)dt, 70, 90, 50, 1);
    test_identity((NumcDType)dt, 64);
    test_kernel_table((NumcDType)dt, 96, 120, 80);
    test_kernel_table((NumcDType)dt, 5, 3, 4);
  }
  test_errors();
  printf("dropin_matmul: %d checks, %d failures\n", g_checks, g_fails);
  return g_fails ? 1 : 0;
}

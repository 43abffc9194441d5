/*
 * numc_oracle_micro.c — register-tile micro-kernels of the oracle's float
 * GEMM (numc_oracle.c).
 *
 * TEST INFRASTRUCTURE ONLY: part of the checker and the timed CPU baseline,
 * never linked into the product library.
 *
 * Each kernel runs one ORACLE_MR x NR tile over one K block: acc = C, then
 * for k in order acc = a[k] * b[k] + acc as ONE fused multiply-add per
 * output, then C = acc — numc's per-output FMA chain (its micro-kernels,
 * e.g. src/intrinsics/gemm_ukernel_f32_6x16_avx2.S:76-105, keep one
 * accumulator per output the same way).  The file is compiled with
 * -ffp-contract=fast so that GCC turns every `av * b + acc` on the vector
 * types below into a vector FMA instruction (AVX2+FMA on x86-64, NEON fmla
 * on aarch64); the oracle tests compare the results with numc's own outputs
 * bit for bit, which would catch an uncontracted add.  This file holds no
 * other arithmetic.
 */
#include <string.h>

#include "numc_oracle_micro.h"

typedef float vf __attribute__((vector_size(ORACLE_VEC_BYTES)));
typedef double vd __attribute__((vector_size(ORACLE_VEC_BYTES)));
enum { VF = ORACLE_VEC_BYTES / 4, VD = ORACLE_VEC_BYTES / 8 };

#define DEFINE_MICRO(NAME, T, V, W, NR)                                        \
  void NAME(const T *restrict a, int64_t lda, const T *restrict bs,           \
            T *restrict c, int64_t ldc, int64_t kc) {                          \
    V acc[ORACLE_MR][ORACLE_NVEC];                                             \
    for (int r = 0; r < ORACLE_MR; r++)                                        \
      for (int v = 0; v < ORACLE_NVEC; v++)                                    \
        memcpy(&acc[r][v], c + r * ldc + W * v, sizeof(V));                    \
    for (int64_t k = 0; k < kc; k++) {                                         \
      V b[ORACLE_NVEC];                                                        \
      for (int v = 0; v < ORACLE_NVEC; v++)                                    \
        memcpy(&b[v], bs + k * NR + W * v, sizeof(V));                         \
      for (int r = 0; r < ORACLE_MR; r++) {                                    \
        const T x = a[r * lda + k]; /* scalar operand: broadcast */           \
        for (int v = 0; v < ORACLE_NVEC; v++) acc[r][v] = x * b[v] + acc[r][v]; \
      }                                                                        \
    }                                                                          \
    for (int r = 0; r < ORACLE_MR; r++)                                        \
      for (int v = 0; v < ORACLE_NVEC; v++)                                    \
        memcpy(c + r * ldc + W * v, &acc[r][v], sizeof(V));                    \
  }

DEFINE_MICRO(oracle_micro_f32, float, vf, VF, ORACLE_NR_F32)
DEFINE_MICRO(oracle_micro_f64, double, vd, VD, ORACLE_NR_F64)

/*
 * numc_oracle_micro.c — register-tile micro-kernels of the oracle's float
 * GEMM (numc_oracle.c).
 *
 * TEST INFRASTRUCTURE ONLY: part of the checker and the timed CPU baseline,
 * never linked into the product library.
 *
 * Each kernel runs one MR x NR tile over one K block: acc = C, then for k in
 * order acc = a[k] * b[k] + acc as ONE fused multiply-add per output, then
 * C = acc — numc's per-output FMA chain (src/intrinsics/gemm_ukernel_f32_
 * 6x16_avx2.S:76-105 keeps the same 6x16 accumulator shape).  The file is
 * compiled with -ffp-contract=fast so that GCC turns every `av * b + acc`
 * on the vector types below into a vector FMA instruction (AVX2+FMA on
 * x86-64, NEON fmla on aarch64); the oracle tests compare the results with
 * numc's own outputs bit for bit, which would catch an uncontracted add.
 * This file holds no other arithmetic.
 */
#include <stdint.h>
#include <string.h>

typedef float vf8 __attribute__((vector_size(32)));
typedef double vd4 __attribute__((vector_size(32)));

/* 6 x 16 float32 tile. */
void oracle_micro_f32(const float *restrict a, int64_t lda,
                      const float *restrict bs, float *restrict c,
                      int64_t ldc, int64_t kc) {
  vf8 acc[6][2];
  for (int r = 0; r < 6; r++) {
    memcpy(&acc[r][0], c + r * ldc, 32);
    memcpy(&acc[r][1], c + r * ldc + 8, 32);
  }
  for (int64_t k = 0; k < kc; k++) {
    vf8 b0, b1;
    memcpy(&b0, bs + k * 16, 32);
    memcpy(&b1, bs + k * 16 + 8, 32);
    for (int r = 0; r < 6; r++) {
      const float x = a[r * lda + k];
      const vf8 av = {x, x, x, x, x, x, x, x};
      acc[r][0] = av * b0 + acc[r][0];
      acc[r][1] = av * b1 + acc[r][1];
    }
  }
  for (int r = 0; r < 6; r++) {
    memcpy(c + r * ldc, &acc[r][0], 32);
    memcpy(c + r * ldc + 8, &acc[r][1], 32);
  }
}

/* 6 x 8 float64 tile. */
void oracle_micro_f64(const double *restrict a, int64_t lda,
                      const double *restrict bs, double *restrict c,
                      int64_t ldc, int64_t kc) {
  vd4 acc[6][2];
  for (int r = 0; r < 6; r++) {
    memcpy(&acc[r][0], c + r * ldc, 32);
    memcpy(&acc[r][1], c + r * ldc + 4, 32);
  }
  for (int64_t k = 0; k < kc; k++) {
    vd4 b0, b1;
    memcpy(&b0, bs + k * 8, 32);
    memcpy(&b1, bs + k * 8 + 4, 32);
    for (int r = 0; r < 6; r++) {
      const double x = a[r * lda + k];
      const vd4 av = {x, x, x, x};
      acc[r][0] = av * b0 + acc[r][0];
      acc[r][1] = av * b1 + acc[r][1];
    }
  }
  for (int r = 0; r < 6; r++) {
    memcpy(c + r * ldc, &acc[r][0], 32);
    memcpy(c + r * ldc + 4, &acc[r][1], 32);
  }
}

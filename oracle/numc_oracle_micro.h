/*
 * numc_oracle_micro.h — register-tile shapes of the oracle's float GEMM
 * micro-kernels (TEST INFRASTRUCTURE ONLY).
 *
 * Each shape fills the host's vector registers: on aarch64 (32 x 128-bit
 * NEON registers) 8 rows x 3 vectors, on other hosts (16 x 256-bit AVX2
 * registers) 6 rows x 2 vectors.  The shape only changes which outputs a
 * call computes together, never the arithmetic of an output.
 */
#ifndef NUMC_ORACLE_MICRO_H
#define NUMC_ORACLE_MICRO_H
#include <stdint.h>

#if defined(__aarch64__)
#define ORACLE_VEC_BYTES 16
#define ORACLE_MR 8
#define ORACLE_NVEC 3
#else
#define ORACLE_VEC_BYTES 32
#define ORACLE_MR 6
#define ORACLE_NVEC 2
#endif
#define ORACLE_NR_F32 (ORACLE_NVEC * ORACLE_VEC_BYTES / 4)
#define ORACLE_NR_F64 (ORACLE_NVEC * ORACLE_VEC_BYTES / 8)

void oracle_micro_f32(const float *a, int64_t lda, const float *bs, float *c, int64_t ldc,
                      int64_t kc);
void oracle_micro_f64(const double *a, int64_t lda, const double *bs, double *c,
                      int64_t ldc, int64_t kc);
#endif

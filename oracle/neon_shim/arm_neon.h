/*
 * arm_neon.h — a scalar model of the AArch64 NEON intrinsics that numc's
 * GEMM kernels use (src/intrinsics/gemm_neon.h, gemmsup_neon.h).
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile.ref puts this directory on the
 * include path when it compiles numc's unmodified src/matmul/matmul.c as its
 * NEON build on an x86-64 host (no AArch64 compiler is available there), so
 * that the golden fixtures of numc's aarch64 results come from numc's own
 * NEON source.  The product library never includes it.
 *
 * Each intrinsic is written from its per-lane definition in Arm's ACLE
 * (Arm C Language Extensions) specification:
 *   - vfmaq_* / vfmaq_laneq_*: a + b * c with one rounding (C99 fma/fmaf),
 *     exactly the AArch64 FMLA instruction;
 *   - vmlaq_* on integer lanes: a + b * c modulo 2^bits (unsigned
 *     arithmetic, no undefined signed overflow);
 *   - vqmovn_*: narrowing with saturation to the destination lane's range
 *     (unsigned sources saturate to the unsigned maximum);
 *   - vmovl_*: widening with sign or zero extension;
 *   - vzip1q/vzip2q, vtrn1q/vtrn2q, vget_low/high, vcombine, vdup, vld1,
 *     vst1, vgetq_lane, vaddq: lane moves, loads, stores and lane adds.
 * Vector types are structs of lane arrays: numc's kernels only pass them by
 * value and through these intrinsics, never through C operators.
 */
#ifndef NUMC_ORACLE_NEON_SHIM_H
#define NUMC_ORACLE_NEON_SHIM_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#define NS_ static inline

typedef struct { float v[4]; } float32x4_t;
typedef struct { float v[2]; } float32x2_t;
typedef struct { double v[2]; } float64x2_t;
typedef struct { int32_t v[4]; } int32x4_t;
typedef struct { uint32_t v[4]; } uint32x4_t;
typedef struct { int16_t v[8]; } int16x8_t;
typedef struct { uint16_t v[8]; } uint16x8_t;
typedef struct { int16_t v[4]; } int16x4_t;
typedef struct { uint16_t v[4]; } uint16x4_t;
typedef struct { int8_t v[8]; } int8x8_t;
typedef struct { uint8_t v[8]; } uint8x8_t;
typedef struct { int64_t v[2]; } int64x2_t;
typedef struct { int64_t v[1]; } int64x1_t;

/* ---- loads, stores, duplicates -------------------------------------------- */
#define NS_LDST(T, E, N, LD, ST)                                   \
  NS_ T LD(const E *p) { T r; memcpy(r.v, p, sizeof(E) * (N)); return r; } \
  NS_ void ST(E *p, T x) { memcpy(p, x.v, sizeof(E) * (N)); }
NS_LDST(float32x4_t, float, 4, vld1q_f32, vst1q_f32)
NS_LDST(float64x2_t, double, 2, vld1q_f64, vst1q_f64)
NS_LDST(int32x4_t, int32_t, 4, vld1q_s32, vst1q_s32)
NS_LDST(int16x8_t, int16_t, 8, vld1q_s16, vst1q_s16)
NS_LDST(int64x2_t, int64_t, 2, vld1q_s64, vst1q_s64)
NS_LDST(int8x8_t, int8_t, 8, vld1_s8, vst1_s8)
NS_LDST(uint8x8_t, uint8_t, 8, vld1_u8, vst1_u8)
#undef NS_LDST

#define NS_DUP(T, E, N, NAME)                                      \
  NS_ T NAME(E x) { T r; for (int i = 0; i < (N); i++) r.v[i] = x; return r; }
NS_DUP(float32x4_t, float, 4, vdupq_n_f32)
NS_DUP(float64x2_t, double, 2, vdupq_n_f64)
NS_DUP(int32x4_t, int32_t, 4, vdupq_n_s32)
NS_DUP(uint32x4_t, uint32_t, 4, vdupq_n_u32)
NS_DUP(int16x8_t, int16_t, 8, vdupq_n_s16)
NS_DUP(int64x2_t, int64_t, 2, vdupq_n_s64)
NS_DUP(int64x1_t, int64_t, 1, vdup_n_s64)
#undef NS_DUP

/* ---- fused multiply-add (one rounding per lane) ---------------------------- */
NS_ float32x4_t vfmaq_f32(float32x4_t a, float32x4_t b, float32x4_t c) {
  for (int i = 0; i < 4; i++) a.v[i] = fmaf(b.v[i], c.v[i], a.v[i]);
  return a;
}
NS_ float64x2_t vfmaq_f64(float64x2_t a, float64x2_t b, float64x2_t c) {
  for (int i = 0; i < 2; i++) a.v[i] = fma(b.v[i], c.v[i], a.v[i]);
  return a;
}
NS_ float32x4_t vfmaq_laneq_f32(float32x4_t a, float32x4_t b, float32x4_t c, int lane) {
  for (int i = 0; i < 4; i++) a.v[i] = fmaf(b.v[i], c.v[lane], a.v[i]);
  return a;
}
NS_ float64x2_t vfmaq_laneq_f64(float64x2_t a, float64x2_t b, float64x2_t c, int lane) {
  for (int i = 0; i < 2; i++) a.v[i] = fma(b.v[i], c.v[lane], a.v[i]);
  return a;
}

/* ---- integer multiply-accumulate, modulo 2^bits ----------------------------- */
NS_ int32x4_t vmlaq_s32(int32x4_t a, int32x4_t b, int32x4_t c) {
  for (int i = 0; i < 4; i++)
    a.v[i] = (int32_t)((uint32_t)a.v[i] + (uint32_t)b.v[i] * (uint32_t)c.v[i]);
  return a;
}
NS_ uint32x4_t vmlaq_u32(uint32x4_t a, uint32x4_t b, uint32x4_t c) {
  for (int i = 0; i < 4; i++) a.v[i] = a.v[i] + b.v[i] * c.v[i];
  return a;
}
NS_ int16x8_t vmlaq_s16(int16x8_t a, int16x8_t b, int16x8_t c) {
  for (int i = 0; i < 8; i++)
    a.v[i] = (int16_t)(uint16_t)((uint32_t)(uint16_t)a.v[i] +
                                 (uint32_t)(uint16_t)b.v[i] * (uint32_t)(uint16_t)c.v[i]);
  return a;
}
NS_ int64x2_t vaddq_s64(int64x2_t a, int64x2_t b) {
  for (int i = 0; i < 2; i++) a.v[i] = (int64_t)((uint64_t)a.v[i] + (uint64_t)b.v[i]);
  return a;
}

/* ---- lane moves ------------------------------------------------------------- */
NS_ float32x2_t vget_low_f32(float32x4_t a) { float32x2_t r = {{a.v[0], a.v[1]}}; return r; }
NS_ float32x2_t vget_high_f32(float32x4_t a) { float32x2_t r = {{a.v[2], a.v[3]}}; return r; }
NS_ float32x4_t vcombine_f32(float32x2_t lo, float32x2_t hi) {
  float32x4_t r = {{lo.v[0], lo.v[1], hi.v[0], hi.v[1]}};
  return r;
}
NS_ float32x4_t vzip1q_f32(float32x4_t a, float32x4_t b) {
  float32x4_t r = {{a.v[0], b.v[0], a.v[1], b.v[1]}};
  return r;
}
NS_ float32x4_t vzip2q_f32(float32x4_t a, float32x4_t b) {
  float32x4_t r = {{a.v[2], b.v[2], a.v[3], b.v[3]}};
  return r;
}
NS_ float64x2_t vtrn1q_f64(float64x2_t a, float64x2_t b) {
  float64x2_t r = {{a.v[0], b.v[0]}};
  return r;
}
NS_ float64x2_t vtrn2q_f64(float64x2_t a, float64x2_t b) {
  float64x2_t r = {{a.v[1], b.v[1]}};
  return r;
}
#define vgetq_lane_s64(a, lane) ((a).v[(lane)])
NS_ int64x2_t vcombine_s64(int64x1_t lo, int64x1_t hi) {
  int64x2_t r = {{lo.v[0], hi.v[0]}};
  return r;
}
NS_ int16x4_t vget_low_s16(int16x8_t a) {
  int16x4_t r; for (int i = 0; i < 4; i++) r.v[i] = a.v[i]; return r;
}
NS_ int16x4_t vget_high_s16(int16x8_t a) {
  int16x4_t r; for (int i = 0; i < 4; i++) r.v[i] = a.v[4 + i]; return r;
}
NS_ uint16x4_t vget_low_u16(uint16x8_t a) {
  uint16x4_t r; for (int i = 0; i < 4; i++) r.v[i] = a.v[i]; return r;
}
NS_ uint16x4_t vget_high_u16(uint16x8_t a) {
  uint16x4_t r; for (int i = 0; i < 4; i++) r.v[i] = a.v[4 + i]; return r;
}
NS_ int16x8_t vcombine_s16(int16x4_t lo, int16x4_t hi) {
  int16x8_t r;
  for (int i = 0; i < 4; i++) { r.v[i] = lo.v[i]; r.v[4 + i] = hi.v[i]; }
  return r;
}
NS_ uint16x8_t vcombine_u16(uint16x4_t lo, uint16x4_t hi) {
  uint16x8_t r;
  for (int i = 0; i < 4; i++) { r.v[i] = lo.v[i]; r.v[4 + i] = hi.v[i]; }
  return r;
}

/* ---- widening and saturating narrowing ----------------------------------------- */
NS_ int16x8_t vmovl_s8(int8x8_t a) {
  int16x8_t r; for (int i = 0; i < 8; i++) r.v[i] = a.v[i]; return r;
}
NS_ uint16x8_t vmovl_u8(uint8x8_t a) {
  uint16x8_t r; for (int i = 0; i < 8; i++) r.v[i] = a.v[i]; return r;
}
NS_ int32x4_t vmovl_s16(int16x4_t a) {
  int32x4_t r; for (int i = 0; i < 4; i++) r.v[i] = a.v[i]; return r;
}
NS_ uint32x4_t vmovl_u16(uint16x4_t a) {
  uint32x4_t r; for (int i = 0; i < 4; i++) r.v[i] = a.v[i]; return r;
}
NS_ int16x4_t vqmovn_s32(int32x4_t a) {
  int16x4_t r;
  for (int i = 0; i < 4; i++)
    r.v[i] = (int16_t)(a.v[i] < -32768 ? -32768 : (a.v[i] > 32767 ? 32767 : a.v[i]));
  return r;
}
NS_ uint16x4_t vqmovn_u32(uint32x4_t a) {
  uint16x4_t r;
  for (int i = 0; i < 4; i++) r.v[i] = (uint16_t)(a.v[i] > 65535u ? 65535u : a.v[i]);
  return r;
}
NS_ int8x8_t vqmovn_s16(int16x8_t a) {
  int8x8_t r;
  for (int i = 0; i < 8; i++)
    r.v[i] = (int8_t)(a.v[i] < -128 ? -128 : (a.v[i] > 127 ? 127 : a.v[i]));
  return r;
}
NS_ uint8x8_t vqmovn_u16(uint16x8_t a) {
  uint8x8_t r;
  for (int i = 0; i < 8; i++) r.v[i] = (uint8_t)(a.v[i] > 255u ? 255u : a.v[i]);
  return r;
}

#undef NS_
#endif /* NUMC_ORACLE_NEON_SHIM_H */

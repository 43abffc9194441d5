/*
 * numc_oracle.c — CPU restatement of numc's matmul arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA backend
 * and the timed CPU baseline; the product library never links, loads or calls
 * it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use it.
 *
 * What it restates (reference paths relative to the numc source tree):
 *
 *  - float32 / float64: an output in a full register tile is a sequential
 *    fused-multiply-add chain over k = 0..K-1 starting from +0: numc's
 *    micro-kernels keep one FMA accumulator per output and reload C between
 *    K blocks (src/intrinsics/gemm_ukernel_f32_6x16_avx2.S:76-105,
 *    src/intrinsics/gemm_avx2.h:852-950).  Remainder tiles follow their own
 *    arithmetic, restated in DEFINE_FLOAT_EDGES below for the x86 AVX2
 *    profile; with that, results equal the compiled reference bit for bit.
 *
 *  - int16/uint16/int32/uint32/int64/uint64: the exact sum reduced modulo
 *    2^bits.  numc wraps in the storage width on every path
 *    (gemm_avx2.h:1841,1986,2312,2456,2550-2591; src/matmul/kernel.h:18-62),
 *    so the result does not depend on summation order.
 *
 *  - int8/uint8: numc's results depend on the host ISA.  Three profiles:
 *
 *    ORACLE_I8_X86_AVX2 (the x86-64 AVX2 build):
 *      if M*K*N <= 192^3 the unpacked path stores the int32 sum truncated to
 *      8 bits (src/matmul/matmul.c:241-256, gemmsup_avx2.h:744-756,865-876).
 *      Otherwise the packed path (gemm_avx2.h:2741-2880, 2983-3125) blocks
 *      K by 512, M by 72 (MR 6) and N by 4080 (NR 16).  With P_b the exact
 *      partial sum of K block b and (i, j) inside a full 6x16 tile:
 *         d = sat(d + P_b), d = 0 before block 0 (the assembly micro-kernel
 *         reloads the stored byte sign/zero-extended and stores through
 *         packssdw/packsswb, or packusdw/packuswb for uint8);
 *      inside a remainder tile:
 *         d = sat(P_0), then d = wrap8(d + sat(P_b)) for b >= 1.
 *      int8 sat clamps to [-128, 127].  uint8 sat is two unsigned packs:
 *      clamp to [0, 65535], reinterpret as int16, clamp to [0, 255] — so
 *      values 256..32767 give 255 and values >= 32768 give 0.
 *
 *    ORACLE_I8_ARM_NEON (the aarch64 NEON build, gemm_neon.h:1440-1630):
 *      no K blocking and no unpacked integer path; M blocked by 72 (MR 6),
 *      N by NR 8 from column 0.  Full 6x8 tiles narrow the wrapped int32 sum
 *      with vqmovn twice (int8: clamp to [-128,127]; uint8: min(u32, 255));
 *      remainder tiles truncate to 8 bits.  Restated from source only.
 *
 *    ORACLE_I8_X86_AVX512 (the x86-64 build on an AVX-512 host, numc's
 *      default -march=native there): M*K*N <= 192^3 keeps AVX2's unpacked
 *      path (truncation; src/matmul/matmul.c:210-226 gives AVX-512 no integer
 *      gemmsup of its own); larger products use gemm_i8_avx512 /
 *      gemm_u8_avx512 (src/intrinsics/gemm_avx512.h:1263-1414): no K
 *      blocking, M blocked by 240 (MR 12) and N by NR 16 from column 0.
 *      Full 12x16 tiles narrow the wrapped int32 sum once with
 *      _mm512_cvtsepi32_epi8 (int8: clamp to [-128,127]) or
 *      _mm512_cvtusepi32_epi8 (uint8: the lane read as unsigned, min(u32,
 *      255)); remainder tiles truncate to 8 bits.
 *
 *    ORACLE_I8_WRAP (numc_matmul_naive, src/matmul/kernel.h:35-62): the sum
 *      truncated to 8 bits.
 *
 *    ORACLE_X86_PACKED: numc's x86 packed kernels called directly, as
 *      numc_dot's GEMM branch does (src/reduction/dot.c:392-398 through
 *      the gemm_*_avx2 wrappers at dot.c:159-231): the x86 rules without the
 *      192^3 unpacked threshold, for every dtype.
 *
 *  - Naive float32/float64 (profile ORACLE_I8_WRAP, numc_matmul_naive,
 *    src/matmul/kernel.h:18-33, and numc_dot's strided kernels,
 *    src/reduction/dot.c:42-72): per output `acc += a * b` in k order from 0
 *    in ISO C without contraction — each product rounded, then each sum.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum {
  DT_I8, DT_I16, DT_I32, DT_I64, DT_U8, DT_U16, DT_U32, DT_U64, DT_F32, DT_F64
};
/* Arithmetic profiles: which numc build's results to reproduce.  They
 * differ for int8/uint8 (store rules) and, in the last bits, for the
 * remainder tiles of float32/float64. */
enum { ORACLE_I8_X86_AVX2 = 0, ORACLE_I8_ARM_NEON = 1, ORACLE_I8_WRAP = 2,
       ORACLE_X86_PACKED = 3, ORACLE_I8_X86_AVX512 = 4 };

static const size_t k_elem[] = {1, 2, 4, 8, 1, 2, 4, 8, 4, 8};

#define MIN(a, b) ((a) < (b) ? (a) : (b))

/* Gather a strided matrix into a dense row-major buffer. */
static void *gather(const void *src, int64_t rows, int64_t cols, int64_t rs,
                    int64_t cs, size_t es) {
  size_t bytes = (size_t)(rows * cols) * es;
  char *dst = (char *)malloc(bytes ? bytes : 1);
  if (!dst) return NULL;
  const char *s = (const char *)src;
  for (int64_t r = 0; r < rows; r++)
    for (int64_t c = 0; c < cols; c++)
      memcpy(dst + (size_t)(r * cols + c) * es,
             s + (size_t)(r * rs + c * cs) * es, es);
  return dst;
}

static void scatter(void *dstv, const void *src, int64_t rows, int64_t cols,
                    int64_t rs, int64_t cs, size_t es) {
  char *d = (char *)dstv;
  const char *s = (const char *)src;
  for (int64_t r = 0; r < rows; r++)
    for (int64_t c = 0; c < cols; c++)
      memcpy(d + (size_t)(r * rs + c * cs) * es,
             s + (size_t)(r * cols + c) * es, es);
}

/* Row block, K block and column block of the cache-blocked loops below.
 * They only change the loop order across outputs, never the k order
 * within one output. */
#define RB 32
#define KB 256
#define JB 128

/* Float kernels: packed, register-blocked GEMM whose arithmetic is exactly
 * numc's full-tile arithmetic — one FMA chain per output in k order from
 * +0 — because each output's accumulator is reloaded from C between K
 * blocks, never split.  B is packed per (column panel, K block) into
 * NR-wide strips shared by all threads; each thread runs MR x NR register
 * tiles over its rows. */
#define FKC 256
#define FNC 512

/* Register-tile micro-kernels (numc_oracle_micro.c, compiled so that each
 * vector multiply-add is one fused multiply-add). */
#include "numc_oracle_micro.h"

#define DEFINE_FLOAT_KERNEL(NAME, T, MICRO, MR_, NR_)                         \
  static void NAME(const T *a, const T *b, T *c, int64_t M, int64_t K,       \
                   int64_t N) {                                               \
    enum { MR = MR_, NR = NR_ };                                              \
    T *bp = (T *)malloc(sizeof(T) * FKC * (FNC + NR));                        \
    for (int64_t i = 0; i < M * N; i++) c[i] = (T)0;                          \
    for (int64_t jc = 0; jc < N; jc += FNC) {                                 \
      const int64_t nc = MIN(FNC, N - jc);                                    \
      const int64_t nstrips = (nc + NR - 1) / NR;                             \
      for (int64_t pc = 0; pc < K; pc += FKC) {                               \
        const int64_t kc = MIN(FKC, K - pc);                                  \
        _Pragma("omp parallel for schedule(static)")                          \
        for (int64_t js = 0; js < nstrips; js++)                              \
          for (int64_t k = 0; k < kc; k++)                                    \
            for (int j = 0; j < NR; j++) {                                    \
              const int64_t col = jc + js * NR + j;                           \
              bp[(js * kc + k) * NR + j] =                                    \
                  col < jc + nc ? b[(pc + k) * N + col] : (T)0;               \
            }                                                                 \
        /* (row block, column strip) tiles shared out in contiguous runs,  \
         * so a few row blocks still keep every thread busy. */              \
        const int64_t nib = (M + MR - 1) / MR;                                \
        _Pragma("omp parallel for schedule(static)")                          \
        for (int64_t t = 0; t < nib * nstrips; t++) {                         \
          const int64_t ib = t / nstrips, js = t % nstrips;                   \
          const int64_t i0 = ib * MR;                                         \
          const int mr = (int)MIN(MR, M - i0);                                \
          T ta[MR * FKC], tc[MR * NR];                                        \
          {                                                                   \
            const int64_t j0 = jc + js * NR;                                  \
            /* the last strip of a panel stops at the panel's end */          \
            const int nr = (int)MIN(NR, jc + nc - j0);                        \
            const T *bs = bp + js * kc * NR;                                  \
            if (mr == MR && nr == NR) {                                       \
              MICRO(a + i0 * K + pc, K, bs, c + i0 * N + j0, N, kc);          \
              continue;                                                       \
            }                                                                 \
            /* Ragged edge: run the same micro-kernel on zero-padded copies   \
             * (padding never reaches a stored output). */                    \
            for (int r = 0; r < MR; r++) {                                    \
              for (int64_t k = 0; k < kc; k++)                                \
                ta[r * kc + k] = r < mr ? a[(i0 + r) * K + pc + k] : (T)0;    \
              for (int j = 0; j < NR; j++)                                    \
                tc[r * NR + j] = (r < mr && j < nr) ? c[(i0 + r) * N + j0 + j] : (T)0; \
            }                                                                 \
            MICRO(ta, kc, bs, tc, NR, kc);                             \
            for (int r = 0; r < mr; r++)                                      \
              for (int j = 0; j < nr; j++)                                    \
                c[(i0 + r) * N + j0 + j] = tc[r * NR + j];                    \
          }                                                                   \
        }                                                                     \
      }                                                                       \
    }                                                                         \
    free(bp);                                                                 \
  }

DEFINE_FLOAT_KERNEL(kern_f32, float, oracle_micro_f32, ORACLE_MR, ORACLE_NR_F32)
DEFINE_FLOAT_KERNEL(kern_f64, double, oracle_micro_f64, ORACLE_MR, ORACLE_NR_F64)

/* Outputs of numc's float kernels that are not a plain FMA chain.
 *
 * Unpacked path (M*K*N <= THR): 6 x NR tiles from the origin; inside a
 * remainder tile the first (nr / VW) * VW columns use vector FMA and the
 * rest scalar `c += a * b`, which the reference's ISO C build (-std=c2x, no
 * FP contraction) rounds twice.  x86 AVX2: gemmsup_avx2.h:97-147 and
 * 221-270 (NR 16 / 8, VW 8 / 4); aarch64 NEON: gemmsup_neon.h:28-155 and
 * 163-300 (NR 12 / 8, VW 4 / 2).
 *
 * Packed path: a remainder tile computes each KC=256 block as an FMA chain
 * from zero and adds it to the stored value; full tiles reload C and keep
 * one chain.  The tile grid is MC x MR rows, NR columns inside NC-column
 * panels.  x86 AVX2 (gemm_avx2.h:852-950 f32, 1377-1475 f64): MC 144 / 72,
 * MR 6, NR 16 / 8, NC 4080.  aarch64 NEON (gemm_neon.h:610-740 f32,
 * 951-1080 f64): MC 128 / 96, MR 8 / 6, NR 12 / 8, NC 4080 / 2048.
 */
#define DEFINE_FLOAT_EDGES(NAME, T, FMA, THR, NR, VW, MC, MR, NC)             \
  /* Packed-path remainder output (i, j): per-KC chains summed in order. */   \
  static T NAME##_packed_one(const T *a, const T *b, int64_t i, int64_t j,   \
                             int64_t K, int64_t N) {                          \
    T d = (T)0;                                                               \
    for (int64_t pc = 0; pc < K; pc += 256) {                                 \
      int64_t pe = MIN(pc + 256, K);                                          \
      T t = (T)0;                                                             \
      for (int64_t k = pc; k < pe; k++) t = FMA(a[i * K + k], b[k * N + j], t); \
      d = (pc == 0) ? t : d + t;                                              \
    }                                                                         \
    return d;                                                                 \
  }                                                                           \
  static void NAME(const T *a, const T *b, T *c, int64_t M, int64_t K,       \
                   int64_t N, int force_packed) {                             \
    int packed = force_packed || (uint64_t)M * (uint64_t)K * (uint64_t)N > (THR); \
    if (packed) {                                                             \
      /* Rows of a remainder row tile: every column is a remainder output;   \
       * computed a whole row at a time (same arithmetic per output, B read  \
       * along rows).  Other rows: only the tail columns of each panel. */   \
      _Pragma("omp parallel")                                                 \
      {                                                                       \
        T *t = (T *)malloc(sizeof(T) * (size_t)(2 * N + 1)), *d = t + N;      \
        _Pragma("omp for schedule(dynamic, 1)")                               \
        for (int64_t i = 0; i < M; i++) {                                     \
          int64_t ic = (i / (MC)) * (MC), mc = MIN((MC), M - ic);             \
          int64_t ir = ((i - ic) / (MR)) * (MR), mr = MIN((MR), mc - ir);     \
          if (mr < (MR)) {                                                    \
            for (int64_t pc = 0; pc < K; pc += 256) {                         \
              int64_t pe = MIN(pc + 256, K);                                  \
              for (int64_t j = 0; j < N; j++) t[j] = (T)0;                    \
              for (int64_t k = pc; k < pe; k++) {                             \
                const T x = a[i * K + k];                                     \
                const T *bk = b + k * N;                                      \
                for (int64_t j = 0; j < N; j++) t[j] = FMA(x, bk[j], t[j]);   \
              }                                                               \
              for (int64_t j = 0; j < N; j++) d[j] = (pc == 0) ? t[j] : d[j] + t[j]; \
            }                                                                 \
            for (int64_t j = 0; j < N; j++) c[i * N + j] = K ? d[j] : (T)0;   \
            continue;                                                         \
          }                                                                   \
          for (int64_t jc = 0; jc < N; jc += (NC)) {                          \
            int64_t nc = MIN((NC), N - jc);                                   \
            for (int64_t j = jc + (nc / (NR)) * (NR); j < jc + nc; j++)       \
              c[i * N + j] = NAME##_packed_one(a, b, i, j, K, N);             \
          }                                                                   \
        }                                                                     \
        free(t);                                                              \
      }                                                                       \
      return;                                                                 \
    }                                                                         \
    _Pragma("omp parallel for schedule(dynamic, 8)")                          \
    for (int64_t i = 0; i < M; i++) {                                         \
      for (int64_t j = 0; j < N; j++) {                                       \
        int64_t mr = MIN(6, M - (i / 6) * 6);                                 \
        int64_t nr = MIN((NR), N - (j / (NR)) * (NR));                        \
        if (mr == 6 && nr == (NR)) continue;                                  \
        int64_t jj = j - (j / (NR)) * (NR);                                   \
        if (jj < (nr / (VW)) * (VW)) continue; /* vector FMA: chain */        \
        T acc = (T)0;                                                         \
        for (int64_t k = 0; k < K; k++) {                                     \
          T p = a[i * K + k] * b[k * N + j];                                  \
          acc = acc + p;                                                      \
        }                                                                     \
        c[i * N + j] = acc;                                                   \
      }                                                                       \
    }                                                                         \
  }

DEFINE_FLOAT_EDGES(edges_f32, float, fmaf, 96ULL * 96 * 96, 16, 8, 144, 6, 4080)
DEFINE_FLOAT_EDGES(edges_f64, double, fma, 48ULL * 48 * 48, 8, 4, 72, 6, 4080)
DEFINE_FLOAT_EDGES(edges_f32_neon, float, fmaf, 96ULL * 96 * 96, 12, 4, 128, 8, 4080)
DEFINE_FLOAT_EDGES(edges_f64_neon, double, fma, 48ULL * 48 * 48, 8, 2, 96, 6, 2048)

/* Naive float kernels: per output `acc = acc + a * b` from 0 in k order,
 * product and sum each rounded (this file is built without contraction). */
#define DEFINE_NAIVE_FLOAT(NAME, T)                                           \
  static void NAME(const T *a, const T *b, T *c, int64_t M, int64_t K,       \
                   int64_t N) {                                               \
    _Pragma("omp parallel for schedule(static)")                              \
    for (int64_t i = 0; i < M; i++)                                           \
      for (int64_t j = 0; j < N; j++) {                                       \
        T acc = (T)0;                                                         \
        for (int64_t k = 0; k < K; k++) {                                     \
          const T p = a[i * K + k] * b[k * N + j];                            \
          acc = acc + p;                                                      \
        }                                                                     \
        c[i * N + j] = acc;                                                   \
      }                                                                       \
  }

DEFINE_NAIVE_FLOAT(naive_f32, float)
DEFINE_NAIVE_FLOAT(naive_f64, double)

/* Wrapping integer kernels: T is the storage type, U the unsigned type of
 * the same width in which every product and sum wraps. */
#define DEFINE_WRAP_KERNEL(NAME, T, U)                                        \
  static void NAME(const T *a, const T *b, T *c, int64_t M, int64_t K,       \
                   int64_t N) {                                               \
    _Pragma("omp parallel for schedule(dynamic, 1)")                          \
    for (int64_t i0 = 0; i0 < M; i0 += RB) {                                  \
      int64_t i1 = MIN(i0 + RB, M);                                           \
      U *acc = (U *)calloc((size_t)((i1 - i0) * N) + 1, sizeof(U));           \
      for (int64_t k0 = 0; k0 < K; k0 += KB) {                                \
        int64_t k1 = MIN(k0 + KB, K);                                         \
        for (int64_t j0 = 0; j0 < N; j0 += JB) {                              \
          int64_t j1 = MIN(j0 + JB, N);                                       \
          for (int64_t i = i0; i < i1; i++) {                                 \
            U *restrict ci = acc + (i - i0) * N;                              \
            for (int64_t k = k0; k < k1; k++) {                               \
              const U aik = (U)a[i * K + k];                                  \
              const T *restrict bk = b + k * N;                               \
              for (int64_t j = j0; j < j1; j++) ci[j] += aik * (U)bk[j];      \
            }                                                                 \
          }                                                                   \
        }                                                                     \
      }                                                                       \
      for (int64_t i = i0; i < i1; i++)                                       \
        for (int64_t j = 0; j < N; j++)                                       \
          c[i * N + j] = (T)acc[(i - i0) * N + j];                            \
      free(acc);                                                              \
    }                                                                         \
  }

/* 16-bit products are formed in 32 bits (promotion), which is exact modulo
 * 2^16 after truncation. */
DEFINE_WRAP_KERNEL(kern_i16, int16_t, uint32_t)
DEFINE_WRAP_KERNEL(kern_u16, uint16_t, uint32_t)
DEFINE_WRAP_KERNEL(kern_i32, int32_t, uint32_t)
DEFINE_WRAP_KERNEL(kern_u32, uint32_t, uint32_t)
DEFINE_WRAP_KERNEL(kern_i64, int64_t, uint64_t)
DEFINE_WRAP_KERNEL(kern_u64, uint64_t, uint64_t)

/* -- 8-bit store rules -------------------------------------------------- */

static inline int32_t sat_s8(int32_t v) {
  return v < -128 ? -128 : (v > 127 ? 127 : v);
}

/* packusdw then packuswb: clamp to [0,65535], view as int16, clamp to
 * [0,255]. */
static inline int32_t sat_u8_x86(int32_t v) {
  int32_t u16 = v < 0 ? 0 : (v > 65535 ? 65535 : v);
  int32_t s16 = u16 >= 32768 ? u16 - 65536 : u16;
  return s16 < 0 ? 0 : (s16 > 255 ? 255 : s16);
}

static inline int32_t wrap8(int32_t v, int is_signed) {
  uint8_t byte = (uint8_t)(uint32_t)v;
  return is_signed ? (int32_t)(int8_t)byte : (int32_t)byte;
}

/* 1 when (i, j) lies in a full register tile of numc's packed x86 path. */
static inline int x86_full_tile(int64_t i, int64_t j, int64_t M, int64_t N) {
  int64_t ic = (i / 72) * 72, mc = MIN(72, M - ic);
  int64_t ir = ((i - ic) / 6) * 6, mr = MIN(6, mc - ir);
  int64_t jc = (j / 4080) * 4080, nc = MIN(4080, N - jc);
  int64_t jr = ((j - jc) / 16) * 16, nr = MIN(16, nc - jr);
  return mr == 6 && nr == 16;
}

/* 1 when (i, j) lies in a full MR x NR tile of a clamp-once path that
 * blocks M by MC (a multiple of MR) and N by NR from column 0: NEON
 * (72, 6, 8; gemm_neon.h:1509-1535) and AVX-512 (240, 12, 16;
 * gemm_avx512.h:1315-1341). */
static inline int clamp_full_tile(int64_t i, int64_t j, int64_t M, int64_t N,
                                  int64_t MC, int64_t MR, int64_t NR) {
  int64_t ic = (i / MC) * MC, mc = MIN(MC, M - ic);
  int64_t full_rows = (mc / MR) * MR;
  int64_t full_cols = (N / NR) * NR;
  return (i - ic) < full_rows && j < full_cols;
}

static void kern_8bit(const void *av, const void *bv, void *cv, int64_t M,
                      int64_t K, int64_t N, int is_signed, int profile) {
  const int8_t *as = (const int8_t *)av, *bs = (const int8_t *)bv;
  const uint8_t *au = (const uint8_t *)av, *bu = (const uint8_t *)bv;
  const int above_sup = (uint64_t)M * (uint64_t)K * (uint64_t)N > 192ULL * 192 * 192;
  int x86_packed = profile == ORACLE_X86_PACKED ||
                   (profile == ORACLE_I8_X86_AVX2 && above_sup);
  if (profile == ORACLE_X86_PACKED) profile = ORACLE_I8_X86_AVX2;
  if (profile == ORACLE_I8_X86_AVX512 && !above_sup) profile = ORACLE_I8_WRAP;
  /* x86 packed blocks K by 512; everything else sums all K in one block. */
  int64_t kblk = x86_packed ? 512 : (K > 0 ? K : 1);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i0 = 0; i0 < M; i0 += RB) {
    int64_t i1 = MIN(i0 + RB, M);
    int64_t rows = i1 - i0;
    uint32_t *part = (uint32_t *)malloc((size_t)(rows * N + 1) * 4);
    int32_t *d = (int32_t *)calloc((size_t)(rows * N + 1), 4);
    for (int64_t pc = 0, b = 0; pc < K || (K == 0 && b == 0); pc += kblk, b++) {
      int64_t kend = MIN(pc + kblk, K);
      memset(part, 0, (size_t)(rows * N) * 4);
      for (int64_t j0 = 0; j0 < N; j0 += JB) {
        int64_t j1 = MIN(j0 + JB, N);
        for (int64_t i = i0; i < i1; i++) {
          uint32_t *restrict pi = part + (i - i0) * N;
          for (int64_t k = pc; k < kend; k++) {
            uint32_t aik = is_signed ? (uint32_t)(int32_t)as[i * K + k]
                                     : (uint32_t)au[i * K + k];
            if (is_signed) {
              const int8_t *restrict bk = bs + k * N;
              for (int64_t j = j0; j < j1; j++)
                pi[j] += aik * (uint32_t)(int32_t)bk[j];
            } else {
              const uint8_t *restrict bk = bu + k * N;
              for (int64_t j = j0; j < j1; j++) pi[j] += aik * (uint32_t)bk[j];
            }
          }
        }
      }
      for (int64_t i = i0; i < i1; i++) {
        for (int64_t j = 0; j < N; j++) {
          int32_t P = (int32_t)part[(i - i0) * N + j];
          int32_t *dij = &d[(i - i0) * N + j];
          if (profile == ORACLE_I8_WRAP ||
              (profile == ORACLE_I8_X86_AVX2 && !x86_packed)) {
            *dij = wrap8((int32_t)((uint32_t)*dij + (uint32_t)P), is_signed);
          } else if (profile == ORACLE_I8_X86_AVX2) {
            int full = x86_full_tile(i, j, M, N);
            if (full) {
              int32_t v = *dij + P;
              *dij = is_signed ? sat_s8(v) : sat_u8_x86(v);
            } else {
              int32_t t = is_signed ? sat_s8(P) : sat_u8_x86(P);
              *dij = (b == 0) ? t : wrap8(*dij + t, is_signed);
            }
          } else { /* NEON or AVX-512: one block over all K, clamp once */
            const int neon = profile == ORACLE_I8_ARM_NEON;
            if (clamp_full_tile(i, j, M, N, neon ? 72 : 240, neon ? 6 : 12, neon ? 8 : 16)) {
              if (is_signed) *dij = sat_s8(P);
              else *dij = (uint32_t)P > 255u ? 255 : P;
            } else {
              *dij = wrap8(P, is_signed);
            }
          }
        }
      }
      if (K == 0) break;
    }
    for (int64_t i = i0; i < i1; i++)
      for (int64_t j = 0; j < N; j++) {
        int32_t v = d[(i - i0) * N + j];
        if (is_signed) ((int8_t *)cv)[i * N + j] = (int8_t)v;
        else ((uint8_t *)cv)[i * N + j] = (uint8_t)v;
      }
    free(part);
    free(d);
  }
}

/*
 * out[M,N] = a[M,K] @ b[K,N] with numc's arithmetic for `dtype` (numc's
 * NumcDType numbering).  Strides are in elements and may be arbitrary.
 * Returns 0, or -1 on a bad argument or allocation failure.
 */
int oracle_matmul(int dtype, const void *a, const void *b, void *out,
                  int64_t M, int64_t K, int64_t N, int64_t rsa, int64_t csa,
                  int64_t rsb, int64_t csb, int64_t rso, int64_t cso,
                  int profile, int nthreads) {
  if (dtype < 0 || dtype > DT_F64 || M < 0 || K < 0 || N < 0) return -1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  size_t es = k_elem[dtype];
  void *ad = gather(a, M, K, rsa, csa, es);
  void *bd = gather(b, K, N, rsb, csb, es);
  void *cd = malloc((size_t)(M * N) * es + 1);
  if (!ad || !bd || !cd) {
    free(ad); free(bd); free(cd);
    return -1;
  }
  /* the AVX-512 profile is an int8/uint8 rule: its floats keep AVX2's tiles */
  const int x86 = profile == ORACLE_I8_X86_AVX2 || profile == ORACLE_X86_PACKED ||
                  profile == ORACLE_I8_X86_AVX512;
  switch (dtype) {
  case DT_F32:
    if (profile == ORACLE_I8_WRAP) {
      naive_f32(ad, bd, cd, M, K, N);
      break;
    }
    kern_f32(ad, bd, cd, M, K, N);
    if (x86) edges_f32(ad, bd, cd, M, K, N, profile == ORACLE_X86_PACKED);
    else if (profile == ORACLE_I8_ARM_NEON) edges_f32_neon(ad, bd, cd, M, K, N, 0);
    break;
  case DT_F64:
    if (profile == ORACLE_I8_WRAP) {
      naive_f64(ad, bd, cd, M, K, N);
      break;
    }
    kern_f64(ad, bd, cd, M, K, N);
    if (x86) edges_f64(ad, bd, cd, M, K, N, profile == ORACLE_X86_PACKED);
    else if (profile == ORACLE_I8_ARM_NEON) edges_f64_neon(ad, bd, cd, M, K, N, 0);
    break;
  case DT_I16: kern_i16(ad, bd, cd, M, K, N); break;
  case DT_U16: kern_u16(ad, bd, cd, M, K, N); break;
  case DT_I32: kern_i32(ad, bd, cd, M, K, N); break;
  case DT_U32: kern_u32(ad, bd, cd, M, K, N); break;
  case DT_I64: kern_i64(ad, bd, cd, M, K, N); break;
  case DT_U64: kern_u64(ad, bd, cd, M, K, N); break;
  case DT_I8: kern_8bit(ad, bd, cd, M, K, N, 1, profile); break;
  case DT_U8: kern_8bit(ad, bd, cd, M, K, N, 0, profile); break;
  }
  scatter(out, cd, M, N, rso, cso, es);
  free(ad); free(bd); free(cd);
  return 0;
}

/* -- Double-double reference for float64 accuracy studies ----------------
 * Compensated dot product "Dot2" (Ogita, Rump and Oishi, "Accurate sum and
 * dot product", SIAM J. Sci. Comput. 26(6), 2005): TwoProduct via FMA and
 * TwoSum, giving a result as accurate as if computed in twice the working
 * precision.  Evaluates `count` outputs (rows[t], cols[t]) of a[M,K]@b[K,N]
 * (dense row-major) into hi[t] + lo[t]. */
void oracle_dot2_f64(const double *a, const double *b, int64_t K, int64_t N,
                     const int64_t *rows, const int64_t *cols, int64_t count,
                     double *hi, double *lo) {
#pragma omp parallel for schedule(static)
  for (int64_t t = 0; t < count; t++) {
    const double *ar = a + rows[t] * K;
    const double *bc = b + cols[t];
    double s = 0.0, c = 0.0;
    for (int64_t k = 0; k < K; k++) {
      double x = ar[k], y = bc[k * N];
      double p = x * y;
      double pe = fma(x, y, -p);          /* TwoProduct error */
      double s2 = s + p;                  /* TwoSum(s, p) */
      double bb = s2 - s;
      double se = (s - (s2 - bb)) + (p - bb);
      s = s2;
      c += pe + se;
    }
    double r = s + c;                     /* FastTwoSum normalisation */
    hi[t] = r;
    lo[t] = c - (r - s);
  }
}

/* Exact float64 accumulation of float32 products for output samples: each
 * float32 x float32 product is exact in float64; the sum uses Dot2 as above
 * so the reference error is far below float32 resolution. */
void oracle_dot_f32_ref(const float *a, const float *b, int64_t K, int64_t N,
                        const int64_t *rows, const int64_t *cols,
                        int64_t count, double *out) {
#pragma omp parallel for schedule(static)
  for (int64_t t = 0; t < count; t++) {
    const float *ar = a + rows[t] * K;
    const float *bc = b + cols[t];
    double s = 0.0, c = 0.0;
    for (int64_t k = 0; k < K; k++) {
      double p = (double)ar[k] * (double)bc[k * N];
      double s2 = s + p;
      double bb = s2 - s;
      c += (s - (s2 - bb)) + (p - bb);
      s = s2;
    }
    out[t] = s + c;
  }
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

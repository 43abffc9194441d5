/*
 * numc_oracle_dot.c — CPU restatement of numc_dot (src/reduction/dot.c).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA backend's numc_dot;
 * the product library never links, loads or calls it.
 *
 * numc_dot(a, b, out) (dot.c:442-447 -> _reduce_dot_op, dot.c:424-436):
 *
 *  - a or b 0-D (dot.c:339-346): out = other * scalar through
 *    numc_mul_scalar: the scalar goes through double and back to the dtype
 *    (elemwise/arithmetic.c:193-203), then one product per element in the
 *    dtype (integers wrap, floats round once).
 *
 *  - both 1-D (dot.c:348-365): contiguous operands use the SIMD dot
 *    (intrinsics/dot_avx2.h:106-158 for floats): 8 vector accumulators of
 *    W lanes (W = 8 float32, 4 float64), lane t of the 8W-element block
 *    chain fma(a, b, acc) over the full blocks; the accumulators are added
 *    pairwise (0+1, 2+3, 4+5, 6+7, then 0+2, 4+6, then 0+4), the lanes
 *    summed by the _hsum order, the tail summed as `tail += a * b` without
 *    contraction, result + tail.  Above 1 MiB of operand bytes the sum is
 *    split into nt = min(4, bytes / 512 KiB) OpenMP chunks
 *    (dot.c:235-258) whose results are added to 0; numc leaves the order of
 *    that addition to the OpenMP runtime, which only matters (for floats)
 *    when nt >= 3 — here chunks are added in order.  Integer sums are the
 *    exact sum modulo 2^bits whatever the order.  Non-contiguous operands
 *    use the strided reduction (reduction/kernel.h:48-78): `acc = acc + a*b`
 *    from 0, in order, in the storage type.
 *
 *  - otherwise (dot.c:367-420): K = a.shape[-1], M = a.size / K,
 *    N = b.dim == 1 ? 1 : b.shape[-1], P = b.size / (K N); row strides
 *    a.strides[0], b.strides[-2] (b.strides[0] for 1-D b), out.strides[0].
 *    P == 1 with unit column strides of b and out: numc's packed GEMM
 *    directly (numc_oracle.c profile ORACLE_X86_PACKED, no gemmsup
 *    threshold).  Otherwise the naive strided kernel (dot.c:42-72): integer
 *    sums promoted and truncated (exact modulo 2^bits), float sums without
 *    contraction; P > 1 runs it per batch, b advanced by K N elements (by
 *    b.strides[0] when b is 3-D) and out by N elements (by out.strides[1]
 *    when out is 3-D).
 *    For a of 3 or more dims numc's row stride a.strides[0] makes rows past
 *    a.shape[0] read beyond the array; here rows of a (and of out) step by
 *    the stride of the second-to-last axis of a (of out's matching axis),
 *    which requires those leading axes to be flattenable, and both a and b
 *    above 2-D is refused (-3).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum {
  DT_I8, DT_I16, DT_I32, DT_I64, DT_U8, DT_U16, DT_U32, DT_U64, DT_F32, DT_F64
};
static const size_t k_es[] = {1, 2, 4, 8, 1, 2, 4, 8, 4, 8};

int oracle_matmul(int dtype, const void *a, const void *b, void *out, int64_t M,
                  int64_t K, int64_t N, int64_t rsa, int64_t csa, int64_t rsb,
                  int64_t csb, int64_t rso, int64_t cso, int profile, int nthreads);

enum { PROFILE_X86_PACKED = 3 };

/* ---- helpers ------------------------------------------------------------ */

static double load_double(int dt, const char *p) {
  switch (dt) {
  case DT_I8: return (double)*(const int8_t *)p;
  case DT_I16: return (double)*(const int16_t *)p;
  case DT_I32: return (double)*(const int32_t *)p;
  case DT_I64: return (double)*(const int64_t *)p;
  case DT_U8: return (double)*(const uint8_t *)p;
  case DT_U16: return (double)*(const uint16_t *)p;
  case DT_U32: return (double)*(const uint32_t *)p;
  case DT_U64: return (double)*(const uint64_t *)p;
  case DT_F32: return (double)*(const float *)p;
  default: return *(const double *)p;
  }
}

/* Bits of an integer element as uint64 (sign-extended for signed types). */
static uint64_t load_bits(int dt, const char *p) {
  switch (dt) {
  case DT_I8: return (uint64_t)(int64_t)*(const int8_t *)p;
  case DT_I16: return (uint64_t)(int64_t)*(const int16_t *)p;
  case DT_I32: return (uint64_t)(int64_t)*(const int32_t *)p;
  case DT_I64: return (uint64_t)*(const int64_t *)p;
  case DT_U8: return *(const uint8_t *)p;
  case DT_U16: return *(const uint16_t *)p;
  case DT_U32: return *(const uint32_t *)p;
  default: return *(const uint64_t *)p;
  }
}

static void store_bits(int dt, char *p, uint64_t v) {
  switch (k_es[dt]) {
  case 1: *(uint8_t *)p = (uint8_t)v; break;
  case 2: *(uint16_t *)p = (uint16_t)v; break;
  case 4: *(uint32_t *)p = (uint32_t)v; break;
  default: *(uint64_t *)p = v; break;
  }
}

/* double -> dtype as a C conversion (numc's _double_to_dtype), as bits. */
static uint64_t int_from_double(int dt, double v) {
  switch (dt) {
  case DT_I8: return (uint64_t)(int64_t)(int8_t)v;
  case DT_I16: return (uint64_t)(int64_t)(int16_t)v;
  case DT_I32: return (uint64_t)(int64_t)(int32_t)v;
  case DT_I64: return (uint64_t)(int64_t)v;
  case DT_U8: return (uint8_t)v;
  case DT_U16: return (uint16_t)v;
  case DT_U32: return (uint32_t)v;
  default: return (uint64_t)v;
  }
}

static int is_float(int dt) { return dt == DT_F32 || dt == DT_F64; }

/* ---- 0-D case ----------------------------------------------------------- */

static void scalar_case(int dt, const char *x, int dim, const int64_t *shape,
                        const int64_t *st, const char *sp, char *out,
                        const int64_t *ost) {
  const size_t es = k_es[dt];
  const double sv = load_double(dt, sp);
  int64_t total = 1;
  for (int d = 0; d < dim; d++) total *= shape[d];
  int64_t idx[16] = {0};
  for (int64_t e = 0; e < total; e++) {
    int64_t xo = 0, oo = 0;
    for (int d = 0; d < dim; d++) {
      xo += idx[d] * st[d];
      oo += idx[d] * ost[d];
    }
    const char *px = x + xo * (int64_t)es;
    char *po = out + oo * (int64_t)es;
    if (dt == DT_F32) {
      const float s = (float)sv;
      *(float *)po = *(const float *)px * s;
    } else if (dt == DT_F64) {
      *(double *)po = *(const double *)px * sv;
    } else {
      store_bits(dt, po, load_bits(dt, px) * int_from_double(dt, sv));
    }
    for (int d = dim - 1; d >= 0; d--) {
      if (++idx[d] < shape[d]) break;
      idx[d] = 0;
    }
  }
}

/* ---- 1-D case ----------------------------------------------------------- */

#define DEFINE_SIMD_DOT(NAME, T, FMA, W)                                       \
  static T NAME(const T *a, const T *b, int64_t n) {                          \
    T acc[8][W];                                                               \
    memset(acc, 0, sizeof acc);                                                \
    int64_t i = 0;                                                             \
    for (; i + 8 * W <= n; i += 8 * W)                                         \
      for (int j = 0; j < 8; j++)                                              \
        for (int l = 0; l < W; l++)                                            \
          acc[j][l] = FMA(a[i + W * j + l], b[i + W * j + l], acc[j][l]);      \
    for (int l = 0; l < W; l++) {                                              \
      acc[0][l] = acc[0][l] + acc[1][l];                                       \
      acc[2][l] = acc[2][l] + acc[3][l];                                       \
      acc[4][l] = acc[4][l] + acc[5][l];                                       \
      acc[6][l] = acc[6][l] + acc[7][l];                                       \
      acc[0][l] = acc[0][l] + acc[2][l];                                       \
      acc[4][l] = acc[4][l] + acc[6][l];                                       \
      acc[0][l] = acc[0][l] + acc[4][l];                                       \
    }                                                                          \
    T result = HSUM_##W(acc[0]);                                               \
    T tail = 0;                                                                \
    for (; i < n; i++) {                                                       \
      const T p = a[i] * b[i];                                                 \
      tail = tail + p;                                                         \
    }                                                                          \
    return result + tail;                                                      \
  }

/* _hsum_ps_avx2: (v0 + v4, v1 + v5, v2 + v6, v3 + v7) = s, then
 * (s0 + s2) + (s1 + s3). */
static float HSUM_8(const float *v) {
  float s0 = v[0] + v[4], s1 = v[1] + v[5], s2 = v[2] + v[6], s3 = v[3] + v[7];
  float t0 = s0 + s2, t1 = s1 + s3;
  return t0 + t1;
}
/* _hsum_pd_avx2: (v0 + v2) + (v1 + v3). */
static double HSUM_4(const double *v) {
  double s0 = v[0] + v[2], s1 = v[1] + v[3];
  return s0 + s1;
}

DEFINE_SIMD_DOT(simd_dot_f32, float, fmaf, 8)
DEFINE_SIMD_DOT(simd_dot_f64, double, fma, 4)

static void dot_1d(int dt, const char *a, int64_t sa, const char *b, int64_t sb,
                   int64_t n, int contiguous, char *out) {
  const size_t es = k_es[dt];
  if (!is_float(dt)) {
    uint64_t acc = 0;   /* exact modulo 2^64, hence modulo 2^bits */
    for (int64_t i = 0; i < n; i++)
      acc += load_bits(dt, a + i * sa * (int64_t)es) * load_bits(dt, b + i * sb * (int64_t)es);
    store_bits(dt, out, acc);
    return;
  }
  if (!contiguous) {
    if (dt == DT_F32) {
      float acc = 0.0f;
      for (int64_t i = 0; i < n; i++) {
        const float p = ((const float *)a)[i * sa] * ((const float *)b)[i * sb];
        acc = acc + p;
      }
      *(float *)out = acc;
    } else {
      double acc = 0.0;
      for (int64_t i = 0; i < n; i++) {
        const double p = ((const double *)a)[i * sa] * ((const double *)b)[i * sb];
        acc = acc + p;
      }
      *(double *)out = acc;
    }
    return;
  }
  const size_t total = (size_t)n * es * 2;
  int nt = (int)(total / (1u << 19));
  if (nt > 4) nt = 4;
  if (total > (1u << 20) && nt >= 2) {
    const int64_t per = n / nt;
    if (dt == DT_F32) {
      float g = 0.0f;
      for (int t = 0; t < nt; t++) {
        const int64_t s = t * per, e = (t == nt - 1) ? n : s + per;
        g = g + simd_dot_f32((const float *)a + s, (const float *)b + s, e - s);
      }
      *(float *)out = g;
    } else {
      double g = 0.0;
      for (int t = 0; t < nt; t++) {
        const int64_t s = t * per, e = (t == nt - 1) ? n : s + per;
        g = g + simd_dot_f64((const double *)a + s, (const double *)b + s, e - s);
      }
      *(double *)out = g;
    }
  } else if (dt == DT_F32) {
    *(float *)out = simd_dot_f32((const float *)a, (const float *)b, n);
  } else {
    *(double *)out = simd_dot_f64((const double *)a, (const double *)b, n);
  }
}

/* ---- N-D case ----------------------------------------------------------- */

/* numc's strided naive kernel (dot.c:42-72) for M x K @ K x N. */
static void naive_strided(int dt, const char *a, const char *b, char *out,
                          int64_t M, int64_t K, int64_t N, int64_t rsa,
                          int64_t csa, int64_t rsb, int64_t csb, int64_t rso,
                          int64_t cso) {
  const int64_t es = (int64_t)k_es[dt];
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < M; i++)
    for (int64_t j = 0; j < N; j++) {
      char *po = out + (i * rso + j * cso) * es;
      if (dt == DT_F32) {
        float acc = 0.0f;
        for (int64_t k = 0; k < K; k++) {
          const float p = ((const float *)a)[i * rsa + k * csa] *
                          ((const float *)b)[k * rsb + j * csb];
          acc = acc + p;
        }
        *(float *)po = acc;
      } else if (dt == DT_F64) {
        double acc = 0.0;
        for (int64_t k = 0; k < K; k++) {
          const double p = ((const double *)a)[i * rsa + k * csa] *
                           ((const double *)b)[k * rsb + j * csb];
          acc = acc + p;
        }
        *(double *)po = acc;
      } else {
        uint64_t acc = 0;
        for (int64_t k = 0; k < K; k++)
          acc += load_bits(dt, a + (i * rsa + k * csa) * es) *
                 load_bits(dt, b + (k * rsb + j * csb) * es);
        store_bits(dt, po, acc);
      }
    }
}

/* Leading axes [0, upto) of (shape, strides) collapse to one row axis. */
static int flattenable(const int64_t *shape, const int64_t *st, int upto) {
  for (int d = 0; d + 1 < upto; d++)
    if (shape[d + 1] != 1 && st[d] != st[d + 1] * shape[d + 1]) return 0;
  return 1;
}

int oracle_dot(int dt, const void *av, int adim, const int64_t *ash,
               const int64_t *ast, int a_contig, const void *bv, int bdim,
               const int64_t *bsh, const int64_t *bst, int b_contig, void *outv,
               int odim, const int64_t *osh, const int64_t *ost) {
  const char *a = (const char *)av, *b = (const char *)bv;
  char *out = (char *)outv;
  if (dt < 0 || dt > DT_F64 || adim > 16 || bdim > 16 || odim > 16) return -1;
  if (adim == 0 || bdim == 0) {
    if (adim == 0) scalar_case(dt, b, bdim, bsh, bst, a, out, ost);
    else scalar_case(dt, a, adim, ash, ast, b, out, ost);
    return 0;
  }
  if (adim == 1 && bdim == 1) {
    dot_1d(dt, a, ast[0], b, bst[0], ash[0], a_contig && b_contig, out);
    return 0;
  }
  if (adim >= 3 && bdim >= 3) return -3;
  int64_t asize = 1, bsize = 1;
  for (int d = 0; d < adim; d++) asize *= ash[d];
  for (int d = 0; d < bdim; d++) bsize *= bsh[d];
  const int64_t K = ash[adim - 1];
  const int64_t N = bdim == 1 ? 1 : bsh[bdim - 1];
  /* numc divides by K here (K = 0 is a division by zero there); an empty
   * contraction gives zeros. */
  if (K == 0) {
    int64_t total = 1, idx[16] = {0};
    for (int d = 0; d < odim; d++) total *= osh[d];
    for (int64_t e = 0; e < total; e++) {
      int64_t o = 0;
      for (int d = 0; d < odim; d++) o += idx[d] * ost[d];
      memset(out + o * (int64_t)k_es[dt], 0, k_es[dt]);
      for (int d = odim - 1; d >= 0; d--) {
        if (++idx[d] < osh[d]) break;
        idx[d] = 0;
      }
    }
    return 0;
  }
  if (N == 0 || asize == 0) return 0;
  const int64_t M = asize / K;
  const int64_t P = bsize / (K * N);
  int64_t rsa = ast[0], rso = odim > 0 ? ost[0] : 0;
  if (adim >= 3) {
    if (!flattenable(ash, ast, adim - 1) || !flattenable(osh, ost, adim - 1)) return -2;
    rsa = ast[adim - 2];
    rso = ost[adim - 2];
  }
  const int64_t csa = ast[adim - 1];
  const int64_t rsb = bdim > 1 ? bst[bdim - 2] : bst[0];
  const int64_t csb = bst[bdim - 1];
  const int64_t cso = odim > 0 ? ost[odim - 1] : 0;
  const int64_t es = (int64_t)k_es[dt];
  if (P <= 1) {
    if (csb == 1 && cso == 1)
      return oracle_matmul(dt, a, b, out, M, K, N, rsa, csa, rsb, 1, rso, 1,
                           PROFILE_X86_PACKED, 0);
    naive_strided(dt, a, b, out, M, K, N, rsa, csa, rsb, csb, rso, cso);
    return 0;
  }
  for (int64_t p = 0; p < P; p++) {
    const char *bp = b + p * K * N * es;
    char *op = out + p * N * es;
    if (odim == 3) op = out + p * ost[1] * es;
    if (bdim == 3) bp = b + p * bst[0] * es;
    naive_strided(dt, a, bp, op, M, K, N, rsa, csa, rsb, csb, rso, cso);
  }
  return 0;
}

/* Matrix multiplication — numc's matmul and dot entry points
 * (include/numc/math.h:573-604 of numc), served by the CUDA backend. */
#ifndef NUMC_MATH_H
#define NUMC_MATH_H

#include "numc/array.h"
#include "numc/export.h"

#ifdef __cplusplus
extern "C" {
#endif

/* out = a @ b for 2-D arrays of one dtype: a is (M, K), b is (K, N) and the
 * caller-allocated out is (M, N).  Replaces numc's numc_matmul
 * (src/matmul/matmul.c:347-389): same validation order and error codes
 * (NULL -> NUMC_ERR_NULL, dtype mismatch -> NUMC_ERR_TYPE, rank or extent
 * mismatch -> NUMC_ERR_SHAPE), same results (integers bit-exact, including
 * numc's int8/uint8 store rules; floats within the stated tolerance).
 * Runs on the GPU; CUDA failures return NUMC_ERR_MALLOC/NUMC_ERR_INTERNAL.
 * Arbitrary byte strides are honoured on all three operands. */
NUMC_API int numc_matmul(const NumcArray *a, const NumcArray *b,
                         NumcArray *out);

/* Reference product (numc's numc_matmul_naive, matmul.c:333-343): integer
 * dtypes accumulate in their storage width (int8/uint8 results are the sum
 * truncated to 8 bits), floats as `acc += a * b` with every product and sum
 * rounded (no fused multiply-add), in k order. */
NUMC_API int numc_matmul_naive(const NumcArray *a, const NumcArray *b,
                               NumcArray *out);

/* numc_dot (numc's math.h:593, src/reduction/dot.c:442-447), numpy.dot's
 * shape rules: a or b 0-D multiplies by the scalar; both 1-D give the inner
 * product (out 0-D or one element); otherwise a's last axis contracts with
 * b's second-to-last (its only axis if 1-D) and out has shape
 * a.shape[:-1] + b.shape[:-2] + b.shape[-1:].  Same validation and error
 * codes as numc, same arithmetic per branch: the GEMM branch (b unbatched,
 * unit column strides of b and out) is numc_matmul's without the small-size
 * int8/uint8 threshold; strided and batched operands use numc's naive sums
 * (floats unfused); 1-D floats follow numc's SIMD lane order.  Deviations:
 * for a of 3+ dims numc's row stride reads past the array, here rows step
 * through a's (and out's) flattenable leading axes (NUMC_ERR_SHAPE if they
 * do not flatten); a and b both above 2-D return NUMC_ERR_SHAPE. */
NUMC_API int numc_dot(const NumcArray *a, const NumcArray *b, NumcArray *out);

/* Fused linear layer out = x @ w + bias (numc's ROADMAP.md "Linear
 * algebra"; not in numc's current API): x (M, K), w (K, N), bias (N,) or
 * NULL, out (M, N).  Results equal numc_matmul(x, w, out) followed by
 * adding bias to every row with numc's elementwise add (floats rounded
 * once, integers modulo 2^bits); the CUDA-core and split kernels add the
 * bias in their store, other algorithms in one extra pass. */
NUMC_API int numc_linear(const NumcArray *x, const NumcArray *w, const NumcArray *bias,
                         NumcArray *out);

/* Batched matrix multiply (numc's ROADMAP.md; not in numc's current API):
 * a (..., M, K), b (..., K, N), out (..., M, N) with the same leading batch
 * axes; every batch is numc_matmul(a[i], b[i], out[i]) with numc_matmul's
 * arithmetic and algorithm choice.  Any strides. */
NUMC_API int numc_bmm(const NumcArray *a, const NumcArray *b, NumcArray *out);

#ifdef __cplusplus
}
#endif

#endif /* NUMC_MATH_H */

/* Matrix multiplication — numc's matmul entry points
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

/* Wrapping reference product (numc's numc_matmul_naive, matmul.c:333-343):
 * every dtype accumulates in its storage width, so int8/uint8 results are
 * the sum truncated to 8 bits. */
NUMC_API int numc_matmul_naive(const NumcArray *a, const NumcArray *b,
                               NumcArray *out);

#ifdef __cplusplus
}
#endif

#endif /* NUMC_MATH_H */

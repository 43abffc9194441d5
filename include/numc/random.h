/* numc's random-array API for the matmul path's inputs (numc's
 * include/numc/random.h:18,32): the same generator, state and results,
 * filled on the GPU. */
#ifndef NUMC_RANDOM_H
#define NUMC_RANDOM_H

#include <stddef.h>
#include <stdint.h>

#include "numc/array.h"
#include "numc/dtype.h"
#include "numc/export.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Seed the calling thread's generator (numc's random.h:18,
 * src/random/random.c:263-266): four xoshiro256** streams, stream 0 from
 * splitmix64(seed), streams 1-3 each 2^128 steps further.  A thread that
 * never seeds uses numc's default seed 0xdeadbeefcafe1234. */
NUMC_API void numc_manual_seed(uint64_t seed);

/* A new array of uniform random values (numc's random.h:32,
 * src/random/random.c:268-272), bit-identical to numc's for every dtype:
 * integers are the low bits of the generator's output, float32/float64
 * uniform in [0, 1).  Arrays up to 1 MiB use numc's single-thread layout;
 * larger ones numc's per-thread chunks, whose layout depends on numc's
 * OpenMP thread count (numc_cuda_rand_set_threads).  Generated on the GPU
 * and copied into the host buffer; the calling thread's state advances as
 * numc's does.  NULL ctx, NULL shape or dim 0: NULL with NUMC_ERR_NULL;
 * no CUDA device: NULL with NUMC_ERR_INTERNAL. */
NUMC_API NumcArray *numc_array_rand(NumcCtx *ctx, const size_t *shape,
                                    size_t dim, NumcDType dtype);

#ifdef __cplusplus
}
#endif

#endif /* NUMC_RANDOM_H */

/* Context and array API — the subset of numc's include/numc/array.h that the
 * matmul path and its callers use, with numc's signatures and semantics:
 *
 *   - a NumcCtx owns every array made from it (arena ownership);
 *     numc_ctx_free releases them all, checkpoint/restore rolls back;
 *   - arrays are row-major with BYTE strides; transpose permutes strides and
 *     slice returns a strided view, neither copies data;
 *   - host data is reachable through numc_array_data(); with the CUDA
 *     backend the host buffer is page-locked so copies to the GPU are DMA.
 */
#ifndef NUMC_ARRAY_H
#define NUMC_ARRAY_H

#include "numc/dtype.h"
#include "numc/export.h"
#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct NumcCtx NumcCtx;
typedef struct NumcArray NumcArray;

typedef struct {
  size_t axis, start, stop, step;
} NumcSlice;

typedef struct {
  void *_block;
  size_t _index;
} NumcCheckpoint;

/* numc array.h:37   */ NUMC_API NumcCtx *numc_ctx_create(void);
/* numc array.h:46   */ NUMC_API void numc_ctx_free(NumcCtx *ctx);
/* numc array.h:54   */ NUMC_API NumcCheckpoint numc_ctx_checkpoint(NumcCtx *ctx);
/* numc array.h:65   */ NUMC_API void numc_ctx_restore(NumcCtx *ctx, NumcCheckpoint cp);

/* numc array.h:78   */
NUMC_API NumcArray *numc_array_create(NumcCtx *ctx, const size_t *shape,
                                      size_t dim, NumcDType dtype);
/* numc array.h:90   */
NUMC_API NumcArray *numc_array_zeros(NumcCtx *ctx, const size_t *shape,
                                     size_t dim, NumcDType dtype);
/* numc array.h:103  */
NUMC_API NumcArray *numc_array_fill(NumcCtx *ctx, const size_t *shape,
                                    size_t dim, NumcDType dtype,
                                    const void *value);
/* numc array.h:113  */ NUMC_API NumcArray *numc_array_copy(const NumcArray *arr);
/* numc array.h:121  */ NUMC_API void numc_array_write(NumcArray *arr, const void *data);
/* numc array.h:176  */ NUMC_API int numc_array_transpose(NumcArray *arr, const size_t *axes);
/* numc array.h:185  */
NUMC_API NumcArray *numc_array_transpose_copy(const NumcArray *arr,
                                              const size_t *axes);
/* numc array.h:198  */
NUMC_API NumcArray *numc_array_slice(const NumcArray *arr, NumcSlice *slice);
/* numc array.h:206  */ NUMC_API bool numc_array_is_contiguous(NumcArray *arr);
/* numc array.h:214  */ NUMC_API int numc_array_contiguous(NumcArray *arr);

/* numc array.h:224-286 */
NUMC_API size_t numc_array_size(const NumcArray *arr);
NUMC_API size_t numc_array_capacity(const NumcArray *arr);
NUMC_API size_t numc_array_elem_size(const NumcArray *arr);
NUMC_API size_t numc_array_ndim(const NumcArray *arr);
NUMC_API void numc_array_shape(const NumcArray *arr, size_t *shape);
NUMC_API void numc_array_strides(const NumcArray *arr, size_t *strides);
NUMC_API NumcDType numc_array_dtype(const NumcArray *arr);
/* Host data pointer.  For an array made device-resident with
 * numc_cuda_array_to_device(), call numc_cuda_array_to_host() first. */
NUMC_API void *numc_array_data(const NumcArray *arr);

#ifdef __cplusplus
}
#endif

#endif /* NUMC_ARRAY_H */

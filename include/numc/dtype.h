/* Element types.  The enumerator order and values are numc's ABI
 * (include/numc/dtype.h:21-32 of numc); code compiled against numc's header
 * passes the same integers. */
#ifndef NUMC_DTYPE_H
#define NUMC_DTYPE_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

typedef enum {
  NUMC_DTYPE_INT8,
  NUMC_DTYPE_INT16,
  NUMC_DTYPE_INT32,
  NUMC_DTYPE_INT64,
  NUMC_DTYPE_UINT8,
  NUMC_DTYPE_UINT16,
  NUMC_DTYPE_UINT32,
  NUMC_DTYPE_UINT64,
  NUMC_DTYPE_FLOAT32,
  NUMC_DTYPE_FLOAT64,
} NumcDType;

#define NUMC_DTYPE_COUNT 10

static inline bool numc_dtype_is_float(NumcDType dt) {
  return dt == NUMC_DTYPE_FLOAT32 || dt == NUMC_DTYPE_FLOAT64;
}

static inline bool numc_dtype_is_signed(NumcDType dt) {
  return dt <= NUMC_DTYPE_INT64 || numc_dtype_is_float(dt);
}

/* Bytes per element. */
static inline size_t numc_dtype_size(NumcDType dt) {
  switch (dt) {
  case NUMC_DTYPE_INT8: case NUMC_DTYPE_UINT8: return 1;
  case NUMC_DTYPE_INT16: case NUMC_DTYPE_UINT16: return 2;
  case NUMC_DTYPE_INT32: case NUMC_DTYPE_UINT32: case NUMC_DTYPE_FLOAT32:
    return 4;
  default: return 8;
  }
}

/* Natural alignment of one element (equal to its size for every dtype). */
static inline size_t numc_dtype_align(NumcDType dt) {
  return numc_dtype_size(dt);
}

#endif /* NUMC_DTYPE_H */

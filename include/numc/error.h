/* Error reporting, ABI-compatible with numc's include/numc/error.h:10-57:
 * functions return 0 or a negative NumcErrorCode and leave a message in
 * thread-local storage, read back with numc_get_error(). */
#ifndef NUMC_ERROR_H
#define NUMC_ERROR_H

#include "numc/export.h"
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  NUMC_ERR_NONE = 0,
  NUMC_ERR_NULL = -1,     /* a required pointer was NULL */
  NUMC_ERR_MALLOC = -2,   /* host or device allocation failed */
  NUMC_ERR_SHAPE = -3,    /* rank or extent mismatch */
  NUMC_ERR_TYPE = -4,     /* dtype mismatch or unsupported dtype */
  NUMC_ERR_BOUNDS = -5,   /* index out of range */
  NUMC_ERR_VALUE = -6,    /* invalid argument value */
  NUMC_ERR_INTERNAL = -99 /* CUDA launch/runtime failure or kernel timeout */
} NumcErrorCode;

typedef struct {
  int code;
  const char *msg;
} NumcError;

/* Record an error for the calling thread; returns `code`. */
NUMC_API int numc_set_error_v(int code, const char *func, const char *file,
                              int line, const char *fmt, ...);
NUMC_API int numc_set_error(int code, const char *msg);
/* Last error recorded on the calling thread. */
NUMC_API NumcError numc_get_error(void);
/* Print an error to stderr. */
NUMC_API void numc_log_error(const NumcError *err);

#define NUMC_SET_ERROR(code, ...) \
  numc_set_error_v(code, __func__, __FILE__, __LINE__, __VA_ARGS__)

#ifdef __cplusplus
}
#endif

#endif /* NUMC_ERROR_H */

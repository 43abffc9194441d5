// Host runtime: thread-local errors, the context arena and array headers.
//
// Semantics follow numc (src/error.c:8-58, src/arena.h, src/array_core.c):
// a context owns a chain of bump-allocated blocks; checkpoint records the
// current (block, offset) and restore frees every block created after it.
// Differences, all deliberate: data is 256-byte aligned (TMA / coalescing),
// and when a GPU is present the arena blocks are page-locked so transfers
// to HBM run as DMA without a bounce buffer.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "runtime.h"

using namespace numc_rt;

// --- errors ---------------------------------------------------------------

namespace {
thread_local int t_err_code = 0;
thread_local char t_err_msg[512] = "";
}  // namespace

extern "C" int numc_set_error_v(int code, const char *func, const char *file,
                                int line, const char *fmt, ...) {
  t_err_code = code;
  int n = snprintf(t_err_msg, sizeof t_err_msg, "[%s:%d %s] ",
                   file ? file : "?", line, func ? func : "?");
  if (n < 0 || (size_t)n >= sizeof t_err_msg) n = 0;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_err_msg + n, sizeof t_err_msg - n, fmt, ap);
  va_end(ap);
  return code;
}

extern "C" int numc_set_error(int code, const char *msg) {
  t_err_code = code;
  snprintf(t_err_msg, sizeof t_err_msg, "%s", msg ? msg : "");
  return code;
}

extern "C" NumcError numc_get_error(void) {
  NumcError e;
  e.code = t_err_code;
  e.msg = t_err_msg;
  return e;
}

extern "C" void numc_log_error(const NumcError *err) {
  if (err && err->code != 0)
    fprintf(stderr, "numc error %d: %s\n", err->code, err->msg ? err->msg : "");
}

// --- arena ----------------------------------------------------------------

namespace numc_rt {

static ArenaBlock *new_block(NumcCtx *ctx, size_t cap) {
  ArenaBlock *b = new (std::nothrow) ArenaBlock();
  if (!b) return nullptr;
  b->pinned = false;
  b->base = nullptr;
  if (ctx->pin_host) {
    b->base = (char *)host_alloc_pinned(cap);
    b->pinned = b->base != nullptr;
  }
  if (!b->base) b->base = (char *)aligned_alloc(kDataAlign, (cap + kDataAlign - 1) / kDataAlign * kDataAlign);
  if (!b->base) {
    delete b;
    return nullptr;
  }
  b->cap = cap;
  b->used = 0;
  b->seq = ctx->next_seq++;
  b->prev = ctx->head;
  ctx->head = b;
  return b;
}

static void free_block(ArenaBlock *b) {
  if (b->pinned) host_free_pinned(b->base);
  else free(b->base);
  delete b;
}

void *arena_alloc(NumcCtx *ctx, size_t bytes, size_t align, ArenaPos *pos) {
  if (bytes == 0) bytes = 1;
  ArenaBlock *b = ctx->head;
  size_t off = 0;
  if (b) off = (b->used + align - 1) / align * align;
  if (!b || off + bytes > b->cap) {
    // Large requests get a dedicated block (numc arena.h:368-376).
    size_t cap = bytes > kArenaBlock ? bytes : kArenaBlock;
    b = new_block(ctx, cap);
    if (!b) return nullptr;
    off = 0;
  }
  b->used = off + bytes;
  if (pos) *pos = ArenaPos{b->seq, off};
  return b->base + off;
}

ArenaPos arena_pos(const NumcCtx *ctx) {
  if (!ctx->head) return ArenaPos{0, 0};
  return ArenaPos{ctx->head->seq, ctx->head->used};
}

size_t array_span_bytes(const NumcArray *arr) {
  if (arr->size == 0) return 0;
  size_t span = arr->elem_size;
  for (size_t d = 0; d < arr->dim; d++)
    span += (arr->shape[d] - 1) * arr->strides[d];
  return span;
}

}  // namespace numc_rt

// --- context --------------------------------------------------------------

extern "C" NumcCtx *numc_ctx_create(void) {
  NumcCtx *ctx = new (std::nothrow) NumcCtx();
  if (!ctx) {
    NUMC_SET_ERROR(NUMC_ERR_MALLOC, "failed to allocate context");
    return nullptr;
  }
  ctx->head = nullptr;
  ctx->next_seq = 1;
  ctx->pin_host = cuda_present();
  ctx->stream = nullptr;
  ctx->copy_in = nullptr;
  ctx->copy_out = nullptr;
  ctx->gemm2 = nullptr;
  ctx->gemm3 = nullptr;
  ctx->device = -1;
  ctx->scratch = nullptr;
  ctx->scratch_bytes = 0;
  ctx->dev_allocs = new (std::nothrow) std::vector<DeviceAlloc>();
  ctx->dev_slabs = new (std::nothrow) std::vector<DeviceSlab>();
  ctx->dev_cur = 0;
  if (!ctx->dev_allocs || !ctx->dev_slabs || !new_block(ctx, kArenaBlock)) {
    delete ctx->dev_allocs;
    delete ctx->dev_slabs;
    delete ctx;
    NUMC_SET_ERROR(NUMC_ERR_MALLOC, "failed to create arena (%zu bytes)",
                   kArenaBlock);
    return nullptr;
  }
  return ctx;
}

extern "C" void numc_ctx_free(NumcCtx *ctx) {
  if (!ctx) return;
  ctx_release_device(ctx, nullptr);
  ArenaBlock *b = ctx->head;
  while (b) {
    ArenaBlock *p = b->prev;
    free_block(b);
    b = p;
  }
  delete ctx->dev_allocs;
  delete ctx->dev_slabs;
  delete ctx;
}

extern "C" NumcCheckpoint numc_ctx_checkpoint(NumcCtx *ctx) {
  NumcCheckpoint cp;
  cp._block = ctx ? ctx->head : nullptr;
  cp._index = (ctx && ctx->head) ? ctx->head->used : 0;
  return cp;
}

extern "C" void numc_ctx_restore(NumcCtx *ctx, NumcCheckpoint cp) {
  if (!ctx) return;
  ArenaBlock *keep = (ArenaBlock *)cp._block;
  ArenaPos pos = keep ? ArenaPos{keep->seq, cp._index} : ArenaPos{0, 0};
  // Device memory of arrays created after the checkpoint goes first.
  ctx_release_device(ctx, &pos);
  while (ctx->head && ctx->head != keep) {
    ArenaBlock *p = ctx->head->prev;
    free_block(ctx->head);
    ctx->head = p;
  }
  if (ctx->head) ctx->head->used = cp._index;
}

// --- arrays ---------------------------------------------------------------

static bool contiguous_strides(size_t *strides, const size_t *shape,
                               size_t dim, size_t elem) {
  if (dim == 0) return true;
  strides[dim - 1] = elem;
  for (size_t i = dim - 1; i > 0; i--)
    if (__builtin_mul_overflow(strides[i], shape[i], &strides[i - 1]))
      return false;
  return true;
}

static NumcArray *new_header(NumcCtx *ctx, size_t dim) {
  ArenaPos pos;
  NumcArray *arr = (NumcArray *)arena_alloc(ctx, sizeof(NumcArray),
                                            alignof(NumcArray), &pos);
  if (!arr) return nullptr;
  memset(arr, 0, sizeof *arr);
  arr->ctx = ctx;
  arr->pos = pos;
  arr->residency = kHostOnly;
  if (dim <= kMaxInlineDims) {
    arr->shape = arr->shape_buf;
    arr->strides = arr->strides_buf;
  } else {
    arr->shape = (size_t *)arena_alloc(ctx, dim * sizeof(size_t),
                                       alignof(size_t), nullptr);
    arr->strides = (size_t *)arena_alloc(ctx, dim * sizeof(size_t),
                                         alignof(size_t), nullptr);
    if (!arr->shape || !arr->strides) return nullptr;
  }
  arr->dim = dim;
  return arr;
}

extern "C" NumcArray *numc_array_create(NumcCtx *ctx, const size_t *shape,
                                        size_t dim, NumcDType dtype) {
  if (!ctx || (!shape && dim > 0)) {
    NUMC_SET_ERROR(NUMC_ERR_NULL, "array_create: NULL argument (ctx=%p shape=%p)",
                   (void *)ctx, (const void *)shape);
    return nullptr;
  }
  if ((int)dtype < 0 || (int)dtype >= NUMC_DTYPE_COUNT) {
    NUMC_SET_ERROR(NUMC_ERR_TYPE, "array_create: unknown dtype %d", (int)dtype);
    return nullptr;
  }
  size_t size = 1, capacity = 0, elem = numc_dtype_size(dtype);
  for (size_t i = 0; i < dim; i++)
    if (__builtin_mul_overflow(size, shape[i], &size)) {
      NUMC_SET_ERROR(NUMC_ERR_SHAPE, "array_create: element count overflow at dim %zu", i);
      return nullptr;
    }
  if (__builtin_mul_overflow(size, elem, &capacity)) {
    NUMC_SET_ERROR(NUMC_ERR_SHAPE, "array_create: byte size overflow");
    return nullptr;
  }
  NumcArray *arr = new_header(ctx, dim);
  if (!arr) {
    NUMC_SET_ERROR(NUMC_ERR_MALLOC, "array_create: header allocation failed");
    return nullptr;
  }
  arr->data = arena_alloc(ctx, capacity, kDataAlign, nullptr);
  if (!arr->data) {
    NUMC_SET_ERROR(NUMC_ERR_MALLOC, "array_create: failed to allocate %zu bytes", capacity);
    return nullptr;
  }
  if (dim) memcpy(arr->shape, shape, dim * sizeof(size_t));
  if (!contiguous_strides(arr->strides, shape, dim, elem)) {
    NUMC_SET_ERROR(NUMC_ERR_SHAPE, "array_create: stride overflow");
    return nullptr;
  }
  arr->elem_size = elem;
  arr->size = size;
  arr->capacity = capacity;
  arr->dtype = dtype;
  arr->is_contiguous = true;
  return arr;
}

extern "C" NumcArray *numc_array_zeros(NumcCtx *ctx, const size_t *shape,
                                       size_t dim, NumcDType dtype) {
  NumcArray *arr = numc_array_create(ctx, shape, dim, dtype);
  if (arr) memset(arr->data, 0, arr->capacity);
  return arr;
}

extern "C" NumcArray *numc_array_fill(NumcCtx *ctx, const size_t *shape,
                                      size_t dim, NumcDType dtype,
                                      const void *value) {
  if (!value) {
    NUMC_SET_ERROR(NUMC_ERR_NULL, "array_fill: value is NULL");
    return nullptr;
  }
  NumcArray *arr = numc_array_create(ctx, shape, dim, dtype);
  if (!arr) return nullptr;
  char *p = (char *)arr->data;
  for (size_t i = 0; i < arr->size || (dim == 0 && i == 0); i++)
    memcpy(p + i * arr->elem_size, value, arr->elem_size);
  return arr;
}

// Visit every element of `arr` in row-major logical order.
template <class F>
static void for_each_elem(const NumcArray *arr, F f) {
  if (arr->size == 0) return;
  size_t coord[64] = {0};
  size_t dim = arr->dim;
  for (size_t n = 0; n < arr->size; n++) {
    size_t off = 0;
    for (size_t d = 0; d < dim; d++) off += coord[d] * arr->strides[d];
    f(n, off);
    for (size_t d = dim; d-- > 0;) {
      if (++coord[d] < arr->shape[d]) break;
      coord[d] = 0;
    }
  }
}

extern "C" void numc_array_write(NumcArray *arr, const void *data) {
  if (!arr || !data) return;
  if (arr->is_contiguous) {
    memcpy(arr->data, data, arr->capacity);
  } else {
    const char *src = (const char *)data;
    for_each_elem(arr, [&](size_t n, size_t off) {
      memcpy((char *)arr->data + off, src + n * arr->elem_size, arr->elem_size);
    });
  }
  if (arr->residency != kHostOnly) {
    // Keep a resident array's device copy in step with the host write.
    arr->residency = kHostOnly;
    numc_cuda_array_to_device(arr);
  }
}

extern "C" NumcArray *numc_array_copy(const NumcArray *arr) {
  if (!arr) {
    NUMC_SET_ERROR(NUMC_ERR_NULL, "array_copy: arr is NULL");
    return nullptr;
  }
  const bool resident = arr->residency != kHostOnly && arr->dev_base;
  NumcArray *copy = numc_array_create(arr->ctx, arr->shape, arr->dim, arr->dtype);
  if (!copy) return nullptr;
  if (resident) {
    // Copy on the GPU: the copy is resident and contiguous there; the host
    // buffer is copied too only when it is current.
    if (device_copy_contiguous(arr, copy) != 0) return nullptr;
    if (arr->residency == kDeviceOnly) return copy;
    copy->residency = kBoth;
  }
  if (arr->is_contiguous) {
    memcpy(copy->data, arr->data, arr->capacity);
  } else {
    char *dst = (char *)copy->data;
    for_each_elem(arr, [&](size_t n, size_t off) {
      memcpy(dst + n * arr->elem_size, (const char *)arr->data + off, arr->elem_size);
    });
  }
  return copy;
}

extern "C" bool numc_array_is_contiguous(NumcArray *arr) {
  size_t expected = arr->elem_size;
  for (size_t i = arr->dim; i-- > 0;) {
    if (arr->strides[i] != expected) return false;
    expected *= arr->shape[i];
  }
  return true;
}

extern "C" int numc_array_contiguous(NumcArray *arr) {
  if (!arr) {
    NUMC_SET_ERROR(NUMC_ERR_NULL, "array_contiguous: arr is NULL");
    return -1;
  }
  if (numc_array_is_contiguous(arr)) return 0;
  const int was = arr->residency;
  const bool resident = was != kHostOnly && arr->dev_base;
  char *fresh = (char *)arena_alloc(arr->ctx, arr->capacity, kDataAlign, nullptr);
  if (!fresh) {
    NUMC_SET_ERROR(NUMC_ERR_MALLOC, "array_contiguous: failed to allocate %zu bytes",
                   arr->capacity);
    return -1;
  }
  char *fresh_dev = nullptr;
  if (resident) {
    // Re-layout on the GPU into a new device buffer owned by this array.
    NumcArray tmp = *arr;
    tmp.data = fresh;
    tmp.dev_base = nullptr;
    if (device_copy_contiguous(arr, &tmp) != 0) return -1;
    fresh_dev = tmp.dev_base;
  }
  if (!resident || was == kBoth) {
    for_each_elem(arr, [&](size_t n, size_t off) {
      memcpy(fresh + n * arr->elem_size, (const char *)arr->data + off, arr->elem_size);
    });
  }
  arr->data = fresh;
  contiguous_strides(arr->strides, arr->shape, arr->dim, arr->elem_size);
  arr->is_contiguous = true;
  arr->residency = resident ? (was == kBoth ? kBoth : kDeviceOnly) : kHostOnly;
  arr->dev_base = fresh_dev;
  return 0;
}

extern "C" int numc_array_transpose(NumcArray *arr, const size_t *axes) {
  if (!arr || !axes) {
    NUMC_SET_ERROR(NUMC_ERR_NULL, "transpose: NULL argument");
    return -1;
  }
  if (arr->dim > 64) {
    NUMC_SET_ERROR(NUMC_ERR_SHAPE, "transpose: rank %zu above 64", arr->dim);
    return -1;
  }
  size_t sh[64], st[64];
  uint64_t seen = 0;
  for (size_t i = 0; i < arr->dim; i++) {
    size_t ax = axes[i];
    if (ax >= arr->dim) {
      NUMC_SET_ERROR(NUMC_ERR_BOUNDS, "transpose: axis %zu out of range (ndim=%zu)",
                     ax, arr->dim);
      return -1;
    }
    if (seen & (1ull << ax)) {
      NUMC_SET_ERROR(NUMC_ERR_SHAPE, "transpose: repeated axis %zu", ax);
      return -1;
    }
    seen |= 1ull << ax;
    sh[i] = arr->shape[ax];
    st[i] = arr->strides[ax];
  }
  memcpy(arr->shape, sh, arr->dim * sizeof(size_t));
  memcpy(arr->strides, st, arr->dim * sizeof(size_t));
  arr->is_contiguous = numc_array_is_contiguous(arr);
  return 0;
}

extern "C" NumcArray *numc_array_transpose_copy(const NumcArray *arr,
                                                const size_t *axes) {
  if (!arr || !axes) {
    NUMC_SET_ERROR(NUMC_ERR_NULL, "transpose_copy: NULL argument");
    return nullptr;
  }
  NumcArray *copy = numc_array_copy(arr);
  if (!copy || numc_array_transpose(copy, axes) < 0) return nullptr;
  return copy;
}

extern "C" NumcArray *numc_array_slice(const NumcArray *arr, NumcSlice *s) {
  if (!arr || !s) {
    NUMC_SET_ERROR(NUMC_ERR_NULL, "slice: NULL argument");
    return nullptr;
  }
  if (s->axis >= arr->dim) {
    NUMC_SET_ERROR(NUMC_ERR_BOUNDS, "slice: axis %zu out of range (ndim=%zu)",
                   s->axis, arr->dim);
    return nullptr;
  }
  size_t extent = arr->shape[s->axis];
  if (extent == 0) {
    NUMC_SET_ERROR(NUMC_ERR_SHAPE, "slice: zero-sized dimension %zu", s->axis);
    return nullptr;
  }
  if (s->step == 0) s->step = 1;
  if (s->stop == 0 || s->stop > extent) s->stop = extent;
  if (s->start >= extent) {
    NUMC_SET_ERROR(NUMC_ERR_BOUNDS, "slice: start %zu out of range (%zu)", s->start, extent);
    return nullptr;
  }
  if (s->start >= s->stop) {
    NUMC_SET_ERROR(NUMC_ERR_VALUE, "slice: empty range [%zu, %zu)", s->start, s->stop);
    return nullptr;
  }
  NumcArray *v = new_header(arr->ctx, arr->dim);
  if (!v) {
    NUMC_SET_ERROR(NUMC_ERR_MALLOC, "slice: header allocation failed");
    return nullptr;
  }
  memcpy(v->shape, arr->shape, arr->dim * sizeof(size_t));
  memcpy(v->strides, arr->strides, arr->dim * sizeof(size_t));
  size_t byte_off = s->start * arr->strides[s->axis];
  v->data = (char *)arr->data + byte_off;
  v->shape[s->axis] = (s->stop - s->start + s->step - 1) / s->step;
  v->strides[s->axis] = arr->strides[s->axis] * s->step;
  v->elem_size = arr->elem_size;
  v->dtype = arr->dtype;
  size_t n = 1;
  for (size_t d = 0; d < v->dim; d++) n *= v->shape[d];
  v->size = n;
  v->capacity = n * v->elem_size;
  v->is_contiguous = false;
  // A view of a resident array is resident at the matching device offset.
  v->residency = arr->residency;
  v->dev_base = arr->dev_base ? arr->dev_base + byte_off : nullptr;
  return v;
}

extern "C" size_t numc_array_size(const NumcArray *a) { return a->size; }
extern "C" size_t numc_array_capacity(const NumcArray *a) { return a->capacity; }
extern "C" size_t numc_array_elem_size(const NumcArray *a) { return a->elem_size; }
extern "C" size_t numc_array_ndim(const NumcArray *a) { return a->dim; }
extern "C" void numc_array_shape(const NumcArray *a, size_t *shape) {
  memcpy(shape, a->shape, a->dim * sizeof(size_t));
}
extern "C" void numc_array_strides(const NumcArray *a, size_t *strides) {
  memcpy(strides, a->strides, a->dim * sizeof(size_t));
}
extern "C" NumcDType numc_array_dtype(const NumcArray *a) { return a->dtype; }
extern "C" void *numc_array_data(const NumcArray *a) { return a->data; }

// Internal structures of the numc-compatible runtime (host side).
//
// NumcCtx/NumcArray keep numc's public meaning (src/internal.h:31-43 of
// numc): a context owns an arena; an array is a header with shape, BYTE
// strides, element size, dtype and a data pointer into the arena.  The CUDA
// backend adds, per array, an optional device mirror and a residency state,
// and, per context, a stream, a device scratch buffer and the list of device
// allocations so that numc_ctx_restore / numc_ctx_free release them.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include "numc/numc.h"

namespace numc_rt {

constexpr size_t kMaxInlineDims = 8;
constexpr size_t kArenaBlock = 8u << 20;   // numc's NUMC_MAX_MEMORY block
constexpr size_t kDataAlign = 256;         // HBM/TMA friendly (numc: 32)

struct ArenaBlock {
  ArenaBlock *prev;
  char *base;
  size_t cap, used;
  uint64_t seq;        // creation order, for checkpoint comparisons
  bool pinned;         // allocated with cudaHostAlloc
};

// Position in the arena's allocation order: (block seq, offset).
struct ArenaPos {
  uint64_t seq;
  size_t off;
  // Strictly earlier: a header allocated at a checkpoint's own position
  // was made after the checkpoint.
  bool before(const ArenaPos &o) const {
    return seq < o.seq || (seq == o.seq && off < o.off);
  }
};

struct DeviceAlloc {
  void *ptr;
  size_t bytes;
  ArenaPos owner;      // arena position of the owning array header
  char *slab;          // base of the device slab holding it
};

// Device memory of a context's arrays comes from slabs of kDeviceSlab bytes
// (an array larger than that gets a slab of its own), handed out by bump
// allocation in the order the arrays first need device memory.
// numc_ctx_restore rewinds each slab to the end of its last surviving
// array and keeps the slabs for reuse; numc_ctx_free releases them.
constexpr size_t kDeviceSlab = 64u << 20;

struct DeviceSlab {
  char *base;
  size_t cap, used;
};

enum Residency : int {
  kHostOnly = 0,       // host buffer authoritative, no device copy
  kDeviceOnly = 1,     // device copy authoritative, host buffer stale
  kBoth = 2,           // both copies hold the same values
};

}  // namespace numc_rt

struct NumcCtx {
  numc_rt::ArenaBlock *head;
  uint64_t next_seq;
  bool pin_host;                      // page-lock arena blocks (GPU present)
  void *stream;                       // cudaStream_t, created lazily
  void *copy_in, *copy_out;           // copy streams of pipelined matmuls (lazy)
  void *gemm2, *gemm3;                // GEMM streams of pipelined matmuls (lazy)
  int device;                         // device the stream belongs to
  void *scratch;                      // device scratch (staging, splits)
  size_t scratch_bytes;
  std::vector<numc_rt::DeviceAlloc> *dev_allocs;
  std::vector<numc_rt::DeviceSlab> *dev_slabs;
  size_t dev_cur;                     // slab that bump allocation continues in
};

struct NumcArray {
  NumcCtx *ctx;
  void *data;
  size_t *shape, *strides;
  size_t shape_buf[numc_rt::kMaxInlineDims];
  size_t strides_buf[numc_rt::kMaxInlineDims];
  size_t dim, elem_size, size, capacity;
  bool is_contiguous;
  NumcDType dtype;
  // CUDA backend state
  numc_rt::ArenaPos pos;              // where the header sits in the arena
  char *dev_base;                     // device address matching `data`
  int residency;                      // numc_rt::Residency
};

namespace numc_rt {

void *arena_alloc(NumcCtx *ctx, size_t bytes, size_t align, ArenaPos *pos);
ArenaPos arena_pos(const NumcCtx *ctx);

// Byte span [lo, hi) of the elements of a 2-D (or N-D) array relative to
// `data` (strides are non-negative in numc).
size_t array_span_bytes(const NumcArray *arr);

// Backend hooks used by the core (implemented in cuda_backend.cpp).
bool cuda_present();
void *host_alloc_pinned(size_t bytes);
void host_free_pinned(void *p);
void ctx_release_device(NumcCtx *ctx, const ArenaPos *keep_upto);
// Device-resident arrays: copy `src` (any strides) into the contiguous
// device buffer of `dst` (allocated here if it has none), on the GPU; dst
// becomes device-resident (kDeviceOnly).  0 or a NumcErrorCode.
int device_copy_contiguous(const NumcArray *src, NumcArray *dst);

}  // namespace numc_rt

// Element-wise helpers of the matmul path: the gather behind numc_array_copy
// / numc_array_contiguous of device-resident arrays, and numc_linear's bias
// add for the GEMM algorithms whose epilogues do not add it themselves.
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#include "kernels.h"

namespace numc_k {
namespace {

template <typename W>
__global__ void gather_kernel(const W *__restrict__ src, W *__restrict__ dst, DotNd ix,
                              int64_t total) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = e, so = 0;
    for (int d = ix.dim - 1; d >= 0; d--) {
      const int64_t q = rem % ix.shape[d];
      rem /= ix.shape[d];
      so += q * ix.xs[d];
    }
    dst[e] = src[so];
  }
}

template <typename W>
cudaError_t gather_t(const void *src, void *dst, const DotNd &ix, int64_t total,
                     cudaStream_t s) {
  const int64_t blocks = (total + 255) / 256;
  gather_kernel<W><<<(unsigned)(blocks < 8192 ? blocks : 8192), 256, 0, s>>>(
      (const W *)src, (W *)dst, ix, total);
  count_launch();
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_gather(const void *src, void *dst, size_t elem_size, const DotNd &ix,
                          cudaStream_t s) {
  int64_t total = 1;
  for (int d = 0; d < ix.dim; d++) total *= ix.shape[d];
  if (total == 0) return cudaSuccess;
  switch (elem_size) {
  case 1: return gather_t<uint8_t>(src, dst, ix, total, s);
  case 2: return gather_t<uint16_t>(src, dst, ix, total, s);
  case 4: return gather_t<uint32_t>(src, dst, ix, total, s);
  case 8: return gather_t<uint64_t>(src, dst, ix, total, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace numc_k

// ---- numc_linear's bias (unfused form) ------------------------------------------

namespace numc_k {
namespace {

template <typename T>
__global__ void bias_add_kernel(T *__restrict__ c, int64_t rso, int64_t cso,
                                const T *__restrict__ bias, int64_t bs, int64_t M, int64_t N) {
  const int64_t total = M * N;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / N, j = e % N;
    T *p = c + i * rso + j * cso;
    if constexpr (std::is_same<T, float>::value) *p = __fadd_rn(*p, bias[j * bs]);
    else if constexpr (std::is_same<T, double>::value) *p = __dadd_rn(*p, bias[j * bs]);
    else *p = (T)((uint64_t)(int64_t)*p + (uint64_t)(int64_t)bias[j * bs]);
  }
}

template <typename T>
cudaError_t bias_t(const Gemm &g, cudaStream_t s) {
  const int64_t total = g.M * g.N;
  if (total == 0) return cudaSuccess;
  const int64_t blocks = (total + 255) / 256;
  bias_add_kernel<T><<<(unsigned)(blocks < 8192 ? blocks : 8192), 256, 0, s>>>(
      (T *)g.c, g.rso, g.cso, (const T *)g.bias, g.bias_stride, g.M, g.N);
  count_launch();
  return cudaGetLastError();
}

}  // namespace

bool fuses_bias(int algo) {
  return algo == NUMC_CUDA_ALGO_SIMT || algo == NUMC_CUDA_ALGO_SPLIT_BF16 ||
         algo == NUMC_CUDA_ALGO_SPLIT_FP16;
}

cudaError_t launch_bias_add(NumcDType dt, const Gemm &g, cudaStream_t s) {
  switch (dt) {
  case NUMC_DTYPE_INT8: return bias_t<int8_t>(g, s);
  case NUMC_DTYPE_INT16: return bias_t<int16_t>(g, s);
  case NUMC_DTYPE_INT32: return bias_t<int32_t>(g, s);
  case NUMC_DTYPE_INT64: return bias_t<int64_t>(g, s);
  case NUMC_DTYPE_UINT8: return bias_t<uint8_t>(g, s);
  case NUMC_DTYPE_UINT16: return bias_t<uint16_t>(g, s);
  case NUMC_DTYPE_UINT32: return bias_t<uint32_t>(g, s);
  case NUMC_DTYPE_UINT64: return bias_t<uint64_t>(g, s);
  case NUMC_DTYPE_FLOAT32: return bias_t<float>(g, s);
  case NUMC_DTYPE_FLOAT64: return bias_t<double>(g, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace numc_k

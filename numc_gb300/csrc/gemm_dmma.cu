// float64 GEMM on the FP64 tensor path (mma.sync.m8n8k4 f64, "DMMA").
//
// Baseline for the Ozaki kernel.  A 64x64 output tile per CTA of four warps
// (2 x 2), each warp owning a 32x32 sub-tile as 4 x 4 m8n8 accumulators; K
// staged through double-buffered shared memory 16 deep.  Operand loads
// honour arbitrary element strides.  Each DMMA adds a 4-term product into
// the accumulator, so results agree with numc's sequential FMA chain to
// rounding, not bit for bit.
#include <cuda_runtime.h>
#include <cstdint>

#include "kernels.h"

namespace numc_k {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, LDS = BM + 4;
constexpr int kThreads = 128;

__device__ __forceinline__ void dmma_8x8x4(double (&d)[2], double a, double b) {
  asm volatile(
      "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 "
      "{%0, %1}, {%2}, {%3}, {%0, %1};\n"
      : "+d"(d[0]), "+d"(d[1])
      : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(kThreads) dmma_gemm(Gemm g) {
  __shared__ double As[2][BK][LDS];   // [k][m]
  __shared__ double Bs[2][BK][LDS];   // [k][n]
  const double *__restrict__ A = (const double *)g.a;
  const double *__restrict__ B = (const double *)g.b;
  double *__restrict__ C = (double *)g.c;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
  const bool a_kfast = g.csa == 1, b_nfast = g.csb == 1 || g.rsb != 1;
  constexpr int L = BM * BK / kThreads;  // 8 elements per thread per operand

  double ra[L], rb[L];
  auto load = [&](int64_t k0) {
#pragma unroll
    for (int q = 0; q < L; q++) {
      int e = tid + kThreads * q;
      int r = a_kfast ? e / BK : e % BM, kk = a_kfast ? e % BK : e / BM;
      int64_t gi = m0 + r, gk = k0 + kk;
      ra[q] = (gi < g.M && gk < g.K) ? A[gi * g.rsa + gk * g.csa] : 0.0;
      int c = b_nfast ? e % BN : e / BK, kb = b_nfast ? e / BN : e % BK;
      int64_t gj = n0 + c, gkb = k0 + kb;
      rb[q] = (gj < g.N && gkb < g.K) ? B[gkb * g.rsb + gj * g.csb] : 0.0;
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int q = 0; q < L; q++) {
      int e = tid + kThreads * q;
      int r = a_kfast ? e / BK : e % BM, kk = a_kfast ? e % BK : e / BM;
      As[buf][kk][r] = ra[q];
      int c = b_nfast ? e % BN : e / BK, kb = b_nfast ? e / BN : e % BK;
      Bs[buf][kb][c] = rb[q];
    }
  };

  double acc[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j][0] = acc[i][j][1] = 0.0;

  // Fragment coordinates (PTX ISA, mma.m8n8k4 f64): A row = lane/4,
  // A col (k) = lane%4; B row (k) = lane%4, B col = lane/4;
  // C row = lane/4, C cols = 2*(lane%4) + {0,1}.
  const int fr = lane >> 2, fk = lane & 3;
  const int64_t ntiles = (g.K + BK - 1) / BK;
  load(0);
  store(0);
  __syncthreads();
  for (int64_t t = 0; t < ntiles; t++) {
    const int buf = (int)(t & 1);
    if (t + 1 < ntiles) load((t + 1) * BK);
#pragma unroll
    for (int k4 = 0; k4 < BK; k4 += 4) {
      double af[4], bf[4];
#pragma unroll
      for (int i = 0; i < 4; i++) af[i] = As[buf][k4 + fk][wm + i * 8 + fr];
#pragma unroll
      for (int j = 0; j < 4; j++) bf[j] = Bs[buf][k4 + fk][wn + j * 8 + fr];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) dmma_8x8x4(acc[i][j], af[i], bf[j]);
    }
    if (t + 1 < ntiles) store(buf ^ 1);
    __syncthreads();
  }

#pragma unroll
  for (int i = 0; i < 4; i++) {
    int64_t gi = m0 + wm + i * 8 + fr;
    if (gi >= g.M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        int64_t gj = n0 + wn + j * 8 + 2 * fk + h;
        if (gj < g.N) C[gi * g.rso + gj * g.cso] = acc[i][j][h];
      }
  }
}

}  // namespace

cudaError_t launch_dmma(const Gemm &g, cudaStream_t s) {
  if (g.M == 0 || g.N == 0) return cudaSuccess;
  int64_t gx = (g.N + BN - 1) / BN, gy = (g.M + BM - 1) / BM;
  if (gy > 65535) return cudaErrorInvalidConfiguration;
  dmma_gemm<<<dim3((unsigned)gx, (unsigned)gy), kThreads, 0, s>>>(g);
  count_launch();
  return cudaGetLastError();
}

}  // namespace numc_k

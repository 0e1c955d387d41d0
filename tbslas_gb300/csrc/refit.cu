// Node values -> Chebyshev coefficients of every leaf (SetTreeGridValues,
// src/tree/tree_utils.h:500-552): one batched dense contraction
//   C[r][n] = sum_p V[r][p] M[p][n],  r = leaf*dof + l,
// V: rows x np node values (row-major), M: np x nc point-to-coefficient
// matrix, C written into the tree's padded per-leaf coefficient layout.
// FP64; 64x64 output tile per CTA, 16-deep K slices staged in shared memory,
// 4x4 outputs per thread (16 FMAs per 8 shared loads).
#include "internal.h"

namespace tbg {

constexpr int kBM = 64, kBN = 64, kBK = 16;

__global__ void __launch_bounds__(256) k_refit(const double* __restrict__ V,
                                               const double* __restrict__ M, int64_t rows,
                                               int np, int nc, int dof, int64_t stride,
                                               double* __restrict__ C) {
  __shared__ double As[kBK][kBM];
  __shared__ double Bs[kBK][kBN];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t row0 = (int64_t)blockIdx.x * kBM;
  const int col0 = blockIdx.y * kBN;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  for (int k0 = 0; k0 < np; k0 += kBK) {
#pragma unroll
    for (int e = threadIdx.x; e < kBM * kBK; e += 256) {
      const int r = e / kBK, k = e % kBK;
      const int64_t row = row0 + r;
      const int kk = k0 + k;
      As[k][r] = (row < rows && kk < np) ? __ldg(V + row * np + kk) : 0.0;
    }
#pragma unroll
    for (int e = threadIdx.x; e < kBK * kBN; e += 256) {
      const int k = e / kBN, c = e % kBN;
      const int kk = k0 + k, col = col0 + c;
      Bs[k][c] = (kk < np && col < nc) ? __ldg(M + (int64_t)kk * nc + col) : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kBK; ++k) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t row = row0 + ty + 16 * i;
    if (row >= rows) continue;
    const int64_t leaf = row / dof;
    const int l = (int)(row - leaf * dof);
    double* out = C + leaf * stride + (int64_t)l * nc;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int col = col0 + tx + 16 * j;
      if (col < nc) out[col] = acc[i][j];
    }
  }
}

void launch_refit(const double* vals, const double* M, int64_t rows, int np, int nc, int dof,
                  int64_t stride, double* coeff, cudaStream_t s) {
  if (rows <= 0) return;
  dim3 grid((unsigned)((rows + kBM - 1) / kBM), (unsigned)((nc + kBN - 1) / kBN));
  k_refit<<<grid, 256, 0, s>>>(vals, M, rows, np, nc, dof, stride, coeff);
}

}  // namespace tbg

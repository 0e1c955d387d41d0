// Node values -> Chebyshev coefficients of every leaf (SetTreeGridValues,
// src/tree/tree_utils.h:500-552): one batched dense contraction
//   C[r][n] = sum_p V[r][p] M[p][n],  r = leaf*dof + l,
// V: rows x np node values (row-major), M: np x nc point-to-coefficient
// matrix, C written into the tree's padded per-leaf coefficient layout.
// FP64; 64x64 output tile per CTA, 16-deep K slices staged in shared memory,
// 4x4 outputs per thread (16 FMAs per 8 shared loads).
#include "internal.h"

namespace tbg {

// One 64x64 output tile of C = V M (rows x nc), written into the padded
// per-leaf coefficient layout.  Shared by the single-tree and batched kernels.
__device__ __forceinline__ void refit_tile(const double* __restrict__ V,
                                           const double* __restrict__ M, int64_t rows, int np,
                                           int nc, int dof, int64_t stride, double* __restrict__ C,
                                           float2* __restrict__ C2, int64_t row0, int col0) {
  __shared__ double As[kRefitBK][kRefitBM];
  __shared__ double Bs[kRefitBK][kRefitBN];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  for (int k0 = 0; k0 < np; k0 += kRefitBK) {
#pragma unroll
    for (int e = threadIdx.x; e < kRefitBM * kRefitBK; e += 256) {
      const int r = e / kRefitBK, k = e % kRefitBK;
      const int64_t row = row0 + r;
      const int kk = k0 + k;
      As[k][r] = (row < rows && kk < np) ? __ldg(V + row * np + kk) : 0.0;
    }
#pragma unroll
    for (int e = threadIdx.x; e < kRefitBK * kRefitBN; e += 256) {
      const int k = e / kRefitBN, c = e % kRefitBN;
      const int kk = k0 + k, col = col0 + c;
      Bs[k][c] = (kk < np && col < nc) ? __ldg(M + (int64_t)kk * nc + col) : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kRefitBK; ++k) {
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
    const int64_t base = leaf * stride + (int64_t)l * nc;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int col = col0 + tx + 16 * j;
      if (col < nc) {
        C[base + col] = acc[i][j];
        if (C2) {
          const df v = df_from_double(acc[i][j]);
          C2[base + col] = make_float2(v.hi, v.lo);
        }
      }
    }
  }
}

__global__ void __launch_bounds__(256) k_refit(const double* __restrict__ V,
                                               const double* __restrict__ M, int64_t rows,
                                               int np, int nc, int dof, int64_t stride,
                                               double* __restrict__ C, float2* __restrict__ C2) {
  refit_tile(V, M, rows, np, nc, dof, stride, C, C2, (int64_t)blockIdx.x * kRefitBM,
             blockIdx.y * kRefitBN);
}

// Batched refit: one CTA per (problem, row tile, column tile) work item.
__global__ void __launch_bounds__(256) k_batch_refit(const RefitJob* __restrict__ jobs,
                                                     const RefitItem* __restrict__ items) {
  const RefitItem it = items[blockIdx.x];
  const RefitJob j = jobs[it.job];
  refit_tile(j.vals, j.M, j.rows, j.np, j.nc, j.dof, j.stride, j.coeff, j.coeff2,
             (int64_t)it.row_tile * kRefitBM, it.col_tile * kRefitBN);
}

void launch_batch_refit(const RefitJob* jobs, const RefitItem* items, int64_t n_items,
                        cudaStream_t s) {
  if (n_items > 0) k_batch_refit<<<(unsigned)n_items, 256, 0, s>>>(jobs, items);
}

void launch_refit(const double* vals, const double* M, int64_t rows, int np, int nc, int dof,
                  int64_t stride, double* coeff, float2* coeff2, cudaStream_t s) {
  if (rows <= 0) return;
  dim3 grid((unsigned)((rows + kRefitBM - 1) / kRefitBM), (unsigned)((nc + kRefitBN - 1) / kRefitBN));
  k_refit<<<grid, 256, 0, s>>>(vals, M, rows, np, nc, dof, stride, coeff, coeff2);
}

// Split FP64 coefficients into their double-float form.
__global__ void k_split(const double* __restrict__ c, float2* __restrict__ c2, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    const df v = df_from_double(c[i]);
    c2[i] = make_float2(v.hi, v.lo);
  }
}

void launch_split(const double* c, float2* c2, int64_t n, cudaStream_t s) {
  if (n > 0) k_split<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(c, c2, n);
}

}  // namespace tbg

// Batched SL kernels for Chebyshev degrees 12..13.
#include "batch_kernels.cuh"

namespace tbg {
void launch_batch_band_2(const BatchLaunch& a, int grid, int block, cudaStream_t s, int what) {
  launch_band<12, 13>(a, grid, block, s, what);
}
}  // namespace tbg

// Batched SL kernels for Chebyshev degrees 1..8.
#include "batch_kernels.cuh"

namespace tbg {
void launch_batch_band_0(const BatchLaunch& a, int grid, int block, cudaStream_t s, int what) {
  launch_band<1, 8>(a, grid, block, s, what);
}
}  // namespace tbg

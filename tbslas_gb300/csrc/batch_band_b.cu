// Batched SL kernels for Chebyshev degrees 9..11.
#include "batch_kernels.cuh"

namespace tbg {
void launch_batch_band_1(const BatchLaunch& a, int grid, int block, cudaStream_t s, int what) {
  launch_band<9, 11>(a, grid, block, s, what);
}
}  // namespace tbg

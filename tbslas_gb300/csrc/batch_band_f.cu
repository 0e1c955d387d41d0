// Batched SL kernels for Chebyshev degrees 16..16.
#include "batch_kernels.cuh"

namespace tbg {
void launch_batch_band_5(const BatchLaunch& a, int grid, int block, cudaStream_t s, int what) {
  launch_band<16, 16>(a, grid, block, s, what);
}
}  // namespace tbg

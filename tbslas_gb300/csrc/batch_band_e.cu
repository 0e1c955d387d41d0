// Batched SL kernels for Chebyshev degrees 15..15.
#include "batch_kernels.cuh"

namespace tbg {
void launch_batch_band_4(const BatchLaunch& a, int grid, int block, cudaStream_t s, int what) {
  launch_band<15, 15>(a, grid, block, s, what);
}
}  // namespace tbg

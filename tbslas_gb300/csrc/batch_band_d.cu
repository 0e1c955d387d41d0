// Batched SL kernels for Chebyshev degrees 14..14.
#include "batch_kernels.cuh"

namespace tbg {
void launch_batch_band_3(const BatchLaunch& a, int grid, int block, cudaStream_t s, int what) {
  launch_band<14, 14>(a, grid, block, s, what);
}
}  // namespace tbg

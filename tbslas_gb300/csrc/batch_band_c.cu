// Batched SL kernel for Chebyshev degrees 13..16.
#include "batch_kernels.cuh"

namespace tbg {
void launch_batch_band_2(const BatchLaunch& a, int grid, int block, cudaStream_t s) {
  k_batch_semilag<13, 16><<<grid, block, 0, s>>>(a);
}
}  // namespace tbg

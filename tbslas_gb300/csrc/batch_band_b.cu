// Batched SL kernel for Chebyshev degrees 9..12.
#include "batch_kernels.cuh"

namespace tbg {
void launch_batch_band_1(const BatchLaunch& a, int grid, int block, cudaStream_t s) {
  k_batch_semilag<9, 12><<<grid, block, 0, s>>>(a);
}
}  // namespace tbg

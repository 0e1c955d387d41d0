// Batched SL kernels for Chebyshev degrees 9..11.
#include "batch_kernels.cuh"

namespace tbg {
void launch_batch_band_1(const BatchLaunch& a, int grid, int block, cudaStream_t s, bool fix) {
  if (fix)
    k_batch_fix<9, 11><<<grid, 128, 0, s>>>(a);
  else
    k_batch_semilag<9, 11><<<grid, block, 0, s>>>(a);
}
}  // namespace tbg

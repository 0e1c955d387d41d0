// Batched SL kernels for Chebyshev degrees 12..13.
#include "batch_kernels.cuh"

namespace tbg {
void launch_batch_band_2(const BatchLaunch& a, int grid, int block, cudaStream_t s, bool fix) {
  if (fix)
    k_batch_fix<12, 13><<<grid, 128, 0, s>>>(a);
  else
    k_batch_semilag<12, 13><<<grid, block, 0, s>>>(a);
}
}  // namespace tbg

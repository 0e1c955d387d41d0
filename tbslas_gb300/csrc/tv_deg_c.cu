// Time-dependent velocity step kernels for Chebyshev degrees 14..16.
#include "tv_kernels.cuh"

namespace tbg {
void register_tv_c(TvFn* table) {
  table[14] = &launch_semilag_tv<15>;
  table[15] = &launch_semilag_tv<16>;
  table[16] = &launch_semilag_tv<17>;
}
}  // namespace tbg

// Time-dependent velocity step kernels for Chebyshev degrees 10..13.
#include "tv_kernels.cuh"

namespace tbg {
void register_tv_b(TvFn* table) {
  table[10] = &launch_semilag_tv<11>;
  table[11] = &launch_semilag_tv<12>;
  table[12] = &launch_semilag_tv<13>;
  table[13] = &launch_semilag_tv<14>;
}
}  // namespace tbg

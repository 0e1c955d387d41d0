// BDF2 two-backtrace step kernels for Chebyshev degrees 10..16.
#include "bdf2_kernels.cuh"

namespace tbg {
void register_bdf2_b(Bdf2Fn* table) {
  table[10] = &launch_semilag_bdf2<11>;
  table[11] = &launch_semilag_bdf2<12>;
  table[12] = &launch_semilag_bdf2<13>;
  table[13] = &launch_semilag_bdf2<14>;
  table[14] = &launch_semilag_bdf2<15>;
  table[15] = &launch_semilag_bdf2<16>;
  table[16] = &launch_semilag_bdf2<17>;
}
}  // namespace tbg

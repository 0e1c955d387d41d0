// BDF2 two-backtrace step kernels for Chebyshev degrees 1..9.
#include "bdf2_kernels.cuh"

namespace tbg {
void register_bdf2_a(Bdf2Fn* table) {
  table[1] = &launch_semilag_bdf2<2>;
  table[2] = &launch_semilag_bdf2<3>;
  table[3] = &launch_semilag_bdf2<4>;
  table[4] = &launch_semilag_bdf2<5>;
  table[5] = &launch_semilag_bdf2<6>;
  table[6] = &launch_semilag_bdf2<7>;
  table[7] = &launch_semilag_bdf2<8>;
  table[8] = &launch_semilag_bdf2<9>;
  table[9] = &launch_semilag_bdf2<10>;
}
}  // namespace tbg

// Adjoint kernels for Chebyshev degrees 6..8.
#include "adjoint_df.cuh"

namespace tbg {
void register_adjoint_b(AdjFn* a, AdjDfFn* d) {
  register_adjoint_degree<7>(a, d);  // q = 6
  register_adjoint_degree<8>(a, d);  // q = 7
  register_adjoint_degree<9>(a, d);  // q = 8
}
}  // namespace tbg

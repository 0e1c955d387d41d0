// Adjoint kernels for Chebyshev degrees 6..8.
#include "adjoint_df.cuh"

namespace tbg {
void register_adjoint_b(AdjFn* a, AdjDfFn* d, JacStepFn* j) {
  register_adjoint_degree<7>(a, d, j);  // q = 6
  register_adjoint_degree<8>(a, d, j);  // q = 7
  register_adjoint_degree<9>(a, d, j);  // q = 8
}
}  // namespace tbg

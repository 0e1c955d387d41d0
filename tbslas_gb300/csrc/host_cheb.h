// Host-side Chebyshev helpers (new_nodes / GetPt2CoeffMatrix).
#pragma once

#include <vector>

namespace tbg {
std::vector<double> cheb_nodes_1d(int q);
std::vector<double> cheb_nodes_3d(int q);
std::vector<double> pt2coeff_matrix(int q);
std::vector<double> refit_factors(int q);
}  // namespace tbg

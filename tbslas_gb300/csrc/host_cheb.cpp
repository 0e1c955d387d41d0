// Host-side Chebyshev helpers: the stretched Chebyshev nodes and the
// point-to-coefficient matrix of the triangular (total-degree) basis.
#include <omp.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "host_cheb.h"

namespace tbg {

// 1-D nodes x_i = -cos((i+1/2)pi/d) / cos(pi/(2d)) / 2 + 1/2: the end nodes
// sit on 0 and 1 so neighbouring leaves share face nodes.  Same expression
// and evaluation order as tbslas::new_nodes, src/utils/cheb.h:50-58.
std::vector<double> cheb_nodes_1d(int q) {
  const int d = q + 1;
  const double pi = 3.14159265358979323846264338327950288;
  std::vector<double> x(d);
  double scal = 1.0 / std::cos(0.5 * pi / d);
  for (int i = 0; i < d; i++) x[i] = -std::cos((i + (double)0.5) * pi / d) * scal * 0.5 + 0.5;
  return x;
}

// (q+1)^3 x 3 tensor nodes, x fastest (src/utils/cheb.h:60-67).
std::vector<double> cheb_nodes_3d(int q) {
  const int d = q + 1;
  std::vector<double> x = cheb_nodes_1d(q);
  std::vector<double> y((size_t)d * d * d * 3);
  for (int k = 0; k < d; k++)
    for (int j = 0; j < d; j++)
      for (int i = 0; i < d; i++) {
        const size_t p = (size_t)i + d * (j + (size_t)d * k);
        y[3 * p + 0] = x[i];
        y[3 * p + 1] = x[j];
        y[3 * p + 2] = x[k];
      }
  return y;
}

static void cheb_poly_1(int q, double xi, double* T) {
  const bool ok = std::fabs(xi) <= 1;
  double x = ok ? xi : 0;
  double y0 = ok ? 1.0 : 0;
  T[0] = y0;
  if (q == 0) return;
  T[1] = x;
  double y1 = x;
  x *= 2;
  for (int i = 2; i <= q; i++) {
    double y2 = x * y1 - y0;
    T[i] = y2;
    y0 = y1;
    y1 = y2;
  }
}

// M = pinv(V)^T, V[p][n] = T_i(z_p) T_j(y_p) T_k(x_p) at the nodes mapped to
// [-1,1], columns in the triangular i/j/k order the evaluator reads
// (GetPt2CoeffMatrix, src/utils/cheb.h:166-196).  pinv via Householder QR:
// V = Q R, M = Q_1 R^{-T}.  Column-major work arrays; reflector updates and
// the triangular solves are parallel over columns / rows.
std::vector<double> pt2coeff_matrix(int q) {
  const int d = q + 1;
  const long m = (long)d * d * d;
  const long n = (long)d * (d + 1) * (d + 2) / 6;
  std::vector<double> nodes = cheb_nodes_3d(q);
  std::vector<double> A((size_t)m * n);  // column-major V
  {
    std::vector<double> tx(d), ty(d), tz(d);
    for (long p = 0; p < m; p++) {
      cheb_poly_1(q, nodes[3 * p + 0] * 2.0 - 1.0, tx.data());
      cheb_poly_1(q, nodes[3 * p + 1] * 2.0 - 1.0, ty.data());
      cheb_poly_1(q, nodes[3 * p + 2] * 2.0 - 1.0, tz.data());
      long c = 0;
      for (int i = 0; i < d; i++)
        for (int j = 0; i + j < d; j++)
          for (int k = 0; i + j + k < d; k++) A[(size_t)c++ * m + p] = tz[i] * ty[j] * tx[k];
    }
  }
  std::vector<double> beta(n);
  for (long j = 0; j < n; j++) {
    double* a = A.data() + (size_t)j * m;
    double norm2 = 0;
    for (long i = j; i < m; i++) norm2 += a[i] * a[i];
    const double norm = std::sqrt(norm2);
    const double alpha = a[j] >= 0 ? -norm : norm;
    const double v0 = a[j] - alpha;
    // v = (a[j:] - alpha e_0) normalised so v[0] = 1; beta = -v0/alpha.
    const double vnorm2 = norm2 - a[j] * a[j] + v0 * v0;
    beta[j] = vnorm2 > 0 ? 2.0 * v0 * v0 / vnorm2 : 0.0;
    for (long i = j + 1; i < m; i++) a[i] /= (v0 != 0 ? v0 : 1.0);
    a[j] = alpha;  // R[j][j]
#pragma omp parallel for schedule(static)
    for (long c = j + 1; c < n; c++) {
      double* b = A.data() + (size_t)c * m;
      double s = b[j];
      for (long i = j + 1; i < m; i++) s += a[i] * b[i];
      s *= beta[j];
      b[j] -= s;
      for (long i = j + 1; i < m; i++) b[i] -= s * a[i];
    }
  }
  // Q1 = H_0 ... H_{n-1} [I; 0], column-major m x n.
  std::vector<double> Q((size_t)m * n, 0.0);
  for (long c = 0; c < n; c++) Q[(size_t)c * m + c] = 1.0;
#pragma omp parallel for schedule(static)
  for (long c = 0; c < n; c++) {
    double* b = Q.data() + (size_t)c * m;
    for (long j = n - 1; j >= 0; j--) {
      const double* a = A.data() + (size_t)j * m;
      double s = b[j];
      for (long i = j + 1; i < m; i++) s += a[i] * b[i];
      s *= beta[j];
      b[j] -= s;
      for (long i = j + 1; i < m; i++) b[i] -= s * a[i];
    }
  }
  // Row r of M solves R M[r]^T = Q1[r]^T (R upper triangular: A[c*m + j], j <= c).
  std::vector<double> M((size_t)m * n);
#pragma omp parallel for schedule(static)
  for (long r = 0; r < m; r++) {
    double* out = M.data() + (size_t)r * n;
    for (long c = n - 1; c >= 0; c--) {
      double s = Q[(size_t)c * m + r];
      for (long k = c + 1; k < n; k++) s -= A[(size_t)k * m + c] * out[k];
      out[c] = s / A[(size_t)c * m + c];
    }
  }
  return M;
}

}  // namespace tbg

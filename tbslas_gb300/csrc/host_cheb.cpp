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

// Factors of the separable refit.  A[a][k] = T_k(xi_a) at the D = q+1
// stretched nodes (xi_a = 2 x_a - 1, as pt2coeff_matrix maps them) has the QR
// factorisation A = Q R.  The 3-D tensor basis on the tensor grid is
// A (x) A (x) A, so the least-squares fit onto the total-degree triangle T =
// {i+j+k < D} that M = pinv(V)^T computes is
//   c = [ (R^-1)^(x)3 ext_T( [ (Q^T)^(x)3 f ]_T ) ]_T :
// with U = R (x) R (x) R the objective is |U (S c - c_full)|^2; U is upper
// triangular on every axis and T is closed downwards, so U's rows outside T
// see only coefficients outside T and the rows in T are solved exactly.
// Returned row-major, 4 D x D blocks: Q[a][k], Q^T, R^-1[k'][k], R^-T.
// Householder QR in long double.
std::vector<double> refit_factors(int q) {
  const int d = q + 1;
  std::vector<double> x = cheb_nodes_1d(q);
  std::vector<long double> A((size_t)d * d), Q((size_t)d * d, 0.0L);
  for (int a = 0; a < d; a++) {
    const long double xi = (long double)(x[a] * 2.0 - 1.0);
    long double t0 = 1.0L, t1 = xi;
    for (int k = 0; k < d; k++) {
      long double t;
      if (k == 0) {
        t = t0;
      } else if (k == 1) {
        t = t1;
      } else {
        t = 2.0L * xi * t1 - t0;
        t0 = t1;
        t1 = t;
      }
      A[(size_t)a * d + k] = t;
    }
  }
  for (int i = 0; i < d; i++) Q[(size_t)i * d + i] = 1.0L;
  // A <- H_{d-1} ... H_0 A = R, Q <- Q H_0 ... H_{d-1}
  std::vector<long double> v(d);
  for (int j = 0; j < d; j++) {
    long double norm2 = 0.0L;
    for (int i = j; i < d; i++) norm2 += A[(size_t)i * d + j] * A[(size_t)i * d + j];
    const long double norm = std::sqrt(norm2);
    if (norm == 0.0L) continue;
    const long double ajj = A[(size_t)j * d + j];
    const long double alpha = ajj >= 0 ? -norm : norm;
    long double vn2 = 0.0L;
    for (int i = 0; i < d; i++) v[i] = i < j ? 0.0L : A[(size_t)i * d + j];
    v[j] -= alpha;
    for (int i = j; i < d; i++) vn2 += v[i] * v[i];
    if (vn2 == 0.0L) continue;
    for (int c = 0; c < d; c++) {  // A = (I - 2 v v^T / vn2) A
      long double s = 0.0L;
      for (int i = j; i < d; i++) s += v[i] * A[(size_t)i * d + c];
      s *= 2.0L / vn2;
      for (int i = j; i < d; i++) A[(size_t)i * d + c] -= s * v[i];
    }
    for (int r = 0; r < d; r++) {  // Q = Q (I - 2 v v^T / vn2)
      long double s = 0.0L;
      for (int i = j; i < d; i++) s += Q[(size_t)r * d + i] * v[i];
      s *= 2.0L / vn2;
      for (int i = j; i < d; i++) Q[(size_t)r * d + i] -= s * v[i];
    }
  }
  // R^-1 by back substitution (R = upper triangle of A)
  std::vector<long double> Ri((size_t)d * d, 0.0L);
  for (int c = 0; c < d; c++) {
    for (int r = c; r >= 0; r--) {
      long double s = r == c ? 1.0L : 0.0L;
      for (int k = r + 1; k <= c; k++) s -= A[(size_t)r * d + k] * Ri[(size_t)k * d + c];
      Ri[(size_t)r * d + c] = s / A[(size_t)r * d + r];
    }
  }
  const size_t dd = (size_t)d * d;
  std::vector<double> out(4 * dd);
  for (int r = 0; r < d; r++)
    for (int c = 0; c < d; c++) {
      out[0 * dd + (size_t)r * d + c] = (double)Q[(size_t)r * d + c];
      out[1 * dd + (size_t)r * d + c] = (double)Q[(size_t)c * d + r];
      out[2 * dd + (size_t)r * d + c] = (double)Ri[(size_t)r * d + c];
      out[3 * dd + (size_t)r * d + c] = (double)Ri[(size_t)c * d + r];
    }
  return out;
}

}  // namespace tbg

// Stand-ins for the PVFMM names the tbslas headers of the SL path use, so
// those headers compile here from the reference's own sources.  PVFMM is not
// vendored; every routine below is this project's restatement of the
// published algorithm, the same one the oracle (oracle/oracle.cpp) restates:
//  - COORD_DIM 3; MAX_DEPTH 30 (the oracle's key resolution);
//  - Vector / Matrix: owning or wrapping dense arrays, row-major matrices;
//    Matrix::GEMM is the plain triple loop; Matrix::pinv is the least-squares
//    pseudo-inverse of a full-column-rank matrix by Householder QR;
//  - MortonId: coordinates quantised to MAX_DEPTH bits per axis, bits
//    interleaved (z, y, x from most to least significant inside a level),
//    ordered by the interleaved key, ties by depth; a point outside [0,1)^3
//    (or NaN) orders after every leaf, as in the oracle;
//  - cheb_poly: T_0..T_q by the three-term recurrence, rows of zeros for
//    |x| > 1; cheb_eval: the total-degree basis T_i(z) T_j(y) T_k(x) at one
//    point, i outer, j, k inner (the order vec_eval reads coefficients);
//  - single-rank sorting and scattering (one process, nothing to exchange).
//
// TEST INFRASTRUCTURE ONLY: compiled with the reference's headers into
// oracle/_ref by oracle/build_ref.py; nothing in the product uses it.
#pragma once
#include <omp.h>

#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <mpi.h>

#define COORD_DIM 3
#define MAX_DEPTH 30

namespace pvfmm {

enum BoundaryType { FreeSpace = 0, Periodic = 1 };

template <class T>
inline T cos(T x) { return std::cos(x); }
template <class T>
inline T sin(T x) { return std::sin(x); }
template <class T>
inline T sqrt(T x) { return std::sqrt(x); }
template <class T>
inline T const_pi() { return (T)3.14159265358979323846264338327950288L; }
template <class T>
inline T pow(T b, int e) {
  T r = 1;
  for (int i = 0; i < e; ++i) r *= b;
  return r;
}

namespace mem {
template <class T>
struct TypeTraits {
  static uintptr_t ID() {
    static char tag;
    return (uintptr_t)&tag;
  }
};
}  // namespace mem

// Scalar forms of the vector-intrinsic helpers vec_eval is written with
// (the driver selects the scalar path, Vec = Real).
template <class V>
inline V zero_intrin() { return (V)0; }
template <class V, class T>
inline V set_intrin(const T& a) { return (V)a; }
template <class V>
inline V load_intrin(const V* p) { return *p; }
template <class V>
inline void store_intrin(V* p, const V& v) { *p = v; }
template <class V>
inline V add_intrin(const V& a, const V& b) { return a + b; }
template <class V>
inline V mul_intrin(const V& a, const V& b) { return a * b; }

template <class T>
class Vector {
 public:
  Vector() {}
  explicit Vector(size_t n) { Resize(n); }
  Vector(size_t n, T* p, bool own = true) {
    if (own) {
      buf_.assign(p, p + n);
      data_ = buf_.data();
    } else {
      data_ = p;
    }
    dim_ = n;
  }
  Vector(const Vector& v) { *this = v; }
  Vector& operator=(const Vector& v) {
    buf_.assign(v.data_, v.data_ + v.dim_);
    data_ = buf_.data();
    dim_ = v.dim_;
    return *this;
  }
  void Resize(size_t n) {
    if (data_ != buf_.data() && data_) {
      std::vector<T> b(data_, data_ + std::min(n, dim_));
      buf_.swap(b);
    }
    buf_.resize(n);
    data_ = buf_.data();
    dim_ = n;
  }
  void ReInit(size_t n, T* p = nullptr, bool own = true) {
    if (p) {
      *this = Vector(n, p, own);
    } else {
      buf_.assign(n, T());
      data_ = buf_.data();
      dim_ = n;
    }
  }
  void SetZero() { std::fill(data_, data_ + dim_, T()); }
  size_t Dim() const { return dim_; }
  T& operator[](size_t i) { return data_[i]; }
  const T& operator[](size_t i) const { return data_[i]; }

 private:
  std::vector<T> buf_;
  T* data_ = nullptr;
  size_t dim_ = 0;
};

template <class T>
class Matrix {
 public:
  Matrix() {}
  Matrix(size_t d0, size_t d1, T* p = nullptr, bool own = true) { ReInit(d0, d1, p, own); }
  Matrix(const Matrix& m) { *this = m; }
  Matrix& operator=(const Matrix& m) {
    d0_ = m.d0_;
    d1_ = m.d1_;
    buf_.assign(m.data_, m.data_ + d0_ * d1_);
    data_ = buf_.data();
    return *this;
  }
  void ReInit(size_t d0, size_t d1, T* p = nullptr, bool own = true) {
    d0_ = d0;
    d1_ = d1;
    if (p && !own) {
      buf_.clear();
      data_ = p;
    } else if (p) {
      buf_.assign(p, p + d0 * d1);
      data_ = buf_.data();
    } else {
      buf_.assign(d0 * d1, T());
      data_ = buf_.data();
    }
  }
  void Resize(size_t d0, size_t d1) { ReInit(d0, d1); }
  void SetZero() { std::fill(data_, data_ + d0_ * d1_, T()); }
  size_t Dim(int i) const { return i == 0 ? d0_ : d1_; }
  T* operator[](size_t i) { return data_ + i * d1_; }
  const T* operator[](size_t i) const { return data_ + i * d1_; }
  Matrix Transpose() const {
    Matrix t(d1_, d0_);
    for (size_t i = 0; i < d0_; ++i)
      for (size_t j = 0; j < d1_; ++j) t[j][i] = (*this)[i][j];
    return t;
  }
  // M_r = A_r * B (plain triple loop, k ascending)
  static void GEMM(Matrix& M_r, const Matrix& A, const Matrix& B, T beta = 0.0) {
    assert(A.d1_ == B.d0_ && M_r.d0_ == A.d0_ && M_r.d1_ == B.d1_);
    for (size_t i = 0; i < A.d0_; ++i)
      for (size_t j = 0; j < B.d1_; ++j) {
        T s = 0;
        for (size_t k = 0; k < A.d1_; ++k) s += A[i][k] * B[k][j];
        M_r[i][j] = beta * M_r[i][j] + s;
      }
  }
  // Least-squares pseudo-inverse (d1 x d0) of a full-column-rank d0 x d1
  // matrix: Householder QR on the columns (kept contiguous), Q's first d1
  // columns formed explicitly, then R X = Q1^T by back substitution.
  Matrix pinv() const {
    const size_t m = d0_, n = d1_;
    std::vector<std::vector<T>> col(n, std::vector<T>(m)), q(n, std::vector<T>(m, T(0)));
    for (size_t i = 0; i < m; ++i)
      for (size_t k = 0; k < n; ++k) col[k][i] = (*this)[i][k];
    std::vector<T> tau(n), diag(n);
    for (size_t k = 0; k < n; ++k) {
      std::vector<T>& v = col[k];
      T nrm = 0;
      for (size_t i = k; i < m; ++i) nrm += v[i] * v[i];
      nrm = std::sqrt(nrm);
      const T alpha = v[k] > 0 ? -nrm : nrm;
      v[k] -= alpha;
      T vv = 0;
      for (size_t i = k; i < m; ++i) vv += v[i] * v[i];
      tau[k] = vv > 0 ? 2 / vv : 0;
      diag[k] = alpha;
      for (size_t j = k + 1; j < n; ++j) {
        std::vector<T>& c = col[j];
        T s = 0;
        for (size_t i = k; i < m; ++i) s += v[i] * c[i];
        s *= tau[k];
        for (size_t i = k; i < m; ++i) c[i] -= s * v[i];
      }
    }
    // Q1 = H_0 ... H_{n-1} [I_n; 0], column by column
    for (size_t j = 0; j < n; ++j) {
      std::vector<T>& e = q[j];
      e[j] = 1;
      for (size_t k = n; k-- > 0;) {
        const std::vector<T>& v = col[k];
        T s = 0;
        for (size_t i = k; i < m; ++i) s += v[i] * e[i];
        s *= tau[k];
        for (size_t i = k; i < m; ++i) e[i] -= s * v[i];
      }
    }
    // R X = Q1^T: row kk of X from the rows below it (R's strict upper part
    // is col[j][kk], j > kk)
    Matrix p(n, m);
    for (size_t kk = n; kk-- > 0;) {
      T* x = p[kk];
      for (size_t i = 0; i < m; ++i) x[i] = q[kk][i];
      for (size_t j = kk + 1; j < n; ++j) {
        const T r = col[j][kk];
        const T* xj = p[j];
        for (size_t i = 0; i < m; ++i) x[i] -= r * xj[i];
      }
      for (size_t i = 0; i < m; ++i) x[i] /= diag[kk];
    }
    return p;
  }

 private:
  std::vector<T> buf_;
  T* data_ = nullptr;
  size_t d0_ = 0, d1_ = 0;
};

class MortonId {
 public:
  MortonId() {}
  MortonId(double x, double y, double z, int depth = MAX_DEPTH) : depth_(depth) {
    const double s = (double)(1UL << MAX_DEPTH);
    const double c[3] = {x, y, z};
    uint64_t q[3];
    for (int k = 0; k < 3; ++k) {
      if (!(c[k] >= 0.0 && c[k] < 1.0)) {
        key_ = ~(unsigned __int128)0;
        return;
      }
      q[k] = (uint64_t)std::floor(c[k] * s);
    }
    key_ = 0;
    for (int b = MAX_DEPTH - 1; b >= 0; --b)
      key_ = (key_ << 3) | (unsigned __int128)((((q[2] >> b) & 1) << 2) |
                                               (((q[1] >> b) & 1) << 1) | ((q[0] >> b) & 1));
  }
  int GetDepth() const { return depth_; }
  bool operator<(const MortonId& o) const {
    return key_ < o.key_ || (key_ == o.key_ && depth_ < o.depth_);
  }
  bool operator>(const MortonId& o) const { return o < *this; }
  bool operator<=(const MortonId& o) const { return !(o < *this); }
  bool operator>=(const MortonId& o) const { return !(*this < o); }
  bool operator==(const MortonId& o) const { return key_ == o.key_ && depth_ == o.depth_; }
  bool operator!=(const MortonId& o) const { return !(*this == o); }

 private:
  unsigned __int128 key_ = 0;
  int depth_ = 0;
};

namespace par {
template <class T>
struct Mpi_datatype {
  static MPI_Datatype value() { return sizeof(T); }
};
template <class A, class B>
struct SortPair {
  A key;
  B data;
  bool operator<(const SortPair& o) const { return key < o.key; }
};
// One rank: the scatter index is the identity and nothing moves.
template <class T>
void SortScatterIndex(const Vector<T>& key, Vector<size_t>& idx, const MPI_Comm&,
                      const T* = nullptr) {
  idx.Resize(key.Dim());
  for (size_t i = 0; i < idx.Dim(); ++i) idx[i] = i;
}
template <class T>
void ScatterForward(Vector<T>&, const Vector<size_t>&, const MPI_Comm&) {}
template <class T>
void ScatterReverse(Vector<T>&, const Vector<size_t>&, const MPI_Comm&, size_t = 0) {}
template <class T>
void HyperQuickSort(const Vector<T>& in, Vector<T>& out, const MPI_Comm&) {
  out = in;
  std::sort(&out[0], &out[0] + out.Dim());
}
template <class T>
void HyperQuickSort(const std::vector<T>& in, std::vector<T>& out, const MPI_Comm&) {
  out = in;
  std::sort(out.begin(), out.end());
}
template <class T>
void partitionW(Vector<T>&, long long*, const MPI_Comm&) {}
}  // namespace par

namespace omp_par {
template <class It>
void merge_sort(It a, It b) {
  std::stable_sort(a, b);
}
}  // namespace omp_par

// T_0..T_q at n points, out[k * n + j]; |x| > 1 (or NaN) gives zero rows.
template <class T>
void cheb_poly(int q, const T* in, int n, T* out) {
  for (int j = 0; j < n; ++j) {
    const bool ok = std::fabs(in[j]) <= 1;
    T x = ok ? in[j] : 0;
    T y0 = ok ? 1 : 0;
    out[j] = y0;
    if (q == 0) continue;
    out[j + n] = x;
    T y1 = x;
    x *= 2;
    for (int i = 2; i <= q; ++i) {
      const T y2 = x * y1 - y0;
      out[i * n + j] = y2;
      y0 = y1;
      y1 = y2;
    }
  }
}

// The total-degree basis at one point (coord in [-1,1]^3, x first):
// out[idx] = T_i(z) T_j(y) T_k(x), i outer, j, k inner, i + j + k <= q.
template <class T>
void cheb_eval(int q, const T* coord, T* out, T* buff) {
  const int d = q + 1;
  T* px = buff;
  T* py = buff + d;
  T* pz = buff + 2 * d;
  cheb_poly(q, coord + 0, 1, px);
  cheb_poly(q, coord + 1, 1, py);
  cheb_poly(q, coord + 2, 1, pz);
  long idx = 0;
  for (int i = 0; i < d; ++i)
    for (int j = 0; i + j < d; ++j)
      for (int k = 0; i + j + k < d; ++k) out[idx++] = pz[i] * py[j] * px[k];
}

template <class T>
std::vector<T> cheb_nodes(int, int);
template <class T, class Y>
void cheb_approx(T*, int, int, T*, T* = nullptr);
template <class T>
void cheb_curl(T*, int, T*);

}  // namespace pvfmm

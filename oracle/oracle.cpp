// Oracle: CPU restatement of the tbslas semi-Lagrangian advection path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product (tbslas_gb300/) links,
// loads or calls this file.  It is used by tests/, by __graft_entry__.smoke()
// and by bench.py's CPU-baseline leg, always as the checker or the timed CPU
// reference, never as the thing measured on the GPU.
//
// Parity status: pinned.  The reference's SL-path sources (traj.inc,
// semilag.inc, tree_functor.h, tree_utils.h, tree_semilag.h, cheb.h) compile
// here against stand-ins for PVFMM and MPI (oracle/ref_stubs/, recipe
// oracle/build_ref.py, library oracle/_ref/libref.so); tests/test_ref_pin.py
// and the fixtures tests/golden/ref_*.npz written from that library check
// this restatement against it: Chebyshev nodes, grid points, tree
// evaluation, trajectories and the tricubic interpolant bit for bit, the
// in-situ step to the pseudo-inverse's and GEMM's rounding.  PVFMM's own
// routines (MortonId, cheb_poly, cheb_eval, pinv, GEMM) are restated in both
// places from their published algorithms; PVFMM is not vendored.  The
// analytic known-answer tests of tests/test_oracle.py pin the physics.
//
// Every routine cites the reference file:line it restates (paths relative to
// the tbslas source tree).  PVFMM routines that the reference calls but that
// are not in the tree (cheb_poly, MortonId, cheb_eval/pinv, GEMM) are restated
// from their published algorithms and named where used.
//
// Build: g++ -O3 -fopenmp -ffp-contract=off -fPIC -shared (see oracle/build.py)

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace orc {

typedef double Real;

// Forward-mode dual number (value, directional derivative) for the
// dual-number gradient of the SL step: the tree path below is templated on
// its number type R, and R = Dual carries d/ds of every quantity along one
// input direction.  Value parts are computed with exactly the operations of
// R = double, so they reproduce the double oracle bit for bit; leaf choices
// and the |x|>1 rule use value parts only (the derivative of the discrete
// map with leaf assignment held fixed).
struct Dual {
  double v, d;
};
static inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
static inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
static inline Dual operator-(Dual a) { return {-a.v, -a.d}; }
static inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.v * b.d + a.d * b.v}; }
static inline Dual operator+(Dual a, double b) { return {a.v + b, a.d}; }
static inline Dual operator-(Dual a, double b) { return {a.v - b, a.d}; }
static inline Dual operator*(Dual a, double b) { return {a.v * b, a.d * b}; }
static inline Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
static inline Dual& operator*=(Dual& a, double b) { a = a * b; return a; }
static inline double val(double x) { return x; }
static inline double val(Dual x) { return x.v; }
template <class R> static inline R mk(double v) { return R(v); }
template <> inline Dual mk<Dual>(double v) { return Dual{v, 0.0}; }
static inline double fmaR(double a, double b, double c) { return std::fma(a, b, c); }
static inline Dual fmaR(Dual a, Dual b, Dual c) {
  return {std::fma(a.v, b.v, c.v), a.v * b.d + a.d * b.v + c.d};
}
static inline Dual fmaR(double a, Dual b, Dual c) {
  return {std::fma(a, b.v, c.v), a * b.d + c.d};
}

// ---------------------------------------------------------------------------
// Chebyshev nodes stretched onto [0,1], x fastest.
// Restates tbslas::new_nodes, src/utils/cheb.h:41-67.
static std::vector<Real> new_nodes(int deg, int dim) {
  const int d = deg + 1;
  std::vector<Real> x(d);
  const Real pi = 3.14159265358979323846264338327950288;
  Real scal = 1.0 / std::cos(0.5 * pi / d);
  for (int i = 0; i < d; i++)
    x[i] = -std::cos((i + (Real)0.5) * pi / d) * scal * 0.5 + 0.5;
  long n1 = 1;
  for (int i = 0; i < dim; i++) n1 *= d;
  std::vector<Real> y(n1 * dim);
  long n2 = 1;
  for (int i = 0; i < dim; i++) {
    for (long j = 0; j < n1; j++) y[j * dim + i] = x[(j / n2) % d];
    n2 *= d;
  }
  return y;
}

// ---------------------------------------------------------------------------
// Chebyshev polynomials T_0..T_q at n points, row k = T_k.  Points with
// |x| > 1 (or NaN) get all-zero rows.  Restates pvfmm::cheb_poly as called at
// src/tree/tree_functor.h:328-330 (three-term recurrence, 2x*T_{k-1}-T_{k-2}).
//
// Multiply-adds are written as explicit fused multiply-adds (std::fma)
// exactly where g++ -O3 -ffp-contract=fast for an FMA target (with a tuning
// that fuses accumulation chains) fuses them when it compiles the
// reference's own sources -- the recurrence, vec_eval's accumulations, the
// RK2 updates, fast_interp's accumulation -- so the oracle's rounding is
// fixed and the same on every host.  tests/test_ref_pin.py checks the oracle
// bit for bit against that build of the reference (oracle/_ref, recipe
// oracle/build_ref.py).
template <class R>
static void cheb_poly(int q, const R* in, int n, R* out) {
  for (int j = 0; j < n; j++) {
    const bool ok = std::fabs(val(in[j])) <= 1;
    R x = ok ? in[j] : mk<R>(0);
    R y0 = mk<R>(ok ? 1.0 : 0.0);
    out[j] = y0;
    if (q == 0) continue;
    out[j + n] = x;
    R y1 = x;
    x *= 2;
    for (int i = 2; i <= q; i++) {
      R y2 = fmaR(x, y1, -y0);
      out[i * n + j] = y2;
      y0 = y1;
      y1 = y2;
    }
  }
}

// ---------------------------------------------------------------------------
// PVFMM MortonId restatement: coordinates quantised to kMaxDepth bits per
// axis, ordered by the interleaved bits (z, y, x from most to least
// significant inside each level), ties broken by depth.  Used at
// src/tree/tree_functor.h:172-184, :195, :467-479.
static const int kMaxDepth = 30;
struct Mid {
  unsigned __int128 key;
  int depth;
};
static inline bool operator<(const Mid& a, const Mid& b) {
  return a.key < b.key || (a.key == b.key && a.depth < b.depth);
}
static unsigned __int128 interleave(uint64_t x, uint64_t y, uint64_t z) {
  unsigned __int128 k = 0;
  for (int b = kMaxDepth - 1; b >= 0; b--) {
    k = (k << 3) | (unsigned __int128)((((z >> b) & 1) << 2) | (((y >> b) & 1) << 1) |
                                       ((x >> b) & 1));
  }
  return k;
}
static const unsigned __int128 kKeyMax = ~(unsigned __int128)0;

// Point MortonId with the reference's shift of 1.0 to 1-2^-MAX_DEPTH when the
// boundary is not periodic (src/tree/tree_functor.h:464-479).  A point
// outside [0,1)^3 (after that shift), or with a NaN coordinate, is ordered
// after every leaf, i.e. it is handed to the last leaf, where cheb_poly's
// |x|>1 rule evaluates it to 0 (the reference reaches the same leaf through
// the wrap-around of its unsigned cast).
template <class R>
static Mid point_mid(const R* c, bool periodic) {
  const Real shift = 1.0 / (Real)(1UL << kMaxDepth);
  uint64_t q[3];
  for (int k = 0; k < 3; k++) {
    Real v = val(c[k]);
    if (v == 1.0 && !periodic) v = v - shift;
    if (!(v >= 0.0 && v < 1.0)) return Mid{kKeyMax, kMaxDepth};
    q[k] = (uint64_t)std::floor(v * (Real)(1UL << kMaxDepth));
  }
  return Mid{interleave(q[0], q[1], q[2]), kMaxDepth};
}

// ---------------------------------------------------------------------------
// A linear octree given by its leaves (anchor, depth) in Morton order with
// per-leaf triangular Chebyshev coefficients [leaf][dof][Nc].
template <class R>
struct TreeT {
  long L;
  const Real* anchor;  // L x 3
  const int* depth;    // L
  int q, dof;
  const R* coeff;      // L x dof x Nc
  std::vector<Mid> mid;
  long nc() const { return (long)(q + 1) * (q + 2) * (q + 3) / 6; }
  void init() {
    mid.resize(L);
    for (long i = 0; i < L; i++) {
      uint64_t a[3];
      for (int k = 0; k < 3; k++)
        a[k] = (uint64_t)std::floor(anchor[3 * i + k] * (Real)(1UL << kMaxDepth));
      mid[i] = Mid{interleave(a[0], a[1], a[2]), depth[i]};
    }
  }
};

// ---------------------------------------------------------------------------
// Triangular tensor Chebyshev sum over a block of n points (n % 16 == 0):
// out[l][p] = sum_i pz_i sum_{j<d-i} py_j sum_{k<d-i-j} c[l][i][j][k] px_k.
// Restates pvfmm::vec_eval, src/tree/tree_functor.h:27-84 (coefficients in a
// padded d0^3 cube, points processed 16 at a time as in the 4xVecLen AVX
// unroll, same i/j/k summation order, fused multiply-add accumulation).
template <class R>
static void vec_eval(int n, int d0, int d, int dof, const R* px, const R* py, const R* pz,
                     const R* coeff, R* tmp_out) {
  const int B = 16;
  for (int l0 = 0; l0 < dof; l0++) {
    for (int l1 = 0; l1 < n; l1 += B) {
      R u[B];
      for (int p = 0; p < B; p++) u[p] = mk<R>(0);
      for (int i = 0; i < d; i++) {
        R v[B];
        for (int p = 0; p < B; p++) v[p] = mk<R>(0);
        const R* pz_ = pz + i * n + l1;
        for (int j = 0; i + j < d; j++) {
          R w[B];
          for (int p = 0; p < B; p++) w[p] = mk<R>(0);
          const R* py_ = py + j * n + l1;
          for (int k = 0; i + j + k < d; k++) {
            const R* px_ = px + k * n + l1;
            const R c = coeff[k + d0 * (j + d0 * (i + d0 * l0))];
            for (int p = 0; p < B; p++) w[p] = fmaR(px_[p], c, w[p]);
          }
          for (int p = 0; p < B; p++) v[p] = fmaR(py_[p], w[p], v[p]);
        }
        for (int p = 0; p < B; p++) u[p] = fmaR(pz_[p], v[p], u[p]);
      }
      for (int p = 0; p < B; p++) tmp_out[l0 * n + l1 + p] = u[p];
    }
  }
}

// ---------------------------------------------------------------------------
// Evaluate the leaves at Morton-sorted points.  Restates EvalNodesLocal,
// src/tree/tree_functor.h:155-395: leaf j owns the sorted points
// [lower_bound(mid_j), lower_bound(mid_{j+1})) (:193-198); each thread takes a
// contiguous point range (:212-243); coefficients repacked into a padded cube
// (:248-268); blocks of 288 points mapped to [-1,1] (:270-295); cheb_poly and
// vec_eval (:303-366); transpose to point-major (:376-383).
template <class R>
static void eval_nodes_local(const TreeT<R>& t, const R* coord, const Mid* trg_mid, size_t N,
                             R* value) {
  const int dof = t.dof;
  const long L = t.L;
  std::vector<size_t> part(L + 1);
  part[L] = N;
#pragma omp parallel for
  for (long j = 0; j < L; j++)
    part[j] = std::lower_bound(trg_mid, trg_mid + N, t.mid[j]) - trg_mid;

  const int omp_p = omp_get_max_threads();
#pragma omp parallel for schedule(static)
  for (int pid = 0; pid < omp_p; pid++) {
    const int d = t.q + 1;
    int d0 = d;
    while (d0 % 4) d0++;
    std::vector<R> coeff_((size_t)d0 * d0 * d0 * dof, mk<R>(0));
    std::vector<R> cx, cy, cz, px, py, pz, tmp_out;

    size_t pt_start0 = (size_t)pid * N / omp_p;
    size_t pt_end0 = (size_t)(pid + 1) * N / omp_p;
    long node_start = std::lower_bound(part.begin(), part.end(), pt_start0) - part.begin() - 1;
    long node_end = std::lower_bound(part.begin(), part.end(), pt_end0) - part.begin();
    node_start = std::max<long>(0, std::min<long>(node_start, L));
    node_end = std::max<long>(0, std::min<long>(node_end, L));
    for (long j = node_start; j < node_end; j++) {
      size_t a = std::max(pt_start0, part[j]);
      size_t b = std::min(pt_end0, part[j + 1]);
      if (a >= b) continue;
      {  // repack the triangular coefficients into the padded cube
        const R* c = t.coeff + (size_t)j * dof * t.nc();
        long indx = 0;
        for (int l0 = 0; l0 < dof; l0++)
          for (int i = 0; i < d; i++)
            for (int jj = 0; i + jj < d; jj++)
              for (int k = 0; i + jj + k < d; k++)
                coeff_[k + d0 * (jj + d0 * (i + d0 * l0))] = c[indx++];
      }
      const Real* anc = t.anchor + 3 * j;
      const Real s = (Real)(1ULL << t.depth[j]);
      const size_t blk = 288;
      for (size_t ps = a; ps < b; ps += blk) {
        const size_t pe = std::min(b, ps + blk);
        const int npts = (int)(pe - ps);
        int n = npts;
        while (n % 16) n++;
        cx.assign(n, mk<R>(0));
        cy.assign(n, mk<R>(0));
        cz.assign(n, mk<R>(0));
        for (int i = 0; i < npts; i++) {
          const R* p = coord + (ps + i) * 3;
          cx[i] = (p[0] - anc[0]) * 2.0 * s - 1.0;
          cy[i] = (p[1] - anc[1]) * 2.0 * s - 1.0;
          cz[i] = (p[2] - anc[2]) * 2.0 * s - 1.0;
        }
        px.assign((size_t)d0 * n, mk<R>(0));
        py.assign((size_t)d0 * n, mk<R>(0));
        pz.assign((size_t)d0 * n, mk<R>(0));
        cheb_poly(t.q, cx.data(), n, px.data());
        cheb_poly(t.q, cy.data(), n, py.data());
        cheb_poly(t.q, cz.data(), n, pz.data());
        tmp_out.resize((size_t)n * dof);
        vec_eval(n, d0, d, dof, px.data(), py.data(), pz.data(), coeff_.data(), tmp_out.data());
        R* out = value + ps * dof;
        for (int i = 0; i < npts; i++)
          for (int l = 0; l < dof; l++) out[i * dof + l] = tmp_out[l * n + i];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Field functor over a tree.  Restates EvalTree, src/tree/tree_functor.h:397-791
// on one rank (lcl_start = 0, lcl_end = N): periodic wrap of the caller's
// array IN PLACE (:442-448), Morton sort with index tracking (:463-489),
// evaluation of the sorted points (:656-677), un-permutation (:683-690).
template <class R>
static void eval_tree(const TreeT<R>& t, R* pos, size_t N, R* value, bool periodic) {
  if (periodic) {
#pragma omp parallel for
    for (size_t i = 0; i < N * 3; i++) {
      R& c = pos[i];
      if (val(c) < 0.0) c = c + 1.0;
      if (val(c) >= 1.0) c = c - 1.0;
    }
  }
  struct Pair {
    Mid key;
    size_t data;
  };
  std::vector<Pair> pr(N);
#pragma omp parallel for
  for (size_t i = 0; i < N; i++) pr[i] = Pair{point_mid(pos + 3 * i, periodic), i};
  std::stable_sort(pr.begin(), pr.end(), [](const Pair& a, const Pair& b) { return a.key < b.key; });

  std::vector<R> coord(N * 3), vals(N * t.dof);
  std::vector<Mid> mids(N);
#pragma omp parallel for
  for (size_t i = 0; i < N; i++) {
    for (int k = 0; k < 3; k++) coord[3 * i + k] = pos[3 * pr[i].data + k];
    mids[i] = pr[i].key;
  }
  eval_nodes_local(t, coord.data(), mids.data(), N, vals.data());
#pragma omp parallel for
  for (size_t i = 0; i < N; i++)
    for (int l = 0; l < t.dof; l++) value[pr[i].data * t.dof + l] = vals[i * t.dof + l];
}

// ---------------------------------------------------------------------------
// Midpoint RK2.  Restates IntegrateRK2 / ComputeTrajRK2,
// src/semilag/traj.inc:20-68: xsol aliases xinit, so the functor's in-place
// periodic wrap of xinit is seen by the final update.
template <class R, class Functor>
static void integrate_rk2(Functor& fn, R* x, size_t N, Real tau) {
  std::vector<R> xtmp(N * 3), vtmp(N * 3);
  fn(x, N, vtmp.data());
#pragma omp parallel for
  for (size_t i = 0; i < N * 3; i++) xtmp[i] = fmaR(0.5 * tau, vtmp[i], x[i]);
  fn(xtmp.data(), N, vtmp.data());
#pragma omp parallel for
  for (size_t i = 0; i < N * 3; i++) x[i] = fmaR(tau, vtmp[i], x[i]);
}

template <class R, class Functor>
static void traj_rk2(Functor& fn, const R* xinit, size_t N, Real tinit, Real tfinal, int nrk,
                     R* xsol) {
  Real tau = (tfinal - tinit) / nrk;
  std::memcpy(xsol, xinit, sizeof(R) * N * 3);
  for (int s = 0; s < nrk; s++) integrate_rk2<R>(fn, xsol, N, tau);
}

template <class R>
struct TreeFunctorT {
  const TreeT<R>* t;
  bool periodic;
  void operator()(R* pos, size_t n, R* out) { eval_tree(*t, pos, n, out, periodic); }
};
typedef TreeT<Real> Tree;
typedef TreeFunctorT<Real> TreeFunctor;

// Leaf Chebyshev nodes of every leaf, leaves in order.  Restates
// CollectChebTreeGridPoints, src/tree/tree_utils.h:442-498.
template <class R>
static void collect_grid_points(const TreeT<R>& t, Real* out) {
  std::vector<Real> nodes = new_nodes(t.q, 3);
  const long np = (long)nodes.size() / 3;
#pragma omp parallel for
  for (long l = 0; l < t.L; l++) {
    const Real len = std::pow(0.5, t.depth[l]);
    const Real* c = t.anchor + 3 * l;
    Real* o = out + (size_t)l * np * 3;
    for (long i = 0; i < np; i++)
      for (int k = 0; k < 3; k++) o[3 * i + k] = c[k] + len * nodes[3 * i + k];
  }
}

// Node values -> coefficients, coeff[row][n] = sum_p vals[row][p] M[p][n] with
// row = leaf*dof + l.  Restates SetTreeGridValues, src/tree/tree_utils.h:500-552
// (per-thread row blocks, GEMM against the point-to-coefficient matrix).
template <class R>
static void set_tree_grid_values(long L, int dof, long np, long nc, const Real* M,
                                 const R* vals, R* coeff) {
  const long rows = L * dof;
  const int RB = 4;
#pragma omp parallel for schedule(static)
  for (long r0 = 0; r0 < rows; r0 += RB) {
    const int rb = (int)std::min<long>(RB, rows - r0);
    std::vector<R> acc((size_t)RB * nc, mk<R>(0));
    for (long p = 0; p < np; p++) {
      const Real* m = M + p * nc;
      for (int rr = 0; rr < rb; rr++) {
        const R v = vals[(r0 + rr) * np + p];
        R* a = acc.data() + rr * nc;
        for (long n = 0; n < nc; n++) a[n] = a[n] + v * m[n];
      }
    }
    for (int rr = 0; rr < rb; rr++)
      std::memcpy(coeff + (r0 + rr) * nc, acc.data() + rr * nc, sizeof(R) * nc);
  }
}

// ---------------------------------------------------------------------------
// Tricubic Lagrange interpolation on an N^3 grid.  Clamped form restates
// tbslas::fast_interp, src/tree/tree_functor.h:89-153 (grid spacing
// 1/(N-1), stencil base floor(x(N-1))-1 clamped to [0,N-4], points outside
// [0,1]^3 give 0, SoA grid vals[x+N(y+Nz)+k N^3], output [pt][dof]).
// Periodic form (defined by this project): grid spacing 1/N on [0,1), the
// query is wrapped in place once as in EvalTree, stencil indices wrap mod N.
static void fast_interp(const Real* grid, int dof, int Nr, Real* pts, size_t n, Real* out,
                        bool periodic) {
  Real lagr_denom[4];
  for (int i = 0; i < 4; i++) {
    lagr_denom[i] = 1;
    for (int j = 0; j < 4; j++)
      if (i != j) lagr_denom[i] /= (Real)(i - j);
  }
  const long N3 = (long)Nr * Nr * Nr;
#pragma omp parallel for
  for (size_t i = 0; i < n; i++) {
    Real* q = pts + 3 * i;
    if (periodic) {
      for (int j = 0; j < 3; j++) {
        if (q[j] < 0.0) q[j] = q[j] + 1.0;
        if (q[j] >= 1.0) q[j] = q[j] - 1.0;
      }
    }
    bool outside = false;
    for (int j = 0; j < 3; j++)
      if (!(q[j] >= 0 && (periodic ? q[j] < 1.0 : q[j] <= 1.0))) outside = true;
    if (outside) {
      for (int k = 0; k < dof; k++) out[i * dof + k] = 0;
      continue;
    }
    Real point[3];
    long gi[3];
    for (int j = 0; j < 3; j++) {
      point[j] = q[j] * (periodic ? Nr : (Nr - 1));
      gi[j] = ((long)point[j]) - 1;
      if (!periodic) {
        if (gi[j] < 0) gi[j] = 0;
        if (gi[j] > Nr - 4) gi[j] = Nr - 4;
      }
      point[j] -= gi[j];
    }
    Real M[3][4];
    for (int j = 0; j < 3; j++) {
      Real x = point[j];
      for (int k = 0; k < 4; k++) {
        M[j][k] = lagr_denom[k];
        for (int l = 0; l < 4; l++)
          if (k != l) M[j][k] *= (x - l);
      }
    }
    long idx[3][4];
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 4; k++) {
        long g = gi[j] + k;
        if (periodic) g = (g % Nr + Nr) % Nr;
        idx[j][k] = g;
      }
    for (int k = 0; k < dof; k++) {
      Real val = 0;
      for (int j2 = 0; j2 < 4; j2++)
        for (int j1 = 0; j1 < 4; j1++) {
          Real M1M2 = M[1][j1] * M[2][j2];
          long ij = Nr * (idx[1][j1] + Nr * idx[2][j2]);
          for (int j0 = 0; j0 < 4; j0++)
            val = std::fma(M[0][j0] * M1M2, grid[idx[0][j0] + ij + k * N3], val);
        }
      out[i * dof + k] = val;
    }
  }
}

struct GridFunctor {
  const Real* grid;
  int dof, Nr;
  bool periodic;
  void operator()(Real* pos, size_t n, Real* out) {
    fast_interp(grid, dof, Nr, pos, n, out, periodic);
  }
};

}  // namespace orc

using namespace orc;

static Tree make_tree(long L, const double* anchor, const int* depth, int q, int dof,
                      const double* coeff) {
  Tree t{L, anchor, depth, q, dof, coeff, {}};
  t.init();
  return t;
}

template <class R>
static TreeT<R> make_tree_t(long L, const double* anchor, const int* depth, int q, int dof,
                            const R* coeff) {
  TreeT<R> t{L, anchor, depth, q, dof, coeff, {}};
  t.init();
  return t;
}

// One in-situ SL step of a concentration tree through a velocity tree.
// Restates SolveSemilagInSitu, src/tree/tree_semilag.h:92-135, with
// SolveSemilagRK2, src/semilag/semilag.inc:26-45.  For dof > 1 the point-major
// values are transposed to the dof-major layout SetTreeGridValues reads.
// Only the target nodes of leaves [leaf_begin, leaf_end) are advected and
// refitted when leaf_end > leaf_begin (bounded CPU samples); coeff_out then
// holds those leaves only.  coeff_out may alias con_coeff only for a full
// step.
template <class R>
static void semilag_in_situ_T(long Lv, const double* av, const int* dv, int qv, const R* cv,
                              long Lc, const double* ac, const int* dc, int qc, int dofc,
                              const R* cc, const double* M, int timestep, double dt, int nrk,
                              int periodic, long leaf_begin, long leaf_end, R* coeff_out) {
  TreeT<R> tv = make_tree_t<R>(Lv, av, dv, qv, 3, cv);
  TreeT<R> tc = make_tree_t<R>(Lc, ac, dc, qc, dofc, cc);
  if (leaf_end <= leaf_begin) {
    leaf_begin = 0;
    leaf_end = Lc;
  }
  const long Ls = leaf_end - leaf_begin;
  TreeT<R> ts = make_tree_t<R>(Ls, ac + 3 * leaf_begin, dc + leaf_begin, qc, dofc, nullptr);
  const int d = qc + 1;
  const long np = (long)d * d * d;
  const size_t N = (size_t)Ls * np;
  std::vector<Real> pts(N * 3);
  std::vector<R> x0(N * 3), xdep(N * 3), vals(N * dofc);
  collect_grid_points(ts, pts.data());
  for (size_t i = 0; i < N * 3; i++) x0[i] = mk<R>(pts[i]);
  Real tinit = timestep * dt;
  Real tfinal = tinit - dt;
  TreeFunctorT<R> fv{&tv, periodic != 0};
  traj_rk2<R>(fv, x0.data(), N, tinit, tfinal, nrk, xdep.data());
  eval_tree(tc, xdep.data(), N, vals.data(), periodic != 0);
  std::vector<R> vdm(N * dofc);
  for (long l = 0; l < Ls; l++)
    for (long p = 0; p < np; p++)
      for (int k = 0; k < dofc; k++)
        vdm[((size_t)l * dofc + k) * np + p] = vals[((size_t)l * np + p) * dofc + k];
  set_tree_grid_values<R>(Ls, dofc, np, (long)d * (d + 1) * (d + 2) / 6, M, vdm.data(),
                          coeff_out);
}

extern "C" {

int orc_num_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
}

int orc_new_nodes(int q, double* out) {
  std::vector<Real> y = new_nodes(q, 3);
  std::memcpy(out, y.data(), sizeof(Real) * y.size());
  return 0;
}

int orc_cheb_poly(int q, const double* x, int n, double* out) {
  cheb_poly(q, x, n, out);
  return 0;
}

// Triangular Chebyshev basis at n points in [-1,1]^3: V[p][idx(i,j,k)] =
// T_i(z) T_j(y) T_k(x) with i outer, j, k inner over i+j+k<=q -- the column
// order vec_eval reads coefficients in (src/tree/tree_functor.h:257-267,
// restating pvfmm::cheb_eval as used at src/utils/cheb.h:177-180).
int orc_cheb_basis(int q, const double* pts, long n, double* V) {
  const int d = q + 1;
  const long nc = (long)d * (d + 1) * (d + 2) / 6;
  std::vector<Real> tx(d), ty(d), tz(d);
  for (long p = 0; p < n; p++) {
    cheb_poly(q, pts + 3 * p + 0, 1, tx.data());
    cheb_poly(q, pts + 3 * p + 1, 1, ty.data());
    cheb_poly(q, pts + 3 * p + 2, 1, tz.data());
    long idx = 0;
    for (int i = 0; i < d; i++)
      for (int j = 0; i + j < d; j++)
        for (int k = 0; i + j + k < d; k++) V[p * nc + idx++] = tz[i] * ty[j] * tx[k];
  }
  return 0;
}

int orc_collect_grid_points(long L, const double* anchor, const int* depth, int q, double* out) {
  Tree t = make_tree(L, anchor, depth, q, 1, nullptr);
  collect_grid_points(t, out);
  return 0;
}

// pos is copied: the caller's array is not mutated here.
int orc_eval_tree(long L, const double* anchor, const int* depth, int q, int dof,
                  const double* coeff, int periodic, const double* pos, long n, double* out) {
  Tree t = make_tree(L, anchor, depth, q, dof, coeff);
  std::vector<Real> p(pos, pos + 3 * n);
  eval_tree(t, p.data(), n, out, periodic != 0);
  return 0;
}

int orc_traj_rk2(long L, const double* anchor, const int* depth, int q, const double* coeff,
                 int periodic, const double* x, long n, double tinit, double tfinal, int nrk,
                 double* xout) {
  Tree t = make_tree(L, anchor, depth, q, 3, coeff);
  TreeFunctor f{&t, periodic != 0};
  traj_rk2(f, x, n, tinit, tfinal, nrk, xout);
  return 0;
}

int orc_set_tree_grid_values(long L, int q, int dof, const double* M, const double* vals,
                             double* coeff) {
  const int d = q + 1;
  set_tree_grid_values(L, dof, (long)d * d * d, (long)d * (d + 1) * (d + 2) / 6, M, vals, coeff);
  return 0;
}

// One in-situ SL step of a concentration tree through a velocity tree.
// Restates SolveSemilagInSitu, src/tree/tree_semilag.h:92-135, with
// SolveSemilagRK2, src/semilag/semilag.inc:26-45.  For dof > 1 the point-major
// values are transposed to the dof-major layout SetTreeGridValues reads.
// Only the target nodes of leaves [leaf_begin, leaf_end) are advected and
// refitted when leaf_end > leaf_begin (bounded CPU samples); coeff_out then
// holds those leaves only.  coeff_out may alias con_coeff only for a full
// step.
int orc_semilag_in_situ(long Lv, const double* av, const int* dv, int qv, const double* cv,
                        long Lc, const double* ac, const int* dc, int qc, int dofc,
                        const double* cc, const double* M, int timestep, double dt, int nrk,
                        int periodic, long leaf_begin, long leaf_end, double* coeff_out) {
  semilag_in_situ_T<Real>(Lv, av, dv, qv, cv, Lc, ac, dc, qc, dofc, cc, M, timestep, dt, nrk,
                          periodic, leaf_begin, leaf_end, coeff_out);
  return 0;
}

// The same step on dual numbers: cv_d / cc_d are the directional
// derivatives of the velocity / concentration coefficients, out_d receives
// the derivative of the new concentration coefficients (whole tree).
int orc_semilag_in_situ_dual(long Lv, const double* av, const int* dv, int qv, const double* cv,
                             const double* cv_d, long Lc, const double* ac, const int* dc, int qc,
                             const double* cc, const double* cc_d, const double* M, int timestep,
                             double dt, int nrk, int periodic, double* out, double* out_d) {
  const long ncv = (long)(qv + 1) * (qv + 2) * (qv + 3) / 6 * 3 * Lv;
  const long ncc = (long)(qc + 1) * (qc + 2) * (qc + 3) / 6 * Lc;
  std::vector<Dual> v(ncv), c(ncc), o(ncc);
  for (long i = 0; i < ncv; i++) v[i] = Dual{cv[i], cv_d[i]};
  for (long i = 0; i < ncc; i++) c[i] = Dual{cc[i], cc_d[i]};
  semilag_in_situ_T<Dual>(Lv, av, dv, qv, v.data(), Lc, ac, dc, qc, 1, c.data(), M, timestep, dt,
                          nrk, periodic, 0, 0, o.data());
  for (long i = 0; i < ncc; i++) {
    out[i] = o[i].v;
    out_d[i] = o[i].d;
  }
  return 0;
}

// pts is copied: the caller's array is not mutated here.
int orc_fast_interp(const double* grid, int dof, int nreg, const double* pts, long n,
                    double* out, int periodic) {
  std::vector<Real> p(pts, pts + 3 * n);
  fast_interp(grid, dof, nreg, p.data(), n, out, periodic != 0);
  return 0;
}

// One SL step on the regular grid: every grid node is a target, RK2 through
// the tricubic velocity, tricubic concentration at the departure points.
// Targets: node (ix,iy,iz) at ix*h with h = 1/(N-1) (clamped, as
// tbslas::get_reg_grid_points, src/utils/common.h:198-208) or h = 1/N
// (periodic).  Only nodes [node_begin, node_end) are computed when
// node_end > node_begin (bounded CPU samples); out is indexed by node.
int orc_semilag_grid(const double* vel, const double* con, int nreg, double dt, int nrk,
                     int periodic, long node_begin, long node_end, double* out) {
  const long N3 = (long)nreg * nreg * nreg;
  if (node_end <= node_begin) {
    node_begin = 0;
    node_end = N3;
  }
  const size_t n = node_end - node_begin;
  const Real h = periodic ? 1.0 / nreg : 1.0 / (nreg - 1);
  std::vector<Real> x(n * 3), xdep(n * 3);
  for (size_t i = 0; i < n; i++) {
    long g = node_begin + (long)i;
    x[3 * i + 0] = (Real)(g % nreg) * h;
    x[3 * i + 1] = (Real)((g / nreg) % nreg) * h;
    x[3 * i + 2] = (Real)(g / ((long)nreg * nreg)) * h;
  }
  GridFunctor fv{vel, 3, nreg, periodic != 0};
  traj_rk2(fv, x.data(), n, 0.0, -dt, nrk, xdep.data());
  fast_interp(con, 1, nreg, xdep.data(), n, out, periodic != 0);
  return 0;
}

}  // extern "C"

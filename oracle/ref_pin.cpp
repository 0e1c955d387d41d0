// The reference's own SL-path code, compiled from its sources where they lie
// (tbslas src/: semilag/traj.inc, semilag/semilag.inc, tree/tree_functor.h,
// tree/tree_utils.h, tree/tree_semilag.h, tree/tree_set_functor.h,
// tree/tree_extrap_functor.h, utils/cheb.h, utils/cubic.h) against the
// stand-ins of oracle/ref_stubs/ for its absent dependencies (PVFMM, MPI),
// and driven on a linear octree given by its leaves.  It pins the oracle:
// tests compare oracle/oracle.cpp with these entry points on the same inputs
// (tests/test_ref_pin.py, fixtures in tests/golden/ref_*.npz).
//
// TEST INFRASTRUCTURE ONLY.  Built into oracle/_ref/libref.so by
// oracle/build_ref.py when the reference's sources are present; nothing in
// the product loads it.
//
// The build contracts multiply-adds (g++ -ffp-contract=fast on an FMA
// target), the rounding of an optimising compiler for a current CPU; the
// scalar form of vec_eval is selected (its per-point arithmetic is the one
// the vector forms repeat lane by lane).
#undef __AVX__
#undef __SSE3__
#undef __MIC__

// utils/common.h first, as the reference's drivers include it (the semilag
// headers use its SimConfigSingleton without including it)
#include <utils/common.h>
#include <tree/tree_semilag.h>
#include <tree/tree_extrap_functor.h>
#include <tree/tree_set_functor.h>

#include <cstdint>
#include <memory>
#include <vector>

namespace refpin {

// A leaf of the octree, with the accessors the reference's tree code calls
// (pvfmm::Cheb_Node's interface as used by tree_functor.h / tree_utils.h).
struct Node {
  double coord[3];
  int depth = 0, deg = 0, dof = 0;
  pvfmm::Vector<double> cheb;
  pvfmm::MortonId mid;
  bool IsLeaf() const { return true; }
  bool IsGhost() const { return false; }
  int DataDOF() const { return dof; }
  int ChebDeg() const { return deg; }
  pvfmm::Vector<double>& ChebData() { return cheb; }
  double* Coord() { return coord; }
  int Depth() const { return depth; }
  pvfmm::MortonId GetMortonId() const { return mid; }
};

// The leaves in Morton order, which is their post-order.
struct Tree {
  typedef Node Node_t;
  typedef double Real_t;
  std::vector<Node> leaves;
  std::vector<Node*> list;
  MPI_Comm comm = MPI_COMM_WORLD;
  Tree(long L, const double* anchor, const int* depth, int q, int dof, const double* coeff) {
    const long nc = (long)(q + 1) * (q + 2) * (q + 3) / 6;
    leaves.resize(L);
    for (long i = 0; i < L; ++i) {
      Node& n = leaves[i];
      for (int k = 0; k < 3; ++k) n.coord[k] = anchor[3 * i + k];
      n.depth = depth[i];
      n.deg = q;
      n.dof = dof;
      n.cheb.Resize(nc * dof);
      for (long c = 0; c < nc * dof; ++c) n.cheb[c] = coeff ? coeff[i * nc * dof + c] : 0.0;
      n.mid = pvfmm::MortonId(n.coord[0], n.coord[1], n.coord[2], n.depth);
    }
    for (Node& n : leaves) list.push_back(&n);
  }
  int Dim() const { return 3; }
  Node* RootNode() { return list[0]; }
  Node* PostorderFirst() { return list.empty() ? nullptr : list[0]; }
  Node* PostorderNxt(Node* n) {
    const long i = n - &leaves[0] + 1;
    return i < (long)list.size() ? list[i] : nullptr;
  }
  const std::vector<Node*>& GetNodeList() { return list; }
  const MPI_Comm* Comm() const { return &comm; }
  void coeffs(double* out) const {
    for (size_t i = 0; i < leaves.size(); ++i) {
      const pvfmm::Vector<double>& c = leaves[i].cheb;
      for (size_t k = 0; k < c.Dim(); ++k) out[i * c.Dim() + k] = c[k];
    }
  }
};

void set_bc(int periodic) {
  tbslas::SimConfigSingleton::Instance()->bc = periodic ? pvfmm::Periodic : pvfmm::FreeSpace;
}

}  // namespace refpin

using refpin::Tree;

extern "C" {

// tbslas::new_nodes<double>(q, 3) (src/utils/cheb.h:41-67): (q+1)^3 x 3.
void ref_new_nodes(int q, double* out) {
  const std::vector<double> y = tbslas::new_nodes<double>(q, 3);
  std::copy(y.begin(), y.end(), out);
}

// pvfmm::vec_eval as tree_functor.h:27-84 defines it, scalar form.
void ref_vec_eval(int n, int d0, int d, int dof, double* px, double* py, double* pz,
                  double* coeff, double* out) {
  pvfmm::vec_eval<double, double>(n, d0, d, dof, px, py, pz, coeff, out);
}

// tbslas::fast_interp (src/tree/tree_functor.h:89-153).
void ref_fast_interp(const double* grid, int dof, int n_reg, const double* pts, long n,
                     double* out) {
  const long n3 = (long)n_reg * n_reg * n_reg;
  std::vector<double> g(grid, grid + n3 * dof), p(pts, pts + 3 * n), v;
  tbslas::fast_interp(g, dof, n_reg, p, v);
  std::copy(v.begin(), v.end(), out);
}

// tbslas::CollectChebTreeGridPoints (src/tree/tree_utils.h:442-498).
void ref_collect_grid_points(long L, const double* anchor, const int* depth, int q,
                             double* out) {
  Tree t(L, anchor, depth, q, 1, nullptr);
  std::vector<double> pts;
  tbslas::CollectChebTreeGridPoints(t, pts);
  std::copy(pts.begin(), pts.end(), out);
}

// tbslas::EvalTree through NodeFieldFunctor (src/tree/tree_functor.h:397-815);
// pos is copied (the reference wraps it in place under periodic bc).
void ref_eval_tree(long L, const double* anchor, const int* depth, int q, int dof,
                   const double* coeff, int periodic, const double* pos, long n, double* out) {
  refpin::set_bc(periodic);
  Tree t(L, anchor, depth, q, dof, coeff);
  std::vector<double> p(pos, pos + 3 * n);
  tbslas::NodeFieldFunctor<double, Tree> f(&t);
  f(p.data(), (int)n, out);
}

// tbslas::ComputeTrajRK2 with a NodeFieldFunctor velocity (src/semilag/traj.inc:20-68).
void ref_traj_rk2(long L, const double* anchor, const int* depth, int q, const double* coeff,
                  int periodic, const double* x, long n, double tinit, double tfinal, int nrk,
                  double* out) {
  refpin::set_bc(periodic);
  Tree t(L, anchor, depth, q, 3, coeff);
  std::vector<double> xi(x, x + 3 * n), xs(3 * n);
  tbslas::ComputeTrajRK2(tbslas::NodeFieldFunctor<double, Tree>(&t), xi, tinit, tfinal, nrk, xs);
  std::copy(xs.begin(), xs.end(), out);
}

// tbslas::GetPt2CoeffMatrix<double> (src/utils/cheb.h:166-196): Np x Nc.
void ref_pt2coeff(int q, double* out) {
  pvfmm::Matrix<double> M;
  tbslas::GetPt2CoeffMatrix<double>(q, M);
  for (size_t i = 0; i < M.Dim(0); ++i)
    for (size_t j = 0; j < M.Dim(1); ++j) out[i * M.Dim(1) + j] = M[i][j];
}

// tbslas::SolveSemilagInSitu (src/tree/tree_semilag.h:92-135): one in-situ
// step of the concentration tree through the velocity tree's functor;
// coeff_out receives the concentration's new coefficients [Lc][dof][Nc].
void ref_semilag_in_situ(long Lv, const double* av, const int* dv, const double* vc, long Lc,
                         const double* ac, const int* dc, int dof, const double* cc, int q,
                         int timestep, double dt, int nrk, int periodic, double* coeff_out) {
  refpin::set_bc(periodic);
  Tree tv(Lv, av, dv, q, 3, vc);
  Tree tc(Lc, ac, dc, q, dof, cc);
  tbslas::NodeFieldFunctor<double, Tree> vel(&tv);
  tbslas::SolveSemilagInSitu(vel, tc, timestep, dt, nrk);
  tc.coeffs(coeff_out);
}

// SolveSemilagInSitu (src/tree/tree_semilag.h:92-135) through a
// FieldSetFunctor (src/tree/tree_set_functor.h:49-72): four velocity trees
// at times[4], cubic in time by CubicInterpPolicy::InterpCubic1D
// (src/utils/cubic.h:42-56).  The trees' leaves are concatenated: tree k has
// Lv[k] leaves (anchors av, depths dv, coefficients vc in that order).
void ref_semilag_in_situ_set(const long* Lv, const double* av, const int* dv, const double* vc,
                             const double* times, long Lc, const double* ac, const int* dc,
                             const double* cc, int q, int timestep, double dt, int nrk,
                             int periodic, double* coeff_out) {
  refpin::set_bc(periodic);
  const long nc = (long)(q + 1) * (q + 2) * (q + 3) / 6;
  std::vector<std::unique_ptr<Tree>> own;
  std::vector<Tree*> tv;
  long o = 0;
  for (int k = 0; k < 4; ++k) {
    own.emplace_back(new Tree(Lv[k], av + 3 * o, dv + o, q, 3, vc + o * 3 * nc));
    tv.push_back(own.back().get());
    o += Lv[k];
  }
  Tree tc(Lc, ac, dc, q, 1, cc);
  tbslas::FieldSetFunctor<double, Tree> vel(tv, std::vector<double>(times, times + 4));
  tbslas::SolveSemilagInSitu(vel, tc, timestep, dt, nrk);
  tc.coeffs(coeff_out);
}

// The two-functor SolveSemilagInSitu (src/tree/tree_semilag.h:137-180): v_n
// (NodeFieldFunctor) at the first stage, FieldExtrapFunctor's
// 1.5 v_n - 0.5 v_{n-1} (src/tree/tree_extrap_functor.h:47-78) at the
// midpoint.  Trees: v_n (Ln leaves), then v_{n-1} (Lp leaves), concatenated.
void ref_semilag_in_situ_extrap(long Ln, long Lp, const double* av, const int* dv,
                                const double* vc, long Lc, const double* ac, const int* dc,
                                const double* cc, int q, int timestep, double dt, int nrk,
                                int periodic, double* coeff_out) {
  refpin::set_bc(periodic);
  const long nc = (long)(q + 1) * (q + 2) * (q + 3) / 6;
  Tree tn(Ln, av, dv, q, 3, vc);
  Tree tp(Lp, av + 3 * Ln, dv + Ln, q, 3, vc + Ln * 3 * nc);
  Tree tc(Lc, ac, dc, q, 1, cc);
  tbslas::NodeFieldFunctor<double, Tree> vel(&tn);
  tbslas::FieldExtrapFunctor<double, Tree> extrap(&tp, &tn);
  tbslas::SolveSemilagInSitu(vel, extrap, tc, timestep, dt, nrk);
  tc.coeffs(coeff_out);
}

// The advection-diffusion driver's BDF2 semi-Lagrangian step
// (src/applications/src/advdiff-ss.cpp:485-521) -- a sequence inside the
// driver's main(), so it is composed here from the reference's own
// CollectChebTreeGridPoints, ComputeTrajRK2 (in place, as the driver calls
// it), NodeFieldFunctor evaluations and SetTreeGridValues in the driver's
// order, with the driver's combination of the two values (4/3 and 1/3).
// Trees: velocity, c_{n-1}, c_n; the target tree's leaves (Ln, an, dn).
void ref_semilag_bdf2(long Lv, const double* av, const int* dv, const double* vc, long Lp,
                      const double* ap, const int* dp, const double* cp, long Lcur,
                      const double* acur, const int* dcur, const double* ccur, long Ln,
                      const double* an, const int* dn, int q, double t, double dt, int nrk,
                      int periodic, double* coeff_out) {
  refpin::set_bc(periodic);
  Tree tv(Lv, av, dv, q, 3, vc);
  Tree tp(Lp, ap, dp, q, 1, cp);
  Tree tc(Lcur, acur, dcur, q, 1, ccur);
  Tree tn(Ln, an, dn, q, 1, nullptr);
  tbslas::NodeFieldFunctor<double, Tree> vel(&tv), cur(&tc), prev(&tp);
  std::vector<double> pts;
  tbslas::CollectChebTreeGridPoints(tn, pts);
  const int n = (int)(pts.size() / 3);
  std::vector<double> vc_n(n), vp_n(n), vals(n);
  tbslas::ComputeTrajRK2(vel, pts, t, t - dt, nrk, pts);
  cur(pts.data(), n, vc_n.data());
  tbslas::ComputeTrajRK2(vel, pts, t - dt, t - dt * 2, nrk, pts);
  prev(pts.data(), n, vp_n.data());
  const double cc = 4.0 / 3, pc = 1.0 / 3;
  for (int i = 0; i < n; ++i) vals[i] = cc * vc_n[i] - pc * vp_n[i];
  tbslas::SetTreeGridValues(tn, q, 1, vals);
  tn.coeffs(coeff_out);
}

// CubicInterpPolicy<double>::InterpCubic1D (src/utils/cubic.h:42-56) for n
// (x, xx[4], pp[4]) triples.
void ref_interp_cubic_1d(long n, const double* x, const double* xx, const double* pp,
                         double* out) {
  for (long i = 0; i < n; ++i) {
    double t[4], p[4];
    for (int k = 0; k < 4; ++k) {
      t[k] = xx[4 * i + k];
      p[k] = pp[4 * i + k];
    }
    out[i] = tbslas::CubicInterpPolicy<double>::InterpCubic1D(x[i], t, p);
  }
}

}  // extern "C"

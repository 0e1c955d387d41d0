// tbslas_gb300.hpp -- header-only C++ layer over the C ABI (tbslas_gb300.h)
// with the shapes of the reference's templates, so code written against
// tbslas's SL path swaps its includes and keeps its call sites:
//
//   tbslas::NodeFieldFunctor<real_t, Tree>   src/tree/tree_functor.h:793-815
//   tbslas::ComputeTrajRK2                   src/semilag/traj.inc:48-68
//   tbslas::SolveSemilagRK2                  src/semilag/semilag.inc:26-45
//   tbslas::SolveSemilagInSitu               src/tree/tree_semilag.h:92-135
//   tbslas::CollectChebTreeGridPoints        src/tree/tree_utils.h:442-498
//   tbslas::SetTreeGridValues                src/tree/tree_utils.h:500-552
//   tbslas::new_nodes / GetPt2CoeffMatrix    src/utils/cheb.h:41-196
//   tbslas::fast_interp                      src/tree/tree_functor.h:89-153
//   tbslas::FieldSetFunctor                  src/tree/tree_set_functor.h:28-103
//   tbslas::FieldExtrapFunctor               src/tree/tree_extrap_functor.h:27-95
//   the two-functor SolveSemilagInSitu       src/tree/tree_semilag.h:137-180
//   Tree::RefineTree + Balance21 after a step src/applications/src/advection.cpp:305-311
//   the BDF2 step of the driver              src/applications/src/advdiff-ss.cpp:485-521
//
// Differences a caller sees: errors throw tbslas_gb300::Error (the reference
// asserts); the boundary condition is an argument, not the SimConfig
// singleton; the functor never writes the periodic wrap back into the
// caller's coordinates; the tree is a Tree object built from the leaf list
// (anchors and depths of the non-ghost leaves in post-order) instead of a
// pvfmm::MPI_Tree.  Link with -ltbslas_gb300.
#ifndef TBSLAS_GB300_HPP_
#define TBSLAS_GB300_HPP_

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "tbslas_gb300.h"

namespace tbslas_gb300 {

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& what)
      : std::runtime_error(what + ": " + tbslas_last_error() + " (" +
                           tbslas_status_string(status) + ")"),
        status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int status, const char* what) {
  if (status != TBSLAS_OK) throw Error(status, what);
}

enum BoundaryType { FreeSpace = TBSLAS_BC_FREESPACE, Periodic = TBSLAS_BC_PERIODIC };

class Context {
 public:
  explicit Context(int device = 0) { check(tbslas_ctx_create(device, &ctx_), "tbslas_ctx_create"); }
  ~Context() { tbslas_ctx_destroy(ctx_); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  tbslas_ctx get() const { return ctx_; }

 private:
  tbslas_ctx ctx_ = nullptr;
};

// A complete linear octree with per-leaf Chebyshev coefficients ([leaf][dof][Nc],
// the concatenated Node::ChebData() of the leaves).
class Tree {
 public:
  typedef double Real_t;
  Tree(Context& ctx, const std::vector<double>& leaf_anchor, const std::vector<int32_t>& leaf_depth,
       int cheb_deg, int data_dof)
      : ctx_(&ctx), q_(cheb_deg), dof_(data_dof), n_(static_cast<int64_t>(leaf_depth.size())) {
    if (leaf_anchor.size() != 3 * leaf_depth.size())
      throw std::invalid_argument("leaf_anchor must hold 3 values per leaf");
    check(tbslas_tree_create(ctx.get(), n_, leaf_anchor.data(), leaf_depth.data(), q_, dof_, &t_),
          "tbslas_tree_create");
  }
  ~Tree() { tbslas_tree_destroy(t_); }
  Tree(const Tree&) = delete;
  Tree& operator=(const Tree&) = delete;

  int ChebDeg() const { return q_; }
  int DataDOF() const { return dof_; }
  int64_t NumLeaves() const { return n_; }
  int64_t NumCoeff() const { return static_cast<int64_t>(q_ + 1) * (q_ + 2) * (q_ + 3) / 6; }
  void SetChebData(const std::vector<double>& coeff) {
    check(static_cast<int64_t>(coeff.size()) == n_ * dof_ * NumCoeff() ? TBSLAS_OK
                                                                       : TBSLAS_ERR_INVALID_ARG,
          "SetChebData size");
    check(tbslas_tree_set_coeffs_host(t_, coeff.data()), "tbslas_tree_set_coeffs_host");
  }
  std::vector<double> ChebData() const {
    std::vector<double> c(static_cast<size_t>(n_ * dof_ * NumCoeff()));
    check(tbslas_tree_get_coeffs_host(t_, c.data()), "tbslas_tree_get_coeffs_host");
    return c;
  }
  tbslas_tree get() const { return t_; }
  Context& ctx() const { return *ctx_; }

  // The driver's `tree.RefineTree(); tree.Balance21(bc);` after a step, on the
  // device (tbslas_tree_remesh: coarsen one level, refine, 2:1 balance by the
  // Chebyshev tail against tol).  The leaf list changes.
  void Remesh(double tol, int min_depth, int max_depth, BoundaryType bc) {
    check(tbslas_tree_remesh(ctx_->get(), t_, tol, min_depth, max_depth, bc, nullptr),
          "tbslas_tree_remesh");
    check(tbslas_tree_info(t_, &n_, nullptr, nullptr, nullptr), "tbslas_tree_info");
  }
  void Leaves(std::vector<double>& anchor, std::vector<int32_t>& depth) const {
    anchor.resize(static_cast<size_t>(3 * n_));
    depth.resize(static_cast<size_t>(n_));
    check(tbslas_tree_get_leaves(t_, anchor.data(), depth.data()), "tbslas_tree_get_leaves");
  }

 private:
  Context* ctx_;
  tbslas_tree t_ = nullptr;
  int q_, dof_;
  int64_t n_;
};

// tbslas::NodeFieldFunctor: f(points[n*3]) -> values[n*dof], host arrays.
template <typename real_t, class NodeType = Tree>
class NodeFieldFunctor {
  static_assert(sizeof(real_t) == sizeof(double), "the GB300 path is FP64");

 public:
  explicit NodeFieldFunctor(NodeType* node, BoundaryType bc = FreeSpace) : node_(node), bc_(bc) {}
  void operator()(const real_t* points_pos, int num_points, real_t* out) {
    check(tbslas_eval_tree_host(node_->ctx().get(), node_->get(), points_pos, num_points, out, bc_),
          "tbslas_eval_tree_host");
  }
  // Stationary velocity: the time argument is ignored, as in the reference
  // (src/tree/tree_functor.h:808-811).
  void operator()(const real_t* points_pos, int num_points, real_t, real_t* out) {
    (*this)(points_pos, num_points, out);
  }
  NodeType* node() const { return node_; }
  BoundaryType bc() const { return bc_; }

 private:
  NodeType* node_;
  BoundaryType bc_;
};

// tbslas::ComputeTrajRK2 with a tree velocity functor.
template <typename real_t>
void ComputeTrajRK2(NodeFieldFunctor<real_t, Tree> field_fn, const std::vector<real_t>& xinit,
                    const real_t tinit, const real_t tfinal, const int num_rk_step,
                    std::vector<real_t>& xsol) {
  xsol.resize(xinit.size());
  Tree* t = field_fn.node();
  check(tbslas_traj_rk2_host(t->ctx().get(), t->get(), xinit.data(),
                             static_cast<int64_t>(xinit.size() / 3), tinit, tfinal, num_rk_step,
                             field_fn.bc(), xsol.data()),
        "tbslas_traj_rk2_host");
}

// tbslas::SolveSemilagRK2 with tree functors for velocity and concentration.
template <typename real_t>
void SolveSemilagRK2(NodeFieldFunctor<real_t, Tree> vel_evaluator,
                     NodeFieldFunctor<real_t, Tree> con_evaluator,
                     const std::vector<real_t>& points_pos, const int sdim, const int timestep,
                     const real_t dt, const int num_rk_step, std::vector<real_t>& points_vals) {
  const real_t tinit = timestep * dt;
  const real_t tfinal = tinit - dt;
  std::vector<real_t> dep;
  ComputeTrajRK2(vel_evaluator, points_pos, tinit, tfinal, num_rk_step, dep);
  points_vals.resize(points_pos.size() / sdim * con_evaluator.node()->DataDOF());
  con_evaluator(dep.data(), static_cast<int>(points_pos.size() / sdim), points_vals.data());
}

// tbslas::SolveSemilagInSitu: one SL step of tree_curr through the velocity
// functor's tree, coefficients refitted in place on the device.
template <class TreeFunc>
void SolveSemilagInSitu(TreeFunc& tvel_func, Tree& tree_curr, const int timestep, const double dt,
                        int num_rk_step = 1) {
  check(tbslas_semilag_in_situ(tree_curr.ctx().get(), tvel_func.node()->get(), tree_curr.get(),
                               timestep, dt, num_rk_step, tvel_func.bc(), nullptr),
        "tbslas_semilag_in_situ");
  check(tbslas_ctx_check(tree_curr.ctx().get(), nullptr), "tbslas_ctx_check");
}

// tbslas::FieldSetFunctor: the velocity cubic in time over four trees at
// increasing times; update() drops the oldest and appends a tree, as the
// reference's does.  Used through SolveSemilagInSitu below.
template <typename real_t, class Tree_t = Tree>
class FieldSetFunctor {
 public:
  FieldSetFunctor(std::vector<Tree_t*> field_set_elems, std::vector<real_t> field_set_times,
                  BoundaryType bc = FreeSpace)
      : elems_(field_set_elems), times_(field_set_times), bc_(bc) {
    if (elems_.size() != 4 || times_.size() != 4)
      throw std::invalid_argument("FieldSetFunctor: four trees and four times");
  }
  void update(Tree_t* new_tree, real_t time) {
    elems_.erase(elems_.begin());
    times_.erase(times_.begin());
    elems_.push_back(new_tree);
    times_.push_back(time);
  }
  const std::vector<Tree_t*>& elems() const { return elems_; }
  const std::vector<real_t>& times() const { return times_; }
  BoundaryType bc() const { return bc_; }

 private:
  std::vector<Tree_t*> elems_;
  std::vector<real_t> times_;
  BoundaryType bc_;
};

// tbslas::FieldExtrapFunctor: 1.5 v_n - 0.5 v_{n-1}; update() shifts in a tree.
template <typename real_t, class Tree_t = Tree>
class FieldExtrapFunctor {
 public:
  FieldExtrapFunctor(Tree_t* tp, Tree_t* tc, BoundaryType bc = FreeSpace)
      : tp_(tp), tc_(tc), bc_(bc) {}
  void update(Tree_t* new_tree, real_t) {
    tp_ = tc_;
    tc_ = new_tree;
  }
  Tree_t* tp() const { return tp_; }
  Tree_t* tc() const { return tc_; }
  BoundaryType bc() const { return bc_; }

 private:
  Tree_t *tp_, *tc_;
  BoundaryType bc_;
};

// SolveSemilagInSitu with a FieldSetFunctor velocity: the cubic's weights at
// the times IntegrateRK2 queries (tinit and tinit + tau/2 of each sub-step,
// src/semilag/traj.inc:20-68), one tbslas_semilag_in_situ_tv call.
template <typename real_t>
void SolveSemilagInSitu(FieldSetFunctor<real_t, Tree>& f, Tree& tree_curr, const int timestep,
                        const double dt, int num_rk_step = 1) {
  std::vector<double> w(static_cast<size_t>(8 * num_rk_step));
  const double tinit = timestep * dt, tfinal = tinit - dt;
  const double tau = (tfinal - tinit) / num_rk_step;
  const double times[4] = {f.times()[0], f.times()[1], f.times()[2], f.times()[3]};
  double cur = tinit;
  for (int s = 0; s < num_rk_step; ++s) {
    check(tbslas_cubic_time_weights(times, cur, &w[8 * s]), "tbslas_cubic_time_weights");
    check(tbslas_cubic_time_weights(times, cur + 0.5 * tau, &w[8 * s + 4]),
          "tbslas_cubic_time_weights");
    cur = cur + tau;
  }
  tbslas_tree v[4];
  for (int k = 0; k < 4; ++k) v[k] = f.elems()[k]->get();
  check(tbslas_semilag_in_situ_tv(tree_curr.ctx().get(), 4, v, w.data(), tree_curr.get(), timestep,
                                  dt, num_rk_step, f.bc(), nullptr),
        "tbslas_semilag_in_situ_tv");
}

// The two-functor SolveSemilagInSitu: tvel_func at X, tvel_extrap at X*.
template <typename real_t>
void SolveSemilagInSitu(NodeFieldFunctor<real_t, Tree>& tvel_func,
                        FieldExtrapFunctor<real_t, Tree>& tvel_extrap, Tree& tree_curr,
                        const int timestep, const double dt, int num_rk_step = 1) {
  tbslas_tree v[3] = {tvel_extrap.tc()->get(), tvel_extrap.tp()->get(), tvel_func.node()->get()};
  const bool same = tvel_func.node() == tvel_extrap.tc();
  const int m = same ? 2 : 3;
  std::vector<double> w;
  for (int s = 0; s < num_rk_step; ++s) {
    const double first[3] = {same ? 1.0 : 0.0, 0.0, same ? 0.0 : 1.0};
    const double second[3] = {1.5, -0.5, 0.0};
    w.insert(w.end(), first, first + m);
    w.insert(w.end(), second, second + m);
  }
  check(tbslas_semilag_in_situ_tv(tree_curr.ctx().get(), m, v, w.data(), tree_curr.get(), timestep,
                                  dt, num_rk_step, tvel_extrap.bc(), nullptr),
        "tbslas_semilag_in_situ_tv");
}

// The advection-diffusion driver's BDF2 step at its running time tcurr:
// treen <- fit of 4/3 treec(X1) - 1/3 treep(X2).
template <typename real_t>
void SemilagBDF2(NodeFieldFunctor<real_t, Tree>& vel_evaluator, Tree& treep, Tree& treec,
                 Tree& treen, const double tcurr, const double dt, int num_rk_step = 1) {
  check(tbslas_semilag_bdf2(treen.ctx().get(), vel_evaluator.node()->get(), treep.get(),
                            treec.get(), treen.get(), tcurr, dt, num_rk_step, vel_evaluator.bc(),
                            nullptr),
        "tbslas_semilag_bdf2");
}

inline std::vector<double> new_nodes(int deg, int dim = 3) {
  if (dim != 3) throw std::invalid_argument("new_nodes: dim must be 3");
  std::vector<double> y(static_cast<size_t>(deg + 1) * (deg + 1) * (deg + 1) * 3);
  check(tbslas_cheb_nodes(deg, y.data()), "tbslas_cheb_nodes");
  return y;
}

// M is (q+1)^3 x Nc, row-major.
inline void GetPt2CoeffMatrix(int cheb_deg, std::vector<double>& M) {
  const size_t d = cheb_deg + 1;
  M.resize(d * d * d * (d * (d + 1) * (d + 2) / 6));
  check(tbslas_pt2coeff_matrix(cheb_deg, M.data()), "tbslas_pt2coeff_matrix");
}

}  // namespace tbslas_gb300

#endif  // TBSLAS_GB300_HPP_

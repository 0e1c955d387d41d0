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

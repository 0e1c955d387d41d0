// Entry points of the checkpointed forward step and its adjoint (the
// differentiation pattern of the SL step; no reference counterpart).
#include <cmath>

#include "adjoint_df.cuh"

namespace tbg {

constexpr int kAdjMaxDegree = 10;


struct AdjTable {
  AdjFn adj[kAdjMaxDegree + 1] = {};
  AdjDfFn adj_df[kAdjMaxDegree + 1] = {};
  JacStepFn jac[kAdjMaxDegree + 1] = {};
  AdjTable() {
    register_adjoint_a(adj, adj_df, jac);
    register_adjoint_b(adj, adj_df, jac);
    register_adjoint_c(adj, adj_df, jac);
  }
};
const AdjTable g_adj;

int launch_semilag_jac(int q, const SemilagTreeArgs& a, cudaStream_t s) {
  if (q < 1 || q > kAdjMaxDegree || !g_adj.jac[q])
    return fail_status(TBSLAS_ERR_UNSUPPORTED,
                       "the velocity Jacobian checkpoint supports Chebyshev degree 1..10");
  g_adj.jac[q](a, s);
  return TBSLAS_OK;
}

int check_pair(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con, double dt, int bc, TreeView* tv,
               TreeView* tc) {
  tbslas_ctx cv = nullptr, cc = nullptr;
  int st = tree_view(vel, tv, &cv);
  if (st != TBSLAS_OK) return st;
  st = tree_view(con, tc, &cc);
  if (st != TBSLAS_OK) return st;
  if (cv != ctx || cc != ctx) return fail_status(TBSLAS_ERR_INVALID_ARG, "trees of another context");
  if (tv->dof != 3 || tc->dof != 1 || tv->q != tc->q)
    return fail_status(TBSLAS_ERR_UNSUPPORTED,
                       "adjoint step needs a dof-3 velocity and a dof-1 concentration tree of one degree");
  if (tc->q < 1 || tc->q > kAdjMaxDegree)
    return fail_status(TBSLAS_ERR_UNSUPPORTED, "adjoint step supports Chebyshev degree 1..10");
  if (!std::isfinite(dt)) return fail_status(TBSLAS_ERR_INVALID_ARG, "dt is not finite");
  if (bc != TBSLAS_BC_FREESPACE && bc != TBSLAS_BC_PERIODIC)
    return fail_status(TBSLAS_ERR_INVALID_ARG, "invalid boundary condition");
  int dev = 0, sms = 0;
  st = ctx_info(ctx, &dev, &sms);
  if (st != TBSLAS_OK) return st;
  if (cudaSetDevice(dev) != cudaSuccess) return fail_status(TBSLAS_ERR_CUDA, "cudaSetDevice");
  return TBSLAS_OK;
}

double step_tau_host(int timestep, double dt) {
  const double tinit = timestep * dt;
  const double tfinal = tinit - dt;
  return (tfinal - tinit) / 1;
}

int launched(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_status(TBSLAS_ERR_CUDA, what);
  return TBSLAS_OK;
}

}  // namespace tbg

using namespace tbg;

extern "C" int tbslas_semilag_in_situ_ckpt(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con,
                                           int timestep, double dt, int bc, double* xmid_dev,
                                           double* xdep_dev, void* stream) {
  // the in-situ step itself (the context's sum mode), storing the points
  DeviceRestore restore;
  TreeView tv, tc;
  int st = check_pair(ctx, vel, con, dt, bc, &tv, &tc);
  if (st != TBSLAS_OK) return st;
  if (!xdep_dev) return fail_status(TBSLAS_ERR_INVALID_ARG, "null departure-point buffer");
  return semilag_in_situ_points(ctx, vel, con, timestep, dt, bc, xmid_dev, xdep_dev,
                                (cudaStream_t)stream);
}

extern "C" int tbslas_semilag_in_situ_ckpt_jac(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con,
                                               int timestep, double dt, int bc, double* xmid_dev,
                                               double* xdep_dev, double* jac_dev, void* stream) {
  DeviceRestore restore;
  TreeView tv, tc;
  int st = check_pair(ctx, vel, con, dt, bc, &tv, &tc);
  if (st != TBSLAS_OK) return st;
  if (!xmid_dev || !xdep_dev || !jac_dev)
    return fail_status(TBSLAS_ERR_INVALID_ARG, "null checkpoint buffer");
  if (ctx_sums(ctx) != TBSLAS_SUMS_FP64)
    return fail_status(TBSLAS_ERR_UNSUPPORTED, "the velocity Jacobian checkpoint needs FP64 sums");
  return semilag_in_situ_points(ctx, vel, con, timestep, dt, bc, xmid_dev, xdep_dev,
                                (cudaStream_t)stream, jac_dev);
}

namespace tbg {

// One adjoint step.  vn_given: the velocity at con's nodes (or null); wnode_acc:
// where the node term's weights are summed over a sequence of steps (null:
// this step scatters its own); jac_dev: the forward's J_v(X*) checkpoint (or
// null).
int semilag_adjoint(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con,
                    const double* con_coeff_k_dev, int timestep, double dt, int bc,
                    const double* lambda_next_dev, double* lambda_k_dev, double* grad_vel_dev,
                    const double* xmid_dev, const double* xdep_dev, const double* vn_given,
                    double* wnode_acc, cudaStream_t s, const double* jac_dev = nullptr) {
  TreeView tv, tc;
  int st = check_pair(ctx, vel, con, dt, bc, &tv, &tc);
  if (st != TBSLAS_OK) return st;
  if (!con_coeff_k_dev || !lambda_next_dev || !lambda_k_dev || !grad_vel_dev)
    return fail_status(TBSLAS_ERR_INVALID_ARG, "null buffer");
  if (xmid_dev && !xdep_dev)
    return fail_status(TBSLAS_ERR_INVALID_ARG, "midpoints without departure points");
  if (jac_dev && (!xmid_dev || !xdep_dev))
    return fail_status(TBSLAS_ERR_INVALID_ARG,
                       "the Jacobian checkpoint needs the midpoints and departure points");
  if (jac_dev && ctx_sums(ctx) != TBSLAS_SUMS_FP64)
    return fail_status(TBSLAS_ERR_UNSUPPORTED, "the velocity Jacobian checkpoint needs FP64 sums");
  const int q = tc.q, d = q + 1;
  const int64_t np = (int64_t)d * d * d, nc = (int64_t)d * (d + 1) * (d + 2) / 6;
  double* mu = nullptr;
  st = ctx_mu_scratch(ctx, tc.L * np, &mu);
  if (st != TBSLAS_OK) return st;
  const double* F = nullptr;
  st = ctx_F(ctx, q, &F);
  if (st != TBSLAS_OK) return st;
  // mu = lambda^{k+1} M^T, one row of Np node weights per leaf
  {
    ProfBracket pb(ctx, "adjoint_refit_t", s);
    launch_refit_t(lambda_next_dev, F, q, tc.L, mu, ctx_sums(ctx) == TBSLAS_SUMS_DOUBLE_FLOAT, s);
  }
  st = launched("transposed refit launch");
  if (st != TBSLAS_OK) return st;
  if (cudaMemsetAsync(lambda_k_dev, 0, sizeof(double) * tc.L * nc, s) != cudaSuccess)
    return fail_status(TBSLAS_ERR_CUDA, "cudaMemsetAsync");
  AdjArgs a;
  a.vel = tv;
  a.con = tc;
  a.con.coeff = con_coeff_k_dev;
  a.con.stride = nc;
  a.nodes = ctx_nodes(q);
  a.tau = step_tau_host(timestep, dt);
  a.periodic = bc;
  a.mu = mu;
  a.xmid = xmid_dev;
  a.xdep = xdep_dev;
  a.lambda = lambda_k_dev;
  a.grad_vel = grad_vel_dev;
  a.wnode = wnode_acc;
  a.wnode_add = wnode_acc ? 1 : 0;
  a.jac = jac_dev;
  const bool df = ctx_sums(ctx) == TBSLAS_SUMS_DOUBLE_FLOAT;
  if (!wnode_acc) {
    st = ctx_wnode_scratch(ctx, tc.L * np * 3, &a.wnode);
    if (st != TBSLAS_OK) return st;
  }
  if (!xdep_dev) {
    // recompute: the step's points by its own kernels (double-float: FP64
    // for the ambiguous targets)
    double *xm = nullptr, *xd = nullptr;
    st = step_points(ctx, vel, con, timestep, dt, bc, &xm, &xd, s, vn_given);
    if (st != TBSLAS_OK) return st;
    a.xmid = xm;
    a.xdep = xd;
  } else if (!xmid_dev) {
    // departure points checkpointed: the midpoints from the node-grid
    // velocity, exactly as the forward formed them
    double* xm = nullptr;
    st = step_midpoints(ctx, vel, con, timestep, dt, bc, &xm, s, vn_given);
    if (st != TBSLAS_OK) return st;
    a.xmid = xm;
  }
  if (df) {
    // the sums in double-float over a hi/lo split of c^k
    float2* c2 = nullptr;
    st = ctx_c2_scratch(ctx, tc.L * nc, &c2);
    if (st != TBSLAS_OK) return st;
    {
      ProfBracket pb(ctx, "adjoint_split", s);
      launch_split(con_coeff_k_dev, c2, tc.L * nc, ctx_err(ctx), s);
    }
    ProfBracket pb(ctx, "adjoint_df", s);
    g_adj.adj_df[q](a, c2, s);
  } else {
    ProfBracket pb(ctx, "adjoint_fp64", s);
    g_adj.adj[q](a, s);
  }
  st = launched("adjoint step launch");
  if (st != TBSLAS_OK) return st;
  if (!wnode_acc) {
    // the node term by the transposed node-grid passes
    ProfBracket pb(ctx, "adjoint_node_scatter", s);
    launch_scatter_on_nodes(tv, tc, bc, a.wnode, grad_vel_dev, 3 * nc, df, s);
  }
  return launched("adjoint step launch");
}

}  // namespace tbg

extern "C" int tbslas_semilag_adjoint(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con,
                                      const double* con_coeff_k_dev, int timestep, double dt,
                                      int bc, const double* lambda_next_dev, double* lambda_k_dev,
                                      double* grad_vel_dev, const double* xmid_dev,
                                      const double* xdep_dev, void* stream) {
  DeviceRestore restore;
  return semilag_adjoint(ctx, vel, con, con_coeff_k_dev, timestep, dt, bc, lambda_next_dev,
                         lambda_k_dev, grad_vel_dev, xmid_dev, xdep_dev, nullptr, nullptr,
                         (cudaStream_t)stream);
}

extern "C" int tbslas_semilag_adjoint_seq(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con,
                                          const double* con_coeff_k_dev, int timestep, double dt,
                                          int bc, const double* lambda_next_dev,
                                          double* lambda_k_dev, double* grad_vel_dev,
                                          const double* xmid_dev, const double* xdep_dev,
                                          const double* vel_at_nodes_dev,
                                          double* node_weights_dev, void* stream) {
  DeviceRestore restore;
  if (!node_weights_dev) return fail_status(TBSLAS_ERR_INVALID_ARG, "null node-weight buffer");
  return semilag_adjoint(ctx, vel, con, con_coeff_k_dev, timestep, dt, bc, lambda_next_dev,
                         lambda_k_dev, grad_vel_dev, xmid_dev, xdep_dev, vel_at_nodes_dev,
                         node_weights_dev, (cudaStream_t)stream);
}

extern "C" int tbslas_semilag_adjoint_jac(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con,
                                          const double* con_coeff_k_dev, int timestep, double dt,
                                          int bc, const double* lambda_next_dev,
                                          double* lambda_k_dev, double* grad_vel_dev,
                                          const double* xmid_dev, const double* xdep_dev,
                                          const double* jac_dev, double* node_weights_dev,
                                          void* stream) {
  DeviceRestore restore;
  if (!jac_dev) return fail_status(TBSLAS_ERR_INVALID_ARG, "null Jacobian checkpoint");
  return semilag_adjoint(ctx, vel, con, con_coeff_k_dev, timestep, dt, bc, lambda_next_dev,
                         lambda_k_dev, grad_vel_dev, xmid_dev, xdep_dev, nullptr,
                         node_weights_dev, (cudaStream_t)stream, jac_dev);
}

extern "C" int tbslas_semilag_adjoint_node_term(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con,
                                                int bc, const double* node_weights_dev,
                                                double* grad_vel_dev, void* stream) {
  DeviceRestore restore;
  TreeView tv, tc;
  int st = check_pair(ctx, vel, con, 0.0, bc, &tv, &tc);
  if (st != TBSLAS_OK) return st;
  if (!node_weights_dev || !grad_vel_dev)
    return fail_status(TBSLAS_ERR_INVALID_ARG, "null buffer");
  const int d = tc.q + 1;
  const int64_t nc = (int64_t)d * (d + 1) * (d + 2) / 6;
  cudaStream_t s = (cudaStream_t)stream;
  {
    ProfBracket pb(ctx, "adjoint_node_scatter", s);
    launch_scatter_on_nodes(tv, tc, bc, node_weights_dev, grad_vel_dev, 3 * nc,
                            ctx_sums(ctx) == TBSLAS_SUMS_DOUBLE_FLOAT, s);
  }
  return launched("adjoint node-term launch");
}

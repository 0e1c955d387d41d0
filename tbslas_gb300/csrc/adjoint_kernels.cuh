// Adjoint kernels of the in-situ SL step (nrk = 1), instantiated per
// Chebyshev degree by adjoint_*.cu.
//
// Forward, per target node X of the concentration tree (c^k -> c^{k+1}):
//   X* = X + tau/2 v(X),  Xd = X + tau v(X*),  u = c^k(Xd),  C^{k+1} = refit(u).
// Adjoint of one step, given lambda^{k+1} = dJ/dC^{k+1}:
//   mu        = lambda^{k+1} M^T                  (transposed refit, per leaf)
//   g         = mu grad c^k(Xd)
//   lambda^k += mu phi(Xd)                        (scatter into Xd's leaf)
//   dJ/dV    += tau g (x) phi(X*)                  (scatter into X*'s velocity leaf)
//   dJ/dV    += tau^2/2 J_v(X*)^T g (x) phi(X)     (scatter into X's velocity leaf)
// phi = the triangular basis T_i(z) T_j(y) T_k(x) at the point's local
// coordinates; J_v = the velocity Jacobian.  The kernels (adjoint_f64.cuh in
// FP64, adjoint_df.cuh in double-float) share the helpers below.
#pragma once

#include "internal.h"
#include "tree_kernels.cuh"

namespace tbg {

struct AdjArgs {
  TreeView vel;        // velocity coefficients (read)
  TreeView con;        // geometry of the concentration tree, coefficients = c^k
  Nodes1D nodes;
  double tau;
  int periodic;
  const double* mu;    // [Lc * Np] dJ/du at the targets
  const double* xmid;  // checkpointed X* or null (recompute)
  const double* xdep;  // checkpointed Xd or null (recompute)
  double* lambda;      // [Lc][Nc] accumulated
  double* grad_vel;    // [Lv][3][Nc] accumulated
  double* wnode;       // [Lc * Np][3]: weights of the tau^2/2 term at the nodes for
                       // the node-grid scatter (launch_scatter_on_nodes)
  int wnode_add = 0;   // 1: the weights are added to wnode (a sequence of steps
                       // through one velocity sums them and scatters once)
  const double* jac = nullptr;  // [Lc * Np][9] the forward's J_v(X*) (row-major
                                // dv_a/dx_b), or null: formed here from vel
};

// T_k and dT_k/dxi for k < D; zero outside [-1,1] like cheb_T.
template <int D>
__device__ __forceinline__ void cheb_TdT(double xi, double (&T)[D], double (&dT)[D]) {
  const bool ok = abs_at_most_one(xi);
  const double x = ok ? xi : 0.0;
  T[0] = ok ? 1.0 : 0.0;
  dT[0] = 0.0;
  if (D > 1) {
    T[1] = x;
    dT[1] = ok ? 1.0 : 0.0;
  }
  const double x2 = twice(x);
#pragma unroll
  for (int k = 2; k < D; ++k) {
    T[k] = fma(x2, T[k - 1], -T[k - 2]);
    dT[k] = fma(x2, dT[k - 1], fma(2.0, T[k - 1], -dT[k - 2]));
  }
}

// Coefficient loaders for tri_grad: one dof, or sum_a g_a c^a over the three
// velocity components (the gradient of g . v in one sweep).
struct OneDof {
  const double* __restrict__ p;
  __device__ __forceinline__ double operator()(int i) const { return __ldg(p + i); }
};
struct Weighted3 {
  const double* __restrict__ p;
  int nc;
  double g0, g1, g2;
  __device__ __forceinline__ double operator()(int i) const {
    return fma(g2, __ldg(p + 2 * nc + i), fma(g1, __ldg(p + nc + i), g0 * __ldg(p + i)));
  }
};

// Gradient (d/dxi) of the triangular expansion with coefficients c(idx).
// Each sum starts from +0.0 and adds its terms by fused multiply-adds; the
// first terms (T_0 = 1 or 0, dT_0 = 0, dT_1 = 1 or 0, from cheb_TdT) are
// formed by fma_t0 with the same bits.
// val receives the expansion's value, bit-identical to tri_sum's (the same
// sums in the same order).
template <int D, class Load>
__device__ __forceinline__ void tri_grad_val(Load c, const double (&tx)[D],
                                             const double (&ty)[D], const double (&tz)[D],
                                             const double (&dx)[D], const double (&dy)[D],
                                             const double (&dz)[D], double (&g)[3],
                                             double& val) {
  double gx = 0.0, gy = 0.0, gz = 0.0, u = 0.0;
  int idx = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    double vx = 0.0, vy = 0.0, vz = 0.0;
#pragma unroll
    for (int j = 0; j < D - i; ++j) {
      const double c0 = c(idx);
      double w = fma_t0(tx[0], c0), wd = fma_t0(dx[0], c0);  // wd: +0, or NaN
      ++idx;
      if (D - i - j > 1) {
        // k = 1: dT_1 is 1 (or 0 outside [-1, 1]) and wd is +0 or NaN, so
        // fma(c1, dT_1, wd) is fma_t0's product unless wd is a NaN
        const double c1 = c(idx);
        w = fma(c1, tx[1], w);
        wd = (dbits(wd) & kBitsAbs) > 0x7FF0000000000000ull ? wd : fma_t0(dx[1], c1);
        ++idx;
      }
#pragma unroll
      for (int k = 2; k < D - i - j; ++k) {
        const double ck = c(idx);
        w = fma(ck, tx[k], w);
        wd = fma(ck, dx[k], wd);
        ++idx;
      }
      if (j == 0) {
        vx = fma_t0(ty[0], wd);
        vy = fma_t0(dy[0], w);
        vz = fma_t0(ty[0], w);
      } else {
        vx = fma(ty[j], wd, vx);
        vy = fma(dy[j], w, vy);
        vz = fma(ty[j], w, vz);
      }
    }
    if (i == 0) {
      gx = fma_t0(tz[0], vx);
      gy = fma_t0(tz[0], vy);
      gz = fma_t0(dz[0], vz);
      u = fma_t0(tz[0], vz);
    } else {
      gx = fma(tz[i], vx, gx);
      gy = fma(tz[i], vy, gy);
      gz = fma(dz[i], vz, gz);
      u = fma(tz[i], vz, u);
    }
  }
  g[0] = gx;
  g[1] = gy;
  g[2] = gz;
  val = u;
}

// Gradient only (the value's sums are dropped by the compiler).
template <int D, class Load>
__device__ __forceinline__ void tri_grad(Load c, const double (&tx)[D],
                                         const double (&ty)[D], const double (&tz)[D],
                                         const double (&dx)[D], const double (&dy)[D],
                                         const double (&dz)[D], double (&g)[3]) {
  double val;
  tri_grad_val<D>(c, tx, ty, tz, dx, dy, dz, g, val);
}

// Locate a point (wrapping it in place under periodic boundaries): leaf index
// or -1 (outside / NaN), its geometry and T_k of the local coordinates.
template <int D>
__device__ __forceinline__ int64_t locate(const TreeView& t, double& x, double& y, double& z,
                                          bool per, Geom& g) {
  if (per) wrap3(x, y, z);
  if (!inside(x, y, z, per)) return -1;
  const int64_t leaf = find_leaf(t, morton3(quantise(x), quantise(y), quantise(z)));
  g = load_geom(t.geom + leaf);
  return leaf;
}

typedef void (*AdjFn)(const AdjArgs&, cudaStream_t);
typedef void (*AdjDfFn)(const AdjArgs&, const float2*, cudaStream_t);
typedef void (*JacStepFn)(const SemilagTreeArgs&, cudaStream_t);
void register_adjoint_a(AdjFn* a, AdjDfFn* d, JacStepFn* j);
void register_adjoint_b(AdjFn* a, AdjDfFn* d, JacStepFn* j);
void register_adjoint_c(AdjFn* a, AdjDfFn* d, JacStepFn* j);

}  // namespace tbg

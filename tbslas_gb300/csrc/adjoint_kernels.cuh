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
// coordinates; J_v = the velocity Jacobian.  Scatters are CTA-cooperative:
// the block's points are staged in shared memory, then for each distinct
// leaf among them (usually one: consecutive targets sit in one leaf and move
// coherently) every thread sums a few coefficients over the block's points of
// that leaf and adds them to global memory with one FP64 atomic each.
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
                       // the node-grid scatter (launch_scatter_on_nodes), or null
};

// T_k and dT_k/dxi for k < D; zero outside [-1,1] like cheb_T.
template <int D>
__device__ __forceinline__ void cheb_TdT(double xi, double (&T)[D], double (&dT)[D]) {
  const bool ok = fabs(xi) <= 1.0;
  const double x = ok ? xi : 0.0;
  T[0] = ok ? 1.0 : 0.0;
  dT[0] = 0.0;
  if (D > 1) {
    T[1] = x;
    dT[1] = ok ? 1.0 : 0.0;
  }
  const double x2 = 2.0 * x;
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
template <int D, class Load>
__device__ __forceinline__ void tri_grad(Load c, const double (&tx)[D],
                                         const double (&ty)[D], const double (&tz)[D],
                                         const double (&dx)[D], const double (&dy)[D],
                                         const double (&dz)[D], double (&g)[3]) {
  double gx = 0.0, gy = 0.0, gz = 0.0;
  int idx = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    double vx = 0.0, vy = 0.0, vz = 0.0;
#pragma unroll
    for (int j = 0; j < D - i; ++j) {
      double w = 0.0, wd = 0.0;
#pragma unroll
      for (int k = 0; k < D - i - j; ++k) {
        const double ck = c(idx);
        w = fma(ck, tx[k], w);
        wd = fma(ck, dx[k], wd);
        ++idx;
      }
      vx = fma(ty[j], wd, vx);
      vy = fma(dy[j], w, vy);
      vz = fma(ty[j], w, vz);
    }
    gx = fma(tz[i], vx, gx);
    gy = fma(tz[i], vy, gy);
    gz = fma(dz[i], vz, gz);
  }
  g[0] = gx;
  g[1] = gy;
  g[2] = gz;
}

// Locate a point (wrapping it in place under periodic boundaries): leaf index
// or -1 (outside / NaN), its geometry and T_k of the local coordinates.
template <int D>
__device__ __forceinline__ int64_t locate(const TreeView& t, double& x, double& y, double& z,
                                          bool per, Geom& g) {
  if (per) {
    x = wrap1(x);
    y = wrap1(y);
    z = wrap1(z);
  }
  if (!inside(x, y, z, per)) return -1;
  const int64_t leaf = find_leaf(t, morton3(quantise(x), quantise(y), quantise(z)));
  g = load_geom(t.geom + leaf);
  return leaf;
}

constexpr int kAdjThreads = 128;

// Shared-memory staging of one block's points for a scatter.
template <int D>
struct AdjSmem {
  static constexpr int NIJ = D * (D + 1) / 2;
  double tx[kAdjThreads][D];
  double tzy[kAdjThreads][NIJ];  // T_i(z) T_j(y) over the (i, j) triangle
  double w[kAdjThreads][3];
  long long leaf[kAdjThreads];
  long long cur;
};

// out[leaf*stride + l*NC + n] += w[l] * phi_n(point), l < DOF, for every
// thread's point (leaf < 0: none).  All threads of the block call it.
template <int D, int DOF>
__device__ __forceinline__ void cta_scatter(AdjSmem<D>& sm, double* __restrict__ out,
                                            int64_t stride, int64_t leaf,
                                            const double (&w)[DOF], const double (&tx)[D],
                                            const double (&ty)[D], const double (&tz)[D]) {
  constexpr int NC = D * (D + 1) * (D + 2) / 6;
  constexpr int PER = (NC + kAdjThreads - 1) / kAdjThreads;
  const int tid = threadIdx.x;
  __syncthreads();  // the staging area is free
  sm.leaf[tid] = leaf;
  if (leaf >= 0) {
#pragma unroll
    for (int k = 0; k < D; ++k) sm.tx[tid][k] = tx[k];
    int ij = 0;
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D - i; ++j) sm.tzy[tid][ij++] = tz[i] * ty[j];
#pragma unroll
    for (int l = 0; l < DOF; ++l) sm.w[tid][l] = w[l];
  }
  // this thread's coefficients n = tid + c*blockDim -> (pair index, k)
  int my_ij[PER], my_k[PER];
#pragma unroll
  for (int c = 0; c < PER; ++c) {
    const int n = tid + c * kAdjThreads;
    int idx = 0, ij = 0;
    my_ij[c] = -1;
    my_k[c] = 0;
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D - i; ++j, ++ij) {
        const int len = D - i - j;
        if (n >= idx && n < idx + len) {
          my_ij[c] = ij;
          my_k[c] = n - idx;
        }
        idx += len;
      }
  }
  __syncthreads();
  for (;;) {
    if (tid < 32) {
      long long first = -1;
#pragma unroll
      for (int chunk = 0; chunk < kAdjThreads / 32; ++chunk) {
        const long long v = sm.leaf[chunk * 32 + tid];
        const unsigned m = __ballot_sync(0xffffffffu, v >= 0);
        if (m) {
          first = __shfl_sync(0xffffffffu, v, __ffs(m) - 1);
          break;
        }
      }
      if (tid == 0) sm.cur = first;
    }
    __syncthreads();
    const long long cur = sm.cur;
    if (cur < 0) break;
#pragma unroll
    for (int c = 0; c < PER; ++c) {
      if (my_ij[c] < 0) continue;
      double acc[DOF];
#pragma unroll
      for (int l = 0; l < DOF; ++l) acc[l] = 0.0;
      for (int p = 0; p < kAdjThreads; ++p) {
        if (sm.leaf[p] != cur) continue;
        const double t = sm.tzy[p][my_ij[c]] * sm.tx[p][my_k[c]];
#pragma unroll
        for (int l = 0; l < DOF; ++l) acc[l] = fma(sm.w[p][l], t, acc[l]);
      }
      const int n = tid + c * kAdjThreads;
#pragma unroll
      for (int l = 0; l < DOF; ++l)
        if (acc[l] != 0.0) atomicAdd(out + cur * stride + l * NC + n, acc[l]);
    }
    __syncthreads();
    if (sm.leaf[tid] == cur) sm.leaf[tid] = -1;
    __syncthreads();
  }
}

template <int D>
__global__ void __launch_bounds__(kAdjThreads) k_adjoint(const AdjArgs a) {
  constexpr int NP = D * D * D;
  constexpr int NC = D * (D + 1) * (D + 2) / 6;
  extern __shared__ __align__(16) unsigned char adj_smem_raw[];
  AdjSmem<D>& sm = *reinterpret_cast<AdjSmem<D>*>(adj_smem_raw);
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool active = t < a.con.L * NP;
  const bool per = a.periodic != 0;
  const int64_t tt = active ? t : 0;
  const int64_t leaf = tt / NP;
  const int p = (int)(tt - leaf * NP);
  const Geom gl = load_geom(a.con.geom + leaf);
  const double h = 2.0 / gl.w;
  double x = gl.x + h * a.nodes.x[p % D];
  double y = gl.y + h * a.nodes.x[(p / D) % D];
  double z = gl.z + h * a.nodes.x[p / (D * D)];
  double xs, ys, zs, xd, yd, zd;
  if (a.xmid) {
    xs = a.xmid[3 * tt];
    ys = a.xmid[3 * tt + 1];
    zs = a.xmid[3 * tt + 2];
    xd = a.xdep[3 * tt];
    yd = a.xdep[3 * tt + 1];
    zd = a.xdep[3 * tt + 2];
  } else {
    double v[3];
    double px = x, py = y, pz = z;
    eval_point<D, 3>(a.vel, px, py, pz, per, v);
    xs = fma(0.5 * a.tau, v[0], px);
    ys = fma(0.5 * a.tau, v[1], py);
    zs = fma(0.5 * a.tau, v[2], pz);
    double qx = xs, qy = ys, qz = zs;
    eval_point<D, 3>(a.vel, qx, qy, qz, per, v);
    xd = fma(a.tau, v[0], px);
    yd = fma(a.tau, v[1], py);
    zd = fma(a.tau, v[2], pz);
  }
  const double mu = active ? a.mu[tt] : 0.0;

  // dJ/du at Xd -> lambda^k, and g = mu grad c^k(Xd).
  double gvec[3] = {0.0, 0.0, 0.0};
  {
    Geom g;
    int64_t lf = locate<D>(a.con, xd, yd, zd, per, g);
    if (!active) lf = -1;
    double tx[D], ty[D], tz[D], dx[D], dy[D], dz[D];
    if (lf >= 0) {
      cheb_TdT<D>((xd - g.x) * g.w - 1.0, tx, dx);
      cheb_TdT<D>((yd - g.y) * g.w - 1.0, ty, dy);
      cheb_TdT<D>((zd - g.z) * g.w - 1.0, tz, dz);
      double gr[3];
      tri_grad<D>(OneDof{a.con.coeff + lf * a.con.stride}, tx, ty, tz, dx, dy, dz, gr);
      gvec[0] = mu * gr[0] * g.w;
      gvec[1] = mu * gr[1] * g.w;
      gvec[2] = mu * gr[2] * g.w;
    } else {
#pragma unroll
      for (int k = 0; k < D; ++k) tx[k] = ty[k] = tz[k] = 0.0;
    }
    const double w[1] = {mu};
    cta_scatter<D, 1>(sm, a.lambda, NC, lf, w, tx, ty, tz);
  }
  // Velocity terms at X*: tau g (x) phi(X*), and J_v(X*)^T g for the X term.
  double jtg[3] = {0.0, 0.0, 0.0};
  {
    Geom g;
    int64_t lf = locate<D>(a.vel, xs, ys, zs, per, g);
    if (!active) lf = -1;
    double tx[D], ty[D], tz[D], dx[D], dy[D], dz[D];
    if (lf >= 0) {
      cheb_TdT<D>((xs - g.x) * g.w - 1.0, tx, dx);
      cheb_TdT<D>((ys - g.y) * g.w - 1.0, ty, dy);
      cheb_TdT<D>((zs - g.z) * g.w - 1.0, tz, dz);
      // J_v^T g = grad (g . v) at X*
      double gr[3];
      tri_grad<D>(Weighted3{a.vel.coeff + lf * a.vel.stride, NC, gvec[0], gvec[1], gvec[2]}, tx,
                  ty, tz, dx, dy, dz, gr);
      jtg[0] = gr[0] * g.w;
      jtg[1] = gr[1] * g.w;
      jtg[2] = gr[2] * g.w;
    } else {
#pragma unroll
      for (int k = 0; k < D; ++k) tx[k] = ty[k] = tz[k] = 0.0;
    }
    const double w[3] = {a.tau * gvec[0], a.tau * gvec[1], a.tau * gvec[2]};
    cta_scatter<D, 3>(sm, a.grad_vel, 3 * NC, lf, w, tx, ty, tz);
  }
  // tau^2/2 J_v(X*)^T g (x) phi(X)
  {
    Geom g;
    int64_t lf = locate<D>(a.vel, x, y, z, per, g);
    if (!active) lf = -1;
    double tx[D], ty[D], tz[D];
    if (lf >= 0) {
      cheb_T<D>((x - g.x) * g.w - 1.0, tx);
      cheb_T<D>((y - g.y) * g.w - 1.0, ty);
      cheb_T<D>((z - g.z) * g.w - 1.0, tz);
    } else {
#pragma unroll
      for (int k = 0; k < D; ++k) tx[k] = ty[k] = tz[k] = 0.0;
    }
    const double c2 = 0.5 * a.tau * a.tau;
    const double w[3] = {c2 * jtg[0], c2 * jtg[1], c2 * jtg[2]};
    cta_scatter<D, 3>(sm, a.grad_vel, 3 * NC, lf, w, tx, ty, tz);
  }
}

typedef void (*AdjFn)(const AdjArgs&, cudaStream_t);
typedef void (*AdjDfFn)(const AdjArgs&, const float2*, cudaStream_t);
void register_adjoint_a(AdjFn* a, AdjDfFn* d);
void register_adjoint_b(AdjFn* a, AdjDfFn* d);
void register_adjoint_c(AdjFn* a, AdjDfFn* d);

template <int D>
void launch_adjoint(const AdjArgs& a, cudaStream_t s) {
  const int64_t n = a.con.L * D * D * D;
  const size_t smem = sizeof(AdjSmem<D>);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_adjoint<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  if (n > 0)
    k_adjoint<D><<<(unsigned)((n + kAdjThreads - 1) / kAdjThreads), kAdjThreads, smem, s>>>(a);
}

}  // namespace tbg

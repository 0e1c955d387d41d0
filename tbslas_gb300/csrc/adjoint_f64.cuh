// The adjoint step (adjoint_kernels.cuh) in FP64, the library's default
// arithmetic: per target, the gradient g = mu grad c^k(Xd) and the scatter
// lambda^k += mu phi(Xd); then J_v(X*)^T g = grad(g . v)(X*) and the scatter
// dJ/dV += tau g (x) phi(X*); the tau^2/2 J_v(X*)^T g (x) phi(X) term is
// written per target for the transposed node-grid passes
// (launch_scatter_on_nodes).  The points X* and Xd are the step's own
// (checkpointed by the forward or recomputed by its FP64 kernel).
//
// Work per target, in FP64 multiply-adds: 2 Nc for grad c^k(Xd), 5 Nc for
// grad(g . v)(X*) (three to form sum_a g_a c_a per coefficient, two for the
// value and derivative sums), and per (point, coefficient) of the scatters
// one multiply-add for lambda (the weight folded into T_i(z) T_j(y)) and
// three for the velocity (each component's weight folded into its own copy
// of T_k(x), 3 D products per point): Nc + 3 Nc -- 11 Nc against the forward
// step's 4 Nc.  Where the three copies would cost the second CTA per SM
// (q >= 9) the velocity scatter forms T_i(z) T_j(y) * T_k(x) once per pair
// instead (4 Nc).
#pragma once

#include "adjoint_kernels.cuh"

namespace tbg {

// Targets (threads) per CTA: every warp owns one coefficient per scatter pass
// at q = 8 (Nc = 165), as in the double-float kernel.
constexpr int kAdjF64Threads = 192;

// Shared memory of the FP64 adjoint.  Every thread owns NS slots of one
// double each (element e of thread t at slots[e * BS + t]; BS odd, so that a
// warp reading different elements of one point's column spreads over the
// banks).  Slot map of a point, written before each scatter:
//   [0, NIJ)          T_i(z) T_j(y) over the (i, j) triangle, i outer (times
//                     the weight when the scatter has one component)
//   one component:    [NIJ, NIJ + D) T_k(x)
//   three, FOLD:      [NIJ + l D, + D) w_l T_k(x) for l = 0, 1, 2
//   three, otherwise: [NIJ, NIJ + D) T_k(x), [NIJ + D, + 3) the weights
template <int D>
struct AdjF64Shared {
  static constexpr int BS = kAdjF64Threads + 1;
  static constexpr int NIJ = D * (D + 1) / 2;
  // the folded layout where two CTAs per SM still fit (228 KB per SM, 1 KB
  // reserved per CTA)
  static constexpr bool FOLD = (size_t)(NIJ + 3 * D) * BS * 8 + 2048 <= 113 * 1024;
  static constexpr int NS = FOLD ? NIJ + 3 * D : NIJ + D + 3;
  double slots[NS * BS];
  int leaf[kAdjF64Threads];            // scatter leaf of each point (-1: none / done)
  unsigned char list[kAdjF64Threads];  // points of the leaf in progress
  int wcount[kAdjF64Threads / 32];
  int cur;
};

// Slot offsets of T_i(z) T_j(y) and T_k(x) for this thread's scatter
// coefficients n = tid + c * blockDim (triangular order; ozy < 0: none).
template <int D, int PER>
__device__ __forceinline__ void scatter_offsets_f64(int (&ozy)[PER], int (&ox)[PER]) {
  constexpr int BS = AdjF64Shared<D>::BS;
  constexpr int NIJ = AdjF64Shared<D>::NIJ;
#pragma unroll
  for (int c = 0; c < PER; ++c) {
    const int n = threadIdx.x + c * kAdjF64Threads;
    int idx = 0, ij = 0;
    ozy[c] = -1;
    ox[c] = 0;
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D - i; ++j, ++ij) {
        const int len = D - i - j;
        if (n >= idx && n < idx + len) {
          ozy[c] = ij * BS;
          ox[c] = (NIJ + n - idx) * BS;
        }
        idx += len;
      }
  }
}

// out[leaf*stride + l*NC + n] += w[l] * phi_n(point) for every thread's point
// (lf < 0: none).  For each distinct leaf among the block's points, in order
// of first appearance, the points of that leaf are listed (ballot
// compaction, in thread order) and every thread sums its coefficients over
// the list, adding each to global memory with one FP64 atomic.  All threads
// of the block call it; it ends after a barrier that every thread passes
// once it has finished reading the slots, so the next call may rewrite them.
template <int D, int DOF, int PER>
__device__ __forceinline__ void scatter_f64(AdjF64Shared<D>& sm, double* __restrict__ out,
                                            int64_t stride, int64_t lf, const double (&tx)[D],
                                            const double (&ty)[D], const double (&tz)[D],
                                            const double (&w)[DOF], const int (&ozy)[PER],
                                            const int (&ox)[PER]) {
  constexpr int NC = D * (D + 1) * (D + 2) / 6;
  constexpr int BS = AdjF64Shared<D>::BS;
  constexpr int NIJ = AdjF64Shared<D>::NIJ;
  constexpr int NW = kAdjF64Threads / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (lf >= 0) {
    // one component: the weight folded into the (i, j) products, so each
    // (point, coefficient) pair costs one multiply-add
    double* const col = sm.slots + tid;
    int ij = 0;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      const double zi = DOF == 1 ? (i == 0 ? mul_t0(tz[0], w[0]) : w[0] * tz[i]) : tz[i];
#pragma unroll
      for (int j = 0; j < D - i; ++j, ++ij) col[ij * BS] = j == 0 ? mul_t0(ty[0], zi) : zi * ty[j];
    }
#pragma unroll
    if (DOF == 1 || !AdjF64Shared<D>::FOLD) {
#pragma unroll
      for (int k = 0; k < D; ++k) col[(NIJ + k) * BS] = tx[k];
      if (DOF > 1) {
#pragma unroll
        for (int l = 0; l < DOF; ++l) col[(NIJ + D + l) * BS] = w[l];
      }
    } else {
#pragma unroll
      for (int l = 0; l < DOF; ++l)
#pragma unroll
        for (int k = 0; k < D; ++k)
          col[(NIJ + l * D + k) * BS] = k == 0 ? mul_t0(tx[0], w[l]) : w[l] * tx[k];
    }
  }
  const int my_leaf = lf >= 0 ? (int)lf : -1;
  sm.leaf[tid] = my_leaf;
  bool pending = my_leaf >= 0;
  __syncthreads();
  for (;;) {
    if (warp == 0) {
      int first = -1;
#pragma unroll
      for (int chunk = 0; chunk < NW; ++chunk) {
        const int v = sm.leaf[chunk * 32 + lane];
        const unsigned m = __ballot_sync(0xffffffffu, v >= 0);
        if (m) {
          first = __shfl_sync(0xffffffffu, v, __ffs(m) - 1);
          break;
        }
      }
      if (lane == 0) sm.cur = first;
    }
    __syncthreads();
    const int cur = sm.cur;
    if (cur < 0) break;
    const bool mine = pending && my_leaf == cur;
    const unsigned m = __ballot_sync(0xffffffffu, mine);
    if (lane == 0) sm.wcount[warp] = __popc(m);
    __syncthreads();
    int base = 0, total = 0;
#pragma unroll
    for (int w2 = 0; w2 < NW; ++w2) {
      const int c = sm.wcount[w2];
      base += w2 < warp ? c : 0;
      total += c;
    }
    if (mine) {
      sm.list[base + __popc(m & ((1u << lane) - 1u))] = (unsigned char)tid;
      sm.leaf[tid] = -1;
      pending = false;
    }
    __syncthreads();
    double acc[PER][DOF];
#pragma unroll
    for (int c = 0; c < PER; ++c)
#pragma unroll
      for (int l = 0; l < DOF; ++l) acc[c][l] = 0.0;
#pragma unroll 2
    for (int k = 0; k < total; ++k) {
      const double* const pc = sm.slots + sm.list[k];
      if (DOF == 1) {
#pragma unroll
        for (int c = 0; c < PER; ++c)
          if (ozy[c] >= 0) acc[c][0] = fma(pc[ozy[c]], pc[ox[c]], acc[c][0]);
        continue;
      }
      if (AdjF64Shared<D>::FOLD) {
#pragma unroll
        for (int c = 0; c < PER; ++c) {
          if (ozy[c] < 0) continue;
          const double zy = pc[ozy[c]];
#pragma unroll
          for (int l = 0; l < DOF; ++l) acc[c][l] = fma(zy, pc[ox[c] + l * D * BS], acc[c][l]);
        }
        continue;
      }
      double wp[DOF];
#pragma unroll
      for (int l = 0; l < DOF; ++l) wp[l] = pc[(NIJ + D + l) * BS];
#pragma unroll
      for (int c = 0; c < PER; ++c) {
        if (ozy[c] < 0) continue;
        const double t = pc[ozy[c]] * pc[ox[c]];
#pragma unroll
        for (int l = 0; l < DOF; ++l) acc[c][l] = fma(wp[l], t, acc[c][l]);
      }
    }
#pragma unroll
    for (int c = 0; c < PER; ++c) {
      if (ozy[c] < 0) continue;
      const int n = tid + c * kAdjF64Threads;
#pragma unroll
      for (int l = 0; l < DOF; ++l)
        // acc != 0.0 as a bit test (integer pipe; NaN counts as nonzero)
        if (dbits(acc[c][l]) & kBitsAbs)
          atomicAdd(out + (int64_t)cur * stride + l * NC + n, acc[c][l]);
    }
  }
}

// One thread per target node, its X* and Xd from a.xmid / a.xdep (required)
// and the node term's weights to a.wnode (required).  Two CTAs per SM up to
// q = 9 (shared memory: 72 doubles per target at q = 8).  JAC: J_v(X*) from
// the forward's checkpoint a.jac, so J_v(X*)^T g is nine multiply-adds
// instead of 5 Nc.
template <int D, bool JAC>
__global__ void __launch_bounds__(kAdjF64Threads, (D <= 10 ? 2 : 1))
    k_adjoint_f64(const AdjArgs a) {
  constexpr int NP = D * D * D;
  constexpr int NC = D * (D + 1) * (D + 2) / 6;
  constexpr int PER = (NC + kAdjF64Threads - 1) / kAdjF64Threads;
  extern __shared__ __align__(16) unsigned char adj_f64_raw[];
  AdjF64Shared<D>& sm = *reinterpret_cast<AdjF64Shared<D>*>(adj_f64_raw);
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool active = t < a.con.L * NP;
  const bool per = a.periodic != 0;
  const int64_t tt = active ? t : 0;
  double xs = a.xmid[3 * tt], ys = a.xmid[3 * tt + 1], zs = a.xmid[3 * tt + 2];
  double xd = a.xdep[3 * tt], yd = a.xdep[3 * tt + 1], zd = a.xdep[3 * tt + 2];
  const double mu = active ? a.mu[tt] : 0.0;
  int ozy[PER], ox[PER];
  scatter_offsets_f64<D, PER>(ozy, ox);

  // g = mu grad c^k(Xd); lambda^k += mu phi(Xd)
  double gvec[3] = {0.0, 0.0, 0.0};
  {
    Geom g;
    int64_t lf = locate<D>(a.con, xd, yd, zd, per, g);
    if (!active) lf = -1;
    double tx[D], ty[D], tz[D];
    if (lf >= 0) {
      double dx[D], dy[D], dz[D];
      cheb_TdT<D>((xd - g.x) * g.w - 1.0, tx, dx);
      cheb_TdT<D>((yd - g.y) * g.w - 1.0, ty, dy);
      cheb_TdT<D>((zd - g.z) * g.w - 1.0, tz, dz);
      double gr[3];
      tri_grad<D>(OneDof{a.con.coeff + lf * a.con.stride}, tx, ty, tz, dx, dy, dz, gr);
      gvec[0] = mu * gr[0] * g.w;
      gvec[1] = mu * gr[1] * g.w;
      gvec[2] = mu * gr[2] * g.w;
    }
    const double w[1] = {mu};
    scatter_f64<D, 1, PER>(sm, a.lambda, NC, lf, tx, ty, tz, w, ozy, ox);
  }
  // tau g (x) phi(X*) and J_v(X*)^T g = grad(g . v)(X*)
  double jtg[3] = {0.0, 0.0, 0.0};
  if (JAC) {
    Geom g;
    int64_t lf = locate<D>(a.vel, xs, ys, zs, per, g);
    if (!active) lf = -1;
    double tx[D], ty[D], tz[D];
    if (lf >= 0) {
      cheb_T<D>((xs - g.x) * g.w - 1.0, tx);
      cheb_T<D>((ys - g.y) * g.w - 1.0, ty);
      cheb_T<D>((zs - g.z) * g.w - 1.0, tz);
      const double* Jp = a.jac + 9 * tt;
#pragma unroll
      for (int b = 0; b < 3; ++b)
        jtg[b] = fma(gvec[2], __ldg(Jp + 6 + b),
                     fma(gvec[1], __ldg(Jp + 3 + b), gvec[0] * __ldg(Jp + b)));
    }
    const double w[3] = {a.tau * gvec[0], a.tau * gvec[1], a.tau * gvec[2]};
    scatter_f64<D, 3, PER>(sm, a.grad_vel, 3 * NC, lf, tx, ty, tz, w, ozy, ox);
  } else {
    Geom g;
    int64_t lf = locate<D>(a.vel, xs, ys, zs, per, g);
    if (!active) lf = -1;
    double tx[D], ty[D], tz[D];
    if (lf >= 0) {
      double dx[D], dy[D], dz[D];
      cheb_TdT<D>((xs - g.x) * g.w - 1.0, tx, dx);
      cheb_TdT<D>((ys - g.y) * g.w - 1.0, ty, dy);
      cheb_TdT<D>((zs - g.z) * g.w - 1.0, tz, dz);
      double gr[3];
      tri_grad<D>(Weighted3{a.vel.coeff + lf * a.vel.stride, NC, gvec[0], gvec[1], gvec[2]}, tx,
                  ty, tz, dx, dy, dz, gr);
      jtg[0] = gr[0] * g.w;
      jtg[1] = gr[1] * g.w;
      jtg[2] = gr[2] * g.w;
    }
    const double w[3] = {a.tau * gvec[0], a.tau * gvec[1], a.tau * gvec[2]};
    scatter_f64<D, 3, PER>(sm, a.grad_vel, 3 * NC, lf, tx, ty, tz, w, ozy, ox);
  }
  // tau^2/2 J_v(X*)^T g (x) phi(X): X is a node, the node-grid scatter adds it
  if (active) {
    const double c2 = 0.5 * a.tau * a.tau;
    double* w = a.wnode + 3 * t;
    if (a.wnode_add) {
      w[0] += c2 * jtg[0];
      w[1] += c2 * jtg[1];
      w[2] += c2 * jtg[2];
    } else {
      w[0] = c2 * jtg[0];
      w[1] = c2 * jtg[1];
      w[2] = c2 * jtg[2];
    }
  }
}

template <int D>
void launch_adjoint_f64(const AdjArgs& a, cudaStream_t s) {
  const int64_t n = a.con.L * D * D * D;
  const size_t smem = sizeof(AdjF64Shared<D>);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_adjoint_f64<D, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    cudaFuncSetAttribute(k_adjoint_f64<D, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    attr = true;
  }
  if (n <= 0) return;
  const unsigned grid = (unsigned)((n + kAdjF64Threads - 1) / kAdjF64Threads);
  if (a.jac)
    k_adjoint_f64<D, true><<<grid, kAdjF64Threads, smem, s>>>(a);
  else
    k_adjoint_f64<D, false><<<grid, kAdjF64Threads, smem, s>>>(a);
}

// ---------------------------------------------------------------------------
// The checkpointed forward step with the velocity Jacobian: v and its
// gradient at a point of a dof-3 tree (wrapped in place under periodic
// boundaries, as eval_point), v bit-identical to eval_point<D, 3>, J[3a+b] =
// dv_a/dx_b; all zero outside the domain.
template <int D>
__device__ __forceinline__ void eval_point_jac(const TreeView& t, double& x, double& y,
                                               double& z, bool per, double (&v)[3],
                                               double (&J)[9]) {
  constexpr int NC = D * (D + 1) * (D + 2) / 6;
  Geom g;
  const int64_t lf = locate<D>(t, x, y, z, per, g);
  if (lf < 0) {
#pragma unroll
    for (int l = 0; l < 3; ++l) v[l] = 0.0;
#pragma unroll
    for (int l = 0; l < 9; ++l) J[l] = 0.0;
    return;
  }
  double tx[D], ty[D], tz[D], dx[D], dy[D], dz[D];
  cheb_TdT<D>((x - g.x) * g.w - 1.0, tx, dx);
  cheb_TdT<D>((y - g.y) * g.w - 1.0, ty, dy);
  cheb_TdT<D>((z - g.z) * g.w - 1.0, tz, dz);
  const double* c = t.coeff + lf * t.stride;
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    double gr[3];
    tri_grad_val<D>(OneDof{c + l * NC}, tx, ty, tz, dx, dy, dz, gr, v[l]);
#pragma unroll
    for (int b = 0; b < 3; ++b) J[3 * l + b] = gr[b] * g.w;
  }
}

// k_semilag_tree<D> with the first stage from the node grid (a.vn), nrk = 1,
// storing X* (a.xmid), Xd (a.xdep) and J_v(X*) (a.jac) of every target:
// the same points and node values, bit for bit (the midpoint velocity by
// tri_grad_val, whose value sums are tri_sum's).
template <int D>
__global__ void __launch_bounds__(128) k_semilag_tree_jac(const SemilagTreeArgs a) {
  constexpr int NP = D * D * D;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= a.con.L * NP) return;
  const int64_t leaf = t / NP;
  const int p = (int)(t - leaf * NP);
  const Geom g = load_geom(a.con.geom + leaf);
  const double h = leaf_side(g);
  double x = g.x + h * a.nodes.x[p % D];
  double y = g.y + h * a.nodes.x[(p / D) % D];
  double z = g.z + h * a.nodes.x[p / (D * D)];
  const bool per = a.periodic != 0;
  if (per) wrap3(x, y, z);
  const double half_tau = 0.5 * a.tau;
  const double* vn = a.vn + 3 * node_source(a.face, t);
  double px = fma(half_tau, __ldg(vn + 0), x);
  double py = fma(half_tau, __ldg(vn + 1), y);
  double pz = fma(half_tau, __ldg(vn + 2), z);
  store_point(a.xmid, t, px, py, pz);
  double v[3], J[9];
  eval_point_jac<D>(a.vel, px, py, pz, per, v, J);
  x = fma(a.tau, v[0], x);
  y = fma(a.tau, v[1], y);
  z = fma(a.tau, v[2], z);
  store_point(a.xdep, t, x, y, z);
  double* Jo = a.jac + 9 * t;
#pragma unroll
  for (int l = 0; l < 9; ++l) Jo[l] = J[l];
  double c[1];
  eval_point<D, 1>(a.con, x, y, z, per, c);
  a.vals[t] = c[0];
}

template <int D>
void launch_semilag_tree_jac(const SemilagTreeArgs& a, cudaStream_t s) {
  const int64_t n = a.con.L * D * D * D;
  if (n > 0) k_semilag_tree_jac<D><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a);
}

}  // namespace tbg

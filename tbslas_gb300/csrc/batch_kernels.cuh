// Persistent batched SL kernel, instantiated per degree band by the
// batch_band_*.cu translation units (so the bands compile in parallel).
#pragma once

#include "tree_kernels.cuh"

namespace tbg {

struct BatchProblem {
  TreeView vel;   // dof 3
  TreeView con;   // dof 1, same degree
  Nodes1D nodes;  // 1-D Chebyshev nodes of degree q
  double* vals;   // [n_targets] node values of this problem
  double dt;
  int64_t n_targets;
  int q;
  int nrk;
};

struct BatchItem {
  int64_t start;
  int32_t problem;
  int32_t count;
};

struct BatchLaunch {
  const BatchProblem* probs;
  const BatchItem* items;  // this band's chunks
  int64_t n_items;
  unsigned long long* counter;
  const int* ts0;  // device scalar: first timestep of the run
  int step;        // step index inside the run
  int periodic;
};

// Degree bands: q 1..8, 9..12, 13..16.
constexpr int kBands = 3;
__host__ __device__ inline int band_of(int q) { return q <= 8 ? 0 : (q <= 12 ? 1 : 2); }



// tau of SolveSemilagRK2 for this timestep (semilag.inc:30-32, traj.inc:55),
// with the host's rounding (no contraction).
__device__ __forceinline__ double step_tau(int ts, double dt, int nrk) {
  const double tinit = __dmul_rn((double)ts, dt);
  const double tfinal = __dsub_rn(tinit, dt);
  return __ddiv_rn(__dsub_rn(tfinal, tinit), (double)nrk);
}

// One target of one problem: the arithmetic of k_semilag_tree<D>.
template <int D>
__device__ __forceinline__ void batch_target(const BatchProblem& p, int64_t t, double tau,
                                             bool per) {
  constexpr int NP = D * D * D;
  const int64_t leaf = t / NP;
  const int pi = (int)(t - leaf * NP);
  const Geom g = load_geom(p.con.geom + leaf);
  const double h = 2.0 / g.w;
  double x = g.x + h * p.nodes.x[pi % D];
  double y = g.y + h * p.nodes.x[(pi / D) % D];
  double z = g.z + h * p.nodes.x[pi / (D * D)];
  rk2_backtrace<D>(p.vel, x, y, z, tau, p.nrk, per);
  double c[1];
  eval_point<D, 1>(p.con, x, y, z, per, c);
  p.vals[t] = c[0];
}

template <int QLO, int QHI>
__device__ __forceinline__ void batch_dispatch(int q, const BatchProblem& p, int64_t t, double tau,
                                               bool per) {
  if constexpr (QLO <= QHI) {
    if (q == QLO)
      batch_target<QLO + 1>(p, t, tau, per);
    else
      batch_dispatch<QLO + 1, QHI>(q, p, t, tau, per);
  }
}

// Persistent CTAs take chunks of targets from an atomic counter; the chunk's
// problem descriptor is staged in shared memory.
template <int QLO, int QHI>
__global__ void __launch_bounds__(256) k_batch_semilag(const BatchLaunch a) {
  __shared__ BatchProblem sp;
  __shared__ int64_t s_item;
  const bool per = a.periodic != 0;
  const int ts = *a.ts0 + a.step;
  for (;;) {
    if (threadIdx.x == 0) s_item = (int64_t)atomicAdd(a.counter, 1ull);
    __syncthreads();
    const int64_t it = s_item;
    if (it >= a.n_items) return;
    const BatchItem w = a.items[it];
    if (threadIdx.x == 0) sp = a.probs[w.problem];
    __syncthreads();
    const double tau = step_tau(ts, sp.dt, sp.nrk);
    const int q = sp.q;
    for (int k = threadIdx.x; k < w.count; k += blockDim.x)
      batch_dispatch<QLO, QHI>(q, sp, w.start + k, tau, per);
    __syncthreads();  // s_item and sp are rewritten for the next chunk
  }
}

}  // namespace tbg

namespace tbg {
void launch_batch_band_0(const BatchLaunch& a, int grid, int block, cudaStream_t s);
void launch_batch_band_1(const BatchLaunch& a, int grid, int block, cudaStream_t s);
void launch_batch_band_2(const BatchLaunch& a, int grid, int block, cudaStream_t s);
inline void launch_batch_band(int band, const BatchLaunch& a, int grid, int block,
                              cudaStream_t s) {
  if (band == 0) launch_batch_band_0(a, grid, block, s);
  else if (band == 1) launch_batch_band_1(a, grid, block, s);
  else launch_batch_band_2(a, grid, block, s);
}
}  // namespace tbg

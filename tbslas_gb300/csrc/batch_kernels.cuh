// Persistent batched SL kernel, instantiated per degree band by the
// batch_band_*.cu translation units (so the bands compile in parallel).
#pragma once

#include <atomic>

#include "tree_kernels.cuh"

namespace tbg {

struct BatchProblem {
  TreeView vel;   // dof 3
  TreeView con;   // dof 1, same degree
  Nodes1D nodes;  // 1-D Chebyshev nodes of degree q
  double* vals;   // [n_targets] node values of this problem
  const double* vn;  // [n_targets][3] velocity at the targets (first RK stage)
  const int32_t* face;  // con's face map: vn holds no shared upper-face nodes, or null
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
  int64_t* fix_list;              // (problem << 40 | target) handed to the FP64 pass
  unsigned long long* fix_count;  // shared by the bands of one step
};
constexpr int kFixShift = 40;

// Degree bands, one translation unit each (the unrolled sums of the high
// degrees dominate compile time): q 1..8, 9..11, 12..13, 14, 15, 16.
constexpr int kBands = 6;
__host__ __device__ inline int band_of(int q) {
  return q <= 8 ? 0 : (q <= 11 ? 1 : (q <= 13 ? 2 : q - 11));
}



// tau of SolveSemilagRK2 for this timestep (semilag.inc:30-32, traj.inc:55),
// with the host's rounding (no contraction).
__device__ __forceinline__ double step_tau(int ts, double dt, int nrk) {
  const double tinit = __dmul_rn((double)ts, dt);
  const double tfinal = __dsub_rn(tinit, dt);
  return __ddiv_rn(__dsub_rn(tfinal, tinit), (double)nrk);
}

// One target of one problem: the arithmetic of k_semilag_tree_df<D>
// (double-float sums, FP64 coordinates, near-face targets listed for the
// FP64 pass).
template <int D>
__device__ __forceinline__ void batch_target_df(const BatchProblem& p, int64_t t, double tau,
                                                bool per, const BatchLaunch& a, int prob,
                                                ThreadSlots slots) {
  constexpr int NP = D * D * D;
  const int64_t leaf = t / NP;
  const int pi = (int)(t - leaf * NP);
  const Geom g = load_geom(p.con.geom + leaf);
  const double h = leaf_side(g);
  double x = g.x + h * p.nodes.x[pi % D];
  double y = g.y + h * p.nodes.x[(pi / D) % D];
  double z = g.z + h * p.nodes.x[pi / (D * D)];
  const double half_tau = 0.5 * tau;
  double xx[3] = {x, y, z};
  double px[3] = {x, y, z};
  double m0[3] = {0.0, 0.0, 0.0}, mp[3] = {0.0, 0.0, 0.0};
  bool amb = false;
  // first stage from the velocity at the nodes (as k_semilag_tree_df)
  const double* vn = p.vn + 3 * node_source(p.face, t);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (per) xx[k] = wrap1(xx[k]);
    px[k] = fma(half_tau, __ldg(vn + k), xx[k]);
  }
#pragma unroll 1
  for (int st = 1; st < 2 * p.nrk; ++st) {
    double v[3], ev[3];
    amb |= eval_point_df<D, 3, true>(p.vel, px[0], px[1], px[2], per, mp, v, ev, slots);
    if ((st & 1) == 0) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        xx[k] = px[k];
        df_update(half_tau, v[k], ev[k], xx[k], m0[k], px[k], mp[k]);
      }
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        df_update(tau, v[k], ev[k], xx[k], m0[k], xx[k], m0[k]);
        px[k] = xx[k];
        mp[k] = m0[k];
      }
    }
  }
  double c[1], ce[1];
  amb |= eval_point_df<D, 1, false>(p.con, xx[0], xx[1], xx[2], per, m0, c, ce, slots);
  p.vals[t] = c[0];
  if (amb) a.fix_list[atomicAdd(a.fix_count, 1ull)] = ((int64_t)prob << kFixShift) | t;
}

// One target of one problem in FP64: the arithmetic of k_semilag_tree<D>
// (first stage from the node grid).
template <int D>
__device__ __forceinline__ void batch_target(const BatchProblem& p, int64_t t, double tau,
                                             bool per) {
  constexpr int NP = D * D * D;
  const int64_t leaf = t / NP;
  const int pi = (int)(t - leaf * NP);
  const Geom g = load_geom(p.con.geom + leaf);
  const double h = leaf_side(g);
  double x = g.x + h * p.nodes.x[pi % D];
  double y = g.y + h * p.nodes.x[(pi / D) % D];
  double z = g.z + h * p.nodes.x[pi / (D * D)];
  rk2_backtrace_from_node<D>(p.vel, p.vn + 3 * node_source(p.face, t), x, y, z, tau, p.nrk, per);
  double c[1];
  eval_point<D, 1>(p.con, x, y, z, per, c);
  p.vals[t] = c[0];
}

template <int QLO, int QHI>
__device__ __forceinline__ void batch_dispatch(int q, const BatchProblem& p, int64_t t, double tau,
                                               bool per, const BatchLaunch& a, int prob,
                                               ThreadSlots slots) {
  if constexpr (QLO <= QHI) {
    if (q == QLO)
      batch_target_df<QLO + 1>(p, t, tau, per, a, prob, slots);
    else
      batch_dispatch<QLO + 1, QHI>(q, p, t, tau, per, a, prob, slots);
  }
}

template <int QLO, int QHI>
__device__ __forceinline__ void batch_dispatch_fp64(int q, const BatchProblem& p, int64_t t,
                                                    double tau, bool per) {
  if constexpr (QLO <= QHI) {
    if (q == QLO)
      batch_target<QLO + 1>(p, t, tau, per);
    else
      batch_dispatch_fp64<QLO + 1, QHI>(q, p, t, tau, per);
  }
}

// Persistent CTAs take chunks of targets from an atomic counter; the chunk's
// problem descriptor is staged in shared memory.
template <int QLO, int QHI>
__global__ void __launch_bounds__(256, 3) k_batch_semilag(const BatchLaunch a) {
  __shared__ BatchProblem sp;
  __shared__ int64_t s_item;
  extern __shared__ float2 s_slots[];  // 2 * (QHI + 1) elements per thread
  const ThreadSlots slots{s_slots + threadIdx.x, (int)blockDim.x};
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
      batch_dispatch<QLO, QHI>(q, sp, w.start + k, tau, per, a, w.problem, slots);
    __syncthreads();  // s_item and sp are rewritten for the next chunk
  }
}

// The TBSLAS_SUMS_FP64 form of k_batch_semilag: every target of a chunk runs
// k_semilag_tree<D>'s FP64 arithmetic (batch_target), so a batch step equals
// the per-problem loop in that mode bit for bit, and no near-face pass
// follows.
template <int QLO, int QHI>
__global__ void __launch_bounds__(256) k_batch_semilag_fp64(const BatchLaunch a) {
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
      batch_dispatch_fp64<QLO, QHI>(q, sp, w.start + k, tau, per);
    __syncthreads();  // s_item and sp are rewritten for the next chunk
  }
}

// FP64 pass over the listed targets whose problem's degree is in this band.
template <int QLO, int QHI>
__global__ void __launch_bounds__(128) k_batch_fix(const BatchLaunch a) {
  const bool per = a.periodic != 0;
  const int ts = *a.ts0 + a.step;
  const int64_t n = (int64_t)*a.fix_count;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = a.fix_list[i];
    const int prob = (int)(e >> kFixShift);
    const int64_t t = e & ((1ll << kFixShift) - 1);
    const BatchProblem& p = a.probs[prob];
    if (p.q < QLO || p.q > QHI) continue;
    batch_dispatch_fp64<QLO, QHI>(p.q, p, t, step_tau(ts, p.dt, p.nrk), per);
  }
}

// What a band launch runs: the double-float step kernel, the FP64 pass over
// its listed targets, or the FP64 step kernel.
enum BandKernel : int { kBandStepDF = 0, kBandFix = 1, kBandStepFP64 = 2 };

// Launch of one band: the double-float step kernel with 2 * (QHI + 1)
// shared-memory elements per thread (its dynamic shared-memory limit raised
// once per device: with the static descriptor, 48 KB of slots already
// exceeds the default), the FP64 pass, or the FP64 step kernel.
template <int QLO, int QHI>
void launch_band(const BatchLaunch& a, int grid, int block, cudaStream_t s, int what) {
  if (what == kBandFix) {
    k_batch_fix<QLO, QHI><<<grid, 128, 0, s>>>(a);
    return;
  }
  if (what == kBandStepFP64) {
    k_batch_semilag_fp64<QLO, QHI><<<grid, block, 0, s>>>(a);
    return;
  }
  constexpr size_t kMaxSmem = 2 * (size_t)(QHI + 1) * 256 * sizeof(float2);
  const size_t smem = 2 * (size_t)(QHI + 1) * block * sizeof(float2);
  static std::atomic<uint64_t> done{0};
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t bit = 1ull << (dev & 63);
  if (!(done.load() & bit)) {
    cudaFuncSetAttribute(k_batch_semilag<QLO, QHI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kMaxSmem);
    done.fetch_or(bit);
  }
  k_batch_semilag<QLO, QHI><<<grid, block, smem, s>>>(a);
}

}  // namespace tbg

namespace tbg {
void launch_batch_band_0(const BatchLaunch& a, int grid, int block, cudaStream_t s, int what);
void launch_batch_band_1(const BatchLaunch& a, int grid, int block, cudaStream_t s, int what);
void launch_batch_band_2(const BatchLaunch& a, int grid, int block, cudaStream_t s, int what);
void launch_batch_band_3(const BatchLaunch& a, int grid, int block, cudaStream_t s, int what);
void launch_batch_band_4(const BatchLaunch& a, int grid, int block, cudaStream_t s, int what);
void launch_batch_band_5(const BatchLaunch& a, int grid, int block, cudaStream_t s, int what);
inline void launch_batch_band(int band, const BatchLaunch& a, int grid, int block,
                              cudaStream_t s, int what) {
  switch (band) {
    case 0: launch_batch_band_0(a, grid, block, s, what); break;
    case 1: launch_batch_band_1(a, grid, block, s, what); break;
    case 2: launch_batch_band_2(a, grid, block, s, what); break;
    case 3: launch_batch_band_3(a, grid, block, s, what); break;
    case 4: launch_batch_band_4(a, grid, block, s, what); break;
    default: launch_batch_band_5(a, grid, block, s, what); break;
  }
}
}  // namespace tbg

// C ABI of libtbslas_gb300.so (include/tbslas_gb300.h): contexts, trees,
// host-side validation, the bucketing kernels of the tree functor, and the
// entry points of the SL path.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "host_cheb.h"
#include "internal.h"
#include "tbslas_gb300.h"

using namespace tbg;

// ---------------------------------------------------------------------------
// errors
namespace {
thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CUDA_TRY(call)                                                                 \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return fail(TBSLAS_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));           \
  } while (0)

#define TRY(expr)            \
  do {                       \
    int s_ = (expr);         \
    if (s_ != TBSLAS_OK) return s_; \
  } while (0)

DegreeKernels g_kernels[TBSLAS_MAX_DEGREE + 1];
Bdf2Fn g_bdf2[TBSLAS_MAX_DEGREE + 1] = {};
TvFn g_tv[TBSLAS_MAX_DEGREE + 1] = {};
std::once_flag g_kernels_once;

void init_kernels() {
  register_tv_a(g_tv);
  register_tv_b(g_tv);
  register_tv_c(g_tv);
  register_bdf2_a(g_bdf2);
  register_bdf2_b(g_bdf2);
  register_degrees_a(g_kernels);
  register_degrees_b(g_kernels);
  register_degrees_c(g_kernels);
  register_degrees_d(g_kernels);
  register_degrees_e(g_kernels);
  register_degrees_f(g_kernels);
  register_degrees_g(g_kernels);
  register_degrees_h(g_kernels);
}

// Point-to-coefficient matrices, computed once per degree per process.
std::mutex g_M_mutex;
std::vector<double> g_M_host[TBSLAS_MAX_DEGREE + 1];

const std::vector<double>& host_M(int q) {
  std::lock_guard<std::mutex> lock(g_M_mutex);
  if (g_M_host[q].empty()) g_M_host[q] = pt2coeff_matrix(q);
  return g_M_host[q];
}

enum Slot {
  kVals,
  kLeafOf,
  kCount,
  kStart,
  kCursor,
  kNTile,
  kTileOff,
  kTiles,
  kPerm,
  kXA,
  kXB,
  kVT,
  kHostIn,
  kHostIn2,
  kHostOut,
  kMu,
  kFixList,
  kFixCount,
  kVN,
  kGridV2,
  kGridC2,
  kGridTmp,
  kAdjC2,
  kAdjW,
  // re-meshing: two sets of leaf arrays (ping-pong) and the temporaries
  kRmKeys0,
  kRmGeom0,
  kRmCoeff0,
  kRmKeys1,
  kRmGeom1,
  kRmCoeff1,
  kRmI64a,
  kRmI64b,
  kRmI64c,
  kRmI64d,
  kRmSrc,
  kRmItems,
  kRmVals,
  kRmSplitC,
  kRmMergeC,
  kRmTail,
  kRmAct,
  kRmAux,
  kRmGroup,
  kRmTable,
  kRmScalars,
  // time-dependent velocity: the two stage blends of a velocity set
  kTvC1,
  kTvC2,
  kTvC2s,
  kTvN2,
  kTvFlag,
  kField,
  kNumSlots
};

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

inline int64_t n_coeff(int q) { return (int64_t)(q + 1) * (q + 2) * (q + 3) / 6; }
inline int64_t n_points(int q) { return (int64_t)(q + 1) * (q + 1) * (q + 1); }
inline bool bc_ok(int bc) { return bc == TBSLAS_BC_FREESPACE || bc == TBSLAS_BC_PERIODIC; }

}  // namespace

// Per-kernel CUDA-event timing (the role of pvfmm::Profile::Tic/Toc in the
// reference, e.g. src/semilag/traj.inc:53, src/tree/tree_functor.h:389-394).
struct ProfRecord {
  const char* name;
  int kernels;
  cudaEvent_t start, stop;
};
struct ProfTotal {
  std::string name;
  int64_t launches = 0;
  int64_t kernels = 0;
  double ms = 0.0;
};

// Leaf-list stamps (tbslas_tree_s::generation), unique across the process.
uint64_t next_generation() {
  static std::atomic<uint64_t> counter{0};
  return counter.fetch_add(1) + 1;
}

// The last leaf-structure comparison of a velocity set
// (tbslas_semilag_in_situ_tv): the trees' stamps and whether their leaves
// were equal.
struct TvStructure {
  int m = 0;
  uint64_t gen[kTvMaxTrees] = {};
  bool same = false;
};

struct tbslas_ctx_s {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;  // used by the synchronous *_host entry points
  uint32_t* d_err = nullptr;
  DevBuf slots[kNumSlots];
  double* d_F[TBSLAS_MAX_DEGREE + 1] = {};  // separable refit factors per degree
  int sums = TBSLAS_SUMS_FP64;  // arithmetic of the SL steps' Chebyshev sums
  uint32_t wait_limit = kWaitLimit;  // polls of the bounded device-side waits
  bool profile = false;
  int64_t live_objects = 0;     // trees and batches created on this context, not yet destroyed
  int64_t* h_pinned = nullptr;  // small pinned host buffer for scalar read-backs
  std::vector<ProfRecord> prof_pending;
  std::vector<cudaEvent_t> prof_pool;
  std::vector<ProfTotal> prof_totals;
  TvStructure tv_structure;
};

struct tbslas_tree_s {
  tbslas_ctx ctx = nullptr;
  int device = 0;        // the context's device (the tree's arrays live there)
  bool counted = false;  // counted in ctx->live_objects
  int64_t L = 0;
  int q = 0, dof = 0, max_depth = 0, T = 0;
  int64_t stride = 0;
  uint64_t* d_keys = nullptr;
  Geom* d_geom = nullptr;
  double* d_coeff = nullptr;
  float2* d_coeff2 = nullptr;  // double-float split of d_coeff, kept in sync
  double* d_cnorm = nullptr;   // [L * dof] sum |c| per leaf and component, kept in sync
  int32_t* d_table = nullptr;
  int64_t cap_L = 0;      // leaves the per-leaf arrays hold (>= L after a re-meshing)
  int64_t cap_table = 0;  // entries d_table holds
  // a process-wide unique stamp of this tree's leaf list, new at creation
  // and whenever the list changes (re-meshing): equal stamps, equal leaves
  uint64_t generation = next_generation();
  // face maps of the node-grid pass, one per boundary condition, built on
  // first use for the current generation (tree_face_map)
  int32_t* d_face[2] = {nullptr, nullptr};
  int64_t face_cap[2] = {0, 0};
  uint64_t face_gen[2] = {0, 0};
  bool face_ok[2] = {false, false};

  TreeView view() const {
    TreeView v;
    v.keys = d_keys;
    v.geom = d_geom;
    v.coeff = d_coeff;
    v.coeff2 = d_coeff2;
    v.cnorm = d_cnorm;
    v.table = d_table;
    v.L = L;
    v.stride = stride;
    v.T = T;
    v.q = q;
    v.dof = dof;
    return v;
  }
};

namespace {

cudaEvent_t prof_event(tbslas_ctx ctx) {
  if (!ctx->prof_pool.empty()) {
    cudaEvent_t e = ctx->prof_pool.back();
    ctx->prof_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Brackets the launches of one named kernel on a stream with events when
// profiling is on; a no-op otherwise.
struct ProfScope {
  tbslas_ctx ctx;
  const char* name;
  cudaStream_t s;
  int kernels;
  cudaEvent_t start = nullptr;
  ProfScope(tbslas_ctx c, const char* n, cudaStream_t st, int nkernels = 1)
      : ctx(c), name(n), s(st), kernels(nkernels) {
    if (ctx->profile) {
      start = prof_event(ctx);
      cudaEventRecord(start, s);
    }
  }
  ~ProfScope() {
    if (start) {
      cudaEvent_t stop = prof_event(ctx);
      cudaEventRecord(stop, s);
      ctx->prof_pending.push_back(ProfRecord{name, kernels, start, stop});
    }
  }
};

// Folds finished event pairs into the per-name totals.
void prof_collect(tbslas_ctx ctx) {
  for (ProfRecord& r : ctx->prof_pending) {
    cudaEventSynchronize(r.stop);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.start, r.stop);
    ProfTotal* t = nullptr;
    for (ProfTotal& x : ctx->prof_totals)
      if (x.name == r.name) t = &x;
    if (!t) {
      ctx->prof_totals.push_back(ProfTotal{r.name});
      t = &ctx->prof_totals.back();
    }
    t->launches += 1;
    t->kernels += r.kernels;
    t->ms += ms;
    ctx->prof_pool.push_back(r.start);
    ctx->prof_pool.push_back(r.stop);
  }
  ctx->prof_pending.clear();
}

int bind(tbslas_ctx ctx) {
  if (!ctx) return fail(TBSLAS_ERR_INVALID_ARG, "null context");
  CUDA_TRY(cudaSetDevice(ctx->device));
  return TBSLAS_OK;
}

// Binds the context's device for the rest of the entry point and restores
// the caller's current device when it returns.
#define BIND(c)                        \
  DeviceRestore device_restore_;       \
  TRY(bind(c))

// Grow-only scratch buffer.  Growing frees the old block (cudaFree waits for
// the device), so no in-flight kernel can still be using it.
int scratch(tbslas_ctx ctx, Slot s, size_t bytes, void** out) {
  DevBuf& b = ctx->slots[s];
  if (b.cap < bytes) {
    if (b.p) CUDA_TRY(cudaFree(b.p));
    b.p = nullptr;
    b.cap = 0;
    size_t want = std::max(bytes, (size_t)256);
    if (cudaMalloc(&b.p, want) != cudaSuccess) {
      cudaGetLastError();
      b.p = nullptr;
      return fail(TBSLAS_ERR_ALLOC, "cudaMalloc of %zu bytes of scratch failed", want);
    }
    b.cap = want;
  }
  *out = b.p;
  return TBSLAS_OK;
}

template <class T>
int scratch_t(tbslas_ctx ctx, Slot s, size_t count, T** out) {
  void* p = nullptr;
  TRY(scratch(ctx, s, count * sizeof(T), &p));
  *out = static_cast<T*>(p);
  return TBSLAS_OK;
}

int device_F(tbslas_ctx ctx, int q, const double** out) {
  if (!ctx->d_F[q]) {
    const std::vector<double> F = refit_factors(q);
    double* d = nullptr;
    CUDA_TRY(cudaMalloc(&d, F.size() * sizeof(double)));
    CUDA_TRY(cudaMemcpy(d, F.data(), F.size() * sizeof(double), cudaMemcpyHostToDevice));
    ctx->d_F[q] = d;
  }
  *out = ctx->d_F[q];
  return TBSLAS_OK;
}

Nodes1D nodes_1d(int q) {
  Nodes1D n;
  std::memset(&n, 0, sizeof(n));
  std::vector<double> x = cheb_nodes_1d(q);
  for (int i = 0; i <= q; ++i) n.x[i] = x[i];
  return n;
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(TBSLAS_ERR_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
  return TBSLAS_OK;
}

// ---------------------------------------------------------------------------
// small kernels

// Chebyshev nodes of every leaf (CollectChebTreeGridPoints,
// src/tree/tree_utils.h:477-495): leaf anchor + 2^-depth * node.
__global__ void k_collect(const TreeView t, const Nodes1D nodes, int d, double* __restrict__ out) {
  const int64_t np = (int64_t)d * d * d;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= t.L * np) return;
  const int64_t leaf = i / np;
  const int p = (int)(i - leaf * np);
  const Geom g = load_geom(t.geom + leaf);
  const double h = leaf_side(g);
  out[3 * i + 0] = g.x + h * nodes.x[p % d];
  out[3 * i + 1] = g.y + h * nodes.x[(p / d) % d];
  out[3 * i + 2] = g.z + h * nodes.x[p / (d * d)];
}

// Leaf of every point (Morton key + coarse table + binary search) and a
// warp-aggregated per-leaf count.  Points that evaluate to 0 (outside the
// domain, NaN) get their output written here and are not bucketed.
__global__ void k_classify(const TreeView t, const double* __restrict__ pos, int64_t n,
                           int periodic, int32_t* __restrict__ leaf_of,
                           unsigned long long* __restrict__ count, double* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int leaf = -2;
  if (i < n) {
    double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    const bool per = periodic != 0;
    if (per) {
      x = wrap1(x);
      y = wrap1(y);
      z = wrap1(z);
    }
    if (inside(x, y, z, per)) {
      leaf = (int)find_leaf(t, morton3(quantise(x), quantise(y), quantise(z)));
    } else {
      leaf = -1;
      for (int l = 0; l < t.dof; ++l) out[i * t.dof + l] = 0.0;
    }
    leaf_of[i] = leaf;
  }
  const unsigned peers = __match_any_sync(0xffffffffu, leaf);
  if (leaf >= 0 && (int)(threadIdx.x & 31) == __ffs(peers) - 1)
    atomicAdd(count + leaf, (unsigned long long)__popc(peers));
}

__global__ void k_ntiles(const unsigned long long* __restrict__ count, int64_t L,
                         int64_t* __restrict__ ntile) {
  const int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (l < L) ntile[l] = (int64_t)((count[l] + kTile - 1) / kTile);
}

// Exclusive scan of in[0..m) into out[0..m], out[m] = total.  One CTA walks
// the array in chunks of 1024 (the arrays are per-leaf, small next to the
// point work).
__global__ void __launch_bounds__(1024) k_scan_excl(const int64_t* __restrict__ in,
                                                    int64_t* __restrict__ out, int64_t m) {
  __shared__ int64_t wsum[32];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t base = 0; base < m; base += 1024) {
    const int64_t i = base + threadIdx.x;
    const int64_t v = i < m ? in[i] : 0;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int64_t w = wsum[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      wsum[lane] = w;
    }
    __syncthreads();
    const int64_t incl = x + (warp > 0 ? wsum[warp - 1] : 0) + carry;
    if (i < m) out[i] = incl - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry = incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) out[m] = carry;
}

__global__ void k_scatter(const int32_t* __restrict__ leaf_of, int64_t n,
                          const int64_t* __restrict__ start, unsigned long long* __restrict__ cursor,
                          int64_t* __restrict__ perm) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int leaf = i < n ? leaf_of[i] : -2;
  const unsigned peers = __match_any_sync(0xffffffffu, leaf);
  if (leaf >= 0) {
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(cursor + leaf, (unsigned long long)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    perm[start[leaf] + (int64_t)base + rank] = i;
  }
}

__global__ void k_make_tiles(const int64_t* __restrict__ start, const int64_t* __restrict__ tileoff,
                             int64_t L, Tile* __restrict__ tiles) {
  const int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (l >= L) return;
  const int64_t s = start[l], c = start[l + 1] - s;
  int64_t o = tileoff[l];
  for (int64_t k = 0; k < c; k += kTile, ++o)
    tiles[o] = Tile{s + k, (int32_t)l, (int32_t)(c - k < kTile ? c - k : kTile)};
}

// [leaf][node][dof] -> [leaf][dof][node]
__global__ void k_point_to_dof_major(const double* __restrict__ in, int64_t L, int np, int dof,
                                     double* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= L * np * dof) return;
  const int64_t leaf = i / ((int64_t)np * dof);
  const int64_t r = i - leaf * np * dof;
  const int p = (int)(r / dof), l = (int)(r % dof);
  out[(leaf * dof + l) * np + p] = in[i];
}

// FMA throughput probe (T = double: FP64 pipe, T = float: FP32 pipe): 8
// independent dependency chains per thread, 64 FMAs per iteration; one store
// per thread.  The shared multiplier and addend sit in registers (b + 0 with
// a run-time 0): taken from the constant bank, as kernel arguments, they
// held the FP64 FMA rate at 1.6 per clock per SM instead of 1.9.
template <class T>
__global__ void __launch_bounds__(256) k_fma_probe(T* out, T b_arg, T c_arg, int iters) {
  const T zero = T(iters < 0);
  const T b = b_arg + zero, c = c_arg + zero;
  T a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5,
    a6 = a0 + 6, a7 = a0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      a0 = fma(a0, b, c);
      a1 = fma(a1, b, c);
      a2 = fma(a2, b, c);
      a3 = fma(a3, b, c);
      a4 = fma(a4, b, c);
      a5 = fma(a5, b, c);
      a6 = fma(a6, b, c);
      a7 = fma(a7, b, c);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

// Per leaf and component: sum of |c| (bounds the double-float sums' error).
__global__ void k_cnorm(const double* __restrict__ c, int64_t L, int dof, int nc, int64_t stride,
                        double* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= L * dof) return;
  const int64_t leaf = i / dof;
  const int l = (int)(i - leaf * dof);
  const double* p = c + leaf * stride + (int64_t)l * nc;
  double s = 0.0;
  for (int n = 0; n < nc; ++n) s += fabs(p[n]);
  out[i] = s;
}

inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// The bucketed tree functor on device buffers.
int eval_tree_dev(tbslas_ctx ctx, tbslas_tree tree, const double* pos, int64_t n, double* out,
                  int bc, cudaStream_t s) {
  if (n == 0) return TBSLAS_OK;
  const TreeView tv = tree->view();
  const int64_t L = tree->L;
  const int64_t max_tiles = (n + kTile - 1) / kTile + L;
  int32_t* leaf_of;
  unsigned long long *count, *cursor;
  int64_t *start, *ntile, *tileoff, *perm;
  Tile* tiles;
  TRY(scratch_t(ctx, kLeafOf, n, &leaf_of));
  TRY(scratch_t(ctx, kCount, L, &count));
  TRY(scratch_t(ctx, kCursor, L, &cursor));
  TRY(scratch_t(ctx, kStart, L + 1, &start));
  TRY(scratch_t(ctx, kNTile, L, &ntile));
  TRY(scratch_t(ctx, kTileOff, L + 1, &tileoff));
  TRY(scratch_t(ctx, kPerm, n, &perm));
  TRY(scratch_t(ctx, kTiles, max_tiles, &tiles));
  CUDA_TRY(cudaMemsetAsync(count, 0, L * sizeof(*count), s));
  CUDA_TRY(cudaMemsetAsync(cursor, 0, L * sizeof(*cursor), s));
  {
    ProfScope p(ctx, "bucket_points", s, 6);
    k_classify<<<blocks_for(n, 256), 256, 0, s>>>(tv, pos, n, bc, leaf_of, count, out);
    k_ntiles<<<blocks_for(L, 256), 256, 0, s>>>(count, L, ntile);
    k_scan_excl<<<1, 1024, 0, s>>>(reinterpret_cast<const int64_t*>(count), start, L);
    k_scan_excl<<<1, 1024, 0, s>>>(ntile, tileoff, L);
    k_scatter<<<blocks_for(n, 256), 256, 0, s>>>(leaf_of, n, start, cursor, perm);
    k_make_tiles<<<blocks_for(L, 256), 256, 0, s>>>(start, tileoff, L, tiles);
    TRY(check_launch("bucketing"));
  }
  EvalTilesArgs a;
  a.tree = tv;
  a.pos = pos;
  a.perm = perm;
  a.tiles = tiles;
  a.ntiles = tileoff + L;
  a.periodic = bc;
  a.out = out;
  a.err = ctx->d_err;
  a.wait_limit = ctx->wait_limit;
  a.grid = (int)std::min<int64_t>(max_tiles, (int64_t)ctx->num_sms * 8);
  ProfScope p(ctx, "eval_tiles", s);
  g_kernels[tree->q].eval_tiles(a, s);
  return check_launch("eval_tiles");
}

int traj_dev(tbslas_ctx ctx, tbslas_tree vel, const double* x, int64_t n, double tau, int nrk,
             int bc, double* xdep, cudaStream_t s) {
  (void)ctx;
  TrajArgs a;
  a.vel = vel->view();
  a.x = x;
  a.n = n;
  a.tau = tau;
  a.nrk = nrk;
  a.periodic = bc;
  a.xdep = xdep;
  ProfScope p(ctx, "traj_rk2", s);
  g_kernels[vel->q].traj(a, s);
  return check_launch("traj");
}

int refit_dev(tbslas_ctx ctx, tbslas_tree tree, const double* vals, cudaStream_t s) {
  const double* F = nullptr;
  TRY(device_F(ctx, tree->q, &F));
  ProfScope p(ctx, "refit", s, tree->dof == 3 ? 2 : 1);
  launch_refit(vals, F, tree->q, tree->L * tree->dof, tree->dof, tree->stride, tree->d_coeff,
               tree->d_coeff2, ctx->d_err, ctx->sums == TBSLAS_SUMS_DOUBLE_FLOAT, s);
  TRY(check_launch("refit"));
  if (tree->dof == 3) {  // a velocity-shaped tree: its norms feed the double-float bounds
    k_cnorm<<<blocks_for(tree->L * 3, 128), 128, 0, s>>>(tree->d_coeff, tree->L, 3,
                                                         (int)n_coeff(tree->q), tree->stride,
                                                         tree->d_cnorm);
    return check_launch("norms");
  }
  return TBSLAS_OK;
}

int collect_dev(tbslas_tree tree, double* out, cudaStream_t s) {
  const int64_t n = tree->L * n_points(tree->q);
  if (n == 0) return TBSLAS_OK;
  ProfScope p(tree->ctx, "collect", s);
  k_collect<<<blocks_for(n, 256), 256, 0, s>>>(tree->view(), nodes_1d(tree->q), tree->q + 1, out);
  return check_launch("collect");
}

// The grid step: double-float stencil sums on periodic grids (unless the
// context asks for FP64 sums), FP64 otherwise.
// split_vel = false: the previous call of this context split the same,
// unchanged velocity grid (a multi-step call), so its hi/lo copy is reused.
int semilag_grid_dev(tbslas_ctx ctx, const double* vel, const double* con, double* cout,
                     int n_reg, double tau, int nrk, int bc, cudaStream_t s,
                     bool split_vel = true) {
  if (bc == TBSLAS_BC_PERIODIC && ctx->sums == TBSLAS_SUMS_DOUBLE_FLOAT) {
    const int64_t n3 = (int64_t)n_reg * n_reg * n_reg;
    float2 *v2, *c2;
    TRY(scratch_t(ctx, kGridV2, n3 * 3, &v2));
    TRY(scratch_t(ctx, kGridC2, n3, &c2));
    ProfScope p(ctx, "semilag_grid", s, split_vel ? 3 : 2);
    launch_semilag_grid_df(vel, con, cout, n_reg, tau, nrk, v2, c2, ctx->d_err, ctx->num_sms,
                           split_vel, s);
    return check_launch("semilag_grid");
  }
  ProfScope p(ctx, "semilag_grid", s);
  launch_semilag_grid(vel, con, cout, n_reg, tau, nrk, bc, s);
  return check_launch("semilag_grid");
}

int check_tree(tbslas_tree t) {
  if (!t || !t->ctx) return fail(TBSLAS_ERR_INVALID_ARG, "null tree");
  return TBSLAS_OK;
}

// The time step of SolveSemilagRK2 (src/semilag/semilag.inc:26-45):
// tinit = timestep*dt, tfinal = tinit - dt, tau = (tfinal - tinit)/nrk.
double sl_tau(int timestep, double dt, int nrk) {
  const double tinit = timestep * dt;
  const double tfinal = tinit - dt;
  return (tfinal - tinit) / nrk;
}

// Do two key arrays differ?  (*flag set to 1 if so)
__global__ void k_keys_differ(const uint64_t* __restrict__ a, const uint64_t* __restrict__ b,
                              int64_t n, int* __restrict__ flag) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n && a[i] != b[i]) *flag = 1;
}

// CubicInterpPolicy::InterpCubic1D (src/utils/cubic.h:42-56): Hermite
// interpolation on [xx1, xx2] with tangents from the neighbouring
// differences, at x, of the values pp.
double interp_cubic_1d(double x, const double* xx, const double* pp) {
  auto tangent = [](double tk_1, double tk, double tk1, double pk_1, double pk, double pk1) {
    return (pk1 - pk) * 0.5 / (tk1 - tk) + (pk - pk_1) * 0.5 / (tk - tk_1);
  };
  const double mk = tangent(xx[0], xx[1], xx[2], pp[0], pp[1], pp[2]);
  const double mk1 = tangent(xx[1], xx[2], xx[3], pp[1], pp[2], pp[3]);
  const double t = (x - xx[1]) / (xx[2] - xx[1]);
  const double h00 = 2 * t * t * t - 3 * t * t + 1, h10 = t * t * t - 2 * t * t + t;
  const double h01 = -2 * t * t * t + 3 * t * t, h11 = t * t * t - t * t;
  return h00 * pp[1] + h10 * (xx[2] - xx[1]) * mk + h01 * pp[2] + h11 * (xx[2] - xx[1]) * mk1;
}

// The fused step of a dof-1 concentration through a velocity of its degree:
// the first RK stage from v1 at the nodes, the others from v2 (one tree for
// the plain step; two blends of a velocity set for the time-dependent one).
int fused_step(tbslas_ctx ctx, const TreeView& v1, const TreeView& v2, tbslas_tree con,
               double tau, int nrk, int bc, cudaStream_t s, double* xmid, double* xdep,
               double* jac = nullptr) {
  const int64_t N = con->L * n_points(con->q);
  double* vals;
  TRY(scratch_t(ctx, kVals, N, &vals));
  SemilagTreeArgs a;
  a.vel = v2;
  a.con = con->view();
  a.nodes = nodes_1d(con->q);
  a.tau = tau;
  a.nrk = nrk;
  a.periodic = bc;
  a.vals = vals;
  a.xmid = xmid;
  a.xdep = xdep;
  {
    // first RK stage: the velocity at the targets by sum factorisation
    double* vn = nullptr;
    TRY(scratch_t(ctx, kVN, N * 3, &vn));
    // shared upper-face nodes are not copied: the step kernels read them
    // through the face map
    const int32_t* face = tree_face_map(con, bc, s);
    ProfScope pv(ctx, "vel_at_nodes", s, 1);
    launch_eval_on_nodes(v1, a.con, bc, vn, s, face, false);
    TRY(check_launch("velocity at nodes"));
    a.vn = vn;
    a.face = face;
  }
  TRY(scratch_t(ctx, kFixList, N, &a.fix_list));
  TRY(scratch_t(ctx, kFixCount, 1, &a.fix_count));
  a.fix_grid = ctx->num_sms * 8;
  if (jac) {
    if (ctx->sums != TBSLAS_SUMS_FP64)
      return fail(TBSLAS_ERR_UNSUPPORTED, "the velocity Jacobian checkpoint needs FP64 sums");
    a.jac = jac;
    ProfScope p(ctx, "semilag_tree_jac", s, 1);
    TRY(launch_semilag_jac(con->q, a, s));
  } else if (ctx->sums == TBSLAS_SUMS_FP64) {
    ProfScope p(ctx, "semilag_tree", s, 1);
    g_kernels[con->q].semilag(a, s);
  } else {
    ProfScope p(ctx, "semilag_tree", s, 2);
    g_kernels[con->q].semilag_df(a, s);
  }
  TRY(check_launch("semilag_tree"));
  return refit_dev(ctx, con, vals, s);
}

int semilag_in_situ_dev(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con, int timestep, double dt,
                        int nrk, int bc, cudaStream_t s, double* xmid = nullptr,
                        double* xdep = nullptr, double* jac = nullptr) {
  const double tau = sl_tau(timestep, dt, nrk);
  const int64_t np = n_points(con->q);
  const int64_t N = con->L * np;
  if (vel->q == con->q && con->dof == 1) {
    const TreeView v = vel->view();
    return fused_step(ctx, v, v, con, tau, nrk, bc, s, xmid, xdep, jac);
  }
  double* vals;
  TRY(scratch_t(ctx, kVals, N * con->dof, &vals));
  {
    double *X, *Xdep, *vt;
    TRY(scratch_t(ctx, kXA, N * 3, &X));
    TRY(scratch_t(ctx, kXB, N * 3, &Xdep));
    TRY(scratch_t(ctx, kVT, N * con->dof, &vt));
    TRY(collect_dev(con, X, s));
    TRY(traj_dev(ctx, vel, X, N, tau, nrk, bc, Xdep, s));
    TRY(eval_tree_dev(ctx, con, Xdep, N, vt, bc, s));
    ProfScope p(ctx, "to_dof_major", s);
    k_point_to_dof_major<<<blocks_for(N * con->dof, 256), 256, 0, s>>>(vt, con->L, (int)np,
                                                                      con->dof, vals);
    TRY(check_launch("transpose"));
  }
  return refit_dev(ctx, con, vals, s);
}

// Validate a leaf list and build the device tree arrays.
int build_tree(tbslas_tree t, const double* anchor, const int32_t* depth) {
  const int64_t L = t->L;
  std::vector<uint64_t> keys(L);
  std::vector<Geom> geom(L);
  int maxd = 0;
  for (int64_t i = 0; i < L; ++i) {
    const int dl = depth[i];
    if (dl < 0 || dl > TBSLAS_MAX_DEPTH)
      return fail(TBSLAS_ERR_TREE, "leaf %lld: depth %d outside [0,%d]", (long long)i, dl,
                  TBSLAS_MAX_DEPTH);
    maxd = std::max(maxd, dl);
    uint64_t a[3];
    for (int k = 0; k < 3; ++k) {
      const double c = anchor[3 * i + k];
      const double s = std::ldexp(c, dl);  // exact
      if (!(c >= 0.0 && c < 1.0) || s != std::floor(s))
        return fail(TBSLAS_ERR_TREE, "leaf %lld: anchor %g is not a multiple of 2^-%d in [0,1)",
                    (long long)i, c, dl);
      a[k] = (uint64_t)std::ldexp(c, kKeyBits);
    }
    keys[i] = morton3(a[0], a[1], a[2]);
    geom[i] = Geom{anchor[3 * i], anchor[3 * i + 1], anchor[3 * i + 2], std::ldexp(2.0, dl)};
  }
  // Complete linear octree in Morton order: each leaf starts where the
  // previous one ends and the last one ends at the domain's end.
  uint64_t expect = 0;
  for (int64_t i = 0; i < L; ++i) {
    if (keys[i] != expect)
      return fail(TBSLAS_ERR_TREE,
                  "leaf %lld: not a complete Morton-ordered octree (gap, overlap or order)",
                  (long long)i);
    expect = keys[i] + (1ull << (3 * (kKeyBits - depth[i])));
  }
  if (expect != (1ull << (3 * kKeyBits)))
    return fail(TBSLAS_ERR_TREE, "leaves do not cover the unit cube");
  const int T = std::min(maxd, 7);
  const int64_t ncell = 1ll << (3 * T);
  std::vector<int32_t> table(ncell + 1);
  {
    int64_t leaf = 0;
    for (int64_t c = 0; c < ncell; ++c) {
      const uint64_t ck = (uint64_t)c << (3 * (kKeyBits - T));
      while (leaf + 1 < L && keys[leaf + 1] <= ck) ++leaf;
      table[c] = (int32_t)leaf;
    }
    table[ncell] = (int32_t)(L - 1);
  }
  t->max_depth = maxd;
  t->T = T;
  CUDA_TRY(cudaMalloc(&t->d_keys, L * sizeof(uint64_t)));
  CUDA_TRY(cudaMalloc(&t->d_geom, L * sizeof(Geom)));
  CUDA_TRY(cudaMalloc(&t->d_table, (ncell + 1) * sizeof(int32_t)));
  CUDA_TRY(cudaMalloc(&t->d_coeff, L * t->stride * sizeof(double)));
  CUDA_TRY(cudaMalloc(&t->d_coeff2, L * t->stride * sizeof(float2)));
  CUDA_TRY(cudaMemset(t->d_coeff2, 0, L * t->stride * sizeof(float2)));
  CUDA_TRY(cudaMalloc(&t->d_cnorm, L * t->dof * sizeof(double)));
  CUDA_TRY(cudaMemset(t->d_cnorm, 0, L * t->dof * sizeof(double)));
  CUDA_TRY(cudaMemcpy(t->d_keys, keys.data(), L * sizeof(uint64_t), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(t->d_geom, geom.data(), L * sizeof(Geom), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(t->d_table, table.data(), (ncell + 1) * sizeof(int32_t),
                      cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemset(t->d_coeff, 0, L * t->stride * sizeof(double)));
  t->cap_L = L;
  t->cap_table = ncell + 1;
  return TBSLAS_OK;
}

// Refresh what is derived from a tree's coefficients: the double-float split
// and the per-leaf coefficient norms.
int derived_coeffs(tbslas_tree t, cudaStream_t s) {
  launch_split(t->d_coeff, t->d_coeff2, t->L * t->stride, t->ctx->d_err, s);
  const int64_t n = t->L * t->dof;
  k_cnorm<<<blocks_for(n, 128), 128, 0, s>>>(t->d_coeff, t->L, t->dof, (int)n_coeff(t->q),
                                             t->stride, t->d_cnorm);
  return check_launch("coefficient split / norms");
}

int copy_coeffs(tbslas_tree t, double* dst, const double* src, bool to_tree, cudaMemcpyKind kind,
                cudaStream_t s) {
  const size_t w = (size_t)t->dof * n_coeff(t->q) * sizeof(double);
  const size_t pitch = (size_t)t->stride * sizeof(double);
  if (to_tree) {
    CUDA_TRY(cudaMemcpy2DAsync(dst, pitch, src, w, w, t->L, kind, s));
    return derived_coeffs(t, s);
  }
  CUDA_TRY(cudaMemcpy2DAsync(dst, w, src, pitch, w, t->L, kind, s));
  return TBSLAS_OK;
}

// ---------------------------------------------------------------------------
// Adaptive re-meshing (tbslas_tree_remesh): host sequence over the kernels of
// remesh.cu.  Leaf arrays ping-pong between two sets of the context's
// grow-only scratch; the host reads back one or two scalars per phase.
constexpr Slot kMeshKeys[2] = {kRmKeys0, kRmKeys1};
constexpr Slot kMeshGeom[2] = {kRmGeom0, kRmGeom1};
constexpr Slot kMeshCoeff[2] = {kRmCoeff0, kRmCoeff1};

struct MeshState {
  int64_t L = 0;
  int set = 0;  // scratch set holding the current leaves
  uint64_t* keys = nullptr;
  Geom* geom = nullptr;
  double* coeff = nullptr;
};

// n (<= 2) int64 device scalars -> host, one synchronisation.
int read_scalars(tbslas_ctx ctx, const int64_t* const* dev, int n, int64_t* host, cudaStream_t s) {
  if (!ctx->h_pinned) CUDA_TRY(cudaMallocHost(&ctx->h_pinned, 4 * sizeof(int64_t)));
  for (int i = 0; i < n; ++i)
    CUDA_TRY(cudaMemcpyAsync(ctx->h_pinned + i, dev[i], sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  for (int i = 0; i < n; ++i) host[i] = ctx->h_pinned[i];
  return TBSLAS_OK;
}

TreeView mesh_view(const tbslas_tree t, const MeshState& m, const int32_t* table, int T) {
  TreeView v;
  v.keys = m.keys;
  v.geom = m.geom;
  v.coeff = m.coeff;
  v.coeff2 = nullptr;
  v.cnorm = nullptr;
  v.table = table;
  v.L = m.L;
  v.stride = t->stride;
  v.T = T;
  v.q = t->q;
  v.dof = t->dof;
  return v;
}

// New leaves from per-leaf actions (keep, split into 8, merge 8 siblings
// into their parent, drop), into the other scratch set: split children get
// the restriction of their parent (transfer + FP64 refit), merged parents the
// rows of merge_c.
// splits >= 0: the actions are keep and split only, with that many splits,
// so the new leaf and transfer counts are known without a read-back.
int apply_actions(tbslas_ctx ctx, tbslas_tree t, MeshState& m, const int8_t* act,
                  const int64_t* aux, const double* merge_c, cudaStream_t s, int64_t* launches,
                  bool coeffs = true, int64_t splits = -1) {
  const int q = t->q, dof = t->dof;
  const int64_t L = m.L, np = n_points(q), stride = t->stride;
  int64_t *nleaf, *nxfer, *pos, *xpos;
  TRY(scratch_t(ctx, kRmI64a, L, &nleaf));
  TRY(scratch_t(ctx, kRmI64b, L, &nxfer));
  TRY(scratch_t(ctx, kRmI64c, L + 1, &pos));
  TRY(scratch_t(ctx, kRmI64d, L + 1, &xpos));
  launch_action_counts(act, L, nleaf, nxfer, s);
  k_scan_excl<<<1, 1024, 0, s>>>(nleaf, pos, L);
  k_scan_excl<<<1, 1024, 0, s>>>(nxfer, xpos, L);
  *launches += 3;
  TRY(check_launch("re-meshing counts"));
  int64_t sz[2] = {L + 7 * splits, 8 * splits};
  if (splits < 0) {
    const int64_t* ends[2] = {pos + L, xpos + L};
    TRY(read_scalars(ctx, ends, 2, sz, s));
  }
  const int64_t Lnew = sz[0], nx = sz[1];
  const int o = 1 - m.set;
  MeshState n;
  n.L = Lnew;
  n.set = o;
  int64_t* src_of;
  XferItem* items;
  TRY(scratch_t(ctx, kMeshKeys[o], Lnew, &n.keys));
  TRY(scratch_t(ctx, kMeshGeom[o], Lnew, &n.geom));
  TRY(scratch_t(ctx, kMeshCoeff[o], Lnew * stride, &n.coeff));
  TRY(scratch_t(ctx, kRmSrc, Lnew, &src_of));
  TRY(scratch_t(ctx, kRmItems, nx > 0 ? nx : 1, &items));
  launch_rebuild(m.keys, m.geom, act, aux, pos, xpos, L, n.keys, n.geom, src_of, items, s);
  *launches += 1;
  TRY(check_launch("re-meshing leaves"));
  if (!coeffs) {  // the leaves only (the caller refits them)
    m = n;
    return TBSLAS_OK;
  }
  double* split_c = nullptr;
  if (nx > 0) {
    const double* F = nullptr;
    double* vals;
    TRY(device_F(ctx, q, &F));
    TRY(scratch_t(ctx, kRmVals, nx * dof * np, &vals));
    TRY(scratch_t(ctx, kRmSplitC, nx * stride, &split_c));
    CUDA_TRY(cudaMemsetAsync(split_c, 0, nx * stride * sizeof(double), s));  // row padding
    launch_transfer(mesh_view(t, m, nullptr, 0), items, nx, nodes_1d(q), vals, s);
    launch_refit(vals, F, q, nx * dof, dof, stride, split_c, nullptr, ctx->d_err, false, s);
    *launches += 2;
    TRY(check_launch("re-meshing transfer"));
  }
  launch_place_coeffs(src_of, Lnew, stride, m.coeff, merge_c, split_c, n.coeff, s);
  *launches += 1;
  TRY(check_launch("re-meshing coefficients"));
  m = n;
  return TBSLAS_OK;
}

// Leaves of a re-meshing or construction into the tree's arrays (grown with
// headroom when the leaf count outgrows them), the lookup table rebuilt and
// the derived coefficient arrays refreshed.
int install_mesh(tbslas_ctx ctx, tbslas_tree t, const MeshState& m, cudaStream_t s,
                 int64_t* launches_out, int known_depth = -1) {
  const int dof = t->dof;
  const int64_t stride = t->stride;
  int64_t launches = 0;
  int maxd = known_depth;
  if (maxd < 0) {
    int64_t* sc;
    TRY(scratch_t(ctx, kRmScalars, 2, &sc));
    CUDA_TRY(cudaMemsetAsync(sc + 1, 0, sizeof(int64_t), s));
    launch_max_depth(m.geom, m.L, reinterpret_cast<int*>(sc + 1), s);
    launches += 1;
    int64_t md = 0;
    const int64_t* mdp = sc + 1;
    TRY(read_scalars(ctx, &mdp, 1, &md, s));
    maxd = (int)(md & 0xffffffff);
  }
  const int T = std::min(maxd, 7);
  const int64_t ntab = (1ll << (3 * T)) + 1;
  // allocate everything that has to grow before touching the tree, so a
  // failed allocation leaves it as it was
  const bool grow = m.L > t->cap_L, grow_tab = ntab > t->cap_table;
  const int64_t cap = grow ? m.L + m.L / 4 : t->cap_L;
  uint64_t* k = nullptr;
  Geom* g = nullptr;
  double *c = nullptr, *cn = nullptr;
  float2* c2 = nullptr;
  int32_t* tab = nullptr;
  bool ok = true;
  if (grow)
    ok = cudaMalloc(&k, cap * sizeof(uint64_t)) == cudaSuccess &&
         cudaMalloc(&g, cap * sizeof(Geom)) == cudaSuccess &&
         cudaMalloc(&c, cap * stride * sizeof(double)) == cudaSuccess &&
         cudaMalloc(&c2, cap * stride * sizeof(float2)) == cudaSuccess &&
         cudaMalloc(&cn, cap * dof * sizeof(double)) == cudaSuccess;
  if (ok && grow_tab) ok = cudaMalloc(&tab, ntab * sizeof(int32_t)) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    cudaFree(k);
    cudaFree(g);
    cudaFree(c);
    cudaFree(c2);
    cudaFree(cn);
    cudaFree(tab);
    return fail(TBSLAS_ERR_ALLOC, "growing the tree to %lld leaves failed", (long long)cap);
  }
  if (grow) {
    CUDA_TRY(cudaMemsetAsync(c2, 0, cap * stride * sizeof(float2), s));
    CUDA_TRY(cudaStreamSynchronize(s));
    cudaFree(t->d_keys);
    cudaFree(t->d_geom);
    cudaFree(t->d_coeff);
    cudaFree(t->d_coeff2);
    cudaFree(t->d_cnorm);
    t->d_keys = k;
    t->d_geom = g;
    t->d_coeff = c;
    t->d_coeff2 = c2;
    t->d_cnorm = cn;
    t->cap_L = cap;
  }
  if (grow_tab) {
    CUDA_TRY(cudaStreamSynchronize(s));
    cudaFree(t->d_table);
    t->d_table = tab;
    t->cap_table = ntab;
  }
  CUDA_TRY(cudaMemcpyAsync(t->d_keys, m.keys, m.L * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(t->d_geom, m.geom, m.L * sizeof(Geom), cudaMemcpyDeviceToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(t->d_coeff, m.coeff, m.L * stride * sizeof(double),
                           cudaMemcpyDeviceToDevice, s));
  t->L = m.L;
  t->max_depth = maxd;
  t->T = T;
  t->generation = next_generation();
  launch_build_table(t->d_keys, t->L, T, t->d_table, s);
  launches += 3;  // the table, then the split and norms of derived_coeffs
  TRY(check_launch("lookup table"));
  TRY(derived_coeffs(t, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  *launches_out += launches;
  return TBSLAS_OK;
}

int tree_remesh(tbslas_ctx ctx, tbslas_tree t, double tol, int min_depth, int max_depth, int bc,
                int64_t* stats) {
  cudaStream_t s = ctx->stream;
  const int q = t->q, dof = t->dof;
  const int64_t stride = t->stride;
  CUDA_TRY(cudaDeviceSynchronize());  // queued work on any stream may still use the tree
  MeshState m;
  m.L = t->L;
  TRY(scratch_t(ctx, kMeshKeys[0], m.L, &m.keys));
  TRY(scratch_t(ctx, kMeshGeom[0], m.L, &m.geom));
  TRY(scratch_t(ctx, kMeshCoeff[0], m.L * stride, &m.coeff));
  CUDA_TRY(cudaMemcpyAsync(m.keys, t->d_keys, m.L * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(m.geom, t->d_geom, m.L * sizeof(Geom), cudaMemcpyDeviceToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(m.coeff, t->d_coeff, m.L * stride * sizeof(double),
                           cudaMemcpyDeviceToDevice, s));
  int64_t merged = 0, split = 0, balanced = 0, launches = 0;
  int final_depth = -1;  // maximum depth of the final leaves, once read
  int64_t* sc;  // device scalars: [0] a count, [1] a maximum depth
  TRY(scratch_t(ctx, kRmScalars, 2, &sc));
  // 1. coarsen one level
  {
    const int64_t L = m.L;
    int64_t *first, *gpos;
    TRY(scratch_t(ctx, kRmI64a, L, &first));
    TRY(scratch_t(ctx, kRmI64c, L + 1, &gpos));
    launch_sibling_groups(m.keys, m.geom, L, min_depth, first, s);
    k_scan_excl<<<1, 1024, 0, s>>>(first, gpos, L);
    launches += 2;
    TRY(check_launch("sibling groups"));
    int64_t G = 0;
    const int64_t* gend = gpos + L;
    TRY(read_scalars(ctx, &gend, 1, &G, s));
    if (G > 0) {
      const double* F = nullptr;
      TRY(device_F(ctx, q, &F));
      XferItem* items;
      int64_t *group_leaf, *aux;
      double *vals, *merge_c, *tail;
      int8_t* act;
      TRY(scratch_t(ctx, kRmItems, G, &items));
      TRY(scratch_t(ctx, kRmGroup, G, &group_leaf));
      TRY(scratch_t(ctx, kRmVals, G * dof * n_points(q), &vals));
      TRY(scratch_t(ctx, kRmMergeC, G * stride, &merge_c));
      TRY(scratch_t(ctx, kRmTail, G, &tail));
      TRY(scratch_t(ctx, kRmAct, L, &act));
      TRY(scratch_t(ctx, kRmAux, L, &aux));
      CUDA_TRY(cudaMemsetAsync(merge_c, 0, G * stride * sizeof(double), s));  // row padding
      launch_group_items(first, gpos, m.geom, L, items, group_leaf, s);
      launch_transfer(mesh_view(t, m, nullptr, 0), items, G, nodes_1d(q), vals, s);
      launch_refit(vals, F, q, G * dof, dof, stride, merge_c, nullptr, ctx->d_err, false, s);
      launch_leaf_tails(merge_c, G, dof, q, stride, tail, s);
      CUDA_TRY(cudaMemsetAsync(act, kActKeep, L, s));
      launch_merge_actions(group_leaf, G, tail, tol, act, aux, s);
      launches += 5;
      TRY(check_launch("coarsening"));
      TRY(apply_actions(ctx, t, m, act, aux, merge_c, s, &launches));
      merged = (L - m.L) / 7;
    }
  }
  // 2. refine
  for (int it = 0; it <= TBSLAS_MAX_DEPTH; ++it) {
    double* tail;
    int8_t* act;
    TRY(scratch_t(ctx, kRmTail, m.L, &tail));
    TRY(scratch_t(ctx, kRmAct, m.L, &act));
    CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(int64_t), s));
    launch_leaf_tails(m.coeff, m.L, dof, q, stride, tail, s);
    launch_split_actions(tail, m.geom, m.L, tol, max_depth, act,
                         reinterpret_cast<unsigned long long*>(sc), s);
    launches += 2;
    TRY(check_launch("refinement flags"));
    int64_t n = 0;
    TRY(read_scalars(ctx, &sc, 1, &n, s));
    if (n == 0) break;
    split += n;
    TRY(apply_actions(ctx, t, m, act, nullptr, nullptr, s, &launches, true, n));
  }
  // 3. balance 2:1 (the lookup table at level 7, which find_leaf accepts at
  // any maximum depth)
  for (int it = 0; it <= TBSLAS_MAX_DEPTH; ++it) {
    int32_t* table;
    int8_t* act;
    TRY(scratch_t(ctx, kRmTable, (1ll << 21) + 1, &table));
    TRY(scratch_t(ctx, kRmAct, m.L, &act));
    launch_build_table(m.keys, m.L, 7, table, s);
    CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(int64_t), s));
    launch_balance_flags(mesh_view(t, m, table, 7), bc, act,
                         reinterpret_cast<unsigned long long*>(sc), s);
    launches += 2;
    TRY(check_launch("balance flags"));
    // the maximum depth of these leaves comes back with the flag count: when
    // nothing is flagged they are the final leaves
    CUDA_TRY(cudaMemsetAsync(sc + 1, 0, sizeof(int64_t), s));
    launch_max_depth(m.geom, m.L, reinterpret_cast<int*>(sc + 1), s);
    launches += 1;
    int64_t n_md[2] = {0, 0};
    const int64_t* both[2] = {sc, sc + 1};
    TRY(read_scalars(ctx, both, 2, n_md, s));
    const int64_t n = n_md[0];
    if (n == 0) {
      final_depth = (int)(n_md[1] & 0xffffffff);
      break;
    }
    balanced += n;
    TRY(apply_actions(ctx, t, m, act, nullptr, nullptr, s, &launches, true, n));
  }
  TRY(install_mesh(ctx, t, m, s, &launches, final_depth));
  if (stats) {
    stats[0] = t->L;
    stats[1] = merged;
    stats[2] = split;
    stats[3] = balanced;
    stats[4] = launches;
  }
  return TBSLAS_OK;
}

// ---------------------------------------------------------------------------
// Analytic input fields (construct.cu) for the device tree construction.
int field_dof(int kind) {
  switch (kind) {
    case TBSLAS_FIELD_GAUSSIANS:
    case TBSLAS_FIELD_GAUSSIAN_3D:
    case TBSLAS_FIELD_EXP_ALPHA:
      return 1;
    case TBSLAS_FIELD_ROTATION:
    case TBSLAS_FIELD_TAYLOR_GREEN:
    case TBSLAS_FIELD_TAYLOR_GREEN_ABC:
    case TBSLAS_FIELD_HOPF:
    case TBSLAS_FIELD_FOURIER:
      return 3;
    default:
      return 0;
  }
}

int64_t field_params(const tbslas_field& f) {
  switch (f.kind) {
    case TBSLAS_FIELD_GAUSSIANS: return 5ll * f.n;
    case TBSLAS_FIELD_GAUSSIAN_3D: return 7;
    case TBSLAS_FIELD_EXP_ALPHA: return 5;
    case TBSLAS_FIELD_ROTATION: return 1;
    case TBSLAS_FIELD_TAYLOR_GREEN: return 0;
    case TBSLAS_FIELD_TAYLOR_GREEN_ABC: return 6;
    case TBSLAS_FIELD_HOPF: return 5;
    case TBSLAS_FIELD_FOURIER: return 9ll * f.n;
    default: return -1;
  }
}

// Validates a field and copies its parameters to the device.
int upload_field(tbslas_ctx ctx, const tbslas_field* f, const double** dev, cudaStream_t s) {
  if (!f) return fail(TBSLAS_ERR_INVALID_ARG, "null field");
  if (field_dof(f->kind) == 0) return fail(TBSLAS_ERR_INVALID_ARG, "field kind %d", f->kind);
  if ((f->kind == TBSLAS_FIELD_GAUSSIANS || f->kind == TBSLAS_FIELD_FOURIER) &&
      (f->n < 1 || f->n > (1 << 20)))
    return fail(TBSLAS_ERR_INVALID_ARG, "field terms %d", f->n);
  const int64_t np = field_params(*f);
  if (np > 0 && !f->p) return fail(TBSLAS_ERR_INVALID_ARG, "null field parameters");
  for (int64_t i = 0; i < np; ++i)
    if (!std::isfinite(f->p[i])) return fail(TBSLAS_ERR_INVALID_ARG, "field parameter %lld",
                                             (long long)i);
  double* d;
  TRY(scratch_t(ctx, kField, np > 0 ? np : 1, &d));
  if (np > 0) CUDA_TRY(cudaMemcpyAsync(d, f->p, np * sizeof(double), cudaMemcpyHostToDevice, s));
  *dev = d;
  return TBSLAS_OK;
}

// Field values at the leaves' nodes, FP64 fit into coeff (SetTreeGridValues).
int fit_field_on(tbslas_ctx ctx, const tbslas_field* f, const double* prm, const Geom* geom,
                 int64_t L, int q, int dof, int64_t stride, double* coeff, cudaStream_t s) {
  const double* F = nullptr;
  TRY(device_F(ctx, q, &F));
  double* vals;
  TRY(scratch_t(ctx, kRmVals, L * dof * n_points(q), &vals));
  launch_field_values(f->kind, f->n, prm, geom, L, nodes_1d(q), q, dof, vals, s);
  launch_refit(vals, F, q, L * dof, dof, stride, coeff, nullptr, ctx->d_err, false, s);
  return check_launch("field fit");
}

// ConstructTree (src/tree/tree_utils.h:83-126) on the device: the uniform
// tree of min_depth; while a leaf's fit has tail > tol below max_depth,
// split it (the children are fitted afresh); 2:1 balance; the final fit.
// *launches_out gets the number of kernels launched.
int tree_construct(tbslas_ctx ctx, tbslas_tree t, const tbslas_field* f, const double* prm,
                   double tol, int min_depth, int max_depth, int bc, cudaStream_t s,
                   int64_t* launches_out) {
  const int q = t->q, dof = t->dof;
  const int64_t stride = t->stride;
  int64_t launches = 0;
  MeshState m;
  m.L = 1ll << (3 * min_depth);
  TRY(scratch_t(ctx, kMeshKeys[0], m.L, &m.keys));
  TRY(scratch_t(ctx, kMeshGeom[0], m.L, &m.geom));
  launch_uniform_leaves(min_depth, m.keys, m.geom, s);
  launches += 1;
  TRY(check_launch("uniform leaves"));
  int64_t* sc;
  TRY(scratch_t(ctx, kRmScalars, 2, &sc));
  for (int it = 0; it <= TBSLAS_MAX_DEPTH + 1; ++it) {
    TRY(scratch_t(ctx, kMeshCoeff[m.set], m.L * stride, &m.coeff));
    CUDA_TRY(cudaMemsetAsync(m.coeff, 0, m.L * stride * sizeof(double), s));  // row padding
    TRY(fit_field_on(ctx, f, prm, m.geom, m.L, q, dof, stride, m.coeff, s));
    double* tail;
    int8_t* act;
    TRY(scratch_t(ctx, kRmTail, m.L, &tail));
    TRY(scratch_t(ctx, kRmAct, m.L, &act));
    CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(int64_t), s));
    launch_leaf_tails(m.coeff, m.L, dof, q, stride, tail, s);
    launch_split_actions(tail, m.geom, m.L, tol, max_depth, act,
                         reinterpret_cast<unsigned long long*>(sc), s);
    launches += 4;  // field values, refit, tails, flags
    TRY(check_launch("refinement flags"));
    int64_t n = 0;
    TRY(read_scalars(ctx, &sc, 1, &n, s));
    if (n == 0) break;
    TRY(apply_actions(ctx, t, m, act, nullptr, nullptr, s, &launches, false));
  }
  bool split = false;
  for (int it = 0; it <= TBSLAS_MAX_DEPTH; ++it) {
    int32_t* table;
    int8_t* act;
    TRY(scratch_t(ctx, kRmTable, (1ll << 21) + 1, &table));
    TRY(scratch_t(ctx, kRmAct, m.L, &act));
    launch_build_table(m.keys, m.L, 7, table, s);
    CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(int64_t), s));
    launch_balance_flags(mesh_view(t, m, table, 7), bc, act,
                         reinterpret_cast<unsigned long long*>(sc), s);
    launches += 2;
    TRY(check_launch("balance flags"));
    int64_t n = 0;
    TRY(read_scalars(ctx, &sc, 1, &n, s));
    if (n == 0) break;
    split = true;
    TRY(apply_actions(ctx, t, m, act, nullptr, nullptr, s, &launches, false));
  }
  if (split) {  // the final leaves' fit
    TRY(scratch_t(ctx, kMeshCoeff[m.set], m.L * stride, &m.coeff));
    CUDA_TRY(cudaMemsetAsync(m.coeff, 0, m.L * stride * sizeof(double), s));
    TRY(fit_field_on(ctx, f, prm, m.geom, m.L, q, dof, stride, m.coeff, s));
    launches += 2;
  }
  TRY(install_mesh(ctx, t, m, s, &launches));
  *launches_out = launches;
  return TBSLAS_OK;
}

template <class T>
int fma_peak(tbslas_ctx ctx, int iters, double* flops_per_s) {
  BIND(ctx);
  if (!flops_per_s) return fail(TBSLAS_ERR_INVALID_ARG, "null output");
  const int blocks = ctx->num_sms * 8, threads = 256;
  double* out;
  TRY(scratch_t(ctx, kHostOut, (size_t)blocks * threads, &out));
  T* o = reinterpret_cast<T*>(out);
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  // b < 1 and c > 0 keep the chains at normal values (a -> c / (1 - b))
  const T b = T(0.999999), c = T(1e-9);
  k_fma_probe<T><<<blocks, threads, 0, ctx->stream>>>(o, b, c, 10);
  cudaEventRecord(e0, ctx->stream);
  k_fma_probe<T><<<blocks, threads, 0, ctx->stream>>>(o, b, c, iters);
  cudaEventRecord(e1, ctx->stream);
  CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  TRY(check_launch("fma_probe"));
  *flops_per_s = 2.0 * 64.0 * iters * (double)blocks * threads / (ms * 1e-3);
  return TBSLAS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// Used only by the allocation-free entry point (noalloc.cu): the bucketed
// functor evaluation on scratch the caller has carved out.  Same kernels and
// launch sequence as eval_tree_dev.
namespace tbg {

int tree_shape(tbslas_tree t, int64_t* L, int* device, int* dof) {
  if (!t || !t->ctx) return fail(TBSLAS_ERR_INVALID_ARG, "null tree");
  *L = t->L;
  *device = t->ctx->device;
  *dof = t->dof;
  return TBSLAS_OK;
}

int bucketed_eval_on(const BucketScratch& b, tbslas_tree tree, const double* pos, int64_t n,
                     double* out, int bc, cudaStream_t s) {
  if (n == 0) return TBSLAS_OK;
  const TreeView tv = tree->view();
  const int64_t L = tree->L;
  const int64_t max_tiles = (n + kTile - 1) / kTile + L;
  CUDA_TRY(cudaMemsetAsync(b.count, 0, L * sizeof(*b.count), s));
  CUDA_TRY(cudaMemsetAsync(b.cursor, 0, L * sizeof(*b.cursor), s));
  k_classify<<<blocks_for(n, 256), 256, 0, s>>>(tv, pos, n, bc, b.leaf_of, b.count, out);
  k_ntiles<<<blocks_for(L, 256), 256, 0, s>>>(b.count, L, b.ntile);
  k_scan_excl<<<1, 1024, 0, s>>>(reinterpret_cast<const int64_t*>(b.count), b.start, L);
  k_scan_excl<<<1, 1024, 0, s>>>(b.ntile, b.tileoff, L);
  k_scatter<<<blocks_for(n, 256), 256, 0, s>>>(b.leaf_of, n, b.start, b.cursor, b.perm);
  k_make_tiles<<<blocks_for(L, 256), 256, 0, s>>>(b.start, b.tileoff, L, b.tiles);
  TRY(check_launch("bucketing"));
  EvalTilesArgs a;
  a.tree = tv;
  a.pos = pos;
  a.perm = b.perm;
  a.tiles = b.tiles;
  a.ntiles = b.tileoff + L;
  a.periodic = bc;
  a.out = out;
  a.err = tree->ctx->d_err;
  a.wait_limit = tree->ctx->wait_limit;
  a.grid = (int)std::min<int64_t>(max_tiles, (int64_t)tree->ctx->num_sms * 8);
  g_kernels[tree->q].eval_tiles(a, s);
  return check_launch("eval_tiles");
}

int fail_status(int code, const char* msg) { return fail(code, "%s", msg); }

// Accessors for batch.cu.
int tree_view(tbslas_tree t, TreeView* v, tbslas_ctx* ctx) {
  if (!t || !t->ctx) return fail(TBSLAS_ERR_INVALID_ARG, "null tree");
  *v = t->view();
  *ctx = t->ctx;
  return TBSLAS_OK;
}

uint64_t tree_generation(tbslas_tree t) { return t ? t->generation : 0; }

const int32_t* tree_face_map(tbslas_tree t, int bc, cudaStream_t s) {
  if (!t || (bc != TBSLAS_BC_FREESPACE && bc != TBSLAS_BC_PERIODIC)) return nullptr;
  const int64_t n = t->L * n_points(t->q);
  if (n <= 0 || n > INT32_MAX) return nullptr;  // node indices must fit the map
  if (t->face_ok[bc] && t->face_gen[bc] == t->generation) return t->d_face[bc];
  if (t->face_cap[bc] < n) {
    int32_t* f = nullptr;
    if (cudaMalloc(&f, n * sizeof(int32_t)) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;  // evaluated without the map: every node, no copy
    }
    if (t->d_face[bc]) {
      cudaStreamSynchronize(s);
      cudaFree(t->d_face[bc]);
    }
    t->d_face[bc] = f;
    t->face_cap[bc] = n;
  }
  launch_face_map(t->view(), bc, t->d_face[bc], s);
  if (cudaGetLastError() != cudaSuccess) return nullptr;
  t->face_ok[bc] = true;
  t->face_gen[bc] = t->generation;
  return t->d_face[bc];
}

int tree_coeff2(tbslas_tree t, float2** coeff2) {
  if (!t || !t->ctx) return fail(TBSLAS_ERR_INVALID_ARG, "null tree");
  *coeff2 = t->d_coeff2;
  return TBSLAS_OK;
}

int tree_coeff(tbslas_tree t, double** coeff, int64_t* n_doubles) {
  if (!t || !t->ctx) return fail(TBSLAS_ERR_INVALID_ARG, "null tree");
  *coeff = t->d_coeff;
  *n_doubles = t->L * t->stride;
  return TBSLAS_OK;
}

int ctx_info(tbslas_ctx ctx, int* device, int* num_sms) {
  if (!ctx) return fail(TBSLAS_ERR_INVALID_ARG, "null context");
  *device = ctx->device;
  *num_sms = ctx->num_sms;
  return TBSLAS_OK;
}

uint32_t* ctx_err(tbslas_ctx ctx) { return ctx ? ctx->d_err : nullptr; }
int ctx_sums(tbslas_ctx ctx) { return ctx->sums; }
void ctx_count_object(tbslas_ctx ctx, int delta) { ctx->live_objects += delta; }
int ctx_c2_scratch(tbslas_ctx ctx, size_t n, float2** out) {
  return scratch_t(ctx, kAdjC2, n, out);
}
int ctx_wnode_scratch(tbslas_ctx ctx, size_t n, double** out) {
  return scratch_t(ctx, kAdjW, n, out);
}
int ctx_vn_scratch(tbslas_ctx ctx, size_t n, double** out) { return scratch_t(ctx, kVN, n, out); }

int ctx_F(tbslas_ctx ctx, int q, const double** F) {
  BIND(ctx);
  return device_F(ctx, q, F);
}

int ctx_mu_scratch(tbslas_ctx ctx, size_t n, double** out) { return scratch_t(ctx, kMu, n, out); }
int ctx_vals_scratch(tbslas_ctx ctx, size_t n, double** out) {
  return scratch_t(ctx, kVals, n, out);
}

Nodes1D ctx_nodes(int q) { return nodes_1d(q); }

}  // namespace tbg

// ===========================================================================
extern "C" {

const char* tbslas_status_string(int status) {
  switch (status) {
    case TBSLAS_OK: return "ok";
    case TBSLAS_ERR_INVALID_ARG: return "invalid argument";
    case TBSLAS_ERR_TREE: return "invalid tree";
    case TBSLAS_ERR_CUDA: return "CUDA error";
    case TBSLAS_ERR_UNSUPPORTED: return "unsupported";
    case TBSLAS_ERR_ALLOC: return "allocation failed";
    case TBSLAS_ERR_SIZE: return "size limit exceeded";
    case TBSLAS_ERR_DEVICE: return "device-side error";
    default: return "unknown status";
  }
}

const char* tbslas_last_error(void) { return g_err.c_str(); }

int tbslas_version(void) { return 1; }

int tbslas_ctx_create(int device, tbslas_ctx* out) {
  if (!out) return fail(TBSLAS_ERR_INVALID_ARG, "null output pointer");
  *out = nullptr;
  std::call_once(g_kernels_once, init_kernels);
  int ndev = 0;
  CUDA_TRY(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev)
    return fail(TBSLAS_ERR_INVALID_ARG, "device %d outside [0,%d)", device, ndev);
  DeviceRestore restore;
  CUDA_TRY(cudaSetDevice(device));
  tbslas_ctx c = new tbslas_ctx_s();
  c->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_err, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(c->d_err, 0, sizeof(uint32_t));
  if (e != cudaSuccess) {
    tbslas_ctx_destroy(c);
    return fail(TBSLAS_ERR_CUDA, "context setup: %s", cudaGetErrorString(e));
  }
  *out = c;
  return TBSLAS_OK;
}

int tbslas_ctx_destroy(tbslas_ctx ctx) {
  if (!ctx) return TBSLAS_OK;
  if (ctx->live_objects > 0)
    return fail(TBSLAS_ERR_INVALID_ARG,
                "%lld trees or batches of this context are still alive; destroy them first",
                (long long)ctx->live_objects);
  DeviceRestore restore;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  for (auto& b : ctx->slots)
    if (b.p) cudaFree(b.p);
  for (auto p : ctx->d_F)
    if (p) cudaFree(p);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  prof_collect(ctx);
  for (cudaEvent_t e : ctx->prof_pool) cudaEventDestroy(e);
  if (ctx->d_err) cudaFree(ctx->d_err);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return TBSLAS_OK;
}

int tbslas_ctx_check(tbslas_ctx ctx, uint32_t* device_error) {
  BIND(ctx);
  CUDA_TRY(cudaDeviceSynchronize());
  uint32_t e = 0;
  CUDA_TRY(cudaMemcpy(&e, ctx->d_err, sizeof(e), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemset(ctx->d_err, 0, sizeof(uint32_t)));
  if (device_error) *device_error = e;
  if (e) return fail(TBSLAS_ERR_DEVICE, "device error word 0x%x", e);
  return TBSLAS_OK;
}

int tbslas_profile_enable(tbslas_ctx ctx, int enable) {
  BIND(ctx);
  ctx->profile = enable != 0;
  return TBSLAS_OK;
}

int tbslas_profile_reset(tbslas_ctx ctx) {
  BIND(ctx);
  prof_collect(ctx);
  ctx->prof_totals.clear();
  return TBSLAS_OK;
}

int tbslas_profile_count(tbslas_ctx ctx, int* n) {
  BIND(ctx);
  if (!n) return fail(TBSLAS_ERR_INVALID_ARG, "null output");
  prof_collect(ctx);
  *n = (int)ctx->prof_totals.size();
  return TBSLAS_OK;
}

int tbslas_profile_get(tbslas_ctx ctx, int i, const char** name, int64_t* launches,
                       int64_t* kernels, double* total_ms) {
  BIND(ctx);
  prof_collect(ctx);
  if (i < 0 || i >= (int)ctx->prof_totals.size())
    return fail(TBSLAS_ERR_INVALID_ARG, "profile index %d", i);
  const ProfTotal& t = ctx->prof_totals[i];
  if (name) *name = t.name.c_str();
  if (launches) *launches = t.launches;
  if (kernels) *kernels = t.kernels;
  if (total_ms) *total_ms = t.ms;
  return TBSLAS_OK;
}

int tbslas_ctx_set_sums(tbslas_ctx ctx, int mode) {
  BIND(ctx);
  if (mode != TBSLAS_SUMS_DOUBLE_FLOAT && mode != TBSLAS_SUMS_FP64)
    return fail(TBSLAS_ERR_INVALID_ARG, "sums mode %d", mode);
  ctx->sums = mode;
  return TBSLAS_OK;
}

int tbslas_ctx_set_wait_limit(tbslas_ctx ctx, uint32_t polls) {
  BIND(ctx);
  ctx->wait_limit = polls;
  return TBSLAS_OK;
}

int tbslas_ctx_get_sums(tbslas_ctx ctx, int* mode) {
  BIND(ctx);
  if (!mode) return fail(TBSLAS_ERR_INVALID_ARG, "null output");
  *mode = ctx->sums;
  return TBSLAS_OK;
}

int tbslas_ctx_last_fp64_targets(tbslas_ctx ctx, int64_t* n) {
  BIND(ctx);
  if (!n) return fail(TBSLAS_ERR_INVALID_ARG, "null output");
  *n = 0;
  if (!ctx->slots[kFixCount].p) return TBSLAS_OK;
  unsigned long long c = 0;
  CUDA_TRY(cudaDeviceSynchronize());
  CUDA_TRY(cudaMemcpy(&c, ctx->slots[kFixCount].p, sizeof(c), cudaMemcpyDeviceToHost));
  *n = (int64_t)c;
  return TBSLAS_OK;
}

int tbslas_fp64_fma_peak(tbslas_ctx ctx, double* flops_per_s) {
  return fma_peak<double>(ctx, 2000, flops_per_s);
}

int tbslas_fp32_fma_peak(tbslas_ctx ctx, double* flops_per_s) {
  return fma_peak<float>(ctx, 40000, flops_per_s);
}

int tbslas_cheb_nodes(int q, double* out_host) {
  if (q < 0 || q > TBSLAS_MAX_DEGREE) return fail(TBSLAS_ERR_UNSUPPORTED, "degree %d", q);
  if (!out_host) return fail(TBSLAS_ERR_INVALID_ARG, "null output");
  std::vector<double> y = cheb_nodes_3d(q);
  std::memcpy(out_host, y.data(), y.size() * sizeof(double));
  return TBSLAS_OK;
}

int tbslas_pt2coeff_matrix(int q, double* M_host) {
  if (q < 1 || q > TBSLAS_MAX_DEGREE) return fail(TBSLAS_ERR_UNSUPPORTED, "degree %d", q);
  if (!M_host) return fail(TBSLAS_ERR_INVALID_ARG, "null output");
  const std::vector<double>& M = host_M(q);
  std::memcpy(M_host, M.data(), M.size() * sizeof(double));
  return TBSLAS_OK;
}

int tbslas_tree_create(tbslas_ctx ctx, int64_t n_leaves, const double* anchor_host,
                       const int32_t* depth_host, int q, int dof, tbslas_tree* out) {
  if (!out) return fail(TBSLAS_ERR_INVALID_ARG, "null output pointer");
  *out = nullptr;
  BIND(ctx);
  if (n_leaves < 1 || n_leaves > (int64_t)INT32_MAX)
    return fail(TBSLAS_ERR_INVALID_ARG, "leaf count %lld", (long long)n_leaves);
  if (!anchor_host || !depth_host) return fail(TBSLAS_ERR_INVALID_ARG, "null leaf arrays");
  if (q < 1 || q > TBSLAS_MAX_DEGREE)
    return fail(TBSLAS_ERR_UNSUPPORTED, "Chebyshev degree %d outside [1,%d]", q,
                TBSLAS_MAX_DEGREE);
  if (dof < 1 || dof > 16) return fail(TBSLAS_ERR_UNSUPPORTED, "dof %d outside [1,16]", dof);
  tbslas_tree t = new tbslas_tree_s();
  t->ctx = ctx;
  t->device = ctx->device;
  t->L = n_leaves;
  t->q = q;
  t->dof = dof;
  t->stride = (dof * n_coeff(q) + 1) & ~(int64_t)1;
  int s = build_tree(t, anchor_host, depth_host);
  if (s != TBSLAS_OK) {
    std::string msg = g_err;
    tbslas_tree_destroy(t);
    g_err = msg;
    return s;
  }
  t->counted = true;
  ctx->live_objects += 1;
  *out = t;
  return TBSLAS_OK;
}

int tbslas_tree_destroy(tbslas_tree t) {
  if (!t) return TBSLAS_OK;
  DeviceRestore restore;
  if (t->counted) t->ctx->live_objects -= 1;
  cudaSetDevice(t->device);
  if (t->d_keys) cudaFree(t->d_keys);
  if (t->d_geom) cudaFree(t->d_geom);
  if (t->d_coeff) cudaFree(t->d_coeff);
  if (t->d_coeff2) cudaFree(t->d_coeff2);
  if (t->d_cnorm) cudaFree(t->d_cnorm);
  if (t->d_table) cudaFree(t->d_table);
  for (int b = 0; b < 2; ++b)
    if (t->d_face[b]) cudaFree(t->d_face[b]);
  delete t;
  return TBSLAS_OK;
}

int tbslas_tree_remesh(tbslas_ctx ctx, tbslas_tree tree, double tol, int min_depth,
                       int max_depth, int bc, int64_t* stats) {
  TRY(check_tree(tree));
  BIND(ctx);
  if (tree->ctx != ctx) return fail(TBSLAS_ERR_INVALID_ARG, "tree belongs to another context");
  if (!(tol >= 0.0))  // +inf: refine nothing
    return fail(TBSLAS_ERR_INVALID_ARG, "tolerance %g is negative or NaN", tol);
  if (min_depth < 0 || max_depth < min_depth || max_depth > TBSLAS_MAX_DEPTH)
    return fail(TBSLAS_ERR_INVALID_ARG, "depth range [%d, %d] outside [0, %d]", min_depth,
                max_depth, TBSLAS_MAX_DEPTH);
  if (!bc_ok(bc)) return fail(TBSLAS_ERR_INVALID_ARG, "boundary condition %d", bc);
  return tree_remesh(ctx, tree, tol, min_depth, max_depth, bc, stats);
}

int tbslas_tree_fit_field(tbslas_ctx ctx, tbslas_tree tree, const tbslas_field* field,
                          void* stream) {
  TRY(check_tree(tree));
  BIND(ctx);
  if (tree->ctx != ctx) return fail(TBSLAS_ERR_INVALID_ARG, "tree belongs to another context");
  cudaStream_t s = (cudaStream_t)stream;
  const double* prm = nullptr;
  TRY(upload_field(ctx, field, &prm, s));
  if (field_dof(field->kind) != tree->dof)
    return fail(TBSLAS_ERR_INVALID_ARG, "field has dof %d, the tree %d", field_dof(field->kind),
                tree->dof);
  TRY(fit_field_on(ctx, field, prm, tree->d_geom, tree->L, tree->q, tree->dof, tree->stride,
                   tree->d_coeff, s));
  return derived_coeffs(tree, s);
}

int tbslas_tree_construct(tbslas_ctx ctx, const tbslas_field* field, int q, double tol,
                          int min_depth, int max_depth, int bc, tbslas_tree* out) {
  if (!out) return fail(TBSLAS_ERR_INVALID_ARG, "null output pointer");
  *out = nullptr;
  BIND(ctx);
  if (q < 1 || q > TBSLAS_MAX_DEGREE)
    return fail(TBSLAS_ERR_UNSUPPORTED, "Chebyshev degree %d outside [1,%d]", q,
                TBSLAS_MAX_DEGREE);
  if (!(tol >= 0.0)) return fail(TBSLAS_ERR_INVALID_ARG, "tolerance %g", tol);
  if (min_depth < 0 || min_depth > 6 || max_depth < min_depth || max_depth > TBSLAS_MAX_DEPTH)
    return fail(TBSLAS_ERR_INVALID_ARG, "depth range [%d, %d] (min_depth <= 6, max_depth <= %d)",
                min_depth, max_depth, TBSLAS_MAX_DEPTH);
  if (!bc_ok(bc)) return fail(TBSLAS_ERR_INVALID_ARG, "boundary condition %d", bc);
  cudaStream_t s = ctx->stream;
  CUDA_TRY(cudaDeviceSynchronize());
  const double* prm = nullptr;
  TRY(upload_field(ctx, field, &prm, s));
  tbslas_tree t = new tbslas_tree_s();
  t->ctx = ctx;
  t->device = ctx->device;
  t->q = q;
  t->dof = field_dof(field->kind);
  t->stride = (t->dof * n_coeff(q) + 1) & ~(int64_t)1;
  ProfBracket pb(ctx, "construct", s, 0);
  int64_t launches = 0;
  int st = tree_construct(ctx, t, field, prm, tol, min_depth, max_depth, bc, s, &launches);
  pb.set_kernels((int)launches);
  if (st != TBSLAS_OK) {
    std::string msg = g_err;
    tbslas_tree_destroy(t);
    g_err = msg;
    return st;
  }
  t->counted = true;
  ctx->live_objects += 1;
  *out = t;
  return TBSLAS_OK;
}

int tbslas_tree_get_leaves(tbslas_tree t, double* anchor_host, int32_t* depth_host) {
  TRY(check_tree(t));
  BIND(t->ctx);
  if (!anchor_host || !depth_host) return fail(TBSLAS_ERR_INVALID_ARG, "null output");
  CUDA_TRY(cudaDeviceSynchronize());  // queued work may still change the leaves
  std::vector<Geom> g(t->L);
  CUDA_TRY(cudaMemcpy(g.data(), t->d_geom, t->L * sizeof(Geom), cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < t->L; ++i) {
    anchor_host[3 * i + 0] = g[i].x;
    anchor_host[3 * i + 1] = g[i].y;
    anchor_host[3 * i + 2] = g[i].z;
    depth_host[i] = std::ilogb(g[i].w) - 1;
  }
  return TBSLAS_OK;
}

int tbslas_tree_info(tbslas_tree t, int64_t* n_leaves, int* q, int* dof, int* max_depth) {
  TRY(check_tree(t));
  if (n_leaves) *n_leaves = t->L;
  if (q) *q = t->q;
  if (dof) *dof = t->dof;
  if (max_depth) *max_depth = t->max_depth;
  return TBSLAS_OK;
}

int tbslas_tree_set_coeffs_host(tbslas_tree t, const double* coeff_host) {
  TRY(check_tree(t));
  BIND(t->ctx);
  if (!coeff_host) return fail(TBSLAS_ERR_INVALID_ARG, "null coefficients");
  CUDA_TRY(cudaDeviceSynchronize());  // queued work on any stream may still use the tree
  TRY(copy_coeffs(t, t->d_coeff, coeff_host, true, cudaMemcpyHostToDevice, t->ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(t->ctx->stream));
  return TBSLAS_OK;
}

int tbslas_tree_get_coeffs_host(tbslas_tree t, double* coeff_host) {
  TRY(check_tree(t));
  BIND(t->ctx);
  if (!coeff_host) return fail(TBSLAS_ERR_INVALID_ARG, "null coefficients");
  CUDA_TRY(cudaDeviceSynchronize());
  TRY(copy_coeffs(t, coeff_host, t->d_coeff, false, cudaMemcpyDeviceToHost, t->ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(t->ctx->stream));
  return TBSLAS_OK;
}

int tbslas_tree_set_coeffs(tbslas_tree t, const double* coeff_dev, void* stream) {
  TRY(check_tree(t));
  BIND(t->ctx);
  if (!coeff_dev) return fail(TBSLAS_ERR_INVALID_ARG, "null coefficients");
  return copy_coeffs(t, t->d_coeff, coeff_dev, true, cudaMemcpyDeviceToDevice,
                     (cudaStream_t)stream);
}

int tbslas_tree_get_coeffs(tbslas_tree t, double* coeff_dev, void* stream) {
  TRY(check_tree(t));
  BIND(t->ctx);
  if (!coeff_dev) return fail(TBSLAS_ERR_INVALID_ARG, "null coefficients");
  return copy_coeffs(t, coeff_dev, t->d_coeff, false, cudaMemcpyDeviceToDevice,
                     (cudaStream_t)stream);
}

int tbslas_collect_grid_points(tbslas_ctx ctx, tbslas_tree tree, double* out_dev, void* stream) {
  TRY(check_tree(tree));
  BIND(ctx);
  if (!out_dev) return fail(TBSLAS_ERR_INVALID_ARG, "null output");
  return collect_dev(tree, out_dev, (cudaStream_t)stream);
}

int tbslas_eval_tree(tbslas_ctx ctx, tbslas_tree tree, const double* pos_dev, int64_t n,
                     double* out_dev, int bc, void* stream) {
  TRY(check_tree(tree));
  BIND(ctx);
  if (n < 0) return fail(TBSLAS_ERR_INVALID_ARG, "negative point count");
  if (n > 0 && (!pos_dev || !out_dev)) return fail(TBSLAS_ERR_INVALID_ARG, "null buffer");
  if (!bc_ok(bc)) return fail(TBSLAS_ERR_INVALID_ARG, "boundary condition %d", bc);
  return eval_tree_dev(ctx, tree, pos_dev, n, out_dev, bc, (cudaStream_t)stream);
}

int tbslas_eval_tree_on_nodes(tbslas_ctx ctx, tbslas_tree src, tbslas_tree dst, double* out_dev,
                              int bc, void* stream) {
  TRY(check_tree(src));
  TRY(check_tree(dst));
  BIND(ctx);
  if (src->ctx != ctx || dst->ctx != ctx)
    return fail(TBSLAS_ERR_INVALID_ARG, "trees belong to another context");
  if (!out_dev) return fail(TBSLAS_ERR_INVALID_ARG, "null buffer");
  if (!bc_ok(bc)) return fail(TBSLAS_ERR_INVALID_ARG, "boundary condition %d", bc);
  cudaStream_t s = (cudaStream_t)stream;
  const int32_t* face = tree_face_map(dst, bc, s);
  ProfScope p(ctx, "eval_on_nodes", s, face ? 2 : 1);
  launch_eval_on_nodes(src->view(), dst->view(), bc, out_dev, s, face);
  return check_launch("eval on nodes");
}

int tbslas_eval_tree_host(tbslas_ctx ctx, tbslas_tree tree, const double* pos_host, int64_t n,
                          double* out_host, int bc) {
  TRY(check_tree(tree));
  BIND(ctx);
  if (n < 0) return fail(TBSLAS_ERR_INVALID_ARG, "negative point count");
  if (n == 0) return TBSLAS_OK;
  if (!pos_host || !out_host) return fail(TBSLAS_ERR_INVALID_ARG, "null buffer");
  if (!bc_ok(bc)) return fail(TBSLAS_ERR_INVALID_ARG, "boundary condition %d", bc);
  CUDA_TRY(cudaDeviceSynchronize());  // the tree may still be written by queued work
  double *pos, *out;
  TRY(scratch_t(ctx, kHostIn, n * 3, &pos));
  TRY(scratch_t(ctx, kHostOut, n * tree->dof, &out));
  cudaStream_t s = ctx->stream;
  CUDA_TRY(cudaMemcpyAsync(pos, pos_host, n * 3 * sizeof(double), cudaMemcpyHostToDevice, s));
  TRY(eval_tree_dev(ctx, tree, pos, n, out, bc, s));
  CUDA_TRY(cudaMemcpyAsync(out_host, out, n * tree->dof * sizeof(double),
                           cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return TBSLAS_OK;
}

int tbslas_traj_rk2(tbslas_ctx ctx, tbslas_tree vel, const double* x_dev, int64_t n,
                    double tinit, double tfinal, int nrk, int bc, double* xdep_dev,
                    void* stream) {
  TRY(check_tree(vel));
  BIND(ctx);
  if (vel->dof != 3) return fail(TBSLAS_ERR_INVALID_ARG, "velocity tree has dof %d, not 3", vel->dof);
  if (n < 0 || nrk < 1) return fail(TBSLAS_ERR_INVALID_ARG, "n=%lld nrk=%d", (long long)n, nrk);
  if (n > 0 && (!x_dev || !xdep_dev)) return fail(TBSLAS_ERR_INVALID_ARG, "null buffer");
  if (!bc_ok(bc)) return fail(TBSLAS_ERR_INVALID_ARG, "boundary condition %d", bc);
  const double tau = (tfinal - tinit) / nrk;
  if (n == 0) return TBSLAS_OK;
  return traj_dev(ctx, vel, x_dev, n, tau, nrk, bc, xdep_dev, (cudaStream_t)stream);
}

int tbslas_traj_rk2_host(tbslas_ctx ctx, tbslas_tree vel, const double* x_host, int64_t n,
                         double tinit, double tfinal, int nrk, int bc, double* xdep_host) {
  TRY(check_tree(vel));
  BIND(ctx);
  if (vel->dof != 3) return fail(TBSLAS_ERR_INVALID_ARG, "velocity tree has dof %d, not 3", vel->dof);
  if (n < 0 || nrk < 1) return fail(TBSLAS_ERR_INVALID_ARG, "n=%lld nrk=%d", (long long)n, nrk);
  if (n == 0) return TBSLAS_OK;
  if (!x_host || !xdep_host) return fail(TBSLAS_ERR_INVALID_ARG, "null buffer");
  if (!bc_ok(bc)) return fail(TBSLAS_ERR_INVALID_ARG, "boundary condition %d", bc);
  CUDA_TRY(cudaDeviceSynchronize());  // the tree may still be written by queued work
  double *x, *xd;
  TRY(scratch_t(ctx, kHostIn, n * 3, &x));
  TRY(scratch_t(ctx, kHostOut, n * 3, &xd));
  cudaStream_t s = ctx->stream;
  CUDA_TRY(cudaMemcpyAsync(x, x_host, n * 3 * sizeof(double), cudaMemcpyHostToDevice, s));
  TRY(traj_dev(ctx, vel, x, n, (tfinal - tinit) / nrk, nrk, bc, xd, s));
  CUDA_TRY(cudaMemcpyAsync(xdep_host, xd, n * 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return TBSLAS_OK;
}

int tbslas_set_tree_grid_values(tbslas_ctx ctx, tbslas_tree tree, const double* vals_dev,
                                void* stream) {
  TRY(check_tree(tree));
  BIND(ctx);
  if (!vals_dev) return fail(TBSLAS_ERR_INVALID_ARG, "null values");
  return refit_dev(ctx, tree, vals_dev, (cudaStream_t)stream);
}

static int check_step_args(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con, double dt, int nrk,
                           int bc) {
  TRY(check_tree(vel));
  TRY(check_tree(con));
  TRY(bind(ctx));
  if (vel->ctx != ctx || con->ctx != ctx)
    return fail(TBSLAS_ERR_INVALID_ARG, "trees belong to another context");
  if (vel->dof != 3) return fail(TBSLAS_ERR_INVALID_ARG, "velocity tree has dof %d, not 3", vel->dof);
  if (nrk < 1) return fail(TBSLAS_ERR_INVALID_ARG, "nrk %d < 1", nrk);
  if (!std::isfinite(dt)) return fail(TBSLAS_ERR_INVALID_ARG, "dt is not finite");
  if (!bc_ok(bc)) return fail(TBSLAS_ERR_INVALID_ARG, "boundary condition %d", bc);
  return TBSLAS_OK;
}

int tbslas_semilag_in_situ(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con, int timestep,
                           double dt, int nrk, int bc, void* stream) {
  DeviceRestore restore;
  TRY(check_step_args(ctx, vel, con, dt, nrk, bc));
  return semilag_in_situ_dev(ctx, vel, con, timestep, dt, nrk, bc, (cudaStream_t)stream);
}

}  // extern "C"

int tbslas_semilag_bdf2(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con_prev,
                        tbslas_tree con_cur, tbslas_tree con_next, double t, double dt, int nrk,
                        int bc, void* stream) {
  DeviceRestore restore;
  TRY(check_step_args(ctx, vel, con_cur, dt, nrk, bc));
  TRY(check_tree(con_prev));
  TRY(check_tree(con_next));
  if (con_prev->ctx != ctx || con_next->ctx != ctx)
    return fail(TBSLAS_ERR_INVALID_ARG, "trees belong to another context");
  if (!std::isfinite(t)) return fail(TBSLAS_ERR_INVALID_ARG, "t is not finite");
  const int q = con_next->q;
  if (vel->q != q || con_cur->q != q || con_prev->q != q || con_cur->dof != 1 ||
      con_prev->dof != 1 || con_next->dof != 1 || !g_bdf2[q])
    return fail(TBSLAS_ERR_UNSUPPORTED, "BDF2 step needs a dof-3 velocity and dof-1 "
                                        "concentration trees of one degree");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t N = con_next->L * n_points(q);
  Bdf2Args a;
  a.vel = vel->view();
  a.prev = con_prev->view();
  a.cur = con_cur->view();
  a.next = con_next->view();
  a.nodes = nodes_1d(q);
  // the two backtraces' sub-steps as the driver computes them: from t to
  // t - dt, then from t - dt to t - 2 dt (ComputeTrajRK2's (tfinal - tinit) / nrk)
  a.tau1 = ((t - dt) - t) / nrk;
  a.tau2 = ((t - dt * 2) - (t - dt)) / nrk;
  a.nrk = nrk;
  a.periodic = bc;
  double* vn = nullptr;
  TRY(scratch_t(ctx, kVals, N, &a.vals));
  TRY(scratch_t(ctx, kVN, N * 3, &vn));
  TRY(scratch_t(ctx, kFixList, N, &a.fix_list));
  TRY(scratch_t(ctx, kFixCount, 1, &a.fix_count));
  a.fix_grid = ctx->num_sms * 8;
  {
    // shared upper-face nodes are read through the face map, not copied
    a.face = tree_face_map(con_next, bc, s);
    ProfScope pv(ctx, "vel_at_nodes", s, 1);
    launch_eval_on_nodes(a.vel, a.next, bc, vn, s, a.face, false);
  }
  TRY(check_launch("velocity at nodes"));
  a.vn = vn;
  {
    const bool df = ctx->sums == TBSLAS_SUMS_DOUBLE_FLOAT;
    ProfScope p(ctx, "semilag_bdf2", s, df ? 2 : 1);
    g_bdf2[q](a, df, s);
  }
  TRY(check_launch("semilag_bdf2"));
  return refit_dev(ctx, con_next, a.vals, s);
}

int tbslas_cubic_time_weights(const double* times, double t, double* w) {
  if (!times || !w) return fail(TBSLAS_ERR_INVALID_ARG, "null pointer");
  if (!(times[0] < times[1] && times[1] < times[2] && times[2] < times[3]) ||
      !std::isfinite(times[0]) || !std::isfinite(times[3]) || !std::isfinite(t))
    return fail(TBSLAS_ERR_INVALID_ARG, "times must be finite and increasing");
  for (int k = 0; k < 4; ++k) {
    double e[4] = {0.0, 0.0, 0.0, 0.0};
    e[k] = 1.0;
    w[k] = interp_cubic_1d(t, times, e);  // the interpolant is linear in the values
  }
  return TBSLAS_OK;
}

int tbslas_semilag_in_situ_tv(tbslas_ctx ctx, int m, const tbslas_tree* vel, const double* w,
                              tbslas_tree con, int timestep, double dt, int nrk, int bc,
                              void* stream) {
  DeviceRestore restore;
  if (m < 1 || m > kTvMaxTrees)
    return fail(TBSLAS_ERR_INVALID_ARG, "%d velocity trees (1..%d)", m, kTvMaxTrees);
  if (!vel || !w) return fail(TBSLAS_ERR_INVALID_ARG, "null pointer");
  if (nrk > kTvMaxSubsteps)
    return fail(TBSLAS_ERR_UNSUPPORTED, "nrk %d > %d with a velocity set", nrk, kTvMaxSubsteps);
  for (int k = 0; k < m; ++k) {
    TRY(check_step_args(ctx, vel[k], con, dt, nrk, bc));
    if (vel[k]->q != con->q)
      return fail(TBSLAS_ERR_UNSUPPORTED, "velocity set: degree %d vs the concentration's %d",
                  vel[k]->q, con->q);
  }
  if (con->dof != 1) return fail(TBSLAS_ERR_UNSUPPORTED, "velocity set: dof-1 concentration only");
  for (int j = 0; j < 2 * nrk * m; ++j)
    if (!std::isfinite(w[j])) return fail(TBSLAS_ERR_INVALID_ARG, "weight %d is not finite", j);
  cudaStream_t s = (cudaStream_t)stream;
  const double tau = sl_tau(timestep, dt, nrk);
  // one leaf structure, nrk = 1 and the double-float mode: blend the
  // coefficients per stage and run the fused step.  The FP64 mode evaluates
  // every tree and blends the values, as the reference's functors do, with
  // one leaf lookup per point when the trees share their structure.
  bool same = true;
  for (int k = 1; k < m && same; ++k) same = vel[k]->L == vel[0]->L;
  // the keys are compared once per set of leaf lists (their stamps)
  TvStructure& known = ctx->tv_structure;
  bool cached = same && m > 1 && known.m == m;
  for (int k = 0; k < m && cached; ++k) cached = known.gen[k] == vel[k]->generation;
  if (cached) {
    same = known.same;
  } else if (same && m > 1) {
    int* flag;
    TRY(scratch_t(ctx, kTvFlag, 1, &flag));
    CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), s));
    for (int k = 1; k < m; ++k)
      k_keys_differ<<<blocks_for(vel[0]->L, 256), 256, 0, s>>>(vel[0]->d_keys, vel[k]->d_keys,
                                                              vel[0]->L, flag);
    TRY(check_launch("velocity set structure"));
    int h = 0;
    CUDA_TRY(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    same = h == 0;
    known.m = m;
    for (int k = 0; k < m; ++k) known.gen[k] = vel[k]->generation;
    known.same = same;
  }
  if (same && nrk == 1 && ctx->sums == TBSLAS_SUMS_DOUBLE_FLOAT) {
    const tbslas_tree v0 = vel[0];
    const int64_t n = v0->L * v0->stride;
    const double* c[kTvMaxTrees];
    for (int k = 0; k < m; ++k) c[k] = vel[k]->d_coeff;
    double *c1, *c2, *n2;
    float2* c2s;
    TRY(scratch_t(ctx, kTvC1, n, &c1));
    TRY(scratch_t(ctx, kTvC2, n, &c2));
    TRY(scratch_t(ctx, kTvC2s, n, &c2s));
    TRY(scratch_t(ctx, kTvN2, v0->L * 3, &n2));
    {
      ProfScope pb(ctx, "velocity_blend", s, 4);
      launch_blend_coeffs(c, w, m, n, c1, s);
      launch_blend_coeffs(c, w + m, m, n, c2, s);
      launch_split(c2, c2s, n, ctx->d_err, s);
      k_cnorm<<<blocks_for(v0->L * 3, 128), 128, 0, s>>>(c2, v0->L, 3, (int)n_coeff(v0->q),
                                                         v0->stride, n2);
    }
    TRY(check_launch("velocity blend"));
    TreeView b1 = v0->view(), b2 = v0->view();
    b1.coeff = c1;
    b2.coeff = c2;
    b2.coeff2 = c2s;
    b2.cnorm = n2;
    return fused_step(ctx, b1, b2, con, tau, 1, bc, s, nullptr, nullptr);
  }
  // general: every tree evaluated at every stage point (FP64)
  TvArgs a;
  for (int k = 0; k < m; ++k) a.vel[k] = vel[k]->view();
  a.m = m;
  a.con = con->view();
  a.nodes = nodes_1d(con->q);
  a.tau = tau;
  a.nrk = nrk;
  a.periodic = bc;
  for (int j = 0; j < 2 * nrk * m; ++j) a.w[j] = w[j];
  a.same_leaves = same ? 1 : 0;
  const int64_t N = con->L * n_points(con->q);
  TRY(scratch_t(ctx, kVals, N, &a.vals));
  {
    // first stage: every tree at the target nodes by sum factorisation
    double* vn = nullptr;
    TRY(scratch_t(ctx, kVN, (size_t)m * N * 3, &vn));
    const int32_t* face = tree_face_map(con, bc, s);
    // shared upper-face nodes are not copied: the step kernel reads them
    // through the face map
    ProfScope pv(ctx, "vel_at_nodes", s, same ? 1 : m);
    if (same) {  // one walk for trees of one structure
      TreeView v[kTvMaxTrees];
      for (int k = 0; k < m; ++k) v[k] = vel[k]->view();
      launch_eval_on_nodes_set(v, m, a.con, bc, vn, 3 * N, s, face);
    } else {
      for (int k = 0; k < m; ++k)
        launch_eval_on_nodes(vel[k]->view(), a.con, bc, vn + 3 * k * N, s, face, false);
    }
    a.face = face;
    TRY(check_launch("velocity set at nodes"));
    a.vn = vn;
  }
  {
    ProfScope p(ctx, "semilag_tv", s);
    g_tv[con->q](a, s);
  }
  TRY(check_launch("semilag_tv"));
  return refit_dev(ctx, con, a.vals, s);
}

// For the adjoint's checkpointed forward (adjoint.cu).
namespace tbg {
int semilag_in_situ_points(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con, int timestep,
                           double dt, int bc, double* xmid, double* xdep, cudaStream_t s,
                           double* jac) {
  TRY(check_step_args(ctx, vel, con, dt, 1, bc));
  if (vel->q != con->q || vel->dof != 3 || con->dof != 1)
    return fail(TBSLAS_ERR_UNSUPPORTED, "points of the step need a dof-3 velocity and a dof-1 "
                                        "concentration tree of one degree");
  if (!xdep) return fail(TBSLAS_ERR_INVALID_ARG, "null departure-point buffer");
  if (jac && !xmid) return fail(TBSLAS_ERR_INVALID_ARG, "the Jacobian checkpoint needs xmid");
  return semilag_in_situ_dev(ctx, vel, con, timestep, dt, 1, bc, s, xmid, xdep, jac);
}

int step_midpoints(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con, int timestep, double dt,
                   int bc, double** xmid, cudaStream_t s, const double* vn_given) {
  TRY(check_step_args(ctx, vel, con, dt, 1, bc));
  const int q = con->q;
  const int64_t N = con->L * n_points(q);
  const double* vn = vn_given;
  if (!vn) {
    double* v = nullptr;
    TRY(scratch_t(ctx, kVN, N * 3, &v));
    ProfScope pv(ctx, "adjoint_vel_at_nodes", s, 2);
    launch_eval_on_nodes(vel->view(), con->view(), bc, v, s, tree_face_map(con, bc, s));
    vn = v;
  }
  TRY(scratch_t(ctx, kXA, N * 3, xmid));
  {
    ProfScope pm(ctx, "adjoint_midpoints", s);
    launch_midpoints(con->view(), nodes_1d(q), q, sl_tau(timestep, dt, 1), bc, vn, *xmid, s);
  }
  return check_launch("midpoints");
}

ProfBracket::ProfBracket(tbslas_ctx ctx, const char* name, cudaStream_t s, int kernels)
    : ctx_(ctx), name_(name), s_(s), kernels_(kernels) {
  if (ctx_->profile) {
    start_ = prof_event(ctx_);
    cudaEventRecord(start_, s_);
  }
}
ProfBracket::~ProfBracket() {
  if (start_) {
    cudaEvent_t stop = prof_event(ctx_);
    cudaEventRecord(stop, s_);
    ctx_->prof_pending.push_back(ProfRecord{name_, kernels_, start_, stop});
  }
}

int step_points(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con, int timestep, double dt,
                int bc, double** xmid, double** xdep, cudaStream_t s, const double* vn_given) {
  TRY(check_step_args(ctx, vel, con, dt, 1, bc));
  const int q = con->q;
  const bool df = ctx->sums == TBSLAS_SUMS_DOUBLE_FLOAT;
  if (vel->q != q || con->dof != 1 || !g_kernels[q].points_df || !g_kernels[q].points_fp64)
    return fail(TBSLAS_ERR_UNSUPPORTED, "step points: degree %d", q);
  const int64_t N = con->L * n_points(q);
  SemilagTreeArgs a;
  a.vel = vel->view();
  a.con = con->view();
  a.nodes = nodes_1d(q);
  a.tau = sl_tau(timestep, dt, 1);
  a.nrk = 1;
  a.periodic = bc;
  a.vals = nullptr;
  if (vn_given) {
    a.vn = vn_given;
  } else {
    double* vn = nullptr;
    TRY(scratch_t(ctx, kVN, N * 3, &vn));
    {
      ProfScope pv(ctx, "adjoint_vel_at_nodes", s, 2);
      launch_eval_on_nodes(a.vel, a.con, bc, vn, s, tree_face_map(con, bc, s));
    }
    TRY(check_launch("velocity at nodes"));
    a.vn = vn;
  }
  TRY(scratch_t(ctx, kXA, N * 3, &a.xmid));
  TRY(scratch_t(ctx, kXB, N * 3, &a.xdep));
  TRY(scratch_t(ctx, kFixList, N, &a.fix_list));
  TRY(scratch_t(ctx, kFixCount, 1, &a.fix_count));
  a.fix_grid = ctx->num_sms * 8;
  {
    ProfScope pp(ctx, "adjoint_points", s, df ? 2 : 1);
    (df ? g_kernels[q].points_df : g_kernels[q].points_fp64)(a, s);
  }
  TRY(check_launch("step points"));
  *xmid = a.xmid;
  *xdep = a.xdep;
  return TBSLAS_OK;
}
}  // namespace tbg

extern "C" {

int tbslas_semilag_in_situ_host(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con,
                                double* con_coeff_host, int timestep, double dt, int nrk,
                                int bc) {
  DeviceRestore restore;
  TRY(check_step_args(ctx, vel, con, dt, nrk, bc));
  if (!con_coeff_host) return fail(TBSLAS_ERR_INVALID_ARG, "null coefficients");
  CUDA_TRY(cudaDeviceSynchronize());  // queued work on any stream may still use the trees
  cudaStream_t s = ctx->stream;
  TRY(copy_coeffs(con, con->d_coeff, con_coeff_host, true, cudaMemcpyHostToDevice, s));
  TRY(semilag_in_situ_dev(ctx, vel, con, timestep, dt, nrk, bc, s));
  TRY(copy_coeffs(con, con_coeff_host, con->d_coeff, false, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return TBSLAS_OK;
}

int tbslas_fast_interp(tbslas_ctx ctx, const double* grid_dev, int dof, int n_reg,
                       const double* pts_dev, int64_t n, double* out_dev, int bc, void* stream) {
  BIND(ctx);
  if (n_reg < 4) return fail(TBSLAS_ERR_INVALID_ARG, "grid size %d < 4", n_reg);
  if ((int64_t)n_reg * n_reg * n_reg > (int64_t)1 << 40)
    return fail(TBSLAS_ERR_SIZE, "grid size %d too large", n_reg);
  if (dof < 1 || n < 0) return fail(TBSLAS_ERR_INVALID_ARG, "dof=%d n=%lld", dof, (long long)n);
  if (n > 0 && (!grid_dev || !pts_dev || !out_dev))
    return fail(TBSLAS_ERR_INVALID_ARG, "null buffer");
  if (!bc_ok(bc)) return fail(TBSLAS_ERR_INVALID_ARG, "boundary condition %d", bc);
  ProfScope p(ctx, "fast_interp", (cudaStream_t)stream);
  launch_fast_interp(grid_dev, dof, n_reg, pts_dev, n, out_dev, bc, (cudaStream_t)stream);
  return check_launch("fast_interp");
}

static int check_grid_args(tbslas_ctx ctx, const void* vel, const void* con, const void* cout,
                           int n_reg, double dt, int nrk, int bc) {
  TRY(bind(ctx));
  if (!vel || !con || !cout) return fail(TBSLAS_ERR_INVALID_ARG, "null buffer");
  if (con == cout) return fail(TBSLAS_ERR_INVALID_ARG, "con_out aliases con");
  if (n_reg < 4) return fail(TBSLAS_ERR_INVALID_ARG, "grid size %d < 4", n_reg);
  if ((int64_t)n_reg * n_reg * n_reg > (int64_t)1 << 40)
    return fail(TBSLAS_ERR_SIZE, "grid size %d too large", n_reg);
  if (nrk < 1) return fail(TBSLAS_ERR_INVALID_ARG, "nrk %d < 1", nrk);
  if (!std::isfinite(dt)) return fail(TBSLAS_ERR_INVALID_ARG, "dt is not finite");
  if (!bc_ok(bc)) return fail(TBSLAS_ERR_INVALID_ARG, "boundary condition %d", bc);
  return TBSLAS_OK;
}

int tbslas_semilag_grid(tbslas_ctx ctx, const double* vel_dev, const double* con_dev,
                        double* con_out_dev, int n_reg, double dt, int nrk, int bc,
                        void* stream) {
  DeviceRestore restore;
  TRY(check_grid_args(ctx, vel_dev, con_dev, con_out_dev, n_reg, dt, nrk, bc));
  const double tau = (-dt - 0.0) / nrk;
  return semilag_grid_dev(ctx, vel_dev, con_dev, con_out_dev, n_reg, tau, nrk, bc,
                          (cudaStream_t)stream);
}

int tbslas_semilag_grid_steps(tbslas_ctx ctx, const double* vel_dev, const double* con_dev,
                              double* con_out_dev, int n_reg, double dt, int nsteps, int nrk,
                              int bc, void* stream) {
  DeviceRestore restore;
  TRY(check_grid_args(ctx, vel_dev, con_dev, con_out_dev, n_reg, dt, nrk, bc));
  if (nsteps < 1) return fail(TBSLAS_ERR_INVALID_ARG, "nsteps %d < 1", nsteps);
  const int64_t n3 = (int64_t)n_reg * n_reg * n_reg;
  double* tmp = nullptr;
  if (nsteps > 1) TRY(scratch_t(ctx, kGridTmp, n3, &tmp));
  const double tau = (-dt - 0.0) / nrk;
  cudaStream_t s = (cudaStream_t)stream;
  const double* in = con_dev;
  for (int k = 0; k < nsteps; ++k) {
    // the last step writes con_out_dev; steps alternate between it and tmp
    double* out = ((nsteps - 1 - k) % 2 == 0) ? con_out_dev : tmp;
    TRY(semilag_grid_dev(ctx, vel_dev, in, out, n_reg, tau, nrk, bc, s, k == 0));
    in = out;
  }
  return TBSLAS_OK;
}

int tbslas_semilag_grid_host(tbslas_ctx ctx, const double* vel_host, const double* con_host,
                             double* con_out_host, int n_reg, double dt, int nrk, int bc) {
  DeviceRestore restore;
  TRY(check_grid_args(ctx, vel_host, con_host, con_out_host, n_reg, dt, nrk, bc));
  CUDA_TRY(cudaDeviceSynchronize());  // earlier queued work may still use the scratch
  const int64_t n3 = (int64_t)n_reg * n_reg * n_reg;
  double *vel, *con, *cout;
  TRY(scratch_t(ctx, kHostIn, n3 * 3, &vel));
  TRY(scratch_t(ctx, kHostIn2, n3, &con));
  TRY(scratch_t(ctx, kHostOut, n3, &cout));
  cudaStream_t s = ctx->stream;
  CUDA_TRY(cudaMemcpyAsync(vel, vel_host, n3 * 3 * sizeof(double), cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(con, con_host, n3 * sizeof(double), cudaMemcpyHostToDevice, s));
  const double tau = (-dt - 0.0) / nrk;
  TRY(semilag_grid_dev(ctx, vel, con, cout, n_reg, tau, nrk, bc, s));
  CUDA_TRY(cudaMemcpyAsync(con_out_host, cout, n3 * sizeof(double), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return TBSLAS_OK;
}

}  // extern "C"

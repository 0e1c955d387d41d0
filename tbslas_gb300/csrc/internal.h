// Declarations shared by the translation units of libtbslas_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace tbg {

// Entry points make their context's device current for their own work and
// put the calling thread's previous current device back when they return
// (on every return path), so a host application that drives several
// devices from one thread keeps its own choice of device.
struct DeviceRestore {
  int prev = -1;
  DeviceRestore() {
    if (cudaGetDevice(&prev) != cudaSuccess) {
      cudaGetLastError();
      prev = -1;
    }
  }
  ~DeviceRestore() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
  DeviceRestore(const DeviceRestore&) = delete;
  DeviceRestore& operator=(const DeviceRestore&) = delete;
};

// One tile of the bucketed functor evaluation: `count` (<= kTile) points of
// one leaf, stored at perm[start, start+count).
struct Tile {
  int64_t start;
  int32_t leaf;
  int32_t count;
};
constexpr int kTile = 128;

struct SemilagTreeArgs {
  TreeView vel;       // dof 3
  TreeView con;       // dof 1, same degree as vel
  Nodes1D nodes;      // 1-D nodes of con's degree
  double tau;         // -dt / nrk
  int nrk;
  int periodic;
  double* vals;       // [Lc * Np] node values at the departure points
  const double* vn;   // [Lc * Np][3] velocity at the targets (first RK stage) or null
  int64_t* fix_list;  // targets the double-float kernel hands to the FP64 pass
  unsigned long long* fix_count;
  int fix_grid;       // CTAs of the FP64 pass (persistent)
  // nrk = 1 with vn given: every target's RK2 midpoint X* and departure point
  // Xd ([Lc * Np][3], unwrapped, as computed -- the FP64 path's points for the
  // targets the FP64 pass recomputes), or null
  double* xmid = nullptr;
  double* xdep = nullptr;
  // with xmid/xdep (FP64 sums): the velocity Jacobian at every midpoint,
  // [Lc * Np][9] row-major dv_a/dx_b (the checkpoint of the adjoint's
  // velocity-gradient term), or null
  double* jac = nullptr;
  // con's face map when vn holds no shared upper-face nodes (node_source),
  // or null
  const int32_t* face = nullptr;
};

struct TrajArgs {
  TreeView vel;
  const double* x;
  int64_t n;
  double tau;
  int nrk;
  int periodic;
  double* xdep;
};

// Polls of a bounded device-side wait before it gives up and sets
// kErrBarrierTimeout (each poll is an mbarrier try_wait, which itself blocks
// for a hardware-defined time slice).
constexpr uint32_t kWaitLimit = 1u << 22;

struct EvalTilesArgs {
  TreeView tree;
  const double* pos;
  const int64_t* perm;
  const Tile* tiles;
  const int64_t* ntiles;  // device scalar
  int periodic;
  double* out;
  uint32_t* err;
  int grid;
  uint32_t wait_limit;  // polls of the wait for each tile's coefficient copy
};

// Scratch of one bucketed tree evaluation, carved by the caller.
struct BucketScratch {
  int32_t* leaf_of;             // [n]
  unsigned long long* count;    // [L], zeroed by the launcher
  unsigned long long* cursor;   // [L], zeroed by the launcher
  int64_t* start;               // [L + 1]
  int64_t* ntile;               // [L]
  int64_t* tileoff;             // [L + 1]
  int64_t* perm;                // [n]
  Tile* tiles;                  // [n / kTile + 1 + L]
};

// The BDF2 two-backtrace step (bdf2_kernels.cuh): value at every node X of
// `next` = 4/3 cur(X1) - 1/3 prev(X2), X1 and X2 the RK2 backtraces over one
// and two steps.
struct Bdf2Args {
  TreeView vel;       // dof 3
  TreeView prev;      // c_{n-1}, dof 1
  TreeView cur;       // c_n, dof 1
  TreeView next;      // the target tree (its nodes); same degree as the others
  Nodes1D nodes;      // 1-D nodes of the degree
  double tau1, tau2;  // sub-step of the first / second backtrace
  int nrk;
  int periodic;
  double* vals;       // [next.L * Np]
  const double* vn;   // [next.L * Np][3] velocity at the targets
  int64_t* fix_list;  // targets the double-float kernel hands to the FP64 pass
  unsigned long long* fix_count;
  int fix_grid;
  const int32_t* face = nullptr;  // next's face map: vn holds no shared upper-face nodes
};

typedef void (*Bdf2Fn)(const Bdf2Args&, bool df_sums, cudaStream_t);
void register_bdf2_a(Bdf2Fn* table);  // index = Chebyshev degree q
void register_bdf2_b(Bdf2Fn* table);

// The in-situ step through a blended set of velocity trees (tv_kernels.cuh):
// the velocity at the stage point of RK2 stage j (2 per sub-step: at X, then
// at X*) is sum_k w[j * m + k] v_k.
constexpr int kTvMaxTrees = 4;
constexpr int kTvMaxSubsteps = 8;
struct TvArgs {
  TreeView vel[kTvMaxTrees];  // dof 3, same degree as con
  int m;                      // trees in use
  TreeView con;               // dof 1
  Nodes1D nodes;
  double tau;
  int nrk;
  int periodic;
  double* vals;  // [con.L * Np]
  // the trees' velocities at the targets (first stage of the first
  // sub-step), tree k at vn + 3 k con.L Np, from the node-grid pass
  // (bit-identical to evaluating them there), or null
  const double* vn = nullptr;
  double w[2 * kTvMaxSubsteps * kTvMaxTrees];
  int same_leaves = 0;  // 1: every tree has vel[0]'s leaves (one lookup per point)
  const int32_t* face = nullptr;  // con's face map: vn holds no shared upper-face nodes
};
typedef void (*TvFn)(const TvArgs&, cudaStream_t);
void register_tv_a(TvFn* table);  // index = Chebyshev degree q
void register_tv_b(TvFn* table);
void register_tv_c(TvFn* table);
// out[i] = sum_k w[k] c_k[i], i < n (tv_deg_a.cu)
void launch_blend_coeffs(const double* const* c, const double* w, int m, int64_t n, double* out,
                         cudaStream_t s);

typedef void (*SemilagTreeFn)(const SemilagTreeArgs&, cudaStream_t);
typedef void (*TrajFn)(const TrajArgs&, cudaStream_t);
typedef void (*EvalTilesFn)(const EvalTilesArgs&, cudaStream_t);

struct DegreeKernels {
  SemilagTreeFn semilag = nullptr;     // FP64 fused step
  SemilagTreeFn semilag_df = nullptr;  // double-float fused step + FP64 pass over near-face targets
  SemilagTreeFn points_df = nullptr;   // its midpoints and departure points only (q <= 10)
  SemilagTreeFn points_fp64 = nullptr;  // the FP64 step's midpoints and departure points (q <= 10)
  TrajFn traj = nullptr;
  EvalTilesFn eval_tiles = nullptr;
  int eval_tiles_max_threads_hint = 0;
};

// Filled by the per-degree translation units (index = Chebyshev degree q).
void register_degrees_a(DegreeKernels* table);
void register_degrees_b(DegreeKernels* table);
void register_degrees_c(DegreeKernels* table);
void register_degrees_d(DegreeKernels* table);
void register_degrees_e(DegreeKernels* table);
void register_degrees_f(DegreeKernels* table);
void register_degrees_g(DegreeKernels* table);
void register_degrees_h(DegreeKernels* table);

// capi.cu, for the allocation-free entry point (noalloc.cu)
int tree_shape(tbslas_tree t, int64_t* L, int* device, int* dof);
int bucketed_eval_on(const BucketScratch& b, tbslas_tree tree, const double* pos,
                     int64_t n, double* out, int bc, cudaStream_t s);
int fail_status(int code, const char* msg);
int tree_view(tbslas_tree t, TreeView* v, tbslas_ctx* ctx);
int tree_coeff(tbslas_tree t, double** coeff, int64_t* n_doubles);
int tree_coeff2(tbslas_tree t, float2** coeff2);
// Changes whenever the tree's leaf list (and with it its device arrays) is
// rebuilt, e.g. by tbslas_tree_remesh.
uint64_t tree_generation(tbslas_tree t);
// The tree's face map for boundary condition bc (launch_eval_on_nodes),
// built on `s` the first time it is asked for at the tree's current leaf
// structure; null when it cannot be had (the evaluation then computes every
// node itself).
const int32_t* tree_face_map(tbslas_tree t, int bc, cudaStream_t s);
int ctx_info(tbslas_ctx ctx, int* device, int* num_sms);
int ctx_F(tbslas_ctx ctx, int q, const double** F);
int ctx_mu_scratch(tbslas_ctx ctx, size_t n, double** out);
int ctx_vals_scratch(tbslas_ctx ctx, size_t n, double** out);
Nodes1D ctx_nodes(int q);
// The in-situ step (nrk = 1, fused path: dof-3 velocity and dof-1
// concentration of one degree) writing every target's RK2 midpoint and
// departure point to xmid / xdep ([Lc * Np][3]) and, when jac is given (FP64
// sums only), the velocity Jacobian at the midpoint ([Lc * Np][9]).
int semilag_in_situ_points(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con, int timestep,
                           double dt, int bc, double* xmid, double* xdep, cudaStream_t s,
                           double* jac = nullptr);
// The fused step kernel that also stores J_v(X*) (adjoint_f64.cuh), for
// degree q (1..10); TBSLAS_ERR_UNSUPPORTED beyond.
int launch_semilag_jac(int q, const SemilagTreeArgs& a, cudaStream_t s);
// Profiling bracket for launch groups of other translation units (the
// context's per-name CUDA-event timing; nothing when profiling is off).
class ProfBracket {
 public:
  ProfBracket(tbslas_ctx ctx, const char* name, cudaStream_t s, int kernels = 1);
  ~ProfBracket();
  ProfBracket(const ProfBracket&) = delete;
  ProfBracket& operator=(const ProfBracket&) = delete;
  // For groups whose launch count is known only at their end.
  void set_kernels(int kernels) { kernels_ = kernels; }

 private:
  tbslas_ctx ctx_;
  const char* name_;
  cudaStream_t s_;
  int kernels_;
  cudaEvent_t start_ = nullptr;
};
// The midpoints of that step, X + tau/2 v(X) with v(X) from the node grid
// (the forward's own arithmetic), into scratch of the context ([Lc * Np][3]).
// vn_given: the velocity at con's nodes when the caller has it (a sequence of
// steps through one stationary velocity), else null (computed here).
int step_midpoints(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con, int timestep, double dt,
                   int bc, double** xmid, cudaStream_t s, const double* vn_given = nullptr);
// xmid[t] = (X_t wrapped under periodic boundaries) + tau/2 vn[t] (construct.cu)
void launch_midpoints(const TreeView& con, const Nodes1D& nodes, int q, double tau, int periodic,
                      const double* vn, double* xmid, cudaStream_t s);
// The midpoints and departure points of that step only, into scratch of the
// context (*xmid, *xdep: [Lc * Np][3]), for the adjoint's recompute: the
// step's own kernels in the context's sums mode (double-float: FP64 for the
// ambiguous targets).
int step_points(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con, int timestep, double dt,
                int bc, double** xmid, double** xdep, cudaStream_t s,
                const double* vn_given = nullptr);

// node_eval.cu: src evaluated at every node of dst's leaves, [dst.L * Np][src.dof]
// (bit-identical to the pointwise FP64 evaluation)
// face: dst's face map for this boundary condition (tree_face_map), or null
// (every node evaluated, no copy)
// copy_faces false: the shared upper-face nodes are left unwritten (the
// consumer reads face[t]'s value instead).
void launch_eval_on_nodes(const TreeView& src, const TreeView& dst, int periodic, double* out,
                          cudaStream_t s, const int32_t* face = nullptr, bool copy_faces = true);
// ntrees source trees of one leaf structure (src[k].keys all equal; the
// walk is src[0]'s), tree k's values at out + k * tstride, each as
// launch_eval_on_nodes writes them with copy_faces false (the shared
// upper-face nodes of a face map left unwritten).  ntrees <= kTvMaxTrees.
void launch_eval_on_nodes_set(const TreeView* src, int ntrees, const TreeView& dst, int periodic,
                              double* out, int64_t tstride, cudaStream_t s,
                              const int32_t* face = nullptr);
// face[t] = the target index whose value the shared upper-face node t takes
// (same point, same source leaf), else -1; [dst.L * Np]
void launch_face_map(const TreeView& dst, int periodic, int32_t* face, cudaStream_t s);
// Transposed: out[V * out_stride + l * Nc + n] += sum over dst's nodes p in
// leaf V of W[p][l] phi_n(X_p) (FP64 atomics); W: [dst.L * Np][src.dof].
void launch_scatter_on_nodes(const TreeView& src, const TreeView& dst, int periodic,
                             const double* W, double* out, int64_t out_stride, bool df_sums,
                             cudaStream_t s);
// Batched: one item per (job, destination leaf); the jobs of one launch
// share the source degree q_src, max_q_dst bounds their destination degrees.
struct NodeEvalJob {
  TreeView src;
  TreeView dst;
  Nodes1D nodes;  // 1-D nodes of dst's degree
  double* out;
  const int32_t* face;  // dst's face map, or null
};
struct NodeEvalItem {
  int32_t job, pad;
  int64_t leaf;
};
// The jobs' shared upper-face nodes (their face maps) are left unwritten.
void launch_batch_eval_on_nodes(const NodeEvalJob* jobs, const NodeEvalItem* items,
                                int64_t n_items, int q_src, int max_q_dst, int periodic,
                                cudaStream_t s);

// Refit (refit.cu): node values -> coefficients through the separable
// factors F = refit_factors(q) (4 D x D blocks on the device).
//   coeff[(r/dof)*stride + (r%dof)*nc + t] = sum_p vals[r*np + p] M[p][t]
// df_sums: the passes in double-float (the default step), else FP64
void launch_refit(const double* vals, const double* F, int q, int64_t rows, int dof,
                  int64_t stride, double* coeff, float2* coeff2, uint32_t* err, bool df_sums,
                  cudaStream_t s);
// mu[r*np + p] = sum_t M[p][t] lam[r*nc + t] (the adjoint's transposed refit)
void launch_refit_t(const double* lam, const double* F, int q, int64_t rows, double* mu,
                    bool df_sums, cudaStream_t s);
// Batched refit: one job per problem, one CTA per (job, row) item.
struct RefitJob {
  const double* vals;
  const double* F;
  double* coeff;
  float2* coeff2;
  uint32_t* err;
  int64_t rows;
  int64_t stride;
  int q, dof;
};
struct RefitItem {
  int32_t job, pad;
  int64_t row;
};
void launch_batch_refit(const RefitJob* jobs, const RefitItem* items, int64_t n_items, int max_q,
                        bool df_sums, cudaStream_t s);
void launch_split(const double* c, float2* c2, int64_t n, uint32_t* err, cudaStream_t s);
uint32_t* ctx_err(tbslas_ctx ctx);
int ctx_sums(tbslas_ctx ctx);
// Trees and batches alive on a context (tbslas_ctx_destroy refuses while any are).
void ctx_count_object(tbslas_ctx ctx, int delta);
int ctx_c2_scratch(tbslas_ctx ctx, size_t n, float2** out);
int ctx_wnode_scratch(tbslas_ctx ctx, size_t n, double** out);
int ctx_vn_scratch(tbslas_ctx ctx, size_t n, double** out);

// Re-meshing (remesh.cu; the host sequence is tree_remesh in capi.cu).
// Transfer item: node values of a new leaf with geometry g, from the old
// tree's leaf src (kXferChild: its parent) or leaves src..src+7 (kXferParent:
// its 8 children, child index x + 2y + 4z).
enum : int32_t { kXferChild = 0, kXferParent = 1 };
struct XferItem {
  Geom g;
  int64_t src;
  int32_t mode, pad;
};
// Per-leaf re-meshing actions.
enum : int8_t { kActKeep = 0, kActSplit = 1, kActMerge = 2, kActDrop = 3 };
// out: [n][S.dof][(q+1)^3] node values (the refit's row layout)
void launch_transfer(const TreeView& S, const XferItem* items, int64_t n, const Nodes1D& nodes,
                     double* out, cudaStream_t s);
void launch_leaf_tails(const double* coeff, int64_t L, int dof, int q, int64_t stride,
                       double* tail, cudaStream_t s);
void launch_sibling_groups(const uint64_t* keys, const Geom* geom, int64_t L, int min_depth,
                           int64_t* first, cudaStream_t s);
void launch_group_items(const int64_t* first, const int64_t* pos, const Geom* geom, int64_t L,
                        XferItem* items, int64_t* group_leaf, cudaStream_t s);
void launch_merge_actions(const int64_t* group_leaf, int64_t G, const double* tail, double tol,
                          int8_t* act, int64_t* aux, cudaStream_t s);
void launch_split_actions(const double* tail, const Geom* geom, int64_t L, double tol,
                          int max_depth, int8_t* act, unsigned long long* count, cudaStream_t s);
void launch_action_counts(const int8_t* act, int64_t L, int64_t* nleaf, int64_t* nxfer,
                          cudaStream_t s);
void launch_rebuild(const uint64_t* keys, const Geom* geom, const int8_t* act, const int64_t* aux,
                    const int64_t* pos, const int64_t* xpos, int64_t L, uint64_t* nkeys,
                    Geom* ngeom, int64_t* src_of, XferItem* items, cudaStream_t s);
void launch_place_coeffs(const int64_t* src_of, int64_t Lnew, int64_t stride, const double* old_c,
                         const double* merge_c, const double* split_c, double* out,
                         cudaStream_t s);
void launch_balance_flags(const TreeView& t, int periodic, int8_t* act, unsigned long long* count,
                          cudaStream_t s);
void launch_build_table(const uint64_t* keys, int64_t L, int T, int32_t* table, cudaStream_t s);
void launch_max_depth(const Geom* geom, int64_t L, int* out, cudaStream_t s);
// Analytic fields (construct.cu): out[(leaf * dof + l) * Np + p] at the
// leaves' nodes; the 8^d leaves of the uniform depth-d tree.
void launch_field_values(int kind, int n, const double* prm, const Geom* geom, int64_t L,
                         const Nodes1D& nodes, int q, int dof, double* out, cudaStream_t s);
void launch_uniform_leaves(int d, uint64_t* keys, Geom* geom, cudaStream_t s);


// grid.cu
void launch_fast_interp(const double* grid, int dof, int nreg, const double* pts, int64_t n,
                        double* out, int periodic, cudaStream_t s);
void launch_semilag_grid(const double* vel, const double* con, double* cout, int nreg,
                         double tau, int nrk, int periodic, cudaStream_t s);
// periodic grids, stencil sums in double-float over hi/lo copies of the grids
// (vel2: 3 n^3, con2: n^3 float2 scratch); split_vel = false reuses vel2 as
// the previous call on the same velocity left it
void launch_semilag_grid_df(const double* vel, const double* con, double* cout, int nreg,
                            double tau, int nrk, float2* vel2, float2* con2, uint32_t* err,
                            int num_sms, bool split_vel, cudaStream_t s);

}  // namespace tbg

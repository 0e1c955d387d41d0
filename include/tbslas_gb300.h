/*
 * tbslas_gb300 -- C ABI of the GB300 (sm_103a) semi-Lagrangian advection step.
 *
 * Drop-in for the tbslas SL path: the field-functor concept
 *   void operator()(const real_t* pos, int n, real_t* out)
 * (src/tree/tree_functor.h:793-815, used by src/semilag/traj.inc:33,:40 and
 * src/semilag/semilag.inc:43), ComputeTrajRK2 (src/semilag/traj.inc:48-68),
 * SolveSemilagInSitu (src/tree/tree_semilag.h:92-135), their tree glue
 * CollectChebTreeGridPoints / SetTreeGridValues (src/tree/tree_utils.h:442-552),
 * the Chebyshev helpers new_nodes / GetPt2CoeffMatrix (src/utils/cheb.h:41-196)
 * and the tricubic regular-grid interpolant fast_interp
 * (src/tree/tree_functor.h:89-153).
 *
 * Conventions
 *  - Every entry point returns a tbslas_status (0 = success).  The reference
 *    has no error codes (asserts only); here bad arguments are rejected on the
 *    host before any launch and tbslas_last_error() gives a message.
 *  - Pointers named *_dev are device pointers owned by the caller; *_host are
 *    host pointers.  `stream` is a cudaStream_t (NULL = legacy default stream).
 *    Device entry points are asynchronous on `stream`; *_host entry points are
 *    synchronous: they first wait for all work queued on the device, then copy,
 *    compute and copy back on the context's own stream.
 *  - All arithmetic is IEEE FP64.
 *  - Boundary condition `bc`: TBSLAS_BC_FREESPACE or TBSLAS_BC_PERIODIC, the
 *    reference's pvfmm::FreeSpace / pvfmm::Periodic (sim_config->bc).
 *  - A point with a NaN coordinate, or outside [0,1]^3 under FreeSpace (after
 *    the single periodic wrap under Periodic), evaluates to 0 -- the value
 *    pvfmm::cheb_poly's |x|>1 rule gives such points in the reference.
 *  - Unlike EvalTree (src/tree/tree_functor.h:442-448, :803), no entry point
 *    writes the periodic wrap back into the caller's coordinate array.
 *  - A tree is a complete linear octree of leaves in Morton order (the
 *    post-order leaf list of the reference's pvfmm::MPI_Tree) with per-leaf
 *    triangular Chebyshev coefficients of degree q, laid out
 *    [leaf][dof][Nc], Nc = (q+1)(q+2)(q+3)/6, index order i (z) outer,
 *    j (y), k (x) inner over i+j+k <= q (src/tree/tree_functor.h:257-267).
 *  - One context per host thread; calls on one context are not re-entrant.
 */
#ifndef TBSLAS_GB300_H_
#define TBSLAS_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  TBSLAS_OK = 0,
  TBSLAS_ERR_INVALID_ARG = 1, /* null pointer, negative size, bad enum      */
  TBSLAS_ERR_TREE = 2,        /* leaves are not a complete Morton-ordered octree */
  TBSLAS_ERR_CUDA = 3,        /* a CUDA runtime call failed                 */
  TBSLAS_ERR_UNSUPPORTED = 4, /* degree outside the compiled range, ...     */
  TBSLAS_ERR_ALLOC = 5,       /* device allocation failed                   */
  TBSLAS_ERR_SIZE = 6,        /* a size exceeds a stated limit              */
  TBSLAS_ERR_DEVICE = 7       /* a kernel reported an error status          */
} tbslas_status;

enum { TBSLAS_BC_FREESPACE = 0, TBSLAS_BC_PERIODIC = 1 };

/* Limits: Chebyshev degree 1..TBSLAS_MAX_DEGREE, leaf depth 0..TBSLAS_MAX_DEPTH. */
#define TBSLAS_MAX_DEGREE 16
#define TBSLAS_MAX_DEPTH 21

typedef struct tbslas_ctx_s* tbslas_ctx;
typedef struct tbslas_tree_s* tbslas_tree;
typedef struct tbslas_batch_s* tbslas_batch;

/* ---- errors / version ---------------------------------------------------- */
const char* tbslas_status_string(int status);
/* Message of the last failing call on this host thread ("" if none). */
const char* tbslas_last_error(void);
int tbslas_version(void);

/* ---- context ------------------------------------------------------------- */
/* Binds `device`, owns cached scratch buffers.  No reference counterpart
 * (the reference keeps static buffers: src/tree/tree_functor.h:166,:519-584). */
int tbslas_ctx_create(int device, tbslas_ctx* out);
/* Destroy a context's trees and batches first: while any are alive the
 * context is left intact and TBSLAS_ERR_INVALID_ARG is returned. */
int tbslas_ctx_destroy(tbslas_ctx ctx);
/* Kernel-side error word (bounded waits that ran out, ...); 0 if clean.
 * Synchronises the context's device; clears the word. */
int tbslas_ctx_check(tbslas_ctx ctx, uint32_t* device_error);
/* Polls a bounded device-side wait makes before it gives up (default
 * TBSLAS_WAIT_LIMIT_DEFAULT).  The functor's per-tile wait for its
 * coefficient copy uses it; a wait that runs out sets bit
 * TBSLAS_DEVICE_ERR_WAIT_TIMEOUT of the error word, lets the copy in flight
 * land, and its kernel returns, leaving the context usable (that call's
 * output is incomplete).  A small limit (0 = give up at once) is how a test
 * drives that path without faulting anything.  No reference counterpart. */
#define TBSLAS_WAIT_LIMIT_DEFAULT (1u << 22)
#define TBSLAS_DEVICE_ERR_WAIT_TIMEOUT 1u
int tbslas_ctx_set_wait_limit(tbslas_ctx ctx, uint32_t polls);

/* ---- profiling --------------------------------------------------------------- */
/* Per-kernel CUDA-event timing, accumulated per kernel name.  Replaces
 * pvfmm::Profile::Enable / Tic / Toc / print as the reference uses them
 * (src/applications/src/advection.cpp:77, :400; src/semilag/traj.inc:53).
 * When enabled, every launch group is bracketed by a pair of events on its
 * stream; reading the totals waits for those events. */
int tbslas_profile_enable(tbslas_ctx ctx, int enable);
int tbslas_profile_reset(tbslas_ctx ctx);
int tbslas_profile_count(tbslas_ctx ctx, int* n);
/* launches: bracketed launch groups; kernels: kernel launches inside them.
 * name: valid until the next reset or destroy of ctx. */
int tbslas_profile_get(tbslas_ctx ctx, int i, const char** name, int64_t* launches,
                       int64_t* kernels, double* total_ms);
/* Arithmetic of the Chebyshev sums of the SL steps on ctx (targets, RK2
 * updates, Morton keys, leaf search and leaf-local coordinates are FP64
 * either way):
 *  - TBSLAS_SUMS_FP64 (default): every sum in FP64 in the reference's order,
 *    as the reference computes them (vec_eval<double>,
 *    src/tree/tree_functor.h:27-84); departure points and node values are
 *    bit-identical to the oracle.
 *  - TBSLAS_SUMS_DOUBLE_FLOAT (opt-in, narrower than FP64): the sums at the
 *    midpoint and the departure point run as double-float (hi + lo float
 *    pairs: 48-bit significand, FP32's exponent range, so magnitudes below
 *    2^-126 flush and above 2^100 are rejected through the device error
 *    word) on the FP32 pipe -- GB300 runs FP64 at 1/72 of its FP32 rate.
 *    Every coordinate carries a rigorous bound on its distance from the
 *    all-FP64 one; targets whose lookup that bound makes ambiguous are
 *    recomputed in FP64, so every leaf choice equals the FP64 path's.
 *    Values agree with the FP64 path to ~1e-14 relative (the parity
 *    tolerance is 1e-12).
 * The first RK2 stage (the velocity at the nodes) is FP64 and exact in both.
 * The batch (tbslas_batch_*) follows the mode its context had when the batch
 * was created. */
enum { TBSLAS_SUMS_DOUBLE_FLOAT = 0, TBSLAS_SUMS_FP64 = 1 };
int tbslas_ctx_set_sums(tbslas_ctx ctx, int mode);
int tbslas_ctx_get_sums(tbslas_ctx ctx, int* mode);
/* Targets of the last double-float in-situ step on ctx that were recomputed
 * in FP64 (ambiguous lookups); synchronises the device.  Diagnostic. */
int tbslas_ctx_last_fp64_targets(tbslas_ctx ctx, int64_t* n);

/* Measured FP64 FMA throughput of the device (FLOP/s, 2 per FMA): the
 * roofline denominator of the FP64-pipe-bound kernels.  Diagnostic; no
 * reference counterpart. */
int tbslas_fp64_fma_peak(tbslas_ctx ctx, double* flops_per_s);
/* Measured FP32 FMA throughput (FLOP/s, 2 per FMA): the denominator of the
 * double-float sums, which run on the FP32 pipe.  Diagnostic; no reference
 * counterpart. */
int tbslas_fp32_fma_peak(tbslas_ctx ctx, double* flops_per_s);

/* ---- Chebyshev helpers (host) ---------------------------------------------- */
/* new_nodes(q,3): (q+1)^3 x 3 nodes in [0,1], x fastest.
 * Replaces tbslas::new_nodes, src/utils/cheb.h:41-67. */
int tbslas_cheb_nodes(int q, double* out_host);
/* (q+1)^3 x Nc matrix M with coeff = values * M (least squares fit of the
 * total-degree basis at new_nodes).  Replaces tbslas::GetPt2CoeffMatrix,
 * src/utils/cheb.h:166-196. */
int tbslas_pt2coeff_matrix(int q, double* M_host);

/* ---- trees ------------------------------------------------------------------- */
/* Leaves: anchor_host[L*3] (lower corner), depth_host[L]; Morton order,
 * complete.  Stands in for the pvfmm::MPI_Tree / Cheb_Node leaf list the
 * reference walks with PostorderFirst/PostorderNxt (src/tree/tree_utils.h:460-495).
 * Coefficients start at zero. */
int tbslas_tree_create(tbslas_ctx ctx, int64_t n_leaves, const double* anchor_host,
                       const int32_t* depth_host, int q, int dof, tbslas_tree* out);
int tbslas_tree_destroy(tbslas_tree tree);
int tbslas_tree_info(tbslas_tree tree, int64_t* n_leaves, int* q, int* dof, int* max_depth);
/* Copy [L][dof][Nc] coefficients in / out (Node::ChebData() of every leaf). */
int tbslas_tree_set_coeffs_host(tbslas_tree tree, const double* coeff_host);
int tbslas_tree_get_coeffs_host(tbslas_tree tree, double* coeff_host);
int tbslas_tree_set_coeffs(tbslas_tree tree, const double* coeff_dev, void* stream);
int tbslas_tree_get_coeffs(tbslas_tree tree, double* coeff_dev, void* stream);
/* Analytic input fields for tree construction and fitting (the input
 * functions of the reference's drivers, src/utils/fields.h).  p: host array
 * of the kind's parameters (copied by the call).
 *   GAUSSIANS        dof 1, sum of n terms amp exp(-|x-c|^2 / (2 sigma^2)),
 *                    p[5i..5i+4] = cx, cy, cz, sigma, amp
 *   GAUSSIAN_3D      dof 1, get_gaussian_field_3d: xc, yc, zc, A, sx, sy, sz
 *   EXP_ALPHA        dof 1, get_exp_alpha_field: xc, yc, zc, R, alpha
 *   ROTATION         dof 3, get_vorticity_field with omega = p[0]
 *   TAYLOR_GREEN     dof 3, (sin 2pi x cos 2pi y cos 2pi z,
 *                    -cos 2pi x sin 2pi y cos 2pi z, 0); no parameters
 *   TAYLOR_GREEN_ABC dof 3, get_taylor_green_field: A, B, C, a, b, c
 *   HOPF             dof 3, get_hopf_field: xc, yc, zc, A, r
 *   FOURIER          dof 3, sum of n modes A cos(2pi k.x) + B sin(2pi k.x),
 *                    p[9i..9i+8] = kx, ky, kz, Ax, Ay, Az, Bx, By, Bz */
enum {
  TBSLAS_FIELD_GAUSSIANS = 0,
  TBSLAS_FIELD_GAUSSIAN_3D = 1,
  TBSLAS_FIELD_EXP_ALPHA = 2,
  TBSLAS_FIELD_ROTATION = 3,
  TBSLAS_FIELD_TAYLOR_GREEN = 4,
  TBSLAS_FIELD_TAYLOR_GREEN_ABC = 5,
  TBSLAS_FIELD_HOPF = 6,
  TBSLAS_FIELD_FOURIER = 7
};
typedef struct {
  int kind;
  int n;
  const double* p;
} tbslas_field;
/* InitTree (src/tree/tree_utils.h:128-178) on the device: the field at every
 * leaf's Chebyshev nodes (new_nodes), fitted as SetTreeGridValues does.  The
 * field's dof must be the tree's. */
int tbslas_tree_fit_field(tbslas_ctx ctx, tbslas_tree tree, const tbslas_field* field,
                          void* stream);
/* ConstructTree (src/tree/tree_utils.h:83-126) on the device: from the
 * uniform tree of min_depth (<= 6), every leaf whose fit of the field has
 * tail > tol (sum over dofs of |c| over the total-degree-q coefficients) and
 * depth < max_depth is split, its children fitted afresh, until none is; then
 * 2:1 balance (periodic images under TBSLAS_BC_PERIODIC) and the final fit.
 * The refinement rule is PVFMM's (not vendored); this is the project's
 * restatement, the one tbslas_tree_remesh applies.  Synchronous.  With
 * profiling on, the whole construction is one launch group "construct" that
 * counts every kernel it launched. */
int tbslas_tree_construct(tbslas_ctx ctx, const tbslas_field* field, int q, double tol,
                          int min_depth, int max_depth, int bc, tbslas_tree* out);

/* The current leaves: anchor_host[L*3], depth_host[L] (L from tbslas_tree_info). */
int tbslas_tree_get_leaves(tbslas_tree tree, double* anchor_host, int32_t* depth_host);

/* Adaptive re-meshing after a step, on the device: the reference's
 * tcon.RefineTree(); tcon.Balance21(bc) (src/applications/src/advection.cpp:
 * 305-311).  Both live in PVFMM (not vendored); this is the project's
 * restatement of their rule, with tail(leaf) = sum over dofs of |c| over the
 * coefficients of total degree q:
 *  1. coarsen, one level: each complete group of 8 sibling leaves deeper than
 *     min_depth becomes its parent when the parent's tail <= tol (the parent
 *     fitted at its nodes from the sibling whose closed half holds each node);
 *  2. refine: while a leaf has tail > tol and depth < max_depth, it is split
 *     into its 8 children (the restriction of its expansion, fitted at the
 *     children's nodes);
 *  3. balance: while a leaf has a face, edge or corner neighbour more than one
 *     level deeper (periodic images under TBSLAS_BC_PERIODIC), it is split.
 * Leaves no rule touches keep their coefficients bit for bit.  The tree's
 * leaf count changes (tbslas_tree_info, tbslas_tree_get_leaves).  stats
 * (optional, 5 values): new leaf count, groups merged, leaves split by
 * refinement, leaves split by balancing, kernels launched.  Synchronous. */
int tbslas_tree_remesh(tbslas_ctx ctx, tbslas_tree tree, double tol, int min_depth,
                       int max_depth, int bc, int64_t* stats);

/* ---- the SL path --------------------------------------------------------------- */
/* Chebyshev nodes of every leaf, leaves in order: out_dev[L*(q+1)^3*3].
 * Replaces CollectChebTreeGridPoints, src/tree/tree_utils.h:442-498. */
int tbslas_collect_grid_points(tbslas_ctx ctx, tbslas_tree tree, double* out_dev, void* stream);

/* Field functor: out_dev[n*dof] (point-major) = tree evaluated at pos_dev[n*3].
 * Points are bucketed by leaf (counting sort on the leaf's Morton rank), each
 * leaf's coefficients staged in shared memory, results un-permuted.
 * Replaces NodeFieldFunctor::operator() -> EvalTree -> EvalNodesLocal,
 * src/tree/tree_functor.h:397-815. */
int tbslas_eval_tree(tbslas_ctx ctx, tbslas_tree tree, const double* pos_dev, int64_t n,
                     double* out_dev, int bc, void* stream);
/* src evaluated at every Chebyshev node of dst's leaves: out_dev
 * [dst leaves * (q_dst+1)^3][src dof], in the order of
 * tbslas_collect_grid_points(dst).  Equals tbslas_eval_tree(src) at those
 * points bit for bit (same sums, same order); computed by sum factorisation
 * over the nodes' tensor grid, ~D^4 instead of D^6/6 work per leaf.  The
 * composition EvalTree(src, CollectChebTreeGridPoints(dst)) that the first
 * RK2 stage of SolveSemilagInSitu performs (src/tree/tree_semilag.h:114-124,
 * src/semilag/traj.inc:20-68). */
int tbslas_eval_tree_on_nodes(tbslas_ctx ctx, tbslas_tree src, tbslas_tree dst, double* out_dev,
                              int bc, void* stream);
/* Synchronous host-buffer form of the same functor (the reference's exact
 * calling convention: host arrays in, host array out). */
int tbslas_eval_tree_host(tbslas_ctx ctx, tbslas_tree tree, const double* pos_host, int64_t n,
                          double* out_host, int bc);

/* Allocation-free form of tbslas_eval_tree, for callers that cannot allocate
 * device memory while they evaluate: a solver loop running under a memory
 * budget fixed up front, or a host application whose own pool owns every
 * device allocation (library-side cudaMalloc/cudaFree would synchronise the
 * device and fragment that pool).  No counterpart in the reference (it
 * allocates freely: static grow-on-demand buffers in EvalTree).  Same inputs,
 * outputs and results as tbslas_eval_tree; the call itself makes no
 * cudaMalloc, cudaFree or allocating library call.  The caller's current
 * device is left as it was.
 *  - Scratch lives in one static device array of TBSLAS_NOALLOC_SCRATCH_BYTES
 *    (about 5 MiB) that every GPU which loads this library holds until the
 *    process exits.
 *  - Limits: n <= TBSLAS_NOALLOC_MAX_POINTS points per call and trees of at
 *    most TBSLAS_NOALLOC_MAX_LEAVES leaves; larger requests return
 *    TBSLAS_ERR_SIZE (split the points over several calls).
 *  - The first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress) with that device current; make that first call
 *    before any stream capture.  If the host application destroys the
 *    device's primary context (cudaDeviceReset), the next call sees a new
 *    context and looks the address up again.
 *  - Every call on a device shares the one array: calls whose work overlaps
 *    on the GPU (other streams, other host threads) race and corrupt each
 *    other.  Serialise them (one stream, or events).  The parts that must
 *    start at zero are cleared by each call. */
#define TBSLAS_NOALLOC_MAX_POINTS (1 << 18)
#define TBSLAS_NOALLOC_MAX_LEAVES (1 << 15)
#define TBSLAS_NOALLOC_SCRATCH_BYTES (5u << 20)
int tbslas_eval_tree_noalloc(tbslas_tree tree, const double* pos_dev, int64_t n, double* out_dev,
                             int bc, void* stream);

/* RK2 backtrace of n points through a dof-3 velocity tree from tinit to tfinal
 * in nrk sub-steps: xdep_dev[n*3].  Replaces ComputeTrajRK2 with a
 * NodeFieldFunctor velocity, src/semilag/traj.inc:20-68. */
int tbslas_traj_rk2(tbslas_ctx ctx, tbslas_tree vel, const double* x_dev, int64_t n,
                    double tinit, double tfinal, int nrk, int bc, double* xdep_dev,
                    void* stream);

/* Synchronous host-buffer form of tbslas_traj_rk2. */
int tbslas_traj_rk2_host(tbslas_ctx ctx, tbslas_tree vel, const double* x_host, int64_t n,
                         double tinit, double tfinal, int nrk, int bc, double* xdep_host);

/* Node values -> coefficients of every leaf: vals_dev[L][dof][(q+1)^3].
 * Replaces SetTreeGridValues, src/tree/tree_utils.h:500-552. */
int tbslas_set_tree_grid_values(tbslas_ctx ctx, tbslas_tree tree, const double* vals_dev,
                                void* stream);

/* One in-situ SL step: every Chebyshev node of `con` is backtraced through
 * `vel` (RK2, nrk sub-steps, from timestep*dt to timestep*dt-dt), `con` is
 * evaluated at the departure points and refitted in place.  Targets are never
 * materialised.  Replaces SolveSemilagInSitu, src/tree/tree_semilag.h:92-135.
 * For dof > 1 the node values are refitted per dof (the reference exercises
 * dof = 1 only). */
int tbslas_semilag_in_situ(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con, int timestep,
                           double dt, int nrk, int bc, void* stream);
/* Same step with the coefficients in host memory: copies con's coefficients
 * in, runs the step, copies them back out (synchronous). */
int tbslas_semilag_in_situ_host(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con,
                                double* con_coeff_host, int timestep, double dt, int nrk,
                                int bc);

/* In-situ step through a time-dependent velocity: m (1..4) velocity trees
 * blended per RK2 stage, the velocity at stage j (two per sub-step: at X,
 * then at X*) being sum_k w[j*m + k] v_k; w: host [2*nrk][m].  The
 * reference's time-dependent functors map to weights:
 *  - FieldSetFunctor (src/tree/tree_set_functor.h:49-72): four trees at times
 *    T[4], cubic in time (CubicInterpPolicy::InterpCubic1D, src/utils/cubic.h:
 *    42-56), queried by IntegrateRK2 at tinit and tinit + tau/2 of each
 *    sub-step (src/semilag/traj.inc:20-45): w[2s*4 + k] and w[(2s+1)*4 + k]
 *    from tbslas_cubic_time_weights;
 *  - FieldExtrapFunctor (src/tree/tree_extrap_functor.h:47-78) with the
 *    current field as the first-stage functor (the two-functor
 *    SolveSemilagInSitu, src/tree/tree_semilag.h:137-180, traj.inc:71-93):
 *    trees {v_n, v_{n-1}}, w = {1, 0, 1.5, -0.5} per sub-step.
 * Trees of one leaf structure with nrk = 1 run, in the double-float mode,
 * the fused step on the per-stage blends of their coefficients; otherwise
 * (and always in TBSLAS_SUMS_FP64) every tree is evaluated at every stage
 * point in FP64 and the values blended -- for trees of one leaf structure
 * with one leaf lookup per point and one node-grid walk, the same values.
 * With m > 1 trees of one leaf count the call compares their leaf keys on
 * the device and waits for the answer (a stream synchronisation), once per
 * set of leaf lists: the context keeps the answer until one of the trees
 * is re-meshed or another set is passed.  Blending
 * coefficients equals blending values up to rounding (~1e-16); where a
 * blended velocity component vanishes at a point on a leaf face or the
 * domain's boundary, that rounding can put the point on the other side than
 * the reference's value blend does.  Velocity trees share the
 * concentration's degree; the concentration has dof 1. */
int tbslas_semilag_in_situ_tv(tbslas_ctx ctx, int m, const tbslas_tree* vel, const double* w,
                              tbslas_tree con, int timestep, double dt, int nrk, int bc,
                              void* stream);
/* w[4] with InterpCubic1D(t, times, p) = sum_k w[k] p[k] for every p (the
 * interpolant is linear in p); times strictly increasing.  Host only. */
int tbslas_cubic_time_weights(const double* times, double t, double* w);

/* Second-order (BDF2) semi-Lagrangian step with two backtraces, the step of
 * the reference's advection-diffusion driver (src/applications/src/
 * advdiff-ss.cpp:485-521): for every Chebyshev node X of con_next,
 *   X1 = ComputeTrajRK2(vel, X, t, t - dt, nrk),
 *   X2 = ComputeTrajRK2(vel, X1, t - dt, t - 2 dt, nrk),
 *   value = 4/3 con_cur(X1) - 1/3 con_prev(X2),
 * refitted into con_next (SetTreeGridValues).  t is the driver's current
 * time (its running tcurr); the sub-steps are computed from it as the
 * reference does.  The four trees share one Chebyshev degree (vel dof 3, the
 * others dof 1); con_next may be con_cur or con_prev itself (it is only
 * written after both are read).  The context's sum mode applies as in
 * tbslas_semilag_in_situ. */
int tbslas_semilag_bdf2(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con_prev,
                        tbslas_tree con_cur, tbslas_tree con_next, double t, double dt, int nrk,
                        int bc, void* stream);

/* ---- differentiation (adjoint of the in-situ step, nrk = 1) ------------------ */
/* No counterpart in the reference.  The forward map of one step is
 * C^{k+1} = refit(c^k(Xd(V))), Xd = X + tau v(X + tau/2 v(X)), for every node
 * X of `con`; the adjoint gives dJ/dC^k and dJ/dV from dJ/dC^{k+1}.  Both
 * support Chebyshev degree 1..10, a dof-3 velocity and a dof-1 concentration
 * tree of the same degree. */
/* tbslas_semilag_in_situ with nrk = 1 (same kernels, same result, the
 * context's sum mode) that also stores, per target node (leaf-major, node
 * order of CollectChebTreeGridPoints), the RK2 midpoint xmid_dev[N*3] (or
 * NULL: departure points only, 24 B per target) and departure point
 * xdep_dev[N*3], N = L (q+1)^3.  In the double-float mode the
 * points lie in the FP64 step's leaves (targets near a face are recomputed in
 * FP64) and within ~1e-15 of its points. */
int tbslas_semilag_in_situ_ckpt(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con, int timestep,
                                double dt, int bc, double* xmid_dev, double* xdep_dev,
                                void* stream);
/* The same checkpointed step that also stores the velocity Jacobian at every
 * midpoint, jac_dev[N*9] (row-major dv_a/dx_b, a the component), for
 * tbslas_semilag_adjoint_jac: 120 B per target with xmid and xdep.  The
 * step's node values and points are bit-identical to tbslas_semilag_in_situ's
 * (the midpoint velocity comes out of the same sums as its gradient).  FP64
 * sums only (TBSLAS_ERR_UNSUPPORTED in the double-float mode); all three
 * buffers required. */
int tbslas_semilag_in_situ_ckpt_jac(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con,
                                    int timestep, double dt, int bc, double* xmid_dev,
                                    double* xdep_dev, double* jac_dev, void* stream);
/* Adjoint of step `timestep`: con_coeff_k_dev [L][Nc] = the concentration
 * coefficients the step started from; lambda_next_dev [L][Nc] = dJ/dC^{k+1};
 * writes lambda_k_dev [L][Nc] = dJ/dC^k and ADDS the step's dJ/dV to
 * grad_vel_dev [Lv][3][Nc].  xmid/xdep: the step's checkpoints; xmid NULL
 * with xdep given rebuilds the midpoints from the node-grid velocity (the
 * forward's own arithmetic); both NULL recompute the points.  Velocity
 * coefficients are read from `vel`. */
int tbslas_semilag_adjoint(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con,
                           const double* con_coeff_k_dev, int timestep, double dt, int bc,
                           const double* lambda_next_dev, double* lambda_k_dev,
                           double* grad_vel_dev, const double* xmid_dev, const double* xdep_dev,
                           void* stream);
/* The same adjoint step inside a sequence of steps through one stationary
 * velocity tree and one concentration tree shape (the in-situ steps of a
 * time loop).  Instead of scattering its node term (tau^2/2 J_v(X*)^T g at
 * every node X) into grad_vel_dev, the step ADDS the per-node weights to
 * node_weights_dev [N][3] (N = L (q+1)^3, zeroed by the caller before the
 * sequence's first step); tbslas_semilag_adjoint_node_term then scatters
 * their sum once, which equals the per-step scatters up to rounding (the
 * scatter is linear and its nodes and velocity leaves do not change).
 * vel_at_nodes_dev [N][3] (optional, NULL to compute it per step): the
 * velocity at the concentration tree's nodes from tbslas_eval_tree_on_nodes,
 * used where the step rebuilds its points (xmid NULL). */
int tbslas_semilag_adjoint_seq(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con,
                               const double* con_coeff_k_dev, int timestep, double dt, int bc,
                               const double* lambda_next_dev, double* lambda_k_dev,
                               double* grad_vel_dev, const double* xmid_dev,
                               const double* xdep_dev, const double* vel_at_nodes_dev,
                               double* node_weights_dev, void* stream);
/* The adjoint step with the forward's Jacobian checkpoint (xmid, xdep and
 * jac from tbslas_semilag_in_situ_ckpt_jac, all required): J_v(X*)^T g is
 * read instead of evaluated, which takes the 5 Nc multiply-adds per target of
 * the velocity-gradient term out of the adjoint pass.  node_weights_dev:
 * as tbslas_semilag_adjoint_seq, or NULL for the step to scatter its own node
 * term into grad_vel_dev (as tbslas_semilag_adjoint).  FP64 sums only.
 * Gradients equal the other modes' up to rounding. */
int tbslas_semilag_adjoint_jac(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con,
                               const double* con_coeff_k_dev, int timestep, double dt, int bc,
                               const double* lambda_next_dev, double* lambda_k_dev,
                               double* grad_vel_dev, const double* xmid_dev,
                               const double* xdep_dev, const double* jac_dev,
                               double* node_weights_dev, void* stream);
/* ADDS the node term of the summed weights to grad_vel_dev [Lv][3][Nc]: the
 * transposed node-grid pass, once per sequence. */
int tbslas_semilag_adjoint_node_term(tbslas_ctx ctx, tbslas_tree vel, tbslas_tree con, int bc,
                                     const double* node_weights_dev, double* grad_vel_dev,
                                     void* stream);

/* ---- batched in-situ SL --------------------------------------------------------- */
/* Many independent in-situ SL problems advanced together: problem i is
 * (vel[i] (dof 3), con[i] (dof 1, same degree), dt[i]); all share nrk and bc.
 * Each step is one node-grid kernel per degree, one persistent kernel per
 * degree band over a flattened worklist of target chunks of every problem
 * (plus, in the double-float mode, the FP64 near-face passes) and one batched
 * refit kernel; results equal a loop of tbslas_semilag_in_situ calls over the
 * problems in the sums mode the context had when the batch was created, bit
 * for bit.  No
 * single-call counterpart in the reference (a driver loops over
 * SolveSemilagInSitu, src/tree/tree_semilag.h:92-135).  The batch keeps
 * pointers to the trees: they must outlive it and keep their shapes (running
 * or tuning a batch whose tree was re-meshed since it was built returns
 * TBSLAS_ERR_INVALID_ARG). */
int tbslas_batch_create(tbslas_ctx ctx, int n_problems, const tbslas_tree* vel,
                        const tbslas_tree* con, const double* dt, int nrk, int bc,
                        tbslas_batch* out);
int tbslas_batch_destroy(tbslas_batch batch);
int tbslas_batch_info(tbslas_batch batch, int64_t* total_targets, int64_t* work_items);
/* Launch parameters: threads per CTA (64/128/256), targets per work chunk,
 * CTAs per SM of the persistent grid. */
int tbslas_batch_set_params(tbslas_batch batch, int block, int targets_per_item,
                            int ctas_per_sm);
int tbslas_batch_get_params(tbslas_batch batch, int* block, int* targets_per_item,
                            int* ctas_per_sm);
/* Times candidate parameter sets on this batch (one step each; the
 * concentration coefficients are saved and restored) and keeps the fastest. */
int tbslas_batch_autotune(tbslas_batch batch, int* block, int* targets_per_item,
                          int* ctas_per_sm);
/* Advance every problem by nsteps steps, timesteps timestep0 .. timestep0 +
 * nsteps - 1.  use_graph != 0: the nsteps-step sequence is captured once as a
 * CUDA graph (re-captured when nsteps or the parameters change) and replayed
 * on `stream`. */
int tbslas_batch_run(tbslas_batch batch, int timestep0, int nsteps, int use_graph, void* stream);

/* ---- tricubic regular grid --------------------------------------------------- */
/* out_dev[n*dof] = tricubic Lagrange interpolant of grid_dev (SoA,
 * vals[x + N(y + N z) + k N^3]) at pts_dev[n*3].  FREESPACE: the reference's
 * clamped stencil on nodes i/(N-1), zero outside [0,1]^3.  PERIODIC: nodes i/N,
 * stencil wrapped mod N.  Replaces tbslas::fast_interp,
 * src/tree/tree_functor.h:89-153.  Requires n_reg >= 4. */
int tbslas_fast_interp(tbslas_ctx ctx, const double* grid_dev, int dof, int n_reg,
                       const double* pts_dev, int64_t n, double* out_dev, int bc, void* stream);
/* One SL step on the grid: every node is a target, RK2 (nrk sub-steps of
 * -dt/nrk) through the 3-component velocity grid, tricubic concentration at
 * the departure points: con_out_dev[N^3].  con_out_dev must not alias
 * con_dev. */
int tbslas_semilag_grid(tbslas_ctx ctx, const double* vel_dev, const double* con_dev,
                        double* con_out_dev, int n_reg, double dt, int nrk, int bc,
                        void* stream);
/* Synchronous host-buffer form: vel_host[3N^3], con_host[N^3] in,
 * con_out_host[N^3] out. */
int tbslas_semilag_grid_host(tbslas_ctx ctx, const double* vel_host, const double* con_host,
                             double* con_out_host, int n_reg, double dt, int nrk, int bc);
/* nsteps grid SL steps through one stationary velocity (a driver's time loop
 * over tbslas_semilag_grid with an unchanged velocity grid): con_dev is the
 * initial concentration, con_out_dev (not aliasing it) the result after
 * nsteps.  The intermediate steps ping-pong through con_out_dev and a
 * context scratch grid.  In the double-float mode the velocity's hi/lo split
 * is made once per call instead of once per step.  No single-call reference
 * counterpart (the reference loops; the velocity is stationary there too,
 * tree_functor.h:808-811). */
int tbslas_semilag_grid_steps(tbslas_ctx ctx, const double* vel_dev, const double* con_dev,
                              double* con_out_dev, int n_reg, double dt, int nsteps, int nrk,
                              int bc, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TBSLAS_GB300_H_ */

// Batched in-situ SL: many independent problems (each a velocity tree and a
// concentration tree of its own size and Chebyshev degree) advanced together.
//
// One persistent kernel per step walks a flattened worklist of target
// chunks across all problems (CTAs take chunks from an atomic counter, so
// problems of uneven size and degree balance across SMs); one batched refit
// kernel per step walks all problems' leaves; before them one kernel
// evaluates each problem's velocity on its concentration nodes (the first RK
// stage, by sum factorisation).  A run of
// nsteps steps is captured once as a CUDA graph and replayed.  Launch
// parameters (threads per CTA, targets per chunk, CTAs per SM) come from the
// autotuner below, which times candidates on the batch itself.
//
// Per target the arithmetic is exactly the single-problem fused step's
// (same device functions), so a batch step reproduces the per-problem loop
// bit for bit.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "host_cheb.h"
#include "internal.h"
#include "batch_kernels.cuh"

namespace tbg {

__global__ void k_set_int(int* p, int v) { *p = v; }

}  // namespace tbg

using namespace tbg;

struct tbslas_batch_s {
  tbslas_ctx ctx = nullptr;
  int device = 0, num_sms = 0;
  int n = 0, nrk = 1, bc = 0;
  bool counted = false;  // counted in the context's live objects
  bool df = false;  // double-float sums (the context's mode at creation), else FP64
  std::vector<BatchProblem> h_probs;
  std::vector<tbslas_tree> trees;   // every velocity and concentration tree
  std::vector<uint64_t> tree_gen;   // their generations when the batch was built
  std::vector<double*> con_coeff;
  std::vector<float2*> con_coeff2;
  std::vector<int64_t> con_coeff_n;
  BatchProblem* d_probs = nullptr;
  RefitJob* d_jobs = nullptr;
  RefitItem* d_ritems = nullptr;
  NodeEvalJob* d_njobs = nullptr;
  NodeEvalItem* d_nitems = nullptr;
  int64_t nitem_begin[TBSLAS_MAX_DEGREE + 2] = {};  // items grouped by degree
  double* d_vn = nullptr;
  int64_t n_ritems = 0;
  int max_q = 0;
  BatchItem* d_items = nullptr;
  int64_t n_items = 0, items_cap = 0;
  int64_t band_begin[kBands + 1] = {};
  double* d_vals = nullptr;
  unsigned long long* d_counters = nullptr;  // per step: kBands chunk counters + 1 fix count
  int counters_cap = 0;
  int64_t* d_fix = nullptr;                  // fix list (total_targets entries)
  int* d_ts0 = nullptr;
  int block = 128, tpi = 256, cps = 4;
  cudaStream_t cap = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_steps = 0;
  int64_t total_targets = 0;
};

namespace {

#define BTRY(expr)                      \
  do {                                  \
    int s_ = (expr);                    \
    if (s_ != TBSLAS_OK) return s_;     \
  } while (0)

int cuda_fail(cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return fail_status(TBSLAS_ERR_CUDA, m.c_str());
}

#define BCUDA(call)                          \
  do {                                       \
    cudaError_t e_ = (call);                 \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

// Chunks of `tpi` consecutive targets grouped by degree band; inside a band
// heavier problems (higher degree) come first so the atomic counter hands
// out the long chunks early.
int build_items(tbslas_batch b) {
  std::vector<int> order(b->n);
  for (int i = 0; i < b->n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int c) { return b->h_probs[a].q > b->h_probs[c].q; });
  std::vector<BatchItem> items;
  for (int band = 0; band < kBands; ++band) {
    b->band_begin[band] = (int64_t)items.size();
    for (int p : order) {
      if (band_of(b->h_probs[p].q) != band) continue;
      for (int64_t s = 0; s < b->h_probs[p].n_targets; s += b->tpi)
        items.push_back(
            BatchItem{s, p, (int32_t)std::min<int64_t>(b->tpi, b->h_probs[p].n_targets - s)});
    }
  }
  b->band_begin[kBands] = (int64_t)items.size();
  if ((int64_t)items.size() > b->items_cap) {
    if (b->d_items) BCUDA(cudaFree(b->d_items));
    b->d_items = nullptr;
    BCUDA(cudaMalloc(&b->d_items, items.size() * sizeof(BatchItem)));
    b->items_cap = (int64_t)items.size();
  }
  BCUDA(cudaMemcpy(b->d_items, items.data(), items.size() * sizeof(BatchItem),
                   cudaMemcpyHostToDevice));
  b->n_items = (int64_t)items.size();
  return TBSLAS_OK;
}

int enqueue_steps(tbslas_batch b, int nsteps, cudaStream_t s) {
  constexpr int kPer = kBands + 1;
  BCUDA(cudaMemsetAsync(b->d_counters, 0, sizeof(unsigned long long) * nsteps * kPer, s));
  const int grid = b->num_sms * b->cps;
  for (int i = 0; i < nsteps; ++i) {
    unsigned long long* fix_count = b->d_counters + (int64_t)i * kPer + kBands;
    for (int q = 0; q <= TBSLAS_MAX_DEGREE; ++q) {
      const int64_t n = b->nitem_begin[q + 1] - b->nitem_begin[q];
      if (n > 0)
        launch_batch_eval_on_nodes(b->d_njobs, b->d_nitems + b->nitem_begin[q], n, q, q, b->bc, s);
    }
    for (int band = 0; band < kBands; ++band) {
      const int64_t n = b->band_begin[band + 1] - b->band_begin[band];
      if (n == 0) continue;
      BatchLaunch a{b->d_probs, b->d_items + b->band_begin[band], n,
                    b->d_counters + (int64_t)i * kPer + band, b->d_ts0, i, b->bc,
                    b->d_fix, fix_count};
      launch_batch_band(band, a, (int)std::min<int64_t>(grid, n), b->block, s,
                        b->df ? kBandStepDF : kBandStepFP64);
    }
    for (int band = 0; band < kBands && b->df; ++band) {
      if (b->band_begin[band + 1] == b->band_begin[band]) continue;
      BatchLaunch a{b->d_probs, nullptr, 0, nullptr, b->d_ts0, i, b->bc, b->d_fix, fix_count};
      launch_batch_band(band, a, b->num_sms * 4, 128, s, kBandFix);
    }
    launch_batch_refit(b->d_jobs, b->d_ritems, b->n_ritems, b->max_q, b->df, s);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "batch step launch");
  return TBSLAS_OK;
}

void drop_graph(tbslas_batch b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->graph_steps = 0;
}

int ensure_counters(tbslas_batch b, int nsteps) {
  if (nsteps > b->counters_cap) {
    if (b->d_counters) BCUDA(cudaFree(b->d_counters));
    b->d_counters = nullptr;
    BCUDA(cudaMalloc(&b->d_counters, sizeof(unsigned long long) * nsteps * (kBands + 1)));
    b->counters_cap = nsteps;
    drop_graph(b);
  }
  return TBSLAS_OK;
}

int run(tbslas_batch b, int timestep0, int nsteps, bool use_graph, cudaStream_t s) {
  BTRY(ensure_counters(b, nsteps));
  if (use_graph && (!b->exec || b->graph_steps != nsteps)) {
    drop_graph(b);
    BCUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
    int st = enqueue_steps(b, nsteps, b->cap);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->cap, &g);
    if (st != TBSLAS_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    b->graph_steps = nsteps;
  }
  k_set_int<<<1, 1, 0, s>>>(b->d_ts0, timestep0);
  if (use_graph) {
    BCUDA(cudaGraphLaunch(b->exec, s));
    return TBSLAS_OK;
  }
  return enqueue_steps(b, nsteps, s);
}

bool params_ok(int block, int tpi, int cps) {
  return (block == 64 || block == 128 || block == 256) && tpi >= 1 && tpi <= (1 << 20) &&
         cps >= 1 && cps <= 32;
}

}  // namespace

extern "C" {

int tbslas_batch_create(tbslas_ctx ctx, int n, const tbslas_tree* vel, const tbslas_tree* con,
                        const double* dt, int nrk, int bc, tbslas_batch* out) {
  if (!out) return fail_status(TBSLAS_ERR_INVALID_ARG, "null output pointer");
  *out = nullptr;
  if (!ctx || n < 1 || !vel || !con || !dt)
    return fail_status(TBSLAS_ERR_INVALID_ARG, "null context/arrays or no problems");
  if (nrk < 1) return fail_status(TBSLAS_ERR_INVALID_ARG, "nrk < 1");
  if (bc != TBSLAS_BC_FREESPACE && bc != TBSLAS_BC_PERIODIC)
    return fail_status(TBSLAS_ERR_INVALID_ARG, "invalid boundary condition");
  DeviceRestore restore;
  tbslas_batch b = new tbslas_batch_s();
  b->ctx = ctx;
  b->n = n;
  b->nrk = nrk;
  b->bc = bc;
  int st = ctx_info(ctx, &b->device, &b->num_sms);
  if (st != TBSLAS_OK) {
    delete b;
    return st;
  }
  b->df = ctx_sums(ctx) == TBSLAS_SUMS_DOUBLE_FLOAT;
  cudaSetDevice(b->device);
  std::vector<RefitJob> jobs;
  std::vector<RefitItem> ritems;
  std::vector<NodeEvalJob> njobs;
  std::vector<NodeEvalItem> nitems;
  int64_t off = 0;
  for (int i = 0; i < n && st == TBSLAS_OK; ++i) {
    BatchProblem p;
    tbslas_ctx cv = nullptr, cc = nullptr;
    st = tree_view(vel[i], &p.vel, &cv);
    if (st == TBSLAS_OK) st = tree_view(con[i], &p.con, &cc);
    if (st != TBSLAS_OK) break;
    for (tbslas_tree tr : {vel[i], con[i]}) {
      b->trees.push_back(tr);
      b->tree_gen.push_back(tree_generation(tr));
    }
    if (cv != ctx || cc != ctx) {
      st = fail_status(TBSLAS_ERR_INVALID_ARG, "batch trees belong to another context");
      break;
    }
    if (p.vel.dof != 3 || p.con.dof != 1 || p.vel.q != p.con.q) {
      st = fail_status(TBSLAS_ERR_UNSUPPORTED,
                       "batched problems need a dof-3 velocity and a dof-1 concentration "
                       "tree of the same degree");
      break;
    }
    if (!(dt[i] == dt[i] && dt[i] - dt[i] == 0.0)) {
      st = fail_status(TBSLAS_ERR_INVALID_ARG, "dt is not finite");
      break;
    }
    p.q = p.con.q;
    p.nrk = nrk;
    {
      std::vector<double> x = cheb_nodes_1d(p.q);
      std::memset(&p.nodes, 0, sizeof(p.nodes));
      for (int k = 0; k <= p.q; ++k) p.nodes.x[k] = x[k];
    }
    p.dt = dt[i];
    const int d = p.q + 1;
    const int np = d * d * d;
    p.n_targets = p.con.L * np;
    p.vals = reinterpret_cast<double*>(off);  // offset; rebased below
    off += p.n_targets;
    b->h_probs.push_back(p);
    double* coeff = nullptr;
    int64_t ncf = 0;
    tree_coeff(con[i], &coeff, &ncf);
    b->con_coeff.push_back(coeff);
    b->con_coeff_n.push_back(ncf);
    {
      float2* c2 = nullptr;
      tree_coeff2(con[i], &c2);
      b->con_coeff2.push_back(c2);
    }
    const double* F = nullptr;
    st = ctx_F(ctx, p.q, &F);
    if (st != TBSLAS_OK) break;
    float2* coeff2 = nullptr;
    tree_coeff2(con[i], &coeff2);
    jobs.push_back(RefitJob{nullptr, F, coeff, coeff2, ctx_err(ctx), p.con.L, p.con.stride, p.q, 1});
    b->max_q = std::max(b->max_q, p.q);
    for (int64_t r = 0; r < p.con.L; ++r) ritems.push_back(RefitItem{i, 0, r});
    NodeEvalJob nj;
    nj.src = p.vel;
    nj.dst = p.con;
    nj.nodes = p.nodes;
    nj.out = nullptr;  // rebased below
    nj.face = tree_face_map(con[i], bc, nullptr);  // built on the legacy stream; synchronised below
    b->h_probs[i].face = nj.face;  // the step reads shared face nodes through it
    njobs.push_back(nj);
    for (int64_t r = 0; r < p.con.L; ++r) nitems.push_back(NodeEvalItem{i, 0, r});
  }
  cudaError_t e = cudaSuccess;
  if (st == TBSLAS_OK) {
    e = cudaDeviceSynchronize();  // the face maps are ready before any run
    if (e != cudaSuccess) st = cuda_fail(e, "batch face maps");
  }
  if (st == TBSLAS_OK) {
    b->total_targets = off;
    e = cudaMalloc(&b->d_vals, sizeof(double) * std::max<int64_t>(off, 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_vn, sizeof(double) * 3 * std::max<int64_t>(off, 1));
    if (e == cudaSuccess) {
      for (size_t i = 0; i < b->h_probs.size(); ++i) {
        const int64_t o = reinterpret_cast<int64_t>(b->h_probs[i].vals);
        b->h_probs[i].vals = b->d_vals + o;
        b->h_probs[i].vn = b->d_vn + 3 * o;
        jobs[i].vals = b->h_probs[i].vals;
        njobs[i].out = b->d_vn + 3 * o;
      }
      e = cudaMalloc(&b->d_probs, sizeof(BatchProblem) * n);
    }
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_probs, b->h_probs.data(), sizeof(BatchProblem) * n,
                     cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_jobs, sizeof(RefitJob) * n);
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_jobs, jobs.data(), sizeof(RefitJob) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_ritems, sizeof(RefitItem) * ritems.size());
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_ritems, ritems.data(), sizeof(RefitItem) * ritems.size(),
                     cudaMemcpyHostToDevice);
    b->n_ritems = (int64_t)ritems.size();
    if (e == cudaSuccess) e = cudaMalloc(&b->d_njobs, sizeof(NodeEvalJob) * n);
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_njobs, njobs.data(), sizeof(NodeEvalJob) * n, cudaMemcpyHostToDevice);
    {
      // group the items by degree (one launch per degree)
      std::stable_sort(nitems.begin(), nitems.end(), [&](const NodeEvalItem& x, const NodeEvalItem& y) {
        return b->h_probs[x.job].q < b->h_probs[y.job].q;
      });
      int64_t k = 0;
      for (int q = 0; q <= TBSLAS_MAX_DEGREE + 1; ++q) {
        while (k < (int64_t)nitems.size() && b->h_probs[nitems[k].job].q < q) ++k;
        b->nitem_begin[q] = k;
      }
    }
    if (e == cudaSuccess) e = cudaMalloc(&b->d_nitems, sizeof(NodeEvalItem) * nitems.size());
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_nitems, nitems.data(), sizeof(NodeEvalItem) * nitems.size(),
                     cudaMemcpyHostToDevice);

    if (e == cudaSuccess) e = cudaMalloc(&b->d_ts0, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_fix, sizeof(int64_t) * std::max<int64_t>(off, 1));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) st = cuda_fail(e, "batch setup");
    if (st == TBSLAS_OK) st = build_items(b);
  }
  if (st != TBSLAS_OK) {
    tbslas_batch_destroy(b);
    return st;
  }
  b->counted = true;
  ctx_count_object(ctx, +1);
  *out = b;
  return TBSLAS_OK;
}

int tbslas_batch_destroy(tbslas_batch b) {
  if (!b) return TBSLAS_OK;
  DeviceRestore restore;
  if (b->counted) ctx_count_object(b->ctx, -1);
  cudaSetDevice(b->device);
  cudaDeviceSynchronize();
  drop_graph(b);
  if (b->cap) cudaStreamDestroy(b->cap);
  for (void* p : {(void*)b->d_probs, (void*)b->d_jobs, (void*)b->d_ritems, (void*)b->d_items,
                  (void*)b->d_vals, (void*)b->d_counters, (void*)b->d_ts0, (void*)b->d_fix,
                  (void*)b->d_njobs, (void*)b->d_nitems, (void*)b->d_vn})
    if (p) cudaFree(p);
  delete b;
  return TBSLAS_OK;
}

int tbslas_batch_info(tbslas_batch b, int64_t* total_targets, int64_t* work_items) {
  if (!b) return fail_status(TBSLAS_ERR_INVALID_ARG, "null batch");
  if (total_targets) *total_targets = b->total_targets;
  if (work_items) *work_items = b->n_items;
  return TBSLAS_OK;
}

int tbslas_batch_set_params(tbslas_batch b, int block, int targets_per_item, int ctas_per_sm) {
  if (!b) return fail_status(TBSLAS_ERR_INVALID_ARG, "null batch");
  if (!params_ok(block, targets_per_item, ctas_per_sm))
    return fail_status(TBSLAS_ERR_INVALID_ARG,
                       "block must be 64/128/256, targets_per_item 1..2^20, ctas_per_sm 1..32");
  DeviceRestore restore;
  cudaSetDevice(b->device);
  b->block = block;
  b->cps = ctas_per_sm;
  if (targets_per_item != b->tpi) {
    b->tpi = targets_per_item;
    BTRY(build_items(b));
  }
  drop_graph(b);
  return TBSLAS_OK;
}

int tbslas_batch_get_params(tbslas_batch b, int* block, int* targets_per_item, int* ctas_per_sm) {
  if (!b) return fail_status(TBSLAS_ERR_INVALID_ARG, "null batch");
  if (block) *block = b->block;
  if (targets_per_item) *targets_per_item = b->tpi;
  if (ctas_per_sm) *ctas_per_sm = b->cps;
  return TBSLAS_OK;
}

// The batch holds its trees' device arrays: a tree re-meshed since the batch
// was built invalidates it.
static int check_generations(const tbslas_batch b) {
  for (size_t i = 0; i < b->trees.size(); ++i)
    if (tree_generation(b->trees[i]) != b->tree_gen[i])
      return fail_status(TBSLAS_ERR_INVALID_ARG,
                         "a tree of the batch was re-meshed after the batch was built; "
                         "rebuild the batch");
  return TBSLAS_OK;
}

int tbslas_batch_run(tbslas_batch b, int timestep0, int nsteps, int use_graph, void* stream) {
  if (!b) return fail_status(TBSLAS_ERR_INVALID_ARG, "null batch");
  if (nsteps < 0) return fail_status(TBSLAS_ERR_INVALID_ARG, "negative step count");
  if (check_generations(b) != TBSLAS_OK) return TBSLAS_ERR_INVALID_ARG;
  if (nsteps == 0) return TBSLAS_OK;
  DeviceRestore restore;
  BCUDA(cudaSetDevice(b->device));
  return run(b, timestep0, nsteps, use_graph != 0, (cudaStream_t)stream);
}

int tbslas_batch_autotune(tbslas_batch b, int* block, int* targets_per_item, int* ctas_per_sm) {
  if (!b) return fail_status(TBSLAS_ERR_INVALID_ARG, "null batch");
  if (check_generations(b) != TBSLAS_OK) return TBSLAS_ERR_INVALID_ARG;
  DeviceRestore restore;
  BCUDA(cudaSetDevice(b->device));
  BCUDA(cudaDeviceSynchronize());
  // Save every concentration tree: each trial step overwrites them.
  int64_t tot = 0;
  for (int64_t c : b->con_coeff_n) tot += c;
  double* backup = nullptr;
  BCUDA(cudaMalloc(&backup, sizeof(double) * std::max<int64_t>(tot, 1)));
  cudaStream_t s = b->cap;
  auto copy_all = [&](bool save) -> cudaError_t {
    int64_t o = 0;
    for (size_t i = 0; i < b->con_coeff.size(); ++i) {
      const size_t bytes = sizeof(double) * b->con_coeff_n[i];
      cudaError_t e = save ? cudaMemcpyAsync(backup + o, b->con_coeff[i], bytes,
                                             cudaMemcpyDeviceToDevice, s)
                           : cudaMemcpyAsync(b->con_coeff[i], backup + o, bytes,
                                             cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return e;
      if (!save)
        launch_split(b->con_coeff[i], b->con_coeff2[i], b->con_coeff_n[i], ctx_err(b->ctx), s);
      o += b->con_coeff_n[i];
    }
    return cudaSuccess;
  };
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int st = TBSLAS_OK;
  cudaError_t ce = copy_all(true);
  const int blocks[] = {64, 128, 256};
  const int mult[] = {1, 4, 16};
  const int cpss[] = {2, 4, 8};
  float best = 1e30f;
  int bb = b->block, bt = b->tpi, bc = b->cps;
  for (int blk : blocks)
    for (int m : mult)
      for (int cps : cpss) {
        if (st != TBSLAS_OK || ce != cudaSuccess) break;
        b->block = blk;
        b->cps = cps;
        if (b->tpi != blk * m) {
          b->tpi = blk * m;
          st = build_items(b);
          if (st != TBSLAS_OK) break;
        }
        float best_trial = 1e30f;
        for (int rep = 0; rep < 2 && st == TBSLAS_OK; ++rep) {
          cudaEventRecord(e0, s);
          st = run(b, 1, 1, false, s);
          cudaEventRecord(e1, s);
          ce = copy_all(false);
          cudaEventSynchronize(e1);
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e0, e1);
          if (rep > 0) best_trial = std::min(best_trial, ms);
        }
        if (best_trial < best) {
          best = best_trial;
          bb = blk;
          bt = blk * m;
          bc = cps;
        }
      }
  cudaStreamSynchronize(s);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(backup);
  if (st != TBSLAS_OK) return st;
  if (ce != cudaSuccess) return cuda_fail(ce, "autotune restore");
  b->block = bb;
  b->cps = bc;
  b->tpi = bt;
  BTRY(build_items(b));
  drop_graph(b);
  if (block) *block = bb;
  if (targets_per_item) *targets_per_item = bt;
  if (ctas_per_sm) *ctas_per_sm = bc;
  return TBSLAS_OK;
}

}  // extern "C"

#!/usr/bin/env python
"""Throughput of the semi-Lagrangian advection step on GB300.

One step = one in-situ SL step of the whole concentration tree: every
Chebyshev node is backtraced (RK2) through the velocity tree, the
concentration is evaluated at the departure points and every leaf is refitted
(SolveSemilagInSitu, src/tree/tree_semilag.h:92-135).  Metric: departure
points per second.  Default workload: the adaptive q=14 configuration
(Taylor-Green velocity, 4 Gaussians, tolerance 1e-6, depths 3..8, CFL 1).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
  python bench.py --impl reference ...   # the reference algorithm on the host cores

With N > 1 (torchrun, one rank per GPU) every rank advances its own replica
(the path is replicated, not partitioned: no collective on the data path);
value = all ranks' departure points / the slowest rank's time.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "SL departure-points/s on 1 GB300 at ≤1e-10 rel err; batched vs plain; adj/fwd"
UNIT = "departure points/s"
L2_FLUSH_BYTES = 256 << 20


def flops_per_point_tree(q, nrk=1):
    """Algorithmic FLOPs of one SL step per departure point, counted as the
    reference counts them: per evaluation 3*d*3 + 2*Nc*dof
    (src/tree/tree_functor.h:389-394), 2*3*3 per RK2 sub-step
    (src/semilag/traj.inc:44), and 2*Nc per node for the refit GEMM
    (src/tree/tree_utils.h:538-551).  Returns (step total, fused-kernel part)."""
    d = q + 1
    nc = d * (d + 1) * (d + 2) // 6
    ev = lambda dof: 9 * d + 2 * nc * dof
    kernel = nrk * (2 * ev(3) + 18) + ev(1)
    return kernel + 2 * nc, kernel


# FP32 instructions per double-float multiply-accumulate (df_fma_acc): one
# FMUL and three FFMA form the exact product, eight FADD/FSUB add it to the
# running sum (TwoSum) and fold the errors into the low word.
DF_FP32_INSTR_PER_MAC = 12


def df_macs_per_point_tree(q, nrk=1):
    """Double-float multiply-accumulates per departure point of the fused
    step: the Nc-term sums of 2*nrk three-component velocity evaluations and
    one concentration evaluation."""
    d = q + 1
    nc = d * (d + 1) * (d + 2) // 6
    return (2 * 3 * nrk + 1) * nc


def bytes_per_point_tree(q, vel_leaves, con_leaves):
    """Compulsory HBM bytes per departure point: each velocity and
    concentration coefficient read once, one node value written and read back
    by the refit, each new coefficient written once."""
    d = q + 1
    nc = d * (d + 1) * (d + 2) // 6
    npt = con_leaves * d ** 3
    coeff_reads = 8.0 * nc * (3 * vel_leaves + con_leaves) / npt
    kernel = coeff_reads + 8.0
    step = kernel + 8.0 + 8.0 * nc * con_leaves / npt
    return step, kernel


# FLOPs per point of the grid step: midpoint velocity (weights 3x12 + 3
# components x 144) + departure concentration (36 + 144) + RK updates 18; the
# first velocity sits on a node (exact read).
GRID_FLOPS_PER_POINT = (36 + 3 * 144) + (36 + 144) + 18
GRID_BYTES_PER_POINT = 40  # 3 velocity + 1 concentration read, 1 written (FP64)
# double-float multiply-adds per node of the periodic grid step: 84 per
# component (64 + 16 + 4) at the midpoint (3 components) and the departure
# point (1)
GRID_DF_MACS_PER_POINT = 4 * 84


# ---------------------------------------------------------------------------
def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def aggregate(points, seconds, world):
    """Whole-job throughput: sum of points over ranks / max time over ranks."""
    if world == 1:
        return points, seconds
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    p = torch.tensor([float(points)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(p, op=dist.ReduceOp.SUM)
    return p.item(), t.item()


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        if self.path and os.path.exists(self.path):
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        try:
            return json.load(open(path)), "measured"
        except ValueError:
            pass
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


_NOMINAL = {}


def fp64_nominal_tflops():
    """The FP64 pipe's nominal rate: 2 FP64 FMA per clock per SM x 2 FLOP x
    SMs x the GPU's maximum SM clock (nvidia-smi; the bench rejects runs whose
    clock sat below it).  Reported beside the measured FMA probe, which
    reaches ~95 % of it: a probe's own FMAs are limited by operand fetch."""
    if "v" not in _NOMINAL:
        import torch
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        mhz = None
        try:
            idx = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or "0"
            out = subprocess.run(["nvidia-smi", "-i", idx, "--query-gpu=clocks.max.sm",
                                  "--format=csv,noheader,nounits"], capture_output=True,
                                 text=True, timeout=20).stdout.strip().splitlines()
            mhz = float(out[0]) if out else None
        except (OSError, ValueError, subprocess.SubprocessError):
            mhz = None
        _NOMINAL["v"] = 4.0 * sms * mhz * 1e6 / 1e12 if mhz else None
    return _NOMINAL["v"]


def nominal_fields(achieved):
    nom = fp64_nominal_tflops()
    return {"nominal_peak": nom, "frac_of_nominal": achieved / nom if nom else None,
            "nominal_source": "2 FP64 FMA per clock per SM x SMs x maximum SM clock"}


# ---------------------------------------------------------------------------
def cpu_baseline_tree(wl, budget_s=12.0, steps=1):
    """The oracle (OpenMP C++ restatement of the reference CPU path) on a
    bounded sample of the workload: the targets of the first k leaves of the
    concentration tree, k sized for ~budget_s of CPU work."""
    from oracle import oracle as ora
    cores = ora.num_threads()
    vel = dict(anchor=wl.va, depth=wl.vd, q=wl.q, dof=3, coeff=wl.vc)
    con = dict(anchor=wl.ca, depth=wl.cd, q=wl.q, dof=1, coeff=wl.cc)
    ora.pt2coeff(wl.q)
    npl = (wl.q + 1) ** 3
    probe = min(4, len(wl.cd))
    t0 = time.perf_counter()
    ora.semilag_in_situ(vel, con, 1, wl.dt, 1, bool(wl.bc), leaf_begin=0, leaf_end=probe)
    per_leaf = max((time.perf_counter() - t0) / probe, 1e-6)
    k = int(max(probe, min(len(wl.cd), budget_s / per_leaf / max(steps, 1))))
    out = None
    t0 = time.perf_counter()
    for s in range(steps):
        out = ora.semilag_in_situ(vel, con, 1, wl.dt, 1, bool(wl.bc), leaf_begin=0, leaf_end=k)
    sec = time.perf_counter() - t0
    return {"value": k * npl * steps / sec, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d of %d concentration leaves (%d departure points) x %d step(s), "
                      "one SL step from the initial state" % (k, len(wl.cd), k * npl, steps),
            "seconds": sec}, out, k


def cpu_baseline_batched(wl, budget_s=10.0):
    """The oracle on a bounded sample of the batched workload: one in-situ
    step of the first leaves of each problem in turn (every problem's
    degree), ~budget_s of CPU work."""
    from oracle import oracle as ora
    cores = ora.num_threads()
    pts, sec, used = 0, 0.0, 0
    for p in wl.problems:
        vel = dict(anchor=p["va"], depth=p["vd"], q=p["q"], dof=3, coeff=p["vc"])
        con = dict(anchor=p["ca"], depth=p["cd"], q=p["q"], dof=1, coeff=p["cc"])
        ora.pt2coeff(p["q"])
        k = min(len(p["cd"]), 8)
        t0 = time.perf_counter()
        ora.semilag_in_situ(vel, con, 1, p["dt"], 1, bool(wl.bc), leaf_begin=0, leaf_end=k)
        sec += time.perf_counter() - t0
        pts += k * (p["q"] + 1) ** 3
        used += 1
        if sec > budget_s:
            break
    return {"value": pts / sec, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "first %s leaves of %d of %d problems (%d departure points), one SL "
                      "step each" % ("8", used, len(wl.problems), pts), "seconds": sec}


def cpu_baseline_grid(wl, budget_s=12.0):
    from oracle import oracle as ora
    cores = ora.num_threads()
    probe = 20000
    t0 = time.perf_counter()
    ora.semilag_grid(wl.vel, wl.con, wl.n, wl.dt, 1, True, 0, probe)
    per = (time.perf_counter() - t0) / probe
    k = int(min(wl.n ** 3, max(probe, budget_s / per)))
    t0 = time.perf_counter()
    out = ora.semilag_grid(wl.vel, wl.con, wl.n, wl.dt, 1, True, 0, k)
    sec = time.perf_counter() - t0
    return {"value": k / sec, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "first %d of %d grid nodes, one SL step" % (k, wl.n ** 3),
            "seconds": sec}, out, k


# ---------------------------------------------------------------------------
def oracle_workload(name):
    """The workload built with the oracle's own Chebyshev nodes and
    pseudo-inverse (the reference arm loads nothing of the library under
    test)."""
    from oracle import oracle as ora
    from tbslas_gb300 import trees
    from tbslas_gb300.workloads import make

    def nodes(q):
        return ora.collect_grid_points(np.zeros((1, 3)), np.zeros(1, dtype=np.int32), q)
    with trees.host_math(trees.HostMath(nodes=nodes, pt2coeff=ora.pt2coeff)):
        return make(name)


def run_reference(args, name):
    """--impl reference: the reference algorithm (oracle port, all host
    threads) timed on bounded samples of the same workload (a name, built
    with the oracle's own set-up math, or a workload object), K steps."""
    wl = oracle_workload(name) if isinstance(name, str) else name
    total_budget = 150.0
    per_step = total_budget / max(1, args.steps + args.warmup)
    timed_steps = args.steps
    unit = UNIT
    if hasattr(wl, "construct"):
        # the oracle's construction of both trees (ConstructTree's rule) per step
        import tbslas_gb300 as tb
        from oracle import construct as oc
        from oracle import oracle as ora
        tol, lo, hi = wl.construct
        fields_ = [tb.Field.gaussians(wl.blobs.centres, wl.blobs.sigmas), tb.Field.taylor_green()]
        nodes = (len(wl.cd) + len(wl.vd)) * (wl.q + 1) ** 3
        secs, pts, n = 0.0, 0, 0
        t_start = time.perf_counter()
        for i in range(args.warmup + args.steps):
            if i > args.warmup and time.perf_counter() - t_start > total_budget:
                break
            t0 = time.perf_counter()
            for f in fields_:
                oc.construct(f.kind, f.n, f.params, wl.q, tol, lo, hi)
            if i >= args.warmup:
                secs += time.perf_counter() - t0
                pts += nodes
                n += 1
        unit = "Chebyshev nodes of the final trees fitted per second (tree construction)"
        cb = {"unit": unit, "cores": ora.num_threads(), "kind": "port",
              "sample": "the oracle's construction of both trees, %d of %d steps" % (n, args.steps)}
        timed_steps = max(n, 1)
    elif hasattr(wl, "remesh"):
        # the reference driver's loop on the CPU: oracle step + oracle re-mesh, advancing
        # the state, as many of the K steps as fit the time budget
        from oracle import oracle as ora
        from oracle import remesh as rm
        tol, lo, hi = wl.remesh
        npl = (wl.q + 1) ** 3
        vel = dict(anchor=wl.va, depth=wl.vd, q=wl.q, dof=3, coeff=wl.vc)
        a, d, c = wl.ca, wl.cd, wl.cc
        ora.pt2coeff(wl.q)
        secs, pts, n = 0.0, 0, 0
        t_start = time.perf_counter()
        for i in range(args.warmup + args.steps):
            if i > args.warmup and time.perf_counter() - t_start > total_budget:
                break
            t0 = time.perf_counter()
            L = d.size
            c1 = ora.semilag_in_situ(vel, dict(anchor=a, depth=d, q=wl.q, dof=1, coeff=c), i + 1,
                                     wl.dt, 1, bool(wl.bc))
            a, d, c = rm.remesh(a, d, wl.q, c1, tol, lo, hi, bool(wl.bc))
            if i >= args.warmup:
                secs += time.perf_counter() - t0
                pts += L * npl
                n += 1
        cb = {"unit": UNIT, "cores": ora.num_threads(), "kind": "port",
              "sample": "%d of the %d timed steps (step + re-mesh, whole tree, state advanced; "
                        "the rest did not fit the %.0f s budget)" % (n, args.steps, total_budget)
              if n < args.steps else "all %d timed steps (step + re-mesh, whole tree)" % n}
        timed_steps = max(n, 1)
    elif hasattr(wl, "vcs"):
        for _ in range(args.warmup):
            cpu_baseline_tv(wl, per_step)
        secs, pts = 0.0, 0
        for _ in range(args.steps):
            cb, _, k = cpu_baseline_tv(wl, per_step)
            secs += cb["seconds"]
            pts += k * (wl.q + 1) ** 3
        cb["sample"] = "per step: " + cb["sample"]
    elif hasattr(wl, "c_prev"):
        for _ in range(args.warmup):
            cpu_baseline_bdf2(wl, per_step)
        secs, pts = 0.0, 0
        for _ in range(args.steps):
            cb, _, k = cpu_baseline_bdf2(wl, per_step)
            secs += cb["seconds"]
            pts += 2 * k * (wl.q + 1) ** 3
        cb["sample"] = "per step: " + cb["sample"]
    elif isinstance(wl, GridWorkloadType()):
        for _ in range(args.warmup):
            cpu_baseline_grid(wl, per_step)
        vals, secs, pts = [], 0.0, 0
        for _ in range(args.steps):
            cb, _, k = cpu_baseline_grid(wl, per_step)
            secs += cb["seconds"]
            pts += k
        cb["sample"] = "per step: " + cb["sample"]
    else:
        note = None
        tw = wl
        if hasattr(wl, "problems"):
            # batched: the reference advances the problems one by one; its
            # CPU path is timed on the problems in turn (a bounded sample each)
            note = "batched: the reference's per-problem CPU step, problems in turn"
        elif not hasattr(wl, "va"):
            # adjoint: the reference has no adjoint; its forward SL step on the
            # same tree and fields is timed
            tw = _TreeView(wl.a, wl.d, wl.vc, wl.a, wl.d, wl.c0, wl.q, wl.dt, wl.bc)
            note = "adjoint: the reference has no adjoint; its forward SL step is timed"
        for i in range(args.warmup):
            cpu_baseline_tree(_pick(tw, i), per_step)
        secs, pts = 0.0, 0
        for i in range(args.steps):
            t = _pick(tw, i)
            cb, _, k = cpu_baseline_tree(t, per_step)
            secs += cb["seconds"]
            pts += k * (t.q + 1) ** 3
        cb["sample"] = "per step: " + cb["sample"] + ("; " + note if note else "")
    value = pts / secs
    cb["value"] = value
    cb.pop("seconds", None)
    line = {"metric": METRIC, "value": value, "unit": unit, "impl": "reference", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / timed_steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded analytic fields)", "config": describe_config(wl),
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


class _TreeView:
    """The tree-workload fields cpu_baseline_tree reads."""

    def __init__(self, va, vd, vc, ca, cd, cc, q, dt, bc):
        self.va, self.vd, self.vc, self.ca, self.cd, self.cc = va, vd, vc, ca, cd, cc
        self.q, self.dt, self.bc = q, dt, bc


def _pick(wl, i):
    """A batch's i-th problem (cyclically) as a tree workload; else wl."""
    if not hasattr(wl, "problems"):
        return wl
    p = wl.problems[i % len(wl.problems)]
    return _TreeView(p["va"], p["vd"], p["vc"], p["ca"], p["cd"], p["cc"], p["q"], p["dt"],
                     wl.bc)


def GridWorkloadType():
    from tbslas_gb300.workloads import GridWorkload
    return GridWorkload


# ---------------------------------------------------------------------------
def fused_flops_per_point_tree(q, nrk=1):
    """Algorithmic FLOPs per target of the fused step kernel, counted as the
    reference counts an evaluation (3*d*3 + 2*Nc*dof, src/tree/tree_functor.h:
    389-394) and an RK2 update (2*3 per sub-step and stage, src/semilag/
    traj.inc:44): the 2*nrk - 1 velocity evaluations after the first (the
    first, at the target node itself, is the node-grid kernel's) and the
    concentration at the departure point."""
    d = q + 1
    nc = d * (d + 1) * (d + 2) // 6
    ev = lambda dof: 9 * d + 2 * nc * dof
    return (2 * nrk - 1) * ev(3) + 18 * nrk + ev(1)


def _traffic(wl_name, kernel):
    """DRAM bytes per launch of `kernel` on workload `wl_name` from one ncu
    capture (profiles/traffic.json), or None."""
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(tpath):
        return None
    return json.load(open(tpath)).get(wl_name, {}).get(kernel)


def fp64_roofline(ctx, kernel, flops_per_point, points_per_launch, prof, name, steps,
                  counting):
    """roofline object of an FP64-pipe-bound kernel: its algorithmic FLOPs per
    launch over its mean launch time (the profiler's brackets named `name`),
    against the FP64 FMA peak measured in this run."""
    groups, _, kms = prof.get(name, (0, 0, 0.0))
    launch_ms = kms / max(groups, 1)
    peak = ctx.fp64_fma_peak() / 1e12
    achieved = flops_per_point * points_per_launch / (max(launch_ms, 1e-9) * 1e-3) / 1e12
    return {"kernel": kernel, "bound": "fp64", "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_source": "FP64 FMA throughput measured in this run (tbslas_fp64_fma_peak); "
                           "MEASURED_PEAKS.json holds no FP64 figure",
            "algorithmic_flops_per_point": flops_per_point, "counting": counting,
            "launch_ms": launch_ms, "traffic": None,
            "kernels_ms_per_step": {k: v[2] / steps for k, v in prof.items()},
            **nominal_fields(achieved)}


def run_gpu(args, wl, rank, world, local_rank):
    """The plain step (tree or grid workload) in the library's default FP64
    arithmetic: K timed steps with inputs resident, a profiled pass for the
    per-kernel split, the same step in the opt-in double-float mode, an
    end-to-end pass through the host-buffer entry point, and (rank 0, N = 1)
    the oracle on a bounded sample.  Returns the bench line on rank 0."""
    import torch
    import tbslas_gb300 as tb

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = tb.Context(local_rank)
    assert ctx.sums == tb.SUMS_FP64
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    is_grid = isinstance(wl, GridWorkloadType())

    if is_grid:
        N = wl.n
        vel = torch.from_numpy(wl.vel).to(dev)
        con0 = torch.from_numpy(wl.con).to(dev)
        bufs = [con0.clone(), torch.empty_like(con0)]

        def step(i, b=bufs):
            tb.semilag_grid(ctx, vel, b[i % 2], N, wl.dt, 1, wl.bc, out=b[(i + 1) % 2])

        def result(b=bufs):
            return b[1].cpu().numpy().ravel()
        flops_kernel = GRID_FLOPS_PER_POINT
        bytes_kernel = GRID_BYTES_PER_POINT
        dominant = "semilag_grid"
    else:
        tv = tb.Tree(ctx, wl.va, wl.vd, wl.q, 3, wl.vc)
        tc = tb.Tree(ctx, wl.ca, wl.cd, wl.q, 1, wl.cc)
        vf = tb.NodeFieldFunctor(tv, wl.bc)

        def step(i, t=tc):
            tb.solve_semilag_in_situ(vf, t, i + 1, wl.dt, 1)

        def result(t=tc):
            return t.get_coeffs()
        flops_kernel = fused_flops_per_point_tree(wl.q)
        _, bytes_kernel = bytes_per_point_tree(wl.q, len(wl.vd), len(wl.cd))
        dominant = "semilag_tree"
    kernel_points = wl.points_per_step

    def timed_steps(k, first_step, stepf):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(k):
            flush.fill_(float(i))  # L2 flush: the step's working set fits in L2
            stepf(first_step + i)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    def profiled(k, first_step, stepf):
        ctx.profile(True)
        ctx.profile_reset()
        for i in range(k):
            flush.fill_(float(i))
            stepf(first_step + i)
        torch.cuda.synchronize()
        prof = ctx.profile_totals()
        ctx.profile(False)
        return prof

    # one step from the initial state, kept for the in-run parity check
    step(0)
    torch.cuda.synchronize()
    first = result()
    for i in range(args.warmup):
        flush.fill_(float(i))  # the flush's own first launch stays out of the timed loop
        step(i + 1)
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        ms = timed_steps(args.steps, args.warmup + 1, step)
    barrier(world)
    # per-kernel breakdown from a separate pass with the library's event
    # profiler on (same steps, same L2 flushes): the timed loop carries no
    # profiling events
    prof = profiled(args.steps, args.warmup + 1 + args.steps, step)
    points = wl.points_per_step * args.steps
    gpu_launches = int(sum(v[1] for v in prof.values()))  # same step sequence as the timed loop

    # the opt-in double-float mode, timed the same way from the initial state
    n_df = max(3, min(args.steps, 10))
    with ctx.sums_mode(tb.SUMS_DOUBLE_FLOAT):
        if is_grid:
            gb = [con0.clone(), torch.empty_like(con0)]
            step_df = lambda i: step(i, gb)
            result_df = lambda: result(gb)
        else:
            tdf = tb.Tree(ctx, wl.ca, wl.cd, wl.q, 1, wl.cc)
            step_df = lambda i: step(i, tdf)
            result_df = lambda: result(tdf)
        step_df(0)
        torch.cuda.synchronize()
        first_df = result_df()
        if is_grid:
            # the velocity is stationary: n_df steps in one call split its
            # hi/lo copy once (tbslas_semilag_grid_steps)
            def steps_df(k, _first_step):
                tb.semilag_grid_steps(ctx, vel, gb[0], N, wl.dt, k, 1, wl.bc, out=gb[1])
            steps_df(3, 1)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            steps_df(n_df, 4)
            e1.record(stream)
            torch.cuda.synchronize()
            ms_df = e0.elapsed_time(e1)
            ctx.profile(True)
            ctx.profile_reset()
            steps_df(n_df, 4)
            torch.cuda.synchronize()
            prof_df = ctx.profile_totals()
            ctx.profile(False)
        else:
            for i in range(3):
                step_df(i + 1)
            torch.cuda.synchronize()
            ms_df = timed_steps(n_df, 4, step_df)
            prof_df = profiled(n_df, 4 + n_df, step_df)
        fixed = None if is_grid else ctx.last_fp64_targets()
    df_launch_ms = prof_df.get(dominant, (1, 0, 0.0))[2] / max(prof_df.get(dominant, (1,))[0], 1)

    tot_points, tot_sec = aggregate(points, ms * 1e-3, world)
    value = tot_points / tot_sec

    # end-to-end through the host-buffer C-ABI entry point: host->device copy of
    # the step's input state and device->host copy of its result every step
    if is_grid:
        vel_h = torch.from_numpy(wl.vel).pin_memory().numpy()
        con_h = torch.from_numpy(wl.con).pin_memory().numpy()
        out_h = torch.empty(wl.con.shape, dtype=torch.float64).pin_memory().numpy()
        h2d = vel_h.nbytes + con_h.nbytes
        d2h = out_h.nbytes

        def e2e_step(i):
            tb.semilag_grid(ctx, vel_h, con_h, N, wl.dt, 1, wl.bc, out=out_h)
    else:
        coeff_h = torch.from_numpy(np.ascontiguousarray(wl.cc)).pin_memory().numpy()
        h2d = d2h = coeff_h.nbytes

        def e2e_step(i):
            tb.solve_semilag_in_situ(vf, tc, i + 1, wl.dt, 1, coeff_host=coeff_h)
    e2e_step(0)
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for i in range(args.steps):
        flush.fill_(float(i))
        e2e_step(i + 1)
    torch.cuda.synchronize()
    e2e_sec = time.perf_counter() - t0
    e_points, e_sec = aggregate(points, e2e_sec, world)

    if rank != 0:
        return None
    peaks, peak_src = measured_peaks()
    fp64_peak = ctx.fp64_fma_peak()
    fp32_peak = ctx.fp32_fma_peak()
    groups, kernels, kms = prof.get(dominant, (0, 0, 0.0))
    launch_ms = kms / max(groups, 1)
    achieved = flops_kernel * kernel_points / (launch_ms * 1e-3) / 1e12
    achieved_gbs = bytes_kernel * kernel_points / (launch_ms * 1e-3) / 1e9
    per_kernel = {k: v[2] / args.steps for k, v in prof.items()}
    roofline = {
        "kernel": dominant + (" (k_semilag_grid, FP64)" if is_grid
                              else " (k_semilag_tree<%d>, FP64)" % (wl.q + 1)),
        "bound": "fp64",
        "achieved": achieved, "peak": fp64_peak / 1e12, "unit": "TFLOP/s",
        "frac": achieved / (fp64_peak / 1e12),
        "peak_source": "FP64 FMA throughput measured in this run (tbslas_fp64_fma_peak); "
                       "MEASURED_PEAKS.json holds no FP64 figure",
        "algorithmic_flops_per_point": flops_kernel,
        "algorithmic_bytes_per_point": bytes_kernel,
        "launch_ms": launch_ms, "traffic": _traffic(wl.name, dominant),
        "hbm": {"achieved": achieved_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved_gbs / peaks["hbm_gbs"], "peak_source": peak_src},
        "kernels_ms_per_step": per_kernel, **nominal_fields(achieved)}

    # the double-float mode's own roofline: its sums are FP32 instructions,
    # each counted as an FMA (2 FLOP) against the measured FP32 FMA peak
    macs = GRID_DF_MACS_PER_POINT if is_grid else df_macs_per_point_tree(wl.q) - 3 * tb.n_coeff(wl.q)
    fp32_flops = 2 * DF_FP32_INSTR_PER_MAC * macs
    achieved32 = fp32_flops * kernel_points / (df_launch_ms * 1e-3) / 1e12
    df64 = {"value": wl.points_per_step / (ms_df / n_df * 1e-3), "unit": UNIT,
            "ms_per_step": ms_df / n_df, "steps": n_df,
            "dtype": "f64 coordinates, double-float sums (hi/lo float pairs: 48-bit "
                     "significand, FP32 exponent range)",
            "rel_diff_vs_fp64_first_step": float(np.abs(first_df - first).max()
                                                 / np.abs(first).max()),
            "roofline": {"kernel": dominant + " (double-float sums%s)"
                         % ("" if is_grid else " + FP64 near-face pass"),
                         "bound": "fp32", "achieved": achieved32, "peak": fp32_peak / 1e12,
                         "unit": "TFLOP/s", "frac": achieved32 / (fp32_peak / 1e12),
                         "peak_source": "FP32 FMA throughput measured in this run "
                                        "(tbslas_fp32_fma_peak)",
                         "counting": "%d double-float multiply-adds per point x %d FP32 "
                                     "instructions, each counted as 2 FLOP"
                                     % (macs, DF_FP32_INSTR_PER_MAC),
                         "launch_ms": df_launch_ms,
                         "traffic": _traffic(wl.name, dominant + "_df")},
            "note": "TBSLAS_SUMS_DOUBLE_FLOAT, opt-in: narrower than the reference's FP64; "
                    "not the headline"}
    if fixed is not None:
        df64["fp64_recomputed_targets_last_step"] = int(fixed)

    cpu = None
    accuracy = None
    if world == 1:
        if is_grid:
            cpu, ref, k = cpu_baseline_grid(wl)
        else:
            cpu, ref, k = cpu_baseline_tree(wl)
        scale = np.abs(ref).max()
        accuracy = {"rel_err_vs_oracle": float(np.abs(first[:k] - ref).max() / scale),
                    "compared": "first GPU step (FP64) vs the oracle on the CPU-baseline sample",
                    "tolerance": 1e-12}
        df64["rel_err_vs_oracle"] = float(np.abs(first_df[:k] - ref).max() / scale)
        cpu.pop("seconds", None)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded analytic fields)", "config": describe_config(wl),
            "e2e": {"value": e_points / e_sec, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": roofline, "cpu_baseline": cpu, "accuracy": accuracy,
            "df64_sums": df64, "clocks": clk.summary(), "gpu_launches": gpu_launches,
            "run_notes": {"l2": "flushed between timed steps (256 MiB write inside the timed "
                                "loop)", "parallelism": "replicas x%d" % world, "nrk": 1}}
    assert ctx.check() == 0
    ctx.close()
    return line


def run_functor(args, wl, rank, world, local_rank):
    """Config 2's step through the reference's separate calls, as
    SolveSemilagInSitu makes them (src/tree/tree_semilag.h:92-135,
    src/semilag/semilag.inc:26-45): CollectChebTreeGridPoints, ComputeTrajRK2
    through the velocity functor, the concentration functor (EvalTree: Morton
    bucketing of the departure points, leaf tiles staged by bulk copy) at the
    departure points, SetTreeGridValues.  Same result as the fused step, bit
    for bit; timed the same way (FP64, L2 flushed between steps)."""
    import torch
    import tbslas_gb300 as tb

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = tb.Context(local_rank)
    assert ctx.sums == tb.SUMS_FP64
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    tv = tb.Tree(ctx, wl.va, wl.vd, wl.q, 3, wl.vc)
    tc = tb.Tree(ctx, wl.ca, wl.cd, wl.q, 1, wl.cc)
    tf = tb.Tree(ctx, wl.ca, wl.cd, wl.q, 1, wl.cc)  # the fused step, for the bitwise check
    vf = tb.NodeFieldFunctor(tv, wl.bc)
    cf = tb.NodeFieldFunctor(tc, wl.bc)
    n = wl.points_per_step
    np_ = (wl.q + 1) ** 3
    pts = torch.empty((n, 3), dtype=torch.float64, device=dev)
    xdep = torch.empty_like(pts)
    vals = torch.empty((len(wl.cd), 1, np_), dtype=torch.float64, device=dev)

    def step(i):
        tinit = (i + 1) * wl.dt
        tb.collect_cheb_tree_grid_points(tc, out=pts)
        tb.compute_traj_rk2(vf, pts, tinit, tinit - wl.dt, 1, xsol=xdep)
        cf(xdep, out=vals.view(n, 1))
        tb.set_tree_grid_values(tc, vals)

    step(0)
    tb.solve_semilag_in_situ(vf, tf, 1, wl.dt, 1)
    torch.cuda.synchronize()
    same = bool(np.array_equal(tc.get_coeffs(), tf.get_coeffs()))
    for i in range(args.warmup):
        flush.fill_(float(i))
        step(i + 1)
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(args.steps):
            flush.fill_(float(i))
            step(args.warmup + 1 + i)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ctx.profile(True)
    ctx.profile_reset()
    for i in range(args.steps):
        flush.fill_(float(i))
        step(args.warmup + 1 + args.steps + i)
    torch.cuda.synchronize()
    prof = ctx.profile_totals()
    ctx.profile(False)
    if rank != 0:
        return None
    fp64_peak = ctx.fp64_fma_peak() / 1e12
    d = wl.q + 1
    nc = tb.n_coeff(wl.q)
    # the reference's count of an evaluation (3 d 3 + 2 Nc dof,
    # src/tree/tree_functor.h:389-394): two velocity evaluations in the
    # trajectory, one concentration evaluation in the functor
    traj_flops = 2 * (3 * d * 3 + 2 * nc * 3) + 18
    eval_flops = 3 * d * 3 + 2 * nc

    def frac(name, flops):
        g, _, kms = prof.get(name, (0, 0, 0.0))
        if not g:
            return None
        launch_ms = kms / g
        ach = flops * n / (launch_ms * 1e-3) / 1e12
        return {"launch_ms": launch_ms, "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": ach / fp64_peak, "algorithmic_flops_per_point": flops,
                **nominal_fields(ach)}
    line = {"metric": METRIC, "value": n * args.steps / (ms * 1e-3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded analytic fields)", "config": describe_config(wl),
            "roofline": {"bound": "fp64", "peak_source": "FP64 FMA throughput measured in this "
                         "run (tbslas_fp64_fma_peak)",
                         "traj_rk2": frac("traj_rk2", traj_flops),
                         "eval_tree (bucket_points + eval_tiles)": frac("eval_tiles", eval_flops),
                         "kernels_ms_per_step": {k: v[2] / args.steps for k, v in prof.items()}},
            "accuracy": {"equals_fused_step_bitwise": same},
            "clocks": clk.summary(),
            "gpu_launches": int(sum(v[1] for v in prof.values())),
            "run_notes": {"l2": "flushed between timed steps (256 MiB write inside the timed "
                                "loop)", "parallelism": "replicas x%d" % world, "nrk": 1}}
    assert ctx.check() == 0
    ctx.close()
    return line


def run_remesh(args, wl, rank, world, local_rank):
    """The adaptive advection loop of the reference's driver: an in-situ SL
    step, then RefineTree and Balance21 (src/applications/src/advection.cpp:
    296-311) -- here tbslas_semilag_in_situ + tbslas_tree_remesh -- every step.
    value: departure points over the K timed steps / their time, re-meshing
    included.  One step + re-mesh from the initial state is checked against
    the oracle (same leaves, coefficients within 1e-12), which is also the
    CPU baseline."""
    import torch
    import tbslas_gb300 as tb
    from oracle import oracle as ora
    from oracle import remesh as rm

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = tb.Context(local_rank)
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    tol, lo, hi = wl.remesh
    npl = (wl.q + 1) ** 3
    tv = tb.Tree(ctx, wl.va, wl.vd, wl.q, 3, wl.vc)
    vf = tb.NodeFieldFunctor(tv, wl.bc)

    def advance(tc, ts):
        tb.solve_semilag_in_situ(vf, tc, ts, wl.dt, 1)
        return tc.remesh(tol, lo, hi, wl.bc)

    # one step + re-mesh from the initial state, for the parity check
    tc = tb.Tree(ctx, wl.ca, wl.cd, wl.q, 1, wl.cc)
    advance(tc, 1)
    ga, gd = tc.leaves()
    gc = tc.get_coeffs()
    tc.close()

    tc = tb.Tree(ctx, wl.ca, wl.cd, wl.q, 1, wl.cc)
    for i in range(args.warmup):
        flush.fill_(float(i))
        advance(tc, i + 1)
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    points, rm_sec, stats, leaves = 0, 0.0, [], []
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        for i in range(args.steps):
            flush.fill_(float(i))
            points += tc.n_leaves * npl
            tb.solve_semilag_in_situ(vf, tc, args.warmup + 1 + i, wl.dt, 1)
            torch.cuda.synchronize()  # the re-meshing waits for the step anyway
            t0 = time.perf_counter()
            stats.append(tc.remesh(tol, lo, hi, wl.bc))
            rm_sec += time.perf_counter() - t0
            leaves.append(tc.n_leaves)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    state_after = (tc.leaves(), tc.get_coeffs())

    # the same K steps again from the same state with the library's event
    # profiler on: the per-kernel split of the SL steps
    tc2 = tb.Tree(ctx, state_after[0][0], state_after[0][1], wl.q, 1, state_after[1])
    ctx.profile(True)
    ctx.profile_reset()
    pts2 = 0
    for i in range(args.steps):
        flush.fill_(float(i))
        pts2 += tc2.n_leaves * npl
        advance(tc2, args.warmup + args.steps + 1 + i)
    torch.cuda.synchronize()
    prof = ctx.profile_totals()
    ctx.profile(False)
    tc2.close()

    # end to end: the field comes from pinned host memory and goes back every
    # step (host-buffer step entry point, re-mesh, coefficients read back)
    tc3 = tb.Tree(ctx, wl.ca, wl.cd, wl.q, 1, wl.cc)
    host = torch.from_numpy(np.ascontiguousarray(wl.cc)).pin_memory().numpy()
    e_points, h2d, d2h = 0, 0, 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(args.steps):
        e_points += tc3.n_leaves * npl
        h2d += host.nbytes
        tb.solve_semilag_in_situ(vf, tc3, i + 1, wl.dt, 1, coeff_host=host)
        tc3.remesh(tol, lo, hi, wl.bc)
        host = torch.empty(tc3.coeff_shape, dtype=torch.float64).pin_memory().numpy()
        tc3.get_coeffs(host)
        d2h += host.nbytes
    torch.cuda.synchronize()
    e2e_sec = time.perf_counter() - t0
    tc3.close()
    tot_points, tot_sec = aggregate(points, ms * 1e-3, world)
    e_points, e2e_sec = aggregate(e_points, e2e_sec, world)
    if rank != 0:
        return

    # the oracle: one step + re-mesh from the initial state (parity and the
    # CPU baseline)
    vel = dict(anchor=wl.va, depth=wl.vd, q=wl.q, dof=3, coeff=wl.vc)
    con = dict(anchor=wl.ca, depth=wl.cd, q=wl.q, dof=1, coeff=wl.cc)
    ora.pt2coeff(wl.q)
    t0 = time.perf_counter()
    c1 = ora.semilag_in_situ(vel, con, 1, wl.dt, 1, bool(wl.bc))
    t_step = time.perf_counter() - t0
    t0 = time.perf_counter()
    ra, rd, rc = rm.remesh(wl.ca, wl.cd, wl.q, c1, tol, lo, hi, bool(wl.bc))
    t_rm = time.perf_counter() - t0
    same = bool(np.array_equal(ga, ra) and np.array_equal(gd, rd))
    accuracy = {"same_leaves_as_oracle": same,
                "rel_err_vs_oracle": (float(np.abs(gc - rc).max() / np.abs(rc).max())
                                      if same else None),
                "compared": "one SL step + re-mesh from the initial state"}
    cpu = {"value": len(wl.cd) * npl / (t_step + t_rm), "unit": UNIT,
           "cores": ora.num_threads(), "kind": "port",
           "sample": "one step + re-mesh of the whole initial tree (%d leaves, %d departure "
                     "points): oracle step %.2f s (OpenMP C++), re-mesh %.2f s (numpy)"
                     % (len(wl.cd), len(wl.cd) * npl, t_step, t_rm)}

    roofline = fp64_roofline(
        ctx, "semilag_tree (k_semilag_tree<%d>, FP64)" % (wl.q + 1),
        fused_flops_per_point_tree(wl.q), pts2 / args.steps, prof, "semilag_tree", args.steps,
        "one velocity evaluation after the node-grid first stage, one concentration evaluation "
        "and the RK2 updates per point, as the reference counts them; points per launch = "
        "the mean leaf count x (q+1)^3")
    step_launches = int(sum(v[1] for v in prof.values()))
    remesh_launches = int(sum(st["kernels"] for st in stats))
    cfg = wl.describe()
    cfg.update({"remesh": {"tol": tol, "min_depth": lo, "max_depth": hi},
                "l2": "flushed between timed steps (256 MiB write inside the timed loop)",
                "parallelism": "replicas x%d" % world, "nrk": 1,
                "departure_points_per_step": "varies with the leaf count"})
    line = {"metric": METRIC, "value": tot_points / tot_sec, "unit": UNIT + " (step + re-mesh)",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded analytic fields)",
            "config": cfg,
            "e2e": {"value": e_points / e2e_sec, "unit": UNIT, "h2d_bytes_per_step": h2d // args.steps,
                    "d2h_bytes_per_step": d2h // args.steps},
            "remesh": {"ms_per_step": rm_sec * 1e3 / args.steps,
                       "share_of_step": rm_sec * 1e3 / ms,
                       "leaves": {"initial": int(len(wl.cd)), "final": leaves[-1],
                                  "min": min(leaves), "max": max(leaves)},
                       "merged_groups": int(sum(st["merged"] for st in stats)),
                       "split_by_refinement": int(sum(st["split"] for st in stats)),
                       "split_by_balance": int(sum(st["balanced"] for st in stats))},
            "roofline": roofline, "cpu_baseline": cpu, "accuracy": accuracy,
            "clocks": clk.summary(), "gpu_launches": step_launches + remesh_launches}
    assert ctx.check() == 0
    return line


def cpu_baseline_bdf2(wl, budget_s=12.0):
    """The oracle's BDF2 step on the first k leaves' targets, k sized for about
    budget_s of CPU work."""
    from oracle import oracle as ora
    vel = dict(anchor=wl.a, depth=wl.d, q=wl.q, dof=3, coeff=wl.vc)
    prev = dict(anchor=wl.a, depth=wl.d, q=wl.q, dof=1, coeff=wl.c_prev)
    cur = dict(anchor=wl.a, depth=wl.d, q=wl.q, dof=1, coeff=wl.c_cur)
    ora.pt2coeff(wl.q)

    def run(k):
        return ora.semilag_bdf2(vel, prev, cur, dict(anchor=wl.a[:k], depth=wl.d[:k], q=wl.q),
                                wl.t0, wl.dt)
    probe = min(8, len(wl.d))
    t0 = time.perf_counter()
    run(probe)
    per_leaf = max((time.perf_counter() - t0) / probe, 1e-6)
    k = int(max(probe, min(len(wl.d), budget_s / per_leaf)))
    t0 = time.perf_counter()
    out = run(k)
    sec = time.perf_counter() - t0
    npl = (wl.q + 1) ** 3
    return {"value": 2 * k * npl / sec, "unit": UNIT, "cores": ora.num_threads(), "kind": "port",
            "sample": "targets of the first %d of %d leaves (%d departure points: two per "
                      "target), one BDF2 step" % (k, len(wl.d), 2 * k * npl),
            "seconds": sec}, out, k


def run_bdf2(args, wl, rank, world, local_rank):
    """BDF2 two-backtrace steps (tbslas_semilag_bdf2), three concentration
    trees rotating roles (next <- 4/3 cur(X1) - 1/3 prev(X2)); value counts
    both departure points of every target."""
    import torch
    import tbslas_gb300 as tb

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = tb.Context(local_rank)
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    tv = tb.Tree(ctx, wl.a, wl.d, wl.q, 3, wl.vc)
    vf = tb.NodeFieldFunctor(tv, wl.bc)
    ts = [tb.Tree(ctx, wl.a, wl.d, wl.q, 1, wl.c_prev), tb.Tree(ctx, wl.a, wl.d, wl.q, 1, wl.c_cur),
          tb.Tree(ctx, wl.a, wl.d, wl.q, 1)]

    def step(i):
        # after i steps: prev = ts[i % 3], cur = ts[(i + 1) % 3], next = ts[(i + 2) % 3]
        tb.solve_semilag_bdf2(vf, ts[i % 3], ts[(i + 1) % 3], ts[(i + 2) % 3],
                              wl.t0 + i * wl.dt, wl.dt)
    step(0)
    torch.cuda.synchronize()
    first = ts[2].get_coeffs()
    for i in range(args.warmup):
        flush.fill_(float(i))
        step(i + 1)
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        for i in range(args.steps):
            flush.fill_(float(i))
            step(args.warmup + 1 + i)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ctx.profile(True)
    ctx.profile_reset()
    for i in range(args.steps):
        flush.fill_(float(i))
        step(args.warmup + args.steps + 1 + i)
    torch.cuda.synchronize()
    prof = ctx.profile_totals()
    ctx.profile(False)
    # end to end: c_{n-1} and c_n from pinned host memory, c_{n+1} back, every step
    hp = torch.from_numpy(np.ascontiguousarray(wl.c_prev)).pin_memory().numpy()
    hc = torch.from_numpy(np.ascontiguousarray(wl.c_cur)).pin_memory().numpy()
    hn = torch.empty(hc.shape, dtype=torch.float64).pin_memory().numpy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(args.steps):
        ts[0].set_coeffs(hp)
        ts[1].set_coeffs(hc)
        tb.solve_semilag_bdf2(vf, ts[0], ts[1], ts[2], wl.t0, wl.dt)
        ts[2].get_coeffs(hn)
    torch.cuda.synchronize()
    e2e_sec = time.perf_counter() - t0
    points = wl.points_per_step * args.steps
    e_points, e2e_sec = aggregate(points, e2e_sec, world)
    tot_points, tot_sec = aggregate(points, ms * 1e-3, world)
    if rank != 0:
        return
    cpu, ref, k = cpu_baseline_bdf2(wl)
    cpu.pop("seconds", None)
    accuracy = {"rel_err_vs_oracle": float(np.abs(first[:k] - ref).max() / np.abs(ref).max()),
                "compared": "first GPU step vs the oracle on the CPU-baseline sample"}
    d = wl.q + 1
    nc = d * (d + 1) * (d + 2) // 6
    ev = lambda dof: 9 * d + 2 * nc * dof
    roofline = fp64_roofline(
        ctx, "semilag_bdf2 (k_semilag_bdf2<%d>, FP64)" % d, 3 * ev(3) + 2 * ev(1) + 36,
        wl.points_per_step // 2, prof, "semilag_bdf2", args.steps,
        "per target: three velocity evaluations (the first stage of the first backtrace is "
        "the node grid's), two concentration evaluations, four RK2 updates")
    cfg = wl.describe()
    cfg.update({"l2": "flushed between timed steps (256 MiB write inside the timed loop)",
                "parallelism": "replicas x%d" % world, "nrk": 1})
    line = {"metric": METRIC, "value": tot_points / tot_sec, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded analytic fields)", "config": cfg,
            "e2e": {"value": e_points / e2e_sec, "unit": UNIT,
                    "h2d_bytes_per_step": int(hp.nbytes + hc.nbytes),
                    "d2h_bytes_per_step": int(hn.nbytes)},
            "targets_per_s": tot_points / 2 / tot_sec,
            "roofline": roofline, "cpu_baseline": cpu, "accuracy": accuracy,
            "clocks": clk.summary(), "gpu_launches": int(sum(v[1] for v in prof.values()))}
    assert ctx.check() == 0
    return line


def cpu_baseline_tv(wl, budget_s=12.0):
    """The oracle's time-dependent step (every tree evaluated, cubic in time)
    on the first k leaves' targets."""
    from oracle import oracle as ora
    vels = [dict(anchor=wl.a, depth=wl.d, q=wl.q, dof=3, coeff=c) for c in wl.vcs]
    con = dict(anchor=wl.a, depth=wl.d, q=wl.q, dof=1, coeff=wl.cc)
    ora.pt2coeff(wl.q)

    def run(k):
        return ora.semilag_in_situ_tv(vels, con, wl.timestep, wl.dt, 1, False, times=wl.times,
                                      leaf_end=k)
    probe = min(8, len(wl.d))
    t0 = time.perf_counter()
    run(probe)
    per_leaf = max((time.perf_counter() - t0) / probe, 1e-6)
    k = int(max(probe, min(len(wl.d), budget_s / per_leaf)))
    t0 = time.perf_counter()
    out = run(k)
    sec = time.perf_counter() - t0
    npl = (wl.q + 1) ** 3
    return {"value": k * npl / sec, "unit": UNIT, "cores": ora.num_threads(), "kind": "port",
            "sample": "targets of the first %d of %d leaves, one step (four velocity trees "
                      "evaluated per stage, numpy composition of the oracle's EvalTree)"
                      % (k, len(wl.d)), "seconds": sec}, out, k


def run_tv(args, wl, rank, world, local_rank):
    """In-situ steps through a FieldSetFunctor velocity (four trees, cubic in
    time; tbslas_semilag_in_situ_tv's blended fused step)."""
    import torch
    import tbslas_gb300 as tb

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = tb.Context(local_rank)
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    vt = [tb.Tree(ctx, wl.a, wl.d, wl.q, 3, c) for c in wl.vcs]
    f = tb.FieldSetFunctor(vt, wl.times, wl.bc)
    tc = tb.Tree(ctx, wl.a, wl.d, wl.q, 1, wl.cc)

    def step(i):
        tb.solve_semilag_in_situ_tv(f, tc, wl.timestep, wl.dt)
    step(0)
    torch.cuda.synchronize()
    first = tc.get_coeffs()
    for i in range(args.warmup):
        flush.fill_(float(i))
        step(i + 1)
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        for i in range(args.steps):
            flush.fill_(float(i))
            step(i)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ctx.profile(True)
    ctx.profile_reset()
    for i in range(args.steps):
        flush.fill_(float(i))
        step(i)
    torch.cuda.synchronize()
    prof = ctx.profile_totals()
    ctx.profile(False)
    host = torch.from_numpy(np.ascontiguousarray(wl.cc)).pin_memory().numpy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(args.steps):
        tc.set_coeffs(host)
        step(i)
        tc.get_coeffs(host)
    torch.cuda.synchronize()
    e2e_sec = time.perf_counter() - t0
    points = wl.points_per_step * args.steps
    e_points, e2e_sec = aggregate(points, e2e_sec, world)
    tot_points, tot_sec = aggregate(points, ms * 1e-3, world)
    if rank != 0:
        return
    cpu, ref, k = cpu_baseline_tv(wl)
    cpu.pop("seconds", None)
    accuracy = {"rel_err_vs_oracle": float(np.abs(first[:k] - ref).max() / np.abs(ref).max()),
                "compared": "first GPU step vs the oracle on the CPU-baseline sample"}
    d = wl.q + 1
    nc = d * (d + 1) * (d + 2) // 6
    ev = lambda dof: 9 * d + 2 * nc * dof
    m = len(wl.vcs)
    roofline = fp64_roofline(
        ctx, "semilag_tv (k_semilag_tv<%d, true>, FP64: every tree at the midpoint)" % d,
        9 * d + m * 2 * nc * 3 + 3 * m + ev(1) + 18, wl.points_per_step, prof, "semilag_tv",
        args.steps,
        "per point: the %d velocity trees evaluated at the RK2 midpoint and blended (as the "
        "reference's FieldSetFunctor does; the trees share their leaves, so one lookup and "
        "one set of T_k serve all of them; the first stage, at the node, is each tree's "
        "node-grid pass, vel_at_nodes), the concentration at the departure point" % m)
    cfg = wl.describe()
    cfg.update({"l2": "flushed between timed steps (256 MiB write inside the timed loop)",
                "parallelism": "replicas x%d" % world, "nrk": 1})
    line = {"metric": METRIC, "value": tot_points / tot_sec, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded analytic fields)", "config": cfg,
            "e2e": {"value": e_points / e2e_sec, "unit": UNIT, "h2d_bytes_per_step": int(host.nbytes),
                    "d2h_bytes_per_step": int(host.nbytes)},
            "roofline": roofline, "cpu_baseline": cpu, "accuracy": accuracy,
            "clocks": clk.summary(), "gpu_launches": int(sum(v[1] for v in prof.values()))}
    assert ctx.check() == 0
    return line


def run_construct(args, wl, rank, world, local_rank):
    """ConstructTree on the device (tbslas_tree_construct) for the two trees of
    the adaptive q=14 configuration (4 Gaussians; Taylor-Green; tol 1e-6,
    depths 3..8): the trees must equal the host construction the other
    workloads use; value = Chebyshev nodes of the final trees fitted per
    second, K constructions timed."""
    import torch
    import tbslas_gb300 as tb
    from oracle import construct as oc

    torch.cuda.set_device(local_rank)
    ctx = tb.Context(local_rank)
    tol, lo, hi = wl.construct
    fc = tb.Field.gaussians(wl.blobs.centres, wl.blobs.sigmas)
    fv = tb.Field.taylor_green()

    def build():
        return (tb.construct_tree(ctx, fc, wl.q, tol, lo, hi),
                tb.construct_tree(ctx, fv, wl.q, tol, lo, hi))
    tcon, tvel = build()
    check = {}
    for name, t, (a, d, c) in (("concentration", tcon, (wl.ca, wl.cd, wl.cc)),
                               ("velocity", tvel, (wl.va, wl.vd, wl.vc))):
        ga, gd = t.leaves()
        same = bool(np.array_equal(ga, a) and np.array_equal(gd, d))
        check[name] = {"leaves": int(len(gd)), "same_leaves_as_host_construction": same,
                       "coeff_rel_diff_vs_host_fit": (float(np.abs(t.get_coeffs() - c).max()
                                                            / np.abs(c).max()) if same else None)}
        t.close()
    nodes = (len(wl.cd) + len(wl.vd)) * (wl.q + 1) ** 3
    for _ in range(args.warmup):
        for t in build():
            t.close()
    torch.cuda.synchronize()
    ctx.profile(True)
    ctx.profile_reset()
    sec = []
    with ClockSampler(local_rank) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            ts = build()
            torch.cuda.synchronize()
            sec.append(time.perf_counter() - t0)
            for t in ts:
                t.close()
    prof = ctx.profile_totals()
    ctx.profile(False)
    ms = 1e3 * float(np.median(sec))
    tot_nodes, tot_sec = aggregate(nodes, ms * 1e-3, world)
    if rank != 0:
        return
    t0 = time.perf_counter()
    oc.construct(fc.kind, fc.n, fc.params, wl.q, tol, lo, hi)
    oc.construct(fv.kind, fv.n, fv.params, wl.q, tol, lo, hi)
    cpu_sec = time.perf_counter() - t0
    from oracle import oracle as ora
    cfg = {"workload": wl.name, "q": wl.q, "tol": tol, "depths": [lo, hi],
           "trees": "4 Gaussians (concentration), Taylor-Green (velocity)",
           "note": "ConstructTree on the device: fit, refine by the Chebyshev tail, "
                   "2:1 balance, final fit"}
    line = {"metric": METRIC, "value": tot_nodes / tot_sec,
            "unit": "Chebyshev nodes of the final trees fitted per second (tree construction)",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded analytic fields)", "config": cfg,
            "timing": "wall clock around each synchronous construction of both trees (median "
                      "of K)",
            "e2e": {"value": tot_nodes / tot_sec, "unit": "fitted nodes/s",
                    "h2d_bytes_per_step": 8 * (fc.params.size + fv.params.size),
                    "d2h_bytes_per_step": 0},
            "cpu_baseline": {"value": nodes / cpu_sec, "unit": "fitted nodes/s",
                             "cores": ora.num_threads(), "kind": "port",
                             "sample": "the oracle's construction of both trees (numpy, the C "
                                       "oracle's fit), once: %.2f s" % cpu_sec},
            "accuracy": check, "clocks": clk.summary(),
            "gpu_launches": int(prof.get("construct", (0, 0, 0.0))[1])}
    assert ctx.check() == 0
    return line


def run_batched(args, wl, rank, world, local_rank):
    """The batched, graph-captured step of 64 uneven problems vs the plain
    per-problem loop of in-situ steps on the same problems, from the same
    state: in the default FP64 arithmetic (the headline of this line) and in
    the opt-in double-float mode.  The plain loop's idle time between its
    launches (wall time minus the summed kernel time the library's event
    profiler brackets) bounds what batching can gain at an equal per-target
    rate."""
    import torch
    import tbslas_gb300 as tb

    torch.cuda.set_device(local_rank)
    ctx = tb.Context(local_rank)
    stream = torch.cuda.current_stream()

    def measure(mode):
        with ctx.sums_mode(mode):
            probs = [(tb.Tree(ctx, p["va"], p["vd"], p["q"], 3, p["vc"]),
                      tb.Tree(ctx, p["ca"], p["cd"], p["q"], 1, p["cc"]), p["dt"])
                     for p in wl.problems]
            funcs = [tb.NodeFieldFunctor(tv, wl.bc) for tv, _, _ in probs]

            def reset():
                for (tv, tc, _), p in zip(probs, wl.problems):
                    tc.set_coeffs(p["cc"])

            def plain(ts0, k):
                for i in range(k):
                    for f, (tv, tc, dt) in zip(funcs, probs):
                        tb.solve_semilag_in_situ(f, tc, ts0 + i, dt)

            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            reset()
            plain(1, args.warmup)
            reset()
            torch.cuda.synchronize()
            e0.record(stream)
            plain(1, args.steps)
            e1.record(stream)
            torch.cuda.synchronize()
            plain_ms = e0.elapsed_time(e1)
            plain_state = [tc.get_coeffs() for _, tc, _ in probs]
            # the plain loop's kernel time (the profiler's event brackets)
            reset()
            ctx.profile(True)
            ctx.profile_reset()
            plain(1, args.steps)
            torch.cuda.synchronize()
            busy_ms = sum(v[2] for v in ctx.profile_totals().values())
            plain_launches = sum(v[1] for v in ctx.profile_totals().values())
            ctx.profile(False)
            batch = tb.Batch(ctx, probs, 1, wl.bc)
        reset()
        tune = batch.autotune()
        reset()
        batch.run(1, args.steps, True)          # capture + warm replay
        reset()
        torch.cuda.synchronize()
        barrier(world)
        with ClockSampler(local_rank) as clk:
            e0.record(stream)
            batch.run(1, args.steps, True)      # the captured K-step graph
            e1.record(stream)
            torch.cuda.synchronize()
        barrier(world)
        ms = e0.elapsed_time(e1)
        same = all(np.array_equal(tc.get_coeffs(), ref)
                   for (_, tc, _), ref in zip(probs, plain_state))
        return dict(probs=probs, batch=batch, plain_ms=plain_ms, busy_ms=busy_ms, ms=ms,
                    same=same, tune=tune, clk=clk, plain_launches=plain_launches)

    r64 = measure(tb.SUMS_FP64)
    # e2e (FP64): host coefficients in, one graph step, host coefficients out, per step
    probs, batch = r64["probs"], r64["batch"]
    pinned = [torch.from_numpy(np.ascontiguousarray(p["cc"])).pin_memory().numpy()
              for p in wl.problems]
    h2d = sum(a.nbytes for a in pinned)
    batch.run(1, 1, True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(args.steps):
        for (_, tc, _), a in zip(probs, pinned):
            tc.set_coeffs(a)
        batch.run(1 + i, 1, True)
        for (_, tc, _), a in zip(probs, pinned):
            tc.get_coeffs(a)
    torch.cuda.synchronize()
    e2e_sec = time.perf_counter() - t0
    batch.close()
    for tv, tc, _ in probs:
        tv.close()
        tc.close()
    rdf = measure(tb.SUMS_DOUBLE_FLOAT)
    rdf["batch"].close()

    points = wl.points_per_step * args.steps
    tot_points, tot_sec = aggregate(points, r64["ms"] * 1e-3, world)
    e_points, e_sec = aggregate(points, e2e_sec, world)
    if rank != 0:
        return None

    def summary(r):
        return {"batched": {"value": points / (r["ms"] * 1e-3), "ms_per_step": r["ms"] / args.steps},
                "plain_loop": {"value": points / (r["plain_ms"] * 1e-3),
                               "ms_per_step": r["plain_ms"] / args.steps,
                               "kernel_ms_per_step": r["busy_ms"] / args.steps,
                               "launch_groups_per_step": r["plain_launches"] / args.steps,
                               "idle_fraction": max(0.0, 1.0 - r["busy_ms"] / r["plain_ms"]),
                               "max_gain_from_removing_idle": r["plain_ms"] / r["busy_ms"]},
                "batched_vs_plain": r["plain_ms"] / r["ms"],
                "batched_equals_plain_bitwise": bool(r["same"]),
                "autotuned": {"block": r["tune"][0], "targets_per_item": r["tune"][1],
                              "ctas_per_sm": r["tune"][2]}}
    cfg = describe_config(wl)
    s64, sdf = summary(r64), summary(rdf)
    # the whole batched step (node-grid kernels, band kernels, refit) over its
    # graph time, counting per target the fused kernel's algorithmic FLOPs (the
    # midpoint velocity and the departure concentration, as the headline's
    # roofline counts them); the node-grid pass and the refit add time only
    step_flops = sum(len(p["cd"]) * (p["q"] + 1) ** 3 * fused_flops_per_point_tree(p["q"])
                     for p in wl.problems)
    ach = step_flops / (r64["ms"] / args.steps * 1e-3) / 1e12
    fp64_peak = ctx.fp64_fma_peak() / 1e12
    roofline = {"kernel": "the batched step (k_batch_eval_on_nodes, k_batch_semilag_fp64 "
                          "bands, k_batch_refit), FP64", "bound": "fp64",
                "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s", "frac": ach / fp64_peak,
                "peak_source": "FP64 FMA throughput measured in this run (tbslas_fp64_fma_peak)",
                "counting": "per problem: targets x the fused step's FLOPs (3*d*3 + 2*Nc*dof "
                            "per evaluation, velocity at the midpoint and concentration at the "
                            "departure point, RK updates) over the whole step's graph time",
                **nominal_fields(ach)}
    cpu = cpu_baseline_batched(wl)
    line = {"metric": METRIC, "value": tot_points / tot_sec, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r64["ms"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded analytic fields)", "config": cfg,
            "batched_vs_plain": s64["batched_vs_plain"],
            "plain_loop": s64["plain_loop"],
            "accuracy": {"batched_equals_plain_bitwise": s64["batched_equals_plain_bitwise"],
                         "plain_loop": "oracle-checked per problem (tests/test_gpu_tree.py)"},
            "autotuned": s64["autotuned"],
            "roofline": roofline, "cpu_baseline": cpu,
            "e2e": {"value": e_points / e_sec, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(h2d)},
            "df64_sums": dict(sdf, dtype="f64 coordinates, double-float sums",
                              note="TBSLAS_SUMS_DOUBLE_FLOAT, opt-in; not the headline"),
            "clocks": r64["clk"].summary(),
            "run_notes": {"l2": "inputs larger than L2 (all problems' trees)",
                          "parallelism": "replicas x%d" % world, "nrk": 1,
                          "graph": "the K-step run is one captured CUDA graph"},
            "gpu_launches": int(args.steps * (len({p["q"] for p in wl.problems})
                                              + len({_band(p["q"]) for p in wl.problems}) + 1))}
    assert ctx.check() == 0
    ctx.close()
    return line


def bubble_directions(wl, rng, n, leaves=None):
    """n seeded velocity-coefficient directions [Lv, 3, Nc] that vanish on
    every leaf face: per leaf and component, (1 - xi^2)(1 - eta^2)(1 - zeta^2)
    times a random polynomial of total degree q - 6 in the leaf's local
    coordinates, fitted at the leaf's nodes (exact: the product has total
    degree q).  Nodes that sit on a leaf face with zero normal velocity -- on
    Taylor-Green, the stagnation planes and every z face (v_z = 0) -- stay
    exactly on that face under such a perturbation.  leaves (optional): per
    direction, the one leaf that carries it (zero elsewhere)."""
    from tbslas_gb300 import trees
    q = wl.q
    d = q + 1
    xi = 2.0 * trees.cheb_nodes(q) - 1.0                      # [Np, 3]
    bub = np.prod(1.0 - xi ** 2, axis=1)                      # [Np]
    r = q - 6
    mono = [(a, b, c) for a in range(r + 1) for b in range(r + 1 - a)
            for c in range(r + 1 - a - b)]
    P = np.stack([xi[:, 0] ** a * xi[:, 1] ** b * xi[:, 2] ** c for a, b, c in mono], axis=1)
    M = trees.pt2coeff(q)
    L = len(wl.d)
    out = []
    for k in range(n):
        w = rng.standard_normal((L, 3, len(mono)))
        if leaves is not None:
            keep = np.zeros(L, dtype=bool)
            keep[leaves[k]] = True
            w[~keep] = 0.0
        vals = np.einsum("pm,lam->lap", P, w) * bub[None, None, :]   # [L, 3, Np]
        out.append((vals.reshape(L * 3, d ** 3) @ M).reshape(L, 3, -1))
    return out


def run_adjoint(args, wl, rank, world, local_rank):
    """The differentiable T-step advection in the default FP64 arithmetic:
    the forward (plain and checkpointed) and adjoint passes timed; gradients
    checked by central differences on the configuration itself (16 c0
    directions, 8 velocity directions that vanish on leaf faces) and by the
    oracle's dual numbers at a reduced depth.  The same passes in the opt-in
    double-float mode are reported beside it."""
    import torch
    import tbslas_gb300 as tb
    from tbslas_gb300 import adjoint

    torch.cuda.set_device(local_rank)
    ctx = tb.Context(local_rank)
    assert ctx.sums == tb.SUMS_FP64
    stream = torch.cuda.current_stream()
    dev = torch.device("cuda", local_rank)
    tv = tb.Tree(ctx, wl.a, wl.d, wl.q, 3, wl.vc)
    tc = tb.Tree(ctx, wl.a, wl.d, wl.q, 1, wl.c0)
    V = torch.from_numpy(adjoint.basis_at_nodes(wl.q)).to(dev)
    vct = torch.from_numpy(wl.vc).to(dev)
    c0 = torch.from_numpy(wl.c0).to(dev)
    T = wl.steps
    with torch.no_grad():
        cobs = adjoint.advect(torch.from_numpy(wl.c0_obs).to(dev), vct, tv, tc, wl.dt, 1, T,
                              wl.bc, False)

    def J(c):
        vals = torch.einsum("ln,pn->lp", c[:, 0, :], V)
        ovals = torch.einsum("ln,pn->lp", cobs[:, 0, :], V)
        return 0.5 * ((vals - ovals) ** 2).sum()

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out

    def fwd_plain():
        with torch.no_grad():
            return adjoint.advect(c0, vct, tv, tc, wl.dt, 1, T, wl.bc, False)

    def grad(checkpoint):
        c = c0.clone().requires_grad_(True)
        v = vct.clone().requires_grad_(True)
        cT = adjoint.advect(c, v, tv, tc, wl.dt, 1, T, wl.bc, checkpoint)
        j = J(cT)
        torch.cuda.synchronize()
        return c, v, j

    def passes(modes):
        fwd_plain()
        fms_plain, _ = timed(fwd_plain)
        for ck in modes:  # the first autograd pass of a process carries one-time setup
            _, _, j0 = grad(ck)
            j0.backward()
        torch.cuda.synchronize()
        res = {}
        for ck in modes:
            fms, (c, v, j) = timed(lambda: grad(ck))
            bms, _ = timed(lambda: j.backward())
            res[ck] = (fms, bms, c.grad.clone(), v.grad.clone(), j.item())
        return fms_plain, res

    with ClockSampler(local_rank) as clk:
        fwd_ms, res = passes(("jacobian", True, "departure", False))
    # per-kernel breakdown of one more adjoint pass each way (profiler on,
    # outside the timed passes)
    by_kernel = {}
    for ck, name in (("jacobian", "checkpoint_jacobian"), (True, "checkpoint"),
                     (False, "recompute")):
        _, _, j1 = grad(ck)
        ctx.profile(True)
        ctx.profile_reset()
        j1.backward()
        torch.cuda.synchronize()
        by_kernel[name] = {k: round(v[2] / T, 3) for k, v in sorted(ctx.profile_totals().items())}
        ctx.profile(False)
    with ctx.sums_mode(tb.SUMS_DOUBLE_FLOAT):
        fwd_df_ms, res_df = passes((True,))
    # the headline mode: every step's points and velocity Jacobian stored
    # (memory is plentiful at this size: 120 B per target per step)
    gc, gv = res["jacobian"][2], res["jacobian"][3]
    rng = np.random.default_rng(123)
    eps = 1e-6

    def J_at(cc, vv):
        with torch.no_grad():
            return J(adjoint.advect(cc, vv, tv, tc, wl.dt, 1, T, wl.bc, False)).item()

    errs_c, errs_v = [], []
    t_fd = time.perf_counter()
    for k in range(16):
        d = torch.from_numpy(rng.standard_normal(wl.c0.shape)).to(dev)
        fd = (J_at(c0 + eps * d, vct) - J_at(c0 - eps * d, vct)) / (2 * eps)
        an = (gc * d).sum().item()
        errs_c.append(abs(fd - an) / abs(an))
    # velocity directions: one face-vanishing bubble each, on a seeded leaf
    # where the concentration is large (so dJ/ds is), i.e. at most a few
    # thousand targets move: an eps-move of a departure point across a leaf
    # face (a jump of J by the fit's face discontinuity) stays improbable
    big = np.flatnonzero(np.abs(wl.c0[:, 0, 0]) > 0.3 * np.abs(wl.c0[:, 0, 0]).max())
    vleaves = rng.choice(big, size=8, replace=False)
    for dvn in bubble_directions(wl, rng, 8, leaves=vleaves):
        dv = torch.from_numpy(dvn).to(dev)
        fd = (J_at(c0, vct + eps * dv) - J_at(c0, vct - eps * dv)) / (2 * eps)
        an = (gv * dv).sum().item()
        errs_v.append(abs(fd - an) / abs(an))
    t_fd = time.perf_counter() - t_fd
    dual = dual_check_adjoint(wl, ctx, dev)
    jk_fms, jk_bms = res["jacobian"][0], res["jacobian"][1]
    ck_fms, ck_bms = res[True][0], res[True][1]
    rc_fms, rc_bms = res[False][0], res[False][1]

    def gap(x, y):
        return max(float((x[2] - y[2]).abs().max() / y[2].abs().max()),
                   float((x[3] - y[3]).abs().max() / y[3].abs().max()))
    ck_gap = gap(res[True], res[False])
    jk_gap = gap(res["jacobian"], res[False])
    df_gap = max(float((res_df[True][2] - gc).abs().max() / gc.abs().max()),
                 float((res_df[True][3] - gv).abs().max() / gv.abs().max()))
    points = wl.points_per_step * T
    # the adjoint kernel against the FP64 peak: per target, grad c^k(Xd)
    # (2 Nc multiply-adds), the lambda scatter (Nc), J_v(X*)^T g (9) and the
    # velocity scatter (3 Nc)
    nc = tb.n_coeff(wl.q)
    adj_flops = 2 * (6 * nc + 9)
    kms = by_kernel["checkpoint_jacobian"].get("adjoint_fp64", 0.0)
    ach = adj_flops * wl.points_per_step / (max(kms, 1e-9) * 1e-3) / 1e12
    fp64_peak = ctx.fp64_fma_peak() / 1e12
    roofline = {"kernel": "adjoint_fp64 (k_adjoint_f64<%d, true>)" % (wl.q + 1),
                "bound": "fp64", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": ach / fp64_peak, "launch_ms": kms,
                "peak_source": "FP64 FMA throughput measured in this run (tbslas_fp64_fma_peak)",
                "algorithmic_flops_per_point": adj_flops,
                "counting": "2 x (6 Nc + 9) per target: grad c^k(Xd) 2 Nc, lambda scatter Nc, "
                            "J_v(X*)^T g 9, velocity scatter 3 Nc multiply-adds",
                **nominal_fields(ach)}
    cpu = {"value": dual["points_per_s"], "unit": UNIT, "cores": dual["cores"], "kind": "port",
           "sample": "the oracle's in-situ step on forward-mode dual numbers (one directional "
                     "derivative of the T-step map, the CPU counterpart of one gradient "
                     "direction; the reference has no adjoint): %s" % dual["tree"],
           "seconds": dual["seconds"]}
    if rank != 0:
        return None
    fd_max = max(errs_c + errs_v)
    line = {"metric": METRIC, "value": points / (jk_bms * 1e-3), "unit": UNIT + " (adjoint pass)",
            "n_gpus": world, "steps": T, "warmup": 1, "ms_per_step": jk_bms / T,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded analytic fields)", "config": describe_config(wl),
            "adj_over_fwd": jk_bms / fwd_ms, "mode": "checkpoint_jacobian",
            "fd_max_rel": fd_max, "dual_max_rel": dual["max_rel_err"],
            "roofline": roofline, "cpu_baseline": cpu,
            "forward": {"ms": fwd_ms, "points_per_s": points / (fwd_ms * 1e-3),
                        "kind": "the in-situ step (FP64 sums), no checkpoints"},
            "checkpoint_jacobian": {"forward_ms": jk_fms, "adjoint_ms": jk_bms,
                                    "adj_over_fwd": jk_bms / fwd_ms,
                                    "grad_over_fwd": (jk_fms + jk_bms) / fwd_ms,
                                    "stored_bytes": int(points * 120),
                                    "note": "midpoints, departure points and the velocity "
                                            "Jacobian at the midpoints stored by the forward"},
            "checkpoint": {"forward_ms": ck_fms, "adjoint_ms": ck_bms,
                           "adj_over_fwd": ck_bms / fwd_ms,
                           "grad_over_fwd": (ck_fms + ck_bms) / fwd_ms,
                           "stored_bytes": int(points * 48)},
            "checkpoint_departure_only": {
                "forward_ms": res["departure"][0], "adjoint_ms": res["departure"][1],
                "adj_over_fwd": res["departure"][1] / fwd_ms,
                "grad_over_fwd": (res["departure"][0] + res["departure"][1]) / fwd_ms,
                "stored_bytes": int(points * 24),
                "note": "departure points stored; midpoints rebuilt from the node-grid "
                        "velocity in the backward pass"},
            "recompute": {"forward_ms": rc_fms, "adjoint_ms": rc_bms,
                          "adj_over_fwd": rc_bms / fwd_ms,
                          "grad_over_fwd": (rc_fms + rc_bms) / fwd_ms, "stored_bytes": 0},
            "fd_check": {"eps": eps, "directions": len(errs_c) + len(errs_v),
                         "directions_kind": "16 N(0,1) c0 directions and 8 velocity directions, "
                                            "each a face bubble times a random polynomial "
                                            "on one seeded leaf inside the Gaussian (zero "
                                            "on every leaf face, so nodes held on faces by "
                                            "zero normal velocity stay there), all on this "
                                            "configuration",
                         "max_rel_err_dJ_dc0": max(errs_c), "max_rel_err_dJ_dV": max(errs_v),
                         "seconds": t_fd, "tolerance": 1e-6},
            "dual_number_check": dual,
            "adjoint_ms_per_step_by_kernel": by_kernel,
            "checkpoint_vs_recompute_rel_diff": ck_gap,
            "jacobian_vs_recompute_rel_diff": jk_gap, "J": res["jacobian"][4],
            "df64_sums": {"forward_ms": fwd_df_ms, "adjoint_ms": res_df[True][1],
                          "adj_over_fwd": res_df[True][1] / fwd_df_ms,
                          "adj_over_fp64_fwd": res_df[True][1] / fwd_ms,
                          "grad_rel_diff_vs_fp64": df_gap,
                          "dtype": "f64 coordinates, double-float sums",
                          "note": "TBSLAS_SUMS_DOUBLE_FLOAT, opt-in; not the headline"},
            "clocks": clk.summary()}
    assert ctx.check() == 0
    ctx.close()
    return line


def dual_check_adjoint(wl, ctx, dev, depth=3, ndir=2):
    """Exact check of the adjoint on the same configuration at a reduced tree
    depth: directional derivative of J through the oracle on forward-mode dual
    numbers (leaf choices held fixed) vs the adjoint gradient, along seeded
    N(0,1) directions in (c0, V) jointly."""
    import torch
    import tbslas_gb300 as tb
    from oracle import oracle as ora
    from tbslas_gb300 import adjoint, workloads
    small = workloads.AdjointWorkload(depth=depth, q=wl.q, steps=wl.steps, dt=wl.dt)
    tv = tb.Tree(ctx, small.a, small.d, small.q, 3, small.vc)
    tc = tb.Tree(ctx, small.a, small.d, small.q, 1, small.c0)
    Vb = adjoint.basis_at_nodes(small.q)
    with torch.no_grad():
        cobs = adjoint.advect(torch.from_numpy(small.c0_obs).to(dev),
                              torch.from_numpy(small.vc).to(dev), tv, tc, small.dt, 1,
                              small.steps, small.bc, False).cpu().numpy()
    c = torch.from_numpy(small.c0).to(dev).requires_grad_(True)
    v = torch.from_numpy(small.vc).to(dev).requires_grad_(True)
    cT = adjoint.advect(c, v, tv, tc, small.dt, 1, small.steps, small.bc, "jacobian")
    Vt = torch.from_numpy(Vb).to(dev)
    J = 0.5 * ((torch.einsum("ln,pn->lp", cT[:, 0, :], Vt) -
                torch.einsum("ln,pn->lp", torch.from_numpy(cobs).to(dev)[:, 0, :], Vt)) ** 2).sum()
    J.backward()
    gc, gv = c.grad.cpu().numpy(), v.grad.cpu().numpy()
    rng = np.random.default_rng(5)
    errs = []
    t0 = time.perf_counter()
    for _ in range(ndir):
        dc, dv = rng.standard_normal(small.c0.shape), rng.standard_normal(small.vc.shape)
        vel = dict(anchor=small.a, depth=small.d, q=small.q, dof=3, coeff=small.vc)
        cc, dcc = small.c0, dc
        for s in range(1, small.steps + 1):
            cc, dcc = ora.semilag_in_situ_dual(
                vel, dv, dict(anchor=small.a, depth=small.d, q=small.q, dof=1, coeff=cc), dcc,
                s, small.dt, 1, bool(small.bc))
        resid = cc[:, 0, :] @ Vb.T - cobs[:, 0, :] @ Vb.T
        dJ = float((resid * (dcc[:, 0, :] @ Vb.T)).sum())
        an = float((gc * dc).sum() + (gv * dv).sum())
        errs.append(abs(dJ - an) / abs(dJ))
    sec = time.perf_counter() - t0
    pts = len(small.d) * (small.q + 1) ** 3 * small.steps * ndir
    return {"tree": "uniform depth %d (%d leaves), same q/velocity/steps" % (depth, len(small.d)),
            "directions": ndir, "max_rel_err": max(errs), "gradient_mode": "checkpoint_jacobian",
            "seconds": sec, "points_per_s": pts / sec, "cores": ora.num_threads()}


def _band(q):
    """Degree band of the batched kernels (band_of in csrc/batch_kernels.cuh)."""
    return 0 if q <= 8 else (1 if q <= 11 else (2 if q <= 13 else q - 11))


# The configurations measured beside the headline in the default run (N = 1):
# key -> (workload, runner name, steps cap).  The headline is the adaptive q = 14
# configuration; these are the uniform q = 8 tree, the tricubic grid, the
# 64-problem batch and the adjoint, each in the library's default FP64
# arithmetic with its own roofline, CPU baseline, accuracy check and clocks,
# and the headline configuration once more through the reference's separate
# calls (the general functor path).
EXTRA_CONFIGS = [
    ("cfg1_uniform_q8", "tree_uniform_q8", "run_gpu", None),
    ("cfg3_grid_256", "grid_periodic_256", "run_gpu", 20),
    ("cfg4_batched_64", "batched_64", "run_batched", 10),
    ("cfg5_adjoint_q8", "adjoint_q8", "run_adjoint", None),
    # config 2 through the reference's separate calls (the functor path)
    ("cfg2_functor_path", "functor_q14", "run_functor", 10),
]


def describe_config(wl):
    """The `config` object of a workload: the same dict in both arms."""
    return wl.describe()


def dispatch(args, wl, rank, world, local_rank):
    if wl.name.startswith("batched"):
        return run_batched(args, wl, rank, world, local_rank)
    if wl.name.startswith("adjoint"):
        return run_adjoint(args, wl, rank, world, local_rank)
    if hasattr(wl, "remesh"):
        return run_remesh(args, wl, rank, world, local_rank)
    if hasattr(wl, "c_prev"):
        return run_bdf2(args, wl, rank, world, local_rank)
    if hasattr(wl, "vcs"):
        return run_tv(args, wl, rank, world, local_rank)
    if hasattr(wl, "construct"):
        return run_construct(args, wl, rank, world, local_rank)
    if hasattr(wl, "functor"):
        return run_functor(args, wl, rank, world, local_rank)
    return run_gpu(args, wl, rank, world, local_rank)


def extra_configs(args, rank, world, local_rank, only=None):
    """{key: line} of EXTRA_CONFIGS (each a complete bench line of its own)."""
    from tbslas_gb300.workloads import make
    out = {}
    for key, name, runner, cap in EXTRA_CONFIGS:
        if only and key not in only:
            continue
        sub = argparse.Namespace(**vars(args))
        if cap is not None:
            sub.steps = min(args.steps, cap)
        t0 = time.perf_counter()
        try:
            line = globals()[runner](sub, make(name), rank, world, local_rank)
        except Exception as e:  # recorded in the line; the headline still prints
            line = {"error": "%s: %s" % (type(e).__name__, e)}
        if line is not None:
            line.pop("metric", None)
            line["wall_s"] = time.perf_counter() - t0
            out[key] = line
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="tree_adaptive_q14")
    ap.add_argument("--extras", default="all",
                    help="with the default workload at N = 1: 'all', 'none' or a comma list "
                         "of %s" % ",".join(k for k, *_ in EXTRA_CONFIGS))
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    rank, world, local_rank = dist_env()
    if args.impl == "reference":
        if rank != 0:
            return
        run_reference(args, args.workload)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    from tbslas_gb300 import build
    build.build()
    from tbslas_gb300.workloads import make
    wl = make(args.workload)
    try:
        line = dispatch(args, wl, rank, world, local_rank)
        if (args.workload == "tree_adaptive_q14" and world == 1 and args.extras != "none"):
            only = None if args.extras == "all" else set(args.extras.split(","))
            extras = extra_configs(args, rank, world, local_rank, only)
            if line is not None:
                line.update(extras)
        if line is not None:
            print(json.dumps(line))
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()

"""The benchmark workloads, built from seeds on the host.

tree_uniform_q8   rotation (omega=2pi) + Gaussian (sigma 0.05 at (0.7,0.5,0.5)) on a
                  uniform depth-4 tree, q=8, dt=0.01, FreeSpace.
tree_adaptive_q14 Taylor-Green velocity + 4 seeded Gaussians (sigma 0.03-0.08,
                  centres U[0.2,0.8]^3) on trees refined to tolerance 1e-6 at
                  depths 3..8, q=14, dt from Chebyshev CFL = dt 2^depth q^2 = 1
                  on the finest leaf (compute_cheb_CFL, src/utils/common.h:246-254),
                  FreeSpace.
grid_periodic_256 divergence-free random Fourier velocity (|k|<=4, amplitudes
                  N(0,1)/|k|^2) on a periodic 256^3 grid, Gaussian blob
                  concentration, dt for a grid CFL of 2.
"""
import math

import numpy as np

from . import fields, trees

SEED = 2024


class TreeWorkload:
    def __init__(self, name, vel_tree, con_tree, q, dt, bc, note):
        self.name, self.q, self.dt, self.bc, self.note = name, q, dt, bc, note
        self.va, self.vd, self.vc = vel_tree
        self.ca, self.cd, self.cc = con_tree

    @property
    def points_per_step(self):
        return len(self.cd) * (self.q + 1) ** 3

    def describe(self):
        return {"workload": self.name, "q": self.q, "dt": self.dt,
                "bc": "periodic" if self.bc else "freespace",
                "vel_leaves": int(len(self.vd)), "con_leaves": int(len(self.cd)),
                "vel_depths": [int(self.vd.min()), int(self.vd.max())],
                "con_depths": [int(self.cd.min()), int(self.cd.max())],
                "departure_points_per_step": int(self.points_per_step), "note": self.note}


def tree_uniform_q8():
    q = 8
    a, d = trees.uniform_tree(4)
    vc = trees.fit(fields.rotation(2 * math.pi), a, d, q, 3)
    cc = trees.fit(fields.gaussian((0.7, 0.5, 0.5), 0.05), a, d, q, 1)
    return TreeWorkload("tree_uniform_q8", (a, d, vc), (a, d, cc), q, 0.01, 0,
                        "uniform depth-4 octree (4096 leaves), q=8, rotation + Gaussian")


def tree_adaptive_q14(seed=SEED, tol=1e-6, depths=(3, 8)):
    q = 14
    lo, hi = depths
    rng = np.random.default_rng(seed)
    blobs = fields.gaussian_blobs(rng, 4)
    ca, cd = trees.adaptive_tree(blobs, q, 1, tol, lo, hi)
    va, vd = trees.adaptive_tree(fields.taylor_green(), q, 3, tol, lo, hi)
    M = None
    cc = trees.fit(blobs, ca, cd, q, 1, M)
    vc = trees.fit(fields.taylor_green(), va, vd, q, 3, M)
    finest = int(max(cd.max(), vd.max()))
    dt = 1.0 / (2.0 ** finest * q * q)
    wl = TreeWorkload("tree_adaptive_q14", (va, vd, vc), (ca, cd, cc), q, dt, 0,
                      "adaptive octrees (tol %g, depth %d..%d), q=14, Taylor-Green + 4 "
                      "Gaussians, CFL=1 on the finest leaf" % (tol, lo, hi))
    wl.blobs = blobs
    return wl


def tree_adaptive_q8_remesh():
    """The adaptive advection loop of the reference's driver
    (SolveSemilagInSitu, then RefineTree and Balance21 after every step,
    src/applications/src/advection.cpp:296-311) on the rotating Gaussian of
    the uniform q = 8 configuration: the concentration tree starts refined for
    the blob (tol 1e-5, depths 3..6) and is re-meshed with the same rule after
    every step while the blob moves through it."""
    q, tol = 8, 1e-5
    va, vd = trees.uniform_tree(4)
    vc = trees.fit(fields.rotation(2 * math.pi), va, vd, q, 3)
    blob = fields.gaussian((0.7, 0.5, 0.5), 0.05)
    ca, cd = trees.adaptive_tree(blob, q, 1, tol, 3, 6)
    cc = trees.fit(blob, ca, cd, q, 1)
    wl = TreeWorkload("tree_adaptive_q8_remesh", (va, vd, vc), (ca, cd, cc), q, 0.01, 0,
                      "rotating Gaussian (sigma 0.05) on an adaptive q=8 concentration tree "
                      "(tol 1e-5, depths 3..6) re-meshed after every step (coarsen, refine, "
                      "2:1 balance); velocity: rotation on the uniform depth-4 tree")
    wl.remesh = (tol, 3, 6)
    return wl


class Bdf2Workload:
    """The BDF2 two-backtrace step (the advection-diffusion driver's step,
    src/applications/src/advdiff-ss.cpp:485-521) on the uniform q = 8
    configuration: rotation on the depth-4 tree, the Gaussian at t - dt and
    t - 2 dt as c_n and c_{n-1}, the three concentration trees of one shape."""

    def __init__(self, q=8, depth=4, dt=0.01, name="bdf2_q8"):
        self.name, self.q, self.dt, self.bc = name, q, dt, 0
        self.a, self.d = trees.uniform_tree(depth)
        self.vc = trees.fit(fields.rotation(2 * math.pi), self.a, self.d, q, 3)
        self.t0 = 2 * dt  # the time of the first step's result

        def blob(time):
            return fields.rotated_gaussian((0.7, 0.5, 0.5), 0.05, 2 * math.pi, time)
        self.c_prev = trees.fit(blob(0.0), self.a, self.d, q, 1)
        self.c_cur = trees.fit(blob(dt), self.a, self.d, q, 1)

    @property
    def points_per_step(self):
        return 2 * len(self.d) * (self.q + 1) ** 3  # two backtraces per target

    def describe(self):
        return {"workload": self.name, "q": self.q, "dt": self.dt, "bc": "freespace",
                "leaves": int(len(self.d)),
                "targets_per_step": int(len(self.d) * (self.q + 1) ** 3),
                "departure_points_per_step": int(self.points_per_step),
                "note": "BDF2 step 4/3 c_n(X1) - 1/3 c_{n-1}(X2), two RK2 backtraces per "
                        "target; uniform depth-4 octree, q=8, rotation + Gaussian"}


class TvWorkload:
    """The uniform q = 8 configuration advected through a time-dependent
    velocity: four rotation trees (omega = 2 pi (1 + k / 4) at times k dt),
    cubic in time (the reference's FieldSetFunctor), one leaf structure -- the
    blended fused step."""

    def __init__(self, q=8, depth=4, dt=0.01, name="tree_uniform_q8_tv"):
        self.name, self.q, self.dt, self.bc = name, q, dt, 0
        self.a, self.d = trees.uniform_tree(depth)
        self.times = [k * dt for k in range(4)]
        self.vcs = [trees.fit(fields.rotation(2 * math.pi * (1 + k / 4)), self.a, self.d, q, 3)
                    for k in range(4)]
        self.cc = trees.fit(fields.gaussian((0.7, 0.5, 0.5), 0.05), self.a, self.d, q, 1)
        self.timestep = 2  # steps query t in [times[1], times[2]]

    @property
    def points_per_step(self):
        return len(self.d) * (self.q + 1) ** 3

    def describe(self):
        return {"workload": self.name, "q": self.q, "dt": self.dt, "bc": "freespace",
                "leaves": int(len(self.d)), "velocity_trees": 4,
                "departure_points_per_step": int(self.points_per_step),
                "note": "uniform depth-4 octree, q=8, Gaussian; velocity cubic in time over four "
                        "rotation trees (FieldSetFunctor), blended per RK2 stage"}


class GridWorkload:
    def __init__(self, n, seed=SEED):
        rng = np.random.default_rng(seed)
        self.name = "grid_periodic_%d" % n
        self.n = n
        self.vel = fields.fourier_velocity_grid(rng, n)
        self.con = fields.periodic_blob_grid(n, (0.45, 0.5, 0.55), 0.1)
        self.dt = 2.0 / n / float(np.abs(self.vel).max())
        self.bc = 1

    @property
    def points_per_step(self):
        return self.n ** 3

    def describe(self):
        return {"workload": self.name, "grid": self.n, "dt": self.dt, "bc": "periodic",
                "departure_points_per_step": self.points_per_step,
                "note": "tricubic SL step on a periodic grid, random divergence-free "
                        "Fourier velocity |k|<=4, Gaussian blob"}


def fourier_fitter(modes, q, M):
    """Fits the Fourier velocity on every leaf: torch on the GPU when one is
    present (the point count runs into the millions), numpy otherwise."""
    ks, A, B = modes
    coef = A - 1j * B

    try:
        import torch
        use_gpu = torch.cuda.is_available()
    except ImportError:
        use_gpu = False

    def fit_gpu(anchor, depth):
        import torch
        dev = "cuda"
        nodes = torch.from_numpy(api_nodes(q)).to(dev)                      # [Np, 3]
        a = torch.from_numpy(anchor).to(dev)
        h = torch.from_numpy(np.ldexp(1.0, -depth.astype(np.int64))).to(dev)
        L, Np = len(depth), nodes.shape[0]
        out = torch.empty((L, 3, M.shape[1]), dtype=torch.float64, device=dev)
        Mt = torch.from_numpy(M).to(dev)
        kt = torch.from_numpy(ks).to(dev)
        ct = torch.from_numpy(coef).to(dev)                                # [m, 3]
        step = max(1, (1 << 21) // Np)
        for l0 in range(0, L, step):
            l1 = min(L, l0 + step)
            pts = (a[l0:l1, None, :] + h[l0:l1, None, None] * nodes[None]).reshape(-1, 3)
            ph = 2 * math.pi * (pts @ kt.T)                                  # [n, m]
            v = torch.cos(ph) @ ct.real + torch.sin(ph) @ (-ct.imag)        # [n, 3]
            vals = v.reshape(l1 - l0, Np, 3).permute(0, 2, 1).reshape(-1, Np)
            out[l0:l1] = (vals @ Mt).reshape(l1 - l0, 3, -1)
        return out.cpu().numpy()

    def fit_cpu(anchor, depth):
        fn = fields.fourier_velocity_from_modes(ks, A, B)
        return trees.fit(fn, anchor, depth, q, 3, M)

    return fit_gpu if use_gpu else fit_cpu


def api_nodes(q):
    return trees.cheb_nodes(q)


class BatchWorkload:
    """Independent problems of uneven size: degree q ~ U{qlo..qhi}, maximum
    depth ~ U{dlo..dhi}; velocity = random divergence-free Fourier field
    (|k| <= 4, amplitudes N(0,1)/|k|^2), concentration = 1..8 Gaussian blobs;
    both trees refined by the coefficient-tail rule at tolerance `tol`
    (minimum depth 2); periodic; dt for Chebyshev CFL 1 on the finest leaf."""

    def __init__(self, n=64, seed=SEED, qs=(8, 14), depths=(4, 7), tol=1e-5, min_depth=2,
                 name="batched_64", qlist=None):
        rng = np.random.default_rng(seed)
        self.name, self.bc, self.problems = name, 1, []
        Ms = {}
        for i in range(n):
            q = int(rng.integers(qs[0], qs[1] + 1))
            if qlist is not None:
                q = int(qlist[i % len(qlist)])
            dmax = int(rng.integers(depths[0], depths[1] + 1))
            M = Ms.setdefault(q, trees.pt2coeff(q))
            modes = fields.fourier_modes(rng)
            blobs = fields.gaussian_blobs(rng, int(rng.integers(1, 9)))
            vfit = fourier_fitter(modes, q, M)
            va, vd = trees.adaptive_tree(None, q, 3, tol, min_depth, dmax, periodic=True, M=M,
                                         fitter=vfit)
            ca, cd = trees.adaptive_tree(blobs, q, 1, tol, min_depth, dmax, periodic=True, M=M)
            vc = vfit(va, vd)
            cc = trees.fit(blobs, ca, cd, q, 1, M)
            finest = int(max(vd.max(), cd.max()))
            dt = 1.0 / (2.0 ** finest * q * q)
            self.problems.append(dict(q=q, dmax=dmax, va=va, vd=vd, vc=vc, ca=ca, cd=cd, cc=cc,
                                      dt=dt))

    @property
    def points_per_step(self):
        return sum(len(p["cd"]) * (p["q"] + 1) ** 3 for p in self.problems)

    def describe(self):
        qs = [p["q"] for p in self.problems]
        return {"workload": self.name, "problems": len(self.problems),
                "q_range": [min(qs), max(qs)],
                "con_leaves": int(sum(len(p["cd"]) for p in self.problems)),
                "vel_leaves": int(sum(len(p["vd"]) for p in self.problems)),
                "departure_points_per_step": int(self.points_per_step),
                "bc": "periodic", "note": self.__doc__.split("\n")[0]}


class AdjointWorkload:
    """Uniform depth-5 octree (32768 leaves), q = 8, stationary Taylor-Green
    velocity, Gaussian c0 (sigma 0.08 at (0.45, 0.5, 0.5)), 20 SL steps of dt
    0.004; the observation is the advected field of a seeded perturbed Gaussian;
    J = 1/2 sum over leaf nodes (c(T) - c_obs)^2."""

    def __init__(self, depth=5, q=8, steps=20, dt=0.004, seed=SEED, name="adjoint_q8"):
        rng = np.random.default_rng(seed)
        self.name, self.q, self.steps, self.dt, self.bc = name, q, steps, dt, 0
        self.depth = depth
        self.a, self.d = trees.uniform_tree(depth)
        self.vc = trees.fit(fields.taylor_green(), self.a, self.d, q, 3)
        self.c0 = trees.fit(fields.gaussian((0.45, 0.5, 0.5), 0.08), self.a, self.d, q, 1)
        shift = rng.uniform(-0.02, 0.02, size=3)
        self.c0_obs = trees.fit(fields.gaussian((0.45 + shift[0], 0.5 + shift[1], 0.5 + shift[2]),
                                                0.08 * (1 + rng.uniform(-0.1, 0.1))),
                                self.a, self.d, q, 1)

    @property
    def points_per_step(self):
        return len(self.d) * (self.q + 1) ** 3

    def describe(self):
        return {"workload": self.name, "q": self.q, "leaves": int(len(self.d)), "steps": self.steps,
                "dt": self.dt, "bc": "freespace",
                "departure_points_per_step": int(self.points_per_step),
                "note": "uniform depth-%d octree, q = %d, stationary Taylor-Green velocity, "
                        "%d SL steps of dt %g" % (self.depth, self.q, self.steps, self.dt)}


def make(name):
    if name == "tree_uniform_q8":
        return tree_uniform_q8()
    if name == "tree_adaptive_q14":
        return tree_adaptive_q14()
    if name == "tree_adaptive_q8_remesh":
        return tree_adaptive_q8_remesh()
    if name == "bdf2_q8":
        return Bdf2Workload()
    if name == "tree_uniform_q8_tv":
        return TvWorkload()
    if name == "functor_q14":
        # config 2 through the reference's separate calls (collect, ComputeTrajRK2,
        # the EvalTree functor, SetTreeGridValues) instead of the fused step
        wl = tree_adaptive_q14()
        wl.name = "functor_q14"
        wl.functor = True
        return wl
    if name == "construct_q14":
        wl = tree_adaptive_q14()
        wl.name = "construct_q14"
        wl.construct = (1e-6, 3, 8)
        return wl
    if name == "adjoint_q8":
        return AdjointWorkload()
    if name == "adjoint_q8_d4":
        return AdjointWorkload(depth=4, steps=4, name=name)
    if name == "batched_64":
        return BatchWorkload()
    if name.startswith("grid_periodic_"):
        return GridWorkload(int(name.rsplit("_", 1)[1]))
    raise ValueError("unknown workload %r" % name)

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


def tree_adaptive_q14(seed=SEED):
    q, tol = 14, 1e-6
    rng = np.random.default_rng(seed)
    blobs = fields.gaussian_blobs(rng, 4)
    ca, cd = trees.adaptive_tree(blobs, q, 1, tol, 3, 8)
    va, vd = trees.adaptive_tree(fields.taylor_green(), q, 3, tol, 3, 8)
    M = None
    cc = trees.fit(blobs, ca, cd, q, 1, M)
    vc = trees.fit(fields.taylor_green(), va, vd, q, 3, M)
    finest = int(max(cd.max(), vd.max()))
    dt = 1.0 / (2.0 ** finest * q * q)
    return TreeWorkload("tree_adaptive_q14", (va, vd, vc), (ca, cd, cc), q, dt, 0,
                        "adaptive octrees (tol 1e-6, depth 3..8), q=14, Taylor-Green + 4 "
                        "Gaussians, CFL=1 on the finest leaf")


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


def make(name):
    if name == "tree_uniform_q8":
        return tree_uniform_q8()
    if name == "tree_adaptive_q14":
        return tree_adaptive_q14()
    if name.startswith("grid_periodic_"):
        return GridWorkload(int(name.rsplit("_", 1)[1]))
    raise ValueError("unknown workload %r" % name)

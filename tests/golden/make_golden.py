"""Writes the golden fixtures of tests/golden/ (run from the repository root:
python tests/golden/make_golden.py).

The reference ships no golden vectors and cannot be built here (PVFMM is not
vendored), so these fixtures are the oracle's outputs on small seeded cases
of every row of the path: a tree step, departure points, a periodic grid
step, a re-meshing, a BDF2 step and a time-dependent step.  They pin the
oracle against later changes and give the GPU parity tests fixed vectors
(tests/test_golden.py)."""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as ora  # noqa: E402
from oracle import remesh as rm  # noqa: E402
from tbslas_gb300 import fields, trees  # noqa: E402


def main():
    out = {}
    # tree step: rotation + Gaussian, uniform depth 2, q = 6
    q = 6
    a, d = trees.uniform_tree(2)
    vc = trees.fit(fields.rotation(2 * math.pi), a, d, q, 3)
    cc = trees.fit(fields.gaussian((0.7, 0.5, 0.5), 0.08), a, d, q, 1)
    vel = dict(anchor=a, depth=d, q=q, dof=3, coeff=vc)
    con = dict(anchor=a, depth=d, q=q, dof=1, coeff=cc)
    out["step_anchor"], out["step_depth"], out["step_vc"], out["step_cc"] = a, d, vc, cc
    out["step_out"] = ora.semilag_in_situ(vel, con, 1, 0.01)
    # departure points of seeded points through Taylor-Green (free space)
    vt = trees.fit(fields.taylor_green(), a, d, 5, 3)
    pts = np.random.default_rng(1).uniform(0, 1, (500, 3))
    out["traj_vc"], out["traj_pts"] = vt, pts
    out["traj_out"] = ora.traj_rk2(a, d, 5, vt, pts, 0.02, 0.0, 2)
    # periodic grid step, N = 16
    rng = np.random.default_rng(16)
    gv = fields.fourier_velocity_grid(rng, 16)
    gc = fields.periodic_blob_grid(16)
    out["grid_vel"], out["grid_con"] = gv, gc
    out["grid_out"] = ora.semilag_grid(gv, gc, 16, 1.0 / 16, 1, True)
    # re-meshing of the step's result
    ra, rd, rc = rm.remesh(a, d, q, out["step_out"], 1e-3, 1, 3)
    out["remesh_anchor"], out["remesh_depth"], out["remesh_coeff"] = ra, rd, rc
    # BDF2 step (c_{n-1} = the initial field, c_n = the step's result)
    cur = dict(anchor=a, depth=d, q=q, dof=1, coeff=out["step_out"])
    out["bdf2_out"] = ora.semilag_bdf2(vel, con, cur, dict(anchor=a, depth=d, q=q), 0.02, 0.01)
    # time-dependent step through four generic Fourier velocity trees, cubic
    # in time, periodic (no velocity component vanishes on a face, where the
    # coefficient blend of the fast path and the reference's value blend could
    # round to different sides)
    a1, d1 = trees.uniform_tree(1)
    vcs = []
    for k in range(4):
        fn = fields.fourier_velocity(np.random.default_rng(40 + k), 2)
        vcs.append(trees.fit(lambda p, fn=fn: 0.5 * fn(p), a1, d1, q, 3))
    c1 = trees.fit(fields.gaussian((0.55, 0.5, 0.45), 0.12), a1, d1, q, 1)
    out["tv_anchor"], out["tv_depth"], out["tv_cc"] = a1, d1, c1
    out["tv_vcs"] = np.stack(vcs)
    out["tv_out"] = ora.semilag_in_situ_tv([dict(anchor=a1, depth=d1, q=q, dof=3, coeff=v)
                                            for v in vcs],
                                           dict(anchor=a1, depth=d1, q=q, dof=1, coeff=c1), 2,
                                           0.01, 1, True, times=[0.0, 0.01, 0.02, 0.03])
    np.savez_compressed(os.path.join(HERE, "path_q6.npz"), **out)


if __name__ == "__main__":
    main()

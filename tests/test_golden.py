"""Golden fixtures (tests/golden/path_q6.npz, written by
tests/golden/make_golden.py from the oracle): the oracle still reproduces
them (CPU), and the device path matches them (GPU) -- a tree step, departure
points, a periodic grid step, a re-meshing, a BDF2 step and a time-dependent
step."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def g():
    return dict(np.load(os.path.join(HERE, "golden", "path_q6.npz")))


def _rel(x, ref):
    return float(np.abs(np.asarray(x) - ref).max() / max(np.abs(ref).max(), 1e-300))


def test_oracle_reproduces_the_fixtures(ora, g):
    from oracle import remesh as rm
    a, d, q = g["step_anchor"], g["step_depth"], 6
    vel = dict(anchor=a, depth=d, q=q, dof=3, coeff=g["step_vc"])
    con = dict(anchor=a, depth=d, q=q, dof=1, coeff=g["step_cc"])
    assert _rel(ora.semilag_in_situ(vel, con, 1, 0.01), g["step_out"]) <= 1e-14
    tr = ora.traj_rk2(a, d, 5, g["traj_vc"], g["traj_pts"], 0.02, 0.0, 2)
    assert np.abs(tr - g["traj_out"]).max() <= 1e-15
    assert _rel(ora.semilag_grid(g["grid_vel"], g["grid_con"], 16, 1.0 / 16, 1, True),
                g["grid_out"]) <= 1e-14
    ra, rd, rc = rm.remesh(a, d, q, g["step_out"], 1e-3, 1, 3)
    assert np.array_equal(rd, g["remesh_depth"]) and np.array_equal(ra, g["remesh_anchor"])
    assert _rel(rc, g["remesh_coeff"]) <= 1e-14


@pytest.mark.gpu
def test_device_matches_the_fixtures(ctx, g):
    import torch
    import tbslas_gb300 as tb
    a, d, q = g["step_anchor"], g["step_depth"], 6
    tv = tb.Tree(ctx, a, d, q, 3, g["step_vc"])
    tc = tb.Tree(ctx, a, d, q, 1, g["step_cc"])
    vf = tb.NodeFieldFunctor(tv)
    tb.solve_semilag_in_situ(vf, tc, 1, 0.01)
    assert _rel(tc.get_coeffs(), g["step_out"]) <= 1e-12
    # departure points: bit-identical arithmetic to the oracle
    t5 = tb.Tree(ctx, a, d, 5, 3, g["traj_vc"])
    x = torch.from_numpy(g["traj_pts"]).cuda()
    dep = tb.compute_traj_rk2(tb.NodeFieldFunctor(t5), x, 0.02, 0.0, 2).cpu().numpy()
    assert np.abs(dep - g["traj_out"]).max() <= 1e-15
    out = tb.semilag_grid(ctx, g["grid_vel"], g["grid_con"], 16, 1.0 / 16, 1, tb.Periodic)
    assert _rel(np.asarray(out).reshape(-1), g["grid_out"].reshape(-1)) <= 1e-12
    # re-meshing of the step's result
    tr = tb.Tree(ctx, a, d, q, 1, g["step_out"])
    tr.remesh(1e-3, 1, 3)
    ra, rd = tr.leaves()
    assert np.array_equal(rd, g["remesh_depth"]) and np.array_equal(ra, g["remesh_anchor"])
    assert _rel(tr.get_coeffs(), g["remesh_coeff"]) <= 1e-12
    # BDF2: c_{n-1} the initial field, c_n the step's result
    tp = tb.Tree(ctx, a, d, q, 1, g["step_cc"])
    tcur = tb.Tree(ctx, a, d, q, 1, g["step_out"])
    tn = tb.Tree(ctx, a, d, q, 1)
    tb.solve_semilag_bdf2(vf, tp, tcur, tn, 0.02, 0.01)
    assert _rel(tn.get_coeffs(), g["bdf2_out"]) <= 1e-12
    # time-dependent velocity, cubic in time over four trees
    a1, d1 = g["tv_anchor"], g["tv_depth"]
    vts = [tb.Tree(ctx, a1, d1, q, 3, v) for v in g["tv_vcs"]]
    t2 = tb.Tree(ctx, a1, d1, q, 1, g["tv_cc"])
    tb.solve_semilag_in_situ_tv(tb.FieldSetFunctor(vts, [0.0, 0.01, 0.02, 0.03], tb.Periodic),
                                t2, 2, 0.01)
    assert _rel(t2.get_coeffs(), g["tv_out"]) <= 1e-12
    for t in [tv, tc, t5, tr, tp, tcur, tn, t2] + vts:
        t.close()

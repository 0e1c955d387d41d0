"""Device re-meshing (tbslas_tree_remesh: coarsen one level, refine, 2:1
balance -- the reference's RefineTree + Balance21 after a step,
src/applications/src/advection.cpp:305-311) against the oracle's
restatement: the same leaves, coefficients within 1e-12 relative (untouched
leaves bit for bit), and the re-meshed tree usable by the SL step."""
import numpy as np
import pytest

import tbslas_gb300 as tb
from tbslas_gb300 import fields, trees

pytestmark = pytest.mark.gpu


def _moved_blob(q, tol):
    """Tree refined for a blob at x = 0.3 carrying a blob at x = 0.62: the
    re-meshing coarsens around the first and refines around the second."""
    a, d = trees.adaptive_tree(fields.gaussian((0.3, 0.5, 0.5), 0.06), q, 1, tol, 2, 5)
    c = trees.fit(fields.gaussian((0.62, 0.52, 0.47), 0.06), a, d, q, 1)
    return a, d, c


def _check(ctx, a, d, q, c, tol, lo, hi, bc):
    from oracle import remesh as rm
    t = tb.Tree(ctx, a, d, q, 1, c)
    st = t.remesh(tol, lo, hi, bc)
    ga, gd = t.leaves()
    gc = t.get_coeffs()
    ra, rd, rc, org = rm.remesh(a, d, q, c, tol, lo, hi, bc == tb.Periodic, origin=True)
    assert np.array_equal(gd, rd) and np.array_equal(ga, ra)
    assert np.abs(gc - rc).max() <= 1e-12 * np.abs(rc).max()
    # leaves no rule touched keep their coefficients bit for bit
    kept = org >= 0
    assert kept.any()
    assert np.array_equal(gc[kept], c[org[kept]])
    assert st["leaves"] == gd.size
    return t, st


@pytest.mark.parametrize("q", [4, 6])
def test_remesh_matches_oracle(ctx, q):
    tol = 1e-4
    a, d, c = _moved_blob(q, tol)
    t, st = _check(ctx, a, d, q, c, tol, 2, 5, tb.FreeSpace)
    assert st["merged"] > 0 and st["split"] > 0
    t.close()


@pytest.mark.parametrize("bc", [tb.FreeSpace, tb.Periodic])
def test_balance_matches_oracle(ctx, bc):
    q = 3
    a, d = trees.uniform_tree(1)
    for _ in range(4):
        k = int(np.argmax(d == d.max()))  # the leaf at the origin
        a = np.concatenate([a[:k], trees.split(a[k:k + 1], d[k:k + 1])[0], a[k + 1:]])
        d = np.concatenate([d[:k], np.full(8, d[k] + 1, dtype=np.int32), d[k + 1:]])
        a, d = trees.sort_leaves(a, d)
    c = trees.fit(fields.gaussian((0.5, 0.5, 0.5), 0.2), a, d, q, 1)
    t, st = _check(ctx, a, d, q, c, np.inf, 5, 5, bc)
    assert (st["balanced"] > 0) == (bc == tb.Periodic)
    t.close()


def test_refinement_keeps_the_function(ctx):
    """Split leaves carry the restriction of their parent: the tree evaluates
    to the same values (up to the fits' rounding) everywhere."""
    import torch
    q = 5
    a, d = trees.uniform_tree(2)
    c = trees.fit(fields.gaussian((0.4, 0.55, 0.5), 0.1), a, d, q, 1)
    t0 = tb.Tree(ctx, a, d, q, 1, c)
    t1 = tb.Tree(ctx, a, d, q, 1, c)
    st = t1.remesh(2e-3, 2, 4)
    assert st["split"] > 0 and st["merged"] == 0
    pts = torch.from_numpy(np.random.default_rng(0).uniform(0, 1, (20000, 3))).cuda()
    v0 = tb.NodeFieldFunctor(t0)(pts).cpu().numpy()
    v1 = tb.NodeFieldFunctor(t1)(pts).cpu().numpy()
    assert np.abs(v0 - v1).max() <= 1e-13 * np.abs(v0).max()
    t0.close()
    t1.close()


def test_step_after_remesh_matches_oracle(ctx, ora):
    """Advect, re-mesh, advect: the second step runs on the re-meshed tree
    (rebuilt keys, geometry and lookup table) and matches the oracle's step on
    the oracle's re-meshed tree."""
    from oracle import remesh as rm
    q, tol = 5, 1e-4
    av, dv = trees.uniform_tree(2)
    vc = trees.fit(fields.rotation(2 * np.pi), av, dv, q, 3)
    tv = tb.Tree(ctx, av, dv, q, 3, vc)
    a, d, c = _moved_blob(q, tol)
    tc = tb.Tree(ctx, a, d, q, 1, c)
    ctx.sums = tb.SUMS_FP64
    try:
        vf = tb.NodeFieldFunctor(tv)
        tb.solve_semilag_in_situ(vf, tc, 1, 0.02)
        c1 = tc.get_coeffs()
        tc.remesh(tol, 2, 5)
        tb.solve_semilag_in_situ(vf, tc, 2, 0.02)
        got_a, got_d = tc.leaves()
        got = tc.get_coeffs()
    finally:
        ctx.sums = tb.SUMS_FP64  # the library default
    vel = dict(anchor=av, depth=dv, q=q, dof=3, coeff=vc)
    ref1 = ora.semilag_in_situ(vel, dict(anchor=a, depth=d, q=q, dof=1, coeff=c), 1, 0.02)
    assert np.abs(c1 - ref1).max() <= 1e-12 * np.abs(ref1).max()
    ra, rd, rc = rm.remesh(a, d, q, c1, tol, 2, 5)
    assert np.array_equal(got_a, ra) and np.array_equal(got_d, rd)
    ref2 = ora.semilag_in_situ(vel, dict(anchor=ra, depth=rd, q=q, dof=1, coeff=rc), 2, 0.02)
    assert np.abs(got - ref2).max() <= 1e-12 * np.abs(ref2).max()
    tv.close()
    tc.close()


def test_remesh_velocity_tree_matches_oracle(ctx):
    """A dof-3 tree (the driver also re-meshes its velocity tree after each
    step): the tail sums over the three components."""
    q, tol = 5, 2e-3
    a, d = trees.adaptive_tree(fields.gaussian((0.5, 0.5, 0.5), 0.1), q, 1, 1e-3, 1, 3)
    vfn = fields.fourier_velocity(np.random.default_rng(8), 2)
    c = trees.fit(lambda p: 0.3 * vfn(p), a, d, q, 3)
    from oracle import remesh as rm
    t = tb.Tree(ctx, a, d, q, 3, c)
    t.remesh(tol, 1, 4, tb.Periodic)
    ga, gd = t.leaves()
    ra, rd, rc = rm.remesh(a, d, q, c, tol, 1, 4, True)
    assert np.array_equal(gd, rd) and np.array_equal(ga, ra)
    assert np.abs(t.get_coeffs() - rc).max() <= 1e-12 * np.abs(rc).max()
    t.close()

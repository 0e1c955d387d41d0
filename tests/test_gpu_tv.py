"""In-situ step through a time-dependent velocity (tbslas_semilag_in_situ_tv)
against the oracle's restatement of the reference's FieldSetFunctor (cubic in
time over four trees) and FieldExtrapFunctor (1.5 v_n - 0.5 v_{n-1}) as
IntegrateRK2 queries them: velocity trees of one leaf structure (the blended
fused step) and of different structures (per-tree evaluation), both sum
modes, to 1e-12 relative."""
import numpy as np
import pytest

import tbslas_gb300 as tb
from tbslas_gb300 import fields, trees

pytestmark = pytest.mark.gpu


def _vel_fn(k, bc):
    """Four related velocity fields (a time series)."""
    if bc == tb.Periodic:
        base = fields.fourier_velocity(np.random.default_rng(20 + k))
        return lambda p: 0.4 * base(p)
    tg = fields.taylor_green()
    rot = fields.rotation(2 * np.pi)
    s = 0.2 * k
    return lambda p: (1.0 - s) * tg(p) + s * rot(p)


def _trees(ctx, q, bc, same):
    out, dicts = [], []
    for k in range(4):
        if same:
            a, d = trees.uniform_tree(2)
        else:
            a, d = trees.adaptive_tree(fields.gaussian((0.3 + 0.1 * k, 0.5, 0.5), 0.1), q, 1,
                                       1e-3, 1, 3)
        c = trees.fit(_vel_fn(k, bc), a, d, q, 3)
        out.append(tb.Tree(ctx, a, d, q, 3, c))
        dicts.append(dict(anchor=a, depth=d, q=q, dof=3, coeff=c))
    return out, dicts


def _con(ctx, q):
    a, d = trees.adaptive_tree(fields.gaussian((0.5, 0.45, 0.55), 0.1), q, 1, 1e-3, 1, 3)
    c = trees.fit(fields.gaussian((0.5, 0.45, 0.55), 0.1), a, d, q, 1)
    return tb.Tree(ctx, a, d, q, 1, c), dict(anchor=a, depth=d, q=q, dof=1, coeff=c)


@pytest.mark.parametrize("same", [True, False])
@pytest.mark.parametrize("bc", [tb.FreeSpace, tb.Periodic])
@pytest.mark.parametrize("mode", ["df", "fp64"])
@pytest.mark.parametrize("kind", ["set", "extrap"])
def test_tv_matches_oracle(ctx, ora, same, bc, mode, kind):
    q, ts, dt = 5, 3, 0.02
    vt, vd = _trees(ctx, q, bc, same)
    tc, cd = _con(ctx, q)
    times = [0.0, 0.02, 0.04, 0.06]
    if kind == "set":
        f = tb.FieldSetFunctor(vt, times, bc)
        ref = ora.semilag_in_situ_tv(vd, cd, ts, dt, 1, bc == tb.Periodic, times=times)
    else:
        f = tb.FieldExtrapFunctor(vt[0], vt[1], bc)
        ref = ora.semilag_in_situ_tv([vd[1], vd[0]], cd, ts, dt, 1, bc == tb.Periodic)
    ctx.sums = tb.SUMS_FP64 if mode == "fp64" else tb.SUMS_DOUBLE_FLOAT
    try:
        tb.solve_semilag_in_situ_tv(f, tc, ts, dt)
        got = tc.get_coeffs()
    finally:
        ctx.sums = tb.SUMS_FP64  # the library default
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    for x in vt + [tc]:
        x.close()


@pytest.mark.parametrize("j", [0, 1, 2, 3])
@pytest.mark.parametrize("bc", [tb.FreeSpace, tb.Periodic])
def test_one_hot_weights_equal_the_plain_step(ctx, j, bc):
    """Four trees of one leaf structure, weight 1 on tree j and 0 on the
    others at both stages: the FP64 step (one node-grid walk and one leaf
    lookup for all four trees) equals the plain step through tree j bit for
    bit -- each tree's values at the nodes and at the midpoints are the ones
    its own evaluation gives."""
    q = 6
    vt, _ = _trees(ctx, q, bc, True)
    tc, cd = _con(ctx, q)
    t2 = tb.Tree(ctx, cd["anchor"], cd["depth"], q, 1, cd["coeff"])
    w = np.zeros(8)
    w[j] = w[4 + j] = 1.0

    class OneHot:
        pass
    f = OneHot()
    f.bc = bc
    f.stage_weights = lambda timestep, dt, nrk: (vt, w)
    tb.solve_semilag_in_situ_tv(f, tc, 1, 0.02)
    tb.solve_semilag_in_situ(tb.NodeFieldFunctor(vt[j], bc), t2, 1, 0.02)
    assert np.array_equal(tc.get_coeffs(), t2.get_coeffs())
    for x in vt + [tc, t2]:
        x.close()


def _same_count_other_leaves():
    """64 leaves like uniform_tree(2), but not its leaves: the depth-1 leaf
    at the origin kept, the other seven split, the depth-2 leaf at
    (3/4, 3/4, 3/4) split again."""
    anchor, depth = [np.zeros(3)], [1]
    for i in range(1, 8):
        a1 = np.array([i & 1, (i >> 1) & 1, (i >> 2) & 1]) / 2.0
        for j in range(8):
            a2 = a1 + np.array([j & 1, (j >> 1) & 1, (j >> 2) & 1]) / 4.0
            if np.all(a2 == 0.75):
                for k in range(8):
                    anchor.append(a2 + np.array([k & 1, (k >> 1) & 1, (k >> 2) & 1]) / 8.0)
                    depth.append(3)
            else:
                anchor.append(a2)
                depth.append(2)
    return trees.sort_leaves(np.array(anchor), np.array(depth, dtype=np.int32))


def test_tv_structure_check_follows_the_trees(ctx, ora):
    """The velocity set's leaf comparison is kept per set of leaf lists: a
    set of one structure, then the same set with one tree swapped for a tree
    of as many leaves but other ones, then the first set again -- each step
    against the oracle."""
    q, ts, dt, bc = 5, 3, 0.02, tb.FreeSpace
    times = [0.0, 0.02, 0.04, 0.06]
    vt, vd = _trees(ctx, q, bc, True)
    a2, d2 = _same_count_other_leaves()
    assert len(d2) == vt[1].n_leaves
    c2 = trees.fit(_vel_fn(1, bc), a2, d2, q, 3)
    other = tb.Tree(ctx, a2, d2, q, 3, c2)
    od = dict(anchor=a2, depth=d2, q=q, dof=3, coeff=c2)
    for vs, ds in ((vt, vd), ([vt[0], other, vt[2], vt[3]], [vd[0], od, vd[2], vd[3]]),
                   (vt, vd)):
        tc, cd = _con(ctx, q)
        ref = ora.semilag_in_situ_tv(ds, cd, ts, dt, 1, False, times=times)
        tb.solve_semilag_in_situ_tv(tb.FieldSetFunctor(vs, times, bc), tc, ts, dt)
        got = tc.get_coeffs()
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
        tc.close()
    for x in vt + [other]:
        x.close()


@pytest.mark.parametrize("q", [9, 11, 14])
@pytest.mark.parametrize("bc", [tb.FreeSpace, tb.Periodic])
def test_tv_shared_leaves_high_degree_matches_oracle(ctx, ora, q, bc):
    """FP64 step through four velocity trees of one leaf structure at the
    degrees of each instantiation unit (one lookup per point for all trees):
    against the oracle, which evaluates every tree on its own."""
    ts, dt = 3, 1.0 / (2 * q * q)
    vt, vd = [], []
    a, d = trees.uniform_tree(1)
    for k in range(4):
        c = trees.fit(_vel_fn(k, bc), a, d, q, 3)
        vt.append(tb.Tree(ctx, a, d, q, 3, c))
        vd.append(dict(anchor=a, depth=d, q=q, dof=3, coeff=c))
    g = fields.gaussian((0.5, 0.45, 0.55), 0.15)
    cc = trees.fit(g, a, d, q, 1)
    tc = tb.Tree(ctx, a, d, q, 1, cc)
    times = [0.0, 0.02, 0.04, 0.06]
    ref = ora.semilag_in_situ_tv(vd, dict(anchor=a, depth=d, q=q, dof=1, coeff=cc), ts, dt, 1,
                                 bc == tb.Periodic, times=times)
    tb.solve_semilag_in_situ_tv(tb.FieldSetFunctor(vt, times, bc), tc, ts, dt)
    got = tc.get_coeffs()
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    for x in vt + [tc]:
        x.close()


def test_tv_two_substeps_matches_oracle(ctx, ora):
    q, ts, dt = 4, 2, 0.03
    vt, vd = _trees(ctx, q, tb.FreeSpace, True)
    tc, cd = _con(ctx, q)
    times = [0.0, 0.02, 0.04, 0.06]
    tb.solve_semilag_in_situ_tv(tb.FieldSetFunctor(vt, times), tc, ts, dt, 2)
    ref = ora.semilag_in_situ_tv(vd, cd, ts, dt, 2, False, times=times)
    got = tc.get_coeffs()
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("mode", ["df", "fp64"])
def test_single_tree_weight_one_is_the_plain_step(ctx, mode):
    """One tree with weight 1 at both stages: the blended coefficients are the
    tree's own, so the step equals tbslas_semilag_in_situ bit for bit."""
    q = 6
    vt, _ = _trees(ctx, q, tb.FreeSpace, True)
    tc, cd = _con(ctx, q)
    t2 = tb.Tree(ctx, cd["anchor"], cd["depth"], q, 1, cd["coeff"])

    class One:
        bc = tb.FreeSpace

        def stage_weights(self, timestep, dt, nrk):
            return [vt[0]], np.ones(2 * nrk)
    ctx.sums = tb.SUMS_FP64 if mode == "fp64" else tb.SUMS_DOUBLE_FLOAT
    try:
        tb.solve_semilag_in_situ_tv(One(), tc, 1, 0.02)
        tb.solve_semilag_in_situ(tb.NodeFieldFunctor(vt[0]), t2, 1, 0.02)
        assert np.array_equal(tc.get_coeffs(), t2.get_coeffs())
    finally:
        ctx.sums = tb.SUMS_FP64  # the library default

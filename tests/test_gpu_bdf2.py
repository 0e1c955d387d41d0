"""BDF2 two-backtrace SL step (tbslas_semilag_bdf2; the advection-diffusion
driver's step, src/applications/src/advdiff-ss.cpp:485-521) against the
oracle's composition of ComputeTrajRK2 / EvalTree / SetTreeGridValues: three
concentration trees of different shapes, free-space and periodic, both sum
modes, to 1e-12 relative."""
import numpy as np
import pytest

import tbslas_gb300 as tb
from tbslas_gb300 import fields, trees

pytestmark = pytest.mark.gpu


def _setup(q, bc):
    rng = np.random.default_rng(11)
    if bc == tb.Periodic:
        fn = fields.fourier_velocity(rng)
        vel_fn = lambda p: 0.5 * fn(p)  # noqa: E731
    else:
        vel_fn = fields.taylor_green()
    av, dv = trees.uniform_tree(2)
    vc = trees.fit(vel_fn, av, dv, q, 3)
    g1 = fields.gaussian((0.45, 0.5, 0.55), 0.1)
    g0 = fields.gaussian((0.47, 0.5, 0.53), 0.1)
    ap, dp = trees.adaptive_tree(g0, q, 1, 1e-3, 1, 3)
    ac, dc = trees.adaptive_tree(g1, q, 1, 1e-3, 1, 3)
    an, dn = trees.adaptive_tree(g1, q, 1, 3e-4, 1, 3)
    return ((av, dv, vc), (ap, dp, trees.fit(g0, ap, dp, q, 1)),
            (ac, dc, trees.fit(g1, ac, dc, q, 1)), (an, dn))


@pytest.mark.parametrize("bc", [tb.FreeSpace, tb.Periodic])
@pytest.mark.parametrize("mode", ["df", "fp64"])
def test_bdf2_matches_oracle(ctx, ora, bc, mode):
    q, t, dt = 6, 0.06, 0.02
    (av, dv, vc), (ap, dp, cp), (ac, dc, cc), (an, dn) = _setup(q, bc)
    tv = tb.Tree(ctx, av, dv, q, 3, vc)
    tp, tcur = tb.Tree(ctx, ap, dp, q, 1, cp), tb.Tree(ctx, ac, dc, q, 1, cc)
    tn = tb.Tree(ctx, an, dn, q, 1)
    ctx.sums = tb.SUMS_FP64 if mode == "fp64" else tb.SUMS_DOUBLE_FLOAT
    try:
        tb.solve_semilag_bdf2(tb.NodeFieldFunctor(tv, bc), tp, tcur, tn, t, dt)
        got = tn.get_coeffs()
    finally:
        ctx.sums = tb.SUMS_FP64  # the library default
    per = bc == tb.Periodic
    ref = ora.semilag_bdf2(dict(anchor=av, depth=dv, q=q, dof=3, coeff=vc),
                           dict(anchor=ap, depth=dp, q=q, dof=1, coeff=cp),
                           dict(anchor=ac, depth=dc, q=q, dof=1, coeff=cc),
                           dict(anchor=an, depth=dn, q=q), t, dt, 1, per)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    for x in (tv, tp, tcur, tn):
        x.close()


def test_bdf2_into_the_current_tree(ctx, ora):
    """con_next may be con_cur itself: both backtraces read it before the refit
    writes it."""
    q, t, dt = 5, 0.04, 0.02
    (av, dv, vc), (ap, dp, cp), (ac, dc, cc), _ = _setup(q, tb.FreeSpace)
    tv = tb.Tree(ctx, av, dv, q, 3, vc)
    tp, tcur = tb.Tree(ctx, ap, dp, q, 1, cp), tb.Tree(ctx, ac, dc, q, 1, cc)
    tb.solve_semilag_bdf2(tb.NodeFieldFunctor(tv), tp, tcur, tcur, t, dt)
    got = tcur.get_coeffs()
    ref = ora.semilag_bdf2(dict(anchor=av, depth=dv, q=q, dof=3, coeff=vc),
                           dict(anchor=ap, depth=dp, q=q, dof=1, coeff=cp),
                           dict(anchor=ac, depth=dc, q=q, dof=1, coeff=cc),
                           dict(anchor=ac, depth=dc, q=q), t, dt)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    for x in (tv, tp, tcur):
        x.close()

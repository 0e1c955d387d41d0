"""A tree evaluated on another tree's node grid by sum factorisation
(tbslas_eval_tree_on_nodes, the first RK2 stage of the in-situ step) is
bit-identical to the oracle's pointwise evaluation at
collect_grid_points(dst), for source trees coarser, equal and finer than the
destination, unequal degrees, both boundary conditions."""
import numpy as np
import pytest

import tbslas_gb300 as tb
from tbslas_gb300 import fields, trees

pytestmark = pytest.mark.gpu


def _src(kind, q, seed):
    if kind == "uniform1":
        a, d = trees.uniform_tree(1)
    elif kind == "uniform2":
        a, d = trees.uniform_tree(2)
    else:
        a, d = trees.adaptive_tree(fields.gaussian((0.3, 0.62, 0.45), 0.08), 4, 1, 1e-3, 1, 4)
    rng = np.random.default_rng(seed)
    c = rng.standard_normal((len(d), 3, tb.n_coeff(q)))
    c /= (1 + np.arange(tb.n_coeff(q)))[None, None, :]
    return a, d, c


@pytest.mark.parametrize("src_kind", ["uniform1", "uniform2", "adaptive"])
@pytest.mark.parametrize("qs,qd", [(3, 3), (8, 8), (14, 14), (5, 9), (9, 4)])
@pytest.mark.parametrize("bc", [0, 1])
def test_eval_on_nodes_bitwise(ctx, ora, src_kind, qs, qd, bc):
    a, d, c = _src(src_kind, qs, seed=qs * 31 + qd)
    src = tb.Tree(ctx, a, d, qs, 3, c)
    da, dd = (trees.adaptive_tree(fields.gaussian((0.6, 0.4, 0.5), 0.1), 4, 1, 1e-3, 1, 3)
              if src_kind == "uniform1" else trees.uniform_tree(2))
    dst = tb.Tree(ctx, da, dd, qd, 1)
    got = tb.NodeFieldFunctor(src, bc).at_nodes(dst).cpu().numpy()
    pts = ora.collect_grid_points(da, dd, qd)
    ref = ora.eval_tree(a, d, qs, 3, c, pts, periodic=bool(bc))
    assert got.shape == ref.shape
    assert np.array_equal(got, ref)


def test_in_situ_step_first_stage_is_exact(ctx, ora):
    """The fused step takes the first-stage velocity from the node grid: the
    step still matches the oracle to 1e-12 on a Taylor-Green case whose
    stagnation planes lie on leaf faces."""
    q = 6
    a, d = trees.uniform_tree(2)
    vc = trees.fit(fields.taylor_green(), a, d, q, 3)
    cc = trees.fit(fields.gaussian((0.4, 0.55, 0.5), 0.1), a, d, q, 1)
    tv, tc = tb.Tree(ctx, a, d, q, 3, vc), tb.Tree(ctx, a, d, q, 1, cc)
    tb.solve_semilag_in_situ(tb.NodeFieldFunctor(tv, 0), tc, 1, 0.02, 1)
    got = tc.get_coeffs()
    ref = ora.semilag_in_situ(dict(anchor=a, depth=d, q=q, dof=3, coeff=vc),
                              dict(anchor=a, depth=d, q=q, dof=1, coeff=cc), 1, 0.02, 1, False)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("bc", [0, 1])
def test_in_situ_fp64_sums_mode(ctx, ora, bc):
    """TBSLAS_SUMS_FP64: every sum in FP64 -- matches the oracle to 1e-12 (the
    refit's summation order is the only difference) and the double-float
    mode to 1e-12; the mode is a context setting, FP64 by default."""
    q = 8
    a, d = trees.adaptive_tree(fields.gaussian((0.45, 0.5, 0.52), 0.08), q, 1, 1e-4, 1, 3)
    vc = trees.fit(fields.taylor_green(), a, d, q, 3)
    cc = trees.fit(fields.gaussian((0.45, 0.5, 0.52), 0.08), a, d, q, 1)
    tv = tb.Tree(ctx, a, d, q, 3, vc)
    ref = ora.semilag_in_situ(dict(anchor=a, depth=d, q=q, dof=3, coeff=vc),
                              dict(anchor=a, depth=d, q=q, dof=1, coeff=cc), 2, 0.01, 1, bool(bc))
    got = {}
    assert ctx.sums == tb.SUMS_FP64  # the library default
    try:
        for mode in (tb.SUMS_FP64, tb.SUMS_DOUBLE_FLOAT):
            ctx.sums = mode
            tc = tb.Tree(ctx, a, d, q, 1, cc)
            tb.solve_semilag_in_situ(tb.NodeFieldFunctor(tv, bc), tc, 2, 0.01, 1)
            got[mode] = tc.get_coeffs()
    finally:
        ctx.sums = tb.SUMS_FP64  # the library default
    scale = np.abs(ref).max()
    assert np.abs(got[tb.SUMS_FP64] - ref).max() <= 1e-12 * scale
    assert np.abs(got[tb.SUMS_DOUBLE_FLOAT] - ref).max() <= 1e-12 * scale
    with pytest.raises(tb.capi.TbslasError):
        ctx.sums = 7

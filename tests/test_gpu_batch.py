"""Batched in-situ SL (one persistent kernel per degree band per step, CUDA
graph replay, autotuned launch parameters) against the per-problem loop of
tbslas_semilag_in_situ calls in the same sums mode (FP64, the default, and
double-float): identical coefficients, bit for bit.  The per-problem loop is
itself checked against the oracle (test_gpu_tree.py)."""
import numpy as np
import pytest

import tbslas_gb300 as tb
from tbslas_gb300 import capi, fields, trees, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_batch():
    return workloads.BatchWorkload(n=7, depths=(2, 3), tol=1e-2, name="batched_small",
                                   qlist=[3, 8, 9, 12, 13, 16, 5])


def _trees(ctx, wl):
    out = []
    for p in wl.problems:
        tv = tb.Tree(ctx, p["va"], p["vd"], p["q"], 3, p["vc"])
        tc = tb.Tree(ctx, p["ca"], p["cd"], p["q"], 1, p["cc"])
        out.append((tv, tc, p["dt"]))
    return out


MODES = {"fp64": tb.SUMS_FP64, "df": tb.SUMS_DOUBLE_FLOAT}


@pytest.mark.parametrize("mode", ["fp64", "df"])
@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_equals_per_problem_loop(ctx, small_batch, use_graph, mode):
    import torch
    wl = small_batch
    with ctx.sums_mode(MODES[mode]):
        ref = _trees(ctx, wl)
        for step in range(1, 4):
            for tv, tc, dt in ref:
                tb.solve_semilag_in_situ(tb.NodeFieldFunctor(tv, wl.bc), tc, step, dt)
        got = _trees(ctx, wl)
        b = tb.Batch(ctx, got, 1, wl.bc)
    # the batch keeps the mode it was created in
    b.set_params(128, 256, 4)
    b.run(1, 2, use_graph)
    b.run(3, 1, use_graph)
    torch.cuda.synchronize()
    for (tv, tc, _), (gv, gc, _) in zip(ref, got):
        assert np.array_equal(gc.get_coeffs(), tc.get_coeffs())
    total, items = b.info()
    assert total == wl.points_per_step and items > len(wl.problems)


@pytest.mark.parametrize("mode", ["fp64", "df"])
def test_batch_graph_replay_and_autotune_keep_state(ctx, small_batch, mode):
    import torch
    wl = small_batch
    with ctx.sums_mode(MODES[mode]):
        ref = _trees(ctx, wl)
        for step in range(1, 5):
            for tv, tc, dt in ref:
                tb.solve_semilag_in_situ(tb.NodeFieldFunctor(tv, wl.bc), tc, step, dt)
        got = _trees(ctx, wl)
        b = tb.Batch(ctx, got, 1, wl.bc)
    blk, tpi, cps = b.autotune()
    assert blk in (64, 128, 256) and tpi % blk == 0 and 1 <= cps <= 32
    assert b.params() == (blk, tpi, cps)
    b.run(1, 2, True)   # captured
    b.run(3, 2, True)   # replayed with a new first timestep
    torch.cuda.synchronize()
    for (tv, tc, _), (gv, gc, _) in zip(ref, got):
        assert np.array_equal(gc.get_coeffs(), tc.get_coeffs())


def test_batch_rejects_mixed_degrees(ctx):
    a, d = trees.uniform_tree(1)
    tv = tb.Tree(ctx, a, d, 4, 3)
    tc = tb.Tree(ctx, a, d, 5, 1)
    with pytest.raises(capi.TbslasError) as e:
        tb.Batch(ctx, [(tv, tc, 0.01)])
    assert e.value.status == 4
    with pytest.raises(capi.TbslasError):
        tb.Batch(ctx, [(tv, tv, 0.01)])


def test_batch_refuses_a_remeshed_tree(ctx):
    """The batch holds its trees' device arrays; after one of its trees is
    re-meshed, running it is refused until it is rebuilt."""
    import math
    a, d = trees.uniform_tree(2)
    q = 4
    v = trees.fit(fields.rotation(2 * math.pi), a, d, q, 3)
    c = trees.fit(fields.gaussian((0.6, 0.5, 0.45), 0.1), a, d, q, 1)
    tv, tc = tb.Tree(ctx, a, d, q, 3, v), tb.Tree(ctx, a, d, q, 1, c)
    b = tb.Batch(ctx, [(tv, tc, 0.01)], 1, tb.FreeSpace)
    b.run(1, 1, False)
    tc.remesh(1e-3, 1, 3)
    with pytest.raises(tb.capi.TbslasError):
        b.run(2, 1, False)
    b.close()
    b = tb.Batch(ctx, [(tv, tc, 0.01)], 1, tb.FreeSpace)
    b.run(2, 1, False)
    b.close()

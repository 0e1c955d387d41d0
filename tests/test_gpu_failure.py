"""Failure detection on the device without a fault: a bounded device-side
wait is made to run out (its poll limit set to zero), the kernel records the
timeout in the context's error word, lets its own copy in flight land and
returns; the host reads the word, and the context stays usable."""
import numpy as np
import pytest

import tbslas_gb300 as tb
from tbslas_gb300 import trees

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.mark.parametrize("q,dof", [(6, 1), (14, 3)])
def test_bounded_wait_runs_out_and_context_stays_usable(ctx, ora, q, dof):
    import torch
    anchor, depth = trees.uniform_tree(2)
    rng = np.random.default_rng(q)
    coeff = rng.standard_normal((len(depth), dof, tb.n_coeff(q)))
    pts = rng.uniform(0.0, 1.0, size=(20000, 3))
    t = tb.Tree(ctx, anchor, depth, q, dof, coeff)
    f = tb.NodeFieldFunctor(t, tb.FreeSpace)
    assert ctx.take_device_error() == 0
    ctx.set_wait_limit(0)  # every per-tile wait gives up at once
    try:
        f(_dev(pts))
        torch.cuda.synchronize()
        word = ctx.take_device_error()
    finally:
        ctx.set_wait_limit(tb.WAIT_LIMIT_DEFAULT)
    assert word & tb.DEVICE_ERR_WAIT_TIMEOUT, word
    assert ctx.take_device_error() == 0  # reading the word cleared it
    # the same context, default limit: the next call is complete and exact
    out = f(_dev(pts)).cpu().numpy()
    ref = ora.eval_tree(anchor, depth, q, dof, coeff, pts)
    assert np.array_equal(out, ref)
    assert ctx.take_device_error() == 0


def test_context_is_destroyed_only_after_its_trees():
    """The C ABI refuses to destroy a context whose trees are alive (it would
    leave them pointing at freed state) and leaves the context usable; the
    Python Context closes its trees first."""
    from tbslas_gb300 import capi
    c = tb.Context(0)
    a, d = trees.uniform_tree(1)
    t = tb.Tree(c, a, d, 3, 1)
    st = capi.lib().tbslas_ctx_destroy(c.handle)
    assert st == 1 and "still alive" in capi.last_error()
    t.set_coeffs(np.ones(t.coeff_shape))  # the context and its tree still work
    assert np.array_equal(t.get_coeffs(), np.ones(t.coeff_shape))
    c.close()
    assert t.handle is None and c.handle is None

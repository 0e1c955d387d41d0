"""tbslas_eval_tree_noalloc: the tree functor for callers that cannot
allocate device memory while they evaluate (a memory budget fixed up front,
or a host application whose own pool owns every device allocation).  Called
through the C ABI and checked against
tbslas_eval_tree on two calls in a row (the scratch array keeps the previous
call's contents, so the second call shows it is cleared where it must be)."""
import ctypes

import numpy as np
import pytest

import tbslas_gb300 as tb
from tbslas_gb300 import capi, fields, trees

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def test_noalloc_matches_eval_tree_two_calls(ctx):
    import torch
    L = capi.lib()
    q = 8
    g = fields.gaussian((0.4, 0.55, 0.5), 0.08)
    anchor, depth = trees.adaptive_tree(g, 4, 1, 1e-3, 1, 4)
    rng = np.random.default_rng(123)
    coeff = rng.standard_normal((len(depth), 3, tb.n_coeff(q)))
    t = tb.Tree(ctx, anchor, depth, q, 3, coeff)
    stream = torch.cuda.current_stream().cuda_stream
    for call, (n, bc) in enumerate([(50000, 0), (20000, 1)]):
        pts = rng.uniform(-0.05, 1.05, size=(n, 3))
        pos = _dev(pts)
        ref = tb.NodeFieldFunctor(t, bc)(pos)
        out = torch.full((n, 3), np.nan, dtype=torch.float64, device="cuda")
        st = L.tbslas_eval_tree_noalloc(t.handle, ctypes.c_void_p(pos.data_ptr()), n,
                                        ctypes.c_void_p(out.data_ptr()), bc, stream)
        assert st == 0, capi.last_error()
        torch.cuda.synchronize()
        o, r = out.cpu().numpy(), ref.cpu().numpy()
        assert np.abs(o - r).max() <= TOL * np.abs(r).max(), call
        assert np.array_equal(o, r), call
    assert ctx.check() == 0


def test_noalloc_rejects_sizes_beyond_its_limit(ctx):
    import torch
    L = capi.lib()
    anchor, depth = trees.uniform_tree(1)
    t = tb.Tree(ctx, anchor, depth, 2, 1)
    buf = torch.zeros(3, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    st = L.tbslas_eval_tree_noalloc(t.handle, p, capi.NOALLOC_MAX_POINTS + 1, p, 0, None)
    assert st == 6 and "TBSLAS_NOALLOC_MAX_POINTS" in capi.last_error()
    big_a, big_d = trees.uniform_tree(6)  # 262144 leaves > the leaf limit
    tbig = tb.Tree(ctx, big_a, big_d, 1, 1)
    st = L.tbslas_eval_tree_noalloc(tbig.handle, p, 1, p, 0, None)
    assert st == 6 and "TBSLAS_NOALLOC_MAX_LEAVES" in capi.last_error()

"""The re-meshing oracle (CPU restatement of RefineTree + Balance21 after a
step, src/applications/src/advection.cpp:305-311): refinement preserves the
represented function (the children carry the restriction of the parent's
expansion), a polynomial of degree < q coarsens exactly, and the result is
2:1 balanced across faces, edges and corners (and periodic images)."""
import numpy as np
import pytest

from tbslas_gb300 import fields, trees


def _eval(ora, a, d, q, c, pts, periodic=False):
    return ora.eval_tree(a, d, q, c.shape[1], c, pts, periodic)


def _balanced(rm, a, d, periodic):
    return not rm.balance_flags(a, d, periodic).any()


def test_refine_preserves_the_function(ora):
    from oracle import remesh as rm
    q = 5
    a, d = trees.uniform_tree(2)
    c = trees.fit(fields.gaussian((0.4, 0.55, 0.5), 0.1), a, d, q, 1)
    tol = 2e-3
    a2, d2, c2 = rm.remesh(a, d, q, c, tol, 2, 4)
    assert d2.size > d.size and d2.min() == 2 and d2.max() <= 4
    # only splits happened (min_depth 2): values equal up to the fits' rounding
    pts = np.random.default_rng(0).uniform(0, 1, (4000, 3))
    v0, v1 = _eval(ora, a, d, q, c, pts), _eval(ora, a2, d2, q, c2, pts)
    leaf0 = np.searchsorted(rm.keys(a), rm.keys(pts), side="right") - 1
    refined_once = d[leaf0] + 1 == d2[np.searchsorted(rm.keys(a2), rm.keys(pts), side="right") - 1]
    assert refined_once.any()
    assert np.abs(v0 - v1).max() <= 1e-13 * np.abs(v0).max()
    assert _balanced(rm, a2, d2, False)
    assert (rm.tails(c2, q)[d2 < 4] <= tol).all()


def test_polynomial_coarsens_exactly(ora):
    from oracle import remesh as rm
    q = 4
    a, d = trees.uniform_tree(3)
    rng = np.random.default_rng(1)
    terms = [(i, j, k) for i in range(q) for j in range(q - i) for k in range(q - i - j)]
    cf = rng.standard_normal(len(terms))

    def fn(p):
        p = np.asarray(p).reshape(-1, 3)
        return sum(w * p[:, 0] ** k * p[:, 1] ** j * p[:, 2] ** i
                   for w, (i, j, k) in zip(cf, terms))[:, None]

    c = trees.fit(fn, a, d, q, 1)
    a2, d2, c2 = rm.remesh(a, d, q, c, 1e-9, 1, 3)
    assert d2.size == 64 and (d2 == 2).all()  # one level per call
    pts = rng.uniform(0, 1, (2000, 3))
    ref = fn(pts)
    assert np.abs(_eval(ora, a2, d2, q, c2, pts) - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("periodic", [False, True])
def test_balance(ora, periodic):
    from oracle import remesh as rm
    q = 3
    # the leaf touching the domain's centre (0.5, 0.5, 0.5) from above, split
    # down to depth 5: its neighbours across the centre stay at depth 1
    a, d = trees.uniform_tree(1)
    for _ in range(4):
        k = int(np.argmin(np.abs(a - 0.5).sum(axis=1) + 10.0 * (d != d.max())))
        a = np.concatenate([a[:k], trees.split(a[k:k + 1], d[k:k + 1])[0], a[k + 1:]])
        d = np.concatenate([d[:k], np.full(8, d[k] + 1, dtype=np.int32), d[k + 1:]])
        a, d = trees.sort_leaves(a, d)
    c = trees.fit(fields.gaussian((0.5, 0.5, 0.5), 0.2), a, d, q, 1)
    assert not _balanced(rm, a, d, periodic)
    a2, d2, c2 = rm.remesh(a, d, q, c, np.inf, 5, 5, periodic)
    assert _balanced(rm, a2, d2, periodic)
    # untouched leaves keep their coefficients bit for bit
    k0, k2 = rm.keys(a), rm.keys(a2)
    same = {(int(kk), int(dd)): i for i, (kk, dd) in enumerate(zip(k0, d))}
    n_same = 0
    for j, (kk, dd) in enumerate(zip(k2, d2)):
        i = same.get((int(kk), int(dd)))
        if i is not None:
            assert np.array_equal(c2[j], c[i])
            n_same += 1
    assert n_same > 0
    assert d2.size > d.size


def test_balance_across_the_periodic_boundary(ora):
    """A corner-graded tree (the origin's leaf split down to depth 5) is 2:1
    balanced in free space but not periodically: the far corner's depth-1
    leaves touch the depth-5 leaves through the wrap."""
    from oracle import remesh as rm
    q = 3
    a, d = trees.uniform_tree(1)
    for _ in range(4):
        k = int(np.argmax(d == d.max()))  # the leaf at the origin
        a = np.concatenate([a[:k], trees.split(a[k:k + 1], d[k:k + 1])[0], a[k + 1:]])
        d = np.concatenate([d[:k], np.full(8, d[k] + 1, dtype=np.int32), d[k + 1:]])
        a, d = trees.sort_leaves(a, d)
    c = trees.fit(fields.gaussian((0.5, 0.5, 0.5), 0.2), a, d, q, 1)
    assert _balanced(rm, a, d, False) and not _balanced(rm, a, d, True)
    a2, d2, _ = rm.remesh(a, d, q, c, np.inf, 5, 5, False)
    assert d2.size == d.size
    a3, d3, _ = rm.remesh(a, d, q, c, np.inf, 5, 5, True)
    assert d3.size > d.size and _balanced(rm, a3, d3, True)


def test_construct_oracle_properties(ora):
    """The construction oracle: a field the degree-q basis represents (a
    Gaussian of huge width is smooth, a rotation is linear) needs no
    refinement; a sharp Gaussian is refined near its centre only, the result
    2:1 balanced and its fit equal to InitTree's on the final leaves."""
    from oracle import construct as oc
    from oracle import remesh as rm
    a, d, c = oc.construct(3, 0, [1.0], 4, 1e-10, 1, 4)  # rotation, linear
    assert len(d) == 8 and (d == 1).all()
    f = (0, 1, [0.3, 0.6, 0.5, 0.05, 1.0])  # one sharp Gaussian
    a, d, c = oc.construct(*f, 5, 1e-4, 1, 4)
    assert d.max() == 4 and d.min() <= 2
    assert not rm.balance_flags(a, d, False).any()
    assert np.array_equal(c, oc.fit(*f, a, d, 5))
    deep = a[d == 4] + 0.5 ** 4 / 2
    assert (np.linalg.norm(deep - [0.3, 0.6, 0.5], axis=1) < 0.4).all()


def test_functor_stage_weights():
    """FieldSetFunctor / FieldExtrapFunctor produce IntegrateRK2's stage
    weights: the cubic's at tinit and tinit + tau/2 of each sub-step, and
    (v_n, 1.5 v_n - 0.5 v_{n-1})."""
    import tbslas_gb300 as tb
    times = [0.0, 0.1, 0.2, 0.3]
    f = tb.FieldSetFunctor([None] * 4, times)
    _, w = f.stage_weights(2, 0.1, 1)
    assert np.allclose(w[:4], tb.cubic_time_weights(times, 0.2), atol=0)
    assert np.allclose(w[4:], tb.cubic_time_weights(times, 0.15), atol=0)
    _, w2 = f.stage_weights(2, 0.1, 2)
    assert len(w2) == 16
    assert np.allclose(w2[12:], tb.cubic_time_weights(times, 0.2 - 0.05 - 0.025), atol=1e-15)
    f.update("new", 0.4)
    assert f.times == [0.1, 0.2, 0.3, 0.4] and f.trees[-1] == "new"
    e = tb.FieldExtrapFunctor("p", "c")
    trees_, w3 = e.stage_weights(1, 0.1, 2)
    assert trees_ == ["c", "p"] and list(w3) == [1.0, 0.0, 1.5, -0.5] * 2
    e.update("n")
    assert (e.tp, e.tc) == ("c", "n")

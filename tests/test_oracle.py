"""Pins the oracle (CPU restatement) against the analytic known answers the
reference's drivers check (the reference ships no golden vectors):
polynomial exactness of the Chebyshev fit/evaluation, the rotation
trajectory returning to its start (traj.cpp:115-131, conv_traj.py:47-60),
translation (advection.cpp tests 3/4), the rotated Gaussian
(advection.cpp test 1), time reversal (advection-inverse.cpp) and the
tricubic interpolant's cubic exactness (tree_functor.h:89-153)."""
import math

import numpy as np
import pytest

from tbslas_gb300 import fields, trees


def _poly(rng, q):
    """Random polynomial of total degree <= q as a point function."""
    terms = [(i, j, k) for i in range(q + 1) for j in range(q + 1 - i) for k in range(q + 1 - i - j)]
    c = rng.standard_normal(len(terms))

    def fn(p):
        p = np.asarray(p).reshape(-1, 3)
        out = np.zeros(len(p))
        for a, (i, j, k) in zip(c, terms):
            out += a * p[:, 0] ** k * p[:, 1] ** j * p[:, 2] ** i
        return out[:, None]
    return fn


def test_new_nodes_layout(ora):
    for q in (1, 4, 8, 14):
        y = ora.new_nodes(q)
        d = q + 1
        assert y.shape == (d ** 3, 3)
        x = y[:d, 0]
        assert abs(x[0]) < 1e-15 and abs(x[-1] - 1) < 1e-15
        assert np.allclose(x + x[::-1], 1.0, atol=1e-15)
        assert np.all(y[:d, 1] == y[0, 1])             # x fastest
        assert np.all(y[d:2 * d, 1] == x[1])


def test_cheb_poly_recurrence_and_outside_zero(ora):
    th = np.linspace(0, math.pi, 17)
    T = ora.cheb_poly(9, np.cos(th))
    for k in range(10):
        assert np.allclose(T[k], np.cos(k * th), atol=1e-13)
    T = ora.cheb_poly(5, np.array([1.0000001, -2.0, np.nan, 1.0]))
    assert np.all(T[:, :3] == 0) and T[0, 3] == 1.0


def test_pt2coeff_reproduces_basis(ora):
    for q in (2, 6):
        M = ora.pt2coeff(q)
        V = ora.cheb_basis(q, 2 * ora.new_nodes(q) - 1)
        assert np.allclose(M.T @ V, np.eye(V.shape[1]), atol=1e-12)


@pytest.mark.parametrize("adaptive", [False, True])
def test_eval_tree_polynomial_exact(ora, adaptive):
    rng = np.random.default_rng(1)
    q = 4
    fn = _poly(rng, q)
    if adaptive:
        g = fields.gaussian((0.3, 0.6, 0.4), 0.08)
        anchor, depth = trees.adaptive_tree(g, q, 1, 1e-3, 1, 3)
        assert len(set(depth)) > 1
    else:
        anchor, depth = trees.uniform_tree(2)
    coeff = trees.fit(fn, anchor, depth, q, 1, ora.pt2coeff(q))
    pts = rng.uniform(0, 1, size=(2000, 3))
    pts[:5] = [[1.0, 0.5, 0.5], [0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [0.5, 0.25, 0.75], [0.25, 1.0, 0]]
    out = ora.eval_tree(anchor, depth, q, 1, coeff, pts)
    ref = fn(pts)
    assert np.abs(out - ref).max() < 1e-11 * max(1.0, np.abs(ref).max())


def test_eval_tree_outside_nan_and_order(ora):
    rng = np.random.default_rng(2)
    q = 3
    anchor, depth = trees.uniform_tree(2)
    coeff = rng.standard_normal((len(depth), 3, ora.n_coeff(q)))
    pts = rng.uniform(-0.2, 1.2, size=(3000, 3))
    pts[0] = [np.nan, 0.5, 0.5]
    out = ora.eval_tree(anchor, depth, q, 3, coeff, pts)
    outside = np.any((pts < 0) | (pts > 1), axis=1) | np.isnan(pts).any(axis=1)
    assert outside.sum() > 100
    assert np.all(out[outside] == 0)
    assert np.all(np.abs(out[~outside]).sum(axis=1) > 0)
    perm = rng.permutation(len(pts))
    out2 = ora.eval_tree(anchor, depth, q, 3, coeff, pts[perm])
    assert np.array_equal(out2, out[perm])
    # periodic: points outside wrap once onto their images
    outp = ora.eval_tree(anchor, depth, q, 3, coeff, pts, periodic=True)
    img = pts - np.floor(pts)
    outi = ora.eval_tree(anchor, depth, q, 3, coeff, img, periodic=True)
    ok = ~np.isnan(pts).any(axis=1)
    assert np.allclose(outp[ok], outi[ok], atol=1e-12)


def test_traj_rotation_returns_second_order(ora):
    """traj.cpp: x0=(0.99,0.5,0.5), omega=1, T=2*pi, RK2; error -> O(dt^2)."""
    q = 3
    anchor, depth = trees.uniform_tree(1)
    coeff = trees.fit(fields.rotation(1.0), anchor, depth, q, 3, ora.pt2coeff(q))
    x0 = np.array([[0.99, 0.5, 0.5]])
    errs = []
    for tn in (50, 100, 200, 400):
        dt = 2 * math.pi / tn
        x = ora.traj_rk2(anchor, depth, q, coeff, x0, 0.0, -tn * dt, tn)
        errs.append(np.linalg.norm(x - x0))
    rates = [errs[i] / errs[i + 1] for i in range(3)]
    assert all(3.5 < r < 4.5 for r in rates), (errs, rates)
    assert errs[-1] < 1e-3


def test_translation_periodic_keeps_linear_field(ora):
    """advection.cpp test 4 shape: v=(-0.5,0,0) with a field of y alone,
    periodic -> every node value is kept (departure points differ in x only;
    nodes on the y=1 face wrap to y=0, so the field is taken y-periodic)."""
    q = 4
    anchor, depth = trees.uniform_tree(2)
    M = ora.pt2coeff(q)
    vel = dict(anchor=anchor, depth=depth, q=q, dof=3,
               coeff=trees.fit(lambda p: np.tile([-0.5, 0.0, 0.0], (len(p), 1)), anchor, depth, q, 3, M))
    c0 = trees.fit(lambda p: np.cos(2 * np.pi * p[:, 1])[:, None], anchor, depth, q, 1, M)
    con = dict(anchor=anchor, depth=depth, q=q, dof=1, coeff=c0)
    c = c0
    for step in range(1, 4):
        con["coeff"] = c
        c = ora.semilag_in_situ(vel, con, step, 0.037, 1, periodic=True)
    assert np.abs(c - c0).max() < 1e-12


def test_translation_polynomial_exact_inside(ora):
    """Constant velocity, polynomial of degree <= q: SL is exact wherever the
    departure points stay inside the domain."""
    rng = np.random.default_rng(3)
    q = 5
    fn = _poly(rng, q)
    anchor, depth = trees.uniform_tree(2)
    M = ora.pt2coeff(q)
    v = np.array([0.3, -0.2, 0.1])
    dt = 0.05
    vel = dict(anchor=anchor, depth=depth, q=q, dof=3,
               coeff=trees.fit(lambda p: np.tile(v, (len(p), 1)), anchor, depth, q, 3, M))
    con = dict(anchor=anchor, depth=depth, q=q, dof=1, coeff=trees.fit(fn, anchor, depth, q, 1, M))
    c1 = ora.semilag_in_situ(vel, con, 1, dt, 1)
    exact = trees.fit(lambda p: fn(p - dt * v), anchor, depth, q, 1, M)
    h = 0.25
    safe = np.all((anchor - dt * v >= 0) & (anchor + h - dt * v <= 1), axis=1)
    assert safe.sum() >= 8
    scale = np.abs(exact).max()
    assert np.abs(c1[safe] - exact[safe]).max() < 1e-11 * scale


def test_rotated_gaussian_accuracy(ora):
    """advection.cpp test 1 shape: rotation + Gaussian vs the exact solution."""
    q, depth_, dt, steps = 8, 3, 0.01, 5
    omega = 2 * math.pi
    anchor, depth = trees.uniform_tree(depth_)
    M = ora.pt2coeff(q)
    g0 = fields.gaussian((0.7, 0.5, 0.5), 0.05)
    vel = dict(anchor=anchor, depth=depth, q=q, dof=3,
               coeff=trees.fit(fields.rotation(omega), anchor, depth, q, 3, M))
    con = dict(anchor=anchor, depth=depth, q=q, dof=1, coeff=trees.fit(g0, anchor, depth, q, 1, M))
    for s in range(1, steps + 1):
        con["coeff"] = ora.semilag_in_situ(vel, con, s, dt, 1)
    pts = trees.leaf_nodes(anchor, depth, q)
    num = ora.eval_tree(anchor, depth, q, 1, con["coeff"], pts)
    ex = fields.rotated_gaussian((0.7, 0.5, 0.5), 0.05, omega, steps * dt)(pts)
    assert np.abs(num - ex).max() < 2e-2


def test_time_reversal(ora):
    """advection-inverse.cpp: N steps forward, negated velocity, N back."""
    q, dt, n = 8, 0.01, 4
    anchor, depth = trees.uniform_tree(2)
    M = ora.pt2coeff(q)
    vc = trees.fit(fields.rotation(2 * math.pi), anchor, depth, q, 3, M)
    c0 = trees.fit(fields.gaussian((0.6, 0.5, 0.5), 0.1), anchor, depth, q, 1, M)
    vel = dict(anchor=anchor, depth=depth, q=q, dof=3, coeff=vc)
    con = dict(anchor=anchor, depth=depth, q=q, dof=1, coeff=c0)
    for s in range(1, n + 1):
        con["coeff"] = ora.semilag_in_situ(vel, con, s, dt, 1)
    moved = np.abs(con["coeff"] - c0).max()
    vel["coeff"] = -vc
    for s in range(n + 1, 2 * n + 1):
        con["coeff"] = ora.semilag_in_situ(vel, con, s, dt, 1)
    back = np.abs(con["coeff"] - c0).max()
    assert back < 0.05 * moved, (back, moved)


def test_fast_interp_cubic_exact_and_outside(ora):
    rng = np.random.default_rng(4)
    N = 12
    x = np.arange(N) / (N - 1)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    f = lambda X, Y, Z: 1 + X - 2 * Y ** 2 + X * Y * Z + 0.5 * Z ** 3 - X ** 3 * Y ** 3 * Z ** 3
    grid = np.stack([f(X, Y, Z), 2 * f(Y, Z, X)]).ravel()
    pts = rng.uniform(0, 1, size=(500, 3))
    out = ora.fast_interp(grid, 2, N, pts)
    ref = np.stack([f(pts[:, 0], pts[:, 1], pts[:, 2]), 2 * f(pts[:, 1], pts[:, 2], pts[:, 0])], 1)
    assert np.abs(out - ref).max() < 1e-12
    bad = np.array([[-1e-9, 0.5, 0.5], [0.5, 1 + 1e-12, 0.5], [np.nan, 0, 0]])
    assert np.all(ora.fast_interp(grid, 2, N, bad) == 0)


def test_fast_interp_periodic_and_grid_shift(ora):
    N = 16
    rng = np.random.default_rng(5)
    con = rng.standard_normal((N, N, N))
    # velocity (-0.5,0,0), dt = 2h: every departure point is the next node in +x
    vel = np.zeros((3, N, N, N))
    vel[0] = -0.5
    out = ora.semilag_grid(vel, con, N, 2.0 / N, 1, periodic=True).reshape(N, N, N)
    assert np.array_equal(out, np.roll(con, -1, axis=2))
    # the periodic interpolant is invariant under a whole-period shift
    pts = rng.uniform(0, 1, size=(200, 3))
    a = ora.fast_interp(con.ravel(), 1, N, pts, periodic=True)
    b = ora.fast_interp(con.ravel(), 1, N, pts - 1.0, periodic=True)
    assert np.allclose(a, b, atol=1e-12)


def test_bdf2_translation_exact(ora):
    """BDF2 two-backtrace step (advdiff-ss.cpp:485-521) under a constant
    velocity with exact c_n, c_{n-1} of a translated polynomial: 4/3 - 1/3 = 1
    times the exact value, on the leaves whose departure points stay inside."""
    q, dt, t = 4, 0.01, 0.05
    a, d = trees.uniform_tree(2)
    v = np.array([0.7, -0.4, 0.3])
    vc = trees.fit(lambda p: np.tile(v, (len(np.asarray(p).reshape(-1, 3)), 1)), a, d, q, 3)
    P = _poly(np.random.default_rng(5), q)

    def at(time):
        return lambda p: P(np.asarray(p).reshape(-1, 3) - v * time)
    vel = dict(anchor=a, depth=d, q=q, dof=3, coeff=vc)
    prev = dict(anchor=a, depth=d, q=q, dof=1, coeff=trees.fit(at(t - 2 * dt), a, d, q, 1))
    cur = dict(anchor=a, depth=d, q=q, dof=1, coeff=trees.fit(at(t - dt), a, d, q, 1))
    out = ora.semilag_bdf2(vel, prev, cur, dict(anchor=a, depth=d, q=q), t, dt)
    pts = np.random.default_rng(6).uniform(0.3, 0.7, (500, 3))
    got = ora.eval_tree(a, d, q, 1, out, pts)
    ref = at(t)(pts)
    assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()


def test_cubic_time_weights_match_interp_cubic(ora):
    """tbslas_cubic_time_weights (host) against the oracle's restatement of
    CubicInterpPolicy::InterpCubic1D (src/utils/cubic.h:42-56): the
    interpolant is linear in the four values."""
    import tbslas_gb300 as tb
    rng = np.random.default_rng(9)
    for _ in range(20):
        times = np.sort(rng.uniform(0, 1, 4)) + np.arange(4) * 0.1
        t = rng.uniform(times[0], times[3])
        w = tb.cubic_time_weights(times, t)
        p = rng.standard_normal(4)
        ref = ora.interp_cubic_1d(t, times, p)
        assert abs(w @ p - ref) <= 1e-14 * max(1.0, abs(ref))
    w = tb.cubic_time_weights([0.0, 1.0, 2.0, 3.0], 1.5)
    assert np.allclose(w, [-0.0625, 0.5625, 0.5625, -0.0625], rtol=0, atol=1e-16)


@pytest.mark.parametrize("functor", ["set", "extrap"])
def test_time_dependent_step_with_one_velocity_is_the_plain_step(ora, functor):
    """FieldSetFunctor over four copies of one tree (cubic weights summing to
    1) and FieldExtrapFunctor over two copies (1.5 v - 0.5 v) are that tree's
    velocity: the time-dependent step equals the plain step up to the
    rounding of the blend, on a generic periodic Fourier velocity (no
    stagnation on leaf faces)."""
    q, dt = 4, 0.01
    a, d = trees.uniform_tree(2)
    vel_fn = fields.fourier_velocity(np.random.default_rng(12))
    vc = trees.fit(vel_fn, a, d, q, 3)
    cc = trees.fit(fields.gaussian_blobs(np.random.default_rng(13), 2, (0.1, 0.15)), a, d, q, 1)
    vel = dict(anchor=a, depth=d, q=q, dof=3, coeff=vc)
    con = dict(anchor=a, depth=d, q=q, dof=1, coeff=cc)
    ref = ora.semilag_in_situ(vel, con, 3, dt, 1, True)
    if functor == "set":
        got = ora.semilag_in_situ_tv([vel] * 4, con, 3, dt, 1, True,
                                     times=[0.0, dt, 2 * dt, 3 * dt])
    else:
        got = ora.semilag_in_situ_tv([vel, vel], con, 3, dt, 1, True)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()

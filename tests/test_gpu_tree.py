"""GPU parity of the tree path (C ABI -> CUDA) against the oracle.

Tolerance: max |gpu - oracle| <= 1e-12 * max |oracle| (L-infinity relative)
on coefficients of the in-situ step, in both sums modes: FP64 (the default;
only the refit's summation order differs from the oracle's) and
double-float (near-face targets are recomputed in FP64, so leaf choices
match the oracle's); bit-exact for the functor values and departure points
(all FP64) and for the collected node coordinates."""
import math

import numpy as np
import pytest

import tbslas_gb300 as tb
from tbslas_gb300 import capi, fields, trees

pytestmark = pytest.mark.gpu
TOL = 1e-12
MODES = {"fp64": tb.SUMS_FP64, "df": tb.SUMS_DOUBLE_FLOAT}


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _tree_case(kind, q, dof, seed=0):
    rng = np.random.default_rng(seed)
    if kind == "uniform":
        anchor, depth = trees.uniform_tree(2)
    else:
        g = fields.gaussian((0.35, 0.6, 0.45), 0.07)
        anchor, depth = trees.adaptive_tree(g, 4, 1, 1e-3, 1, 4)
    coeff = rng.standard_normal((len(depth), dof, tb.n_coeff(q)))
    coeff /= (1 + np.arange(tb.n_coeff(q)))[None, None, :]
    return anchor, depth, coeff


def _points(rng, n):
    pts = rng.uniform(-0.05, 1.05, size=(n, 3))
    special = np.array([[1.0, 0.5, 0.5], [0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [0.5, 0.5, 0.5],
                        [0.25, 0.75, 1.0], [np.nan, 0.5, 0.5], [0.5, -0.0, 0.5],
                        [1.0 - 2 ** -53, 0.5, 0.5], [0.125, 0.125, 0.125]])
    pts[:len(special)] = special
    return pts


@pytest.mark.parametrize("kind", ["uniform", "adaptive"])
@pytest.mark.parametrize("q,dof", [(2, 1), (5, 3), (8, 1), (8, 3), (14, 1)])
@pytest.mark.parametrize("bc", [0, 1])
def test_eval_tree_matches_oracle(ctx, ora, kind, q, dof, bc):
    anchor, depth, coeff = _tree_case(kind, q, dof, seed=q)
    rng = np.random.default_rng(10 + q)
    pts = _points(rng, 20000)
    t = tb.Tree(ctx, anchor, depth, q, dof, coeff)
    f = tb.NodeFieldFunctor(t, bc)
    out = f(_dev(pts)).cpu().numpy()
    ref = ora.eval_tree(anchor, depth, q, dof, coeff, pts, periodic=bool(bc))
    assert rel_err(out, ref) <= TOL
    assert np.array_equal(out == 0, ref == 0)
    host = f(pts)
    assert np.array_equal(host, out)


@pytest.mark.parametrize("bc", [0, 1])
def test_eval_tree_special_values_match_oracle(ctx, ora, bc):
    """Coefficients with exact zeros and -0.0 (the first term of every row of
    the Chebyshev sums is formed on the integer pipe: c_0 with -0 read as +0,
    as the FP64 fma gives it) and coordinates at 0, -0.0, just below 0 and
    above 1, subnormal, tiny, infinite and NaN (the domain tests, the
    periodic wrap and the Morton quantisation run on the coordinates' bits):
    the functor's values equal the oracle's exactly."""
    q, dof = 6, 3
    anchor, depth, coeff = _tree_case("adaptive", q, dof, seed=7)
    coeff[::3, :, 0] = -0.0
    coeff[1::5, :, ::4] = 0.0
    coeff[2::7] = -0.0
    rng = np.random.default_rng(77)
    pts = _points(rng, 4000)
    extra = np.array([[5e-324, 0.5, 0.5], [np.inf, 0.5, 0.5], [-np.inf, 0.5, 0.5],
                      [-1e-300, 0.5, 0.5], [1 + 2 ** -52, 0.5, 0.5], [0.5, 2 ** -30, 0.5],
                      [0.5, 0.5, -0.0], [-0.0, -0.0, -0.0], [np.nan, 0.1, 0.1],
                      [0.5, -np.nan, 0.5], [2 ** -21, 2 ** -21 - 2 ** -74, 0.5]])
    pts[20:20 + len(extra)] = extra
    t = tb.Tree(ctx, anchor, depth, q, dof, coeff)
    out = tb.NodeFieldFunctor(t, bc)(_dev(pts)).cpu().numpy()
    ref = ora.eval_tree(anchor, depth, q, dof, coeff, pts.copy(), periodic=bool(bc))
    assert np.array_equal(out, ref)


def test_eval_tree_empty_and_errors(ctx):
    import torch
    anchor, depth = trees.uniform_tree(1)
    t = tb.Tree(ctx, anchor, depth, 3, 1)
    out = tb.NodeFieldFunctor(t)(torch.empty((0, 3), dtype=torch.float64, device="cuda"))
    assert out.shape == (0, 1)
    with pytest.raises(capi.TbslasError) as e:
        tb.Tree(ctx, anchor[:-1], depth[:-1], 3, 1)
    assert e.value.status == 2
    with pytest.raises(capi.TbslasError) as e:
        tb.Tree(ctx, anchor[::-1], depth[::-1], 3, 1)
    assert e.value.status == 2
    bad = anchor.copy()
    bad[0, 0] = 0.1
    with pytest.raises(capi.TbslasError) as e:
        tb.Tree(ctx, bad, depth, 3, 1)
    assert e.value.status == 2
    with pytest.raises(capi.TbslasError) as e:
        tb.Tree(ctx, anchor, depth, 17, 1)
    assert e.value.status == 4
    with pytest.raises(capi.TbslasError) as e:
        tb.NodeFieldFunctor(t, bc=7)(np.zeros((4, 3)))
    assert e.value.status == 1


def test_collect_grid_points_exact(ctx, ora):
    g = fields.gaussian((0.5, 0.4, 0.6), 0.06)
    anchor, depth = trees.adaptive_tree(g, 3, 1, 1e-3, 1, 4)
    for q in (3, 8):
        t = tb.Tree(ctx, anchor, depth, q, 1)
        out = tb.collect_cheb_tree_grid_points(t).cpu().numpy()
        assert np.array_equal(out, ora.collect_grid_points(anchor, depth, q))


@pytest.mark.parametrize("q,dof", [(4, 1), (8, 3), (14, 1)])
def test_set_tree_grid_values_matches_oracle(ctx, ora, q, dof):
    rng = np.random.default_rng(q)
    anchor, depth = trees.uniform_tree(2)
    L, np_ = len(depth), (q + 1) ** 3
    vals = rng.standard_normal((L, dof, np_))
    t = tb.Tree(ctx, anchor, depth, q, dof)
    tb.set_tree_grid_values(t, _dev(vals))
    ref = ora.set_tree_grid_values(L, q, dof, vals)
    assert rel_err(t.get_coeffs(), ref) <= TOL


@pytest.mark.parametrize("bc,nrk", [(0, 1), (1, 1), (0, 3)])
def test_traj_rk2_matches_oracle(ctx, ora, bc, nrk):
    q = 8
    anchor, depth = trees.uniform_tree(2)
    vc = trees.fit(fields.taylor_green(), anchor, depth, q, 3)
    t = tb.Tree(ctx, anchor, depth, q, 3, vc)
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 1, size=(5000, 3))
    out = tb.compute_traj_rk2(tb.NodeFieldFunctor(t, bc), _dev(x), 0.3, 0.3 - 0.05, nrk)
    ref = ora.traj_rk2(anchor, depth, q, vc, x, 0.3, 0.3 - 0.05, nrk, periodic=bool(bc))
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-14


def _sl_case(kind, qv, qc, dofc, rng):
    if kind == "uniform":
        av, dv = trees.uniform_tree(2)
        ac, dc = trees.uniform_tree(2)
    else:
        av, dv = trees.adaptive_tree(fields.taylor_green(), 4, 3, 1e-2, 1, 3)
        g = fields.gaussian_blobs(rng, 3, (0.05, 0.1))
        ac, dc = trees.adaptive_tree(g, 4, 1, 1e-3, 1, 4)
    vc = trees.fit(fields.taylor_green(), av, dv, qv, 3)
    blobs = fields.gaussian_blobs(rng, 2, (0.08, 0.12))
    cc = trees.fit(lambda p: np.repeat(blobs(p), dofc, axis=1) * (1 + np.arange(dofc)),
                   ac, dc, qc, dofc)
    return (av, dv, vc), (ac, dc, cc)


@pytest.mark.parametrize("mode", ["fp64", "df"])
@pytest.mark.parametrize("kind", ["uniform", "adaptive"])
@pytest.mark.parametrize("qv,qc,dofc", [(8, 8, 1), (5, 5, 1), (6, 4, 1), (4, 4, 2)])
@pytest.mark.parametrize("bc,nrk", [(0, 1), (1, 2)])
def test_semilag_in_situ_matches_oracle(ctx, ora, kind, qv, qc, dofc, bc, nrk, mode):
    rng = np.random.default_rng(qv * 10 + qc)
    (av, dv, vc), (ac, dc, cc) = _sl_case(kind, qv, qc, dofc, rng)
    tv = tb.Tree(ctx, av, dv, qv, 3, vc)
    tc = tb.Tree(ctx, ac, dc, qc, dofc, cc)
    vel = tb.NodeFieldFunctor(tv, bc)
    ref_con = dict(anchor=ac, depth=dc, q=qc, dof=dofc, coeff=cc.copy())
    ref_vel = dict(anchor=av, depth=dv, q=qv, dof=3, coeff=vc)
    dt = 0.02
    with ctx.sums_mode(MODES[mode]):
        for step in (1, 2):
            tb.solve_semilag_in_situ(vel, tc, step, dt, nrk)
            ref_con["coeff"] = ora.semilag_in_situ(ref_vel, ref_con, step, dt, nrk,
                                                   periodic=bool(bc))
            assert rel_err(tc.get_coeffs(), ref_con["coeff"]) <= TOL, step


@pytest.mark.parametrize("mode", ["fp64", "df"])
@pytest.mark.parametrize("bc", [0, 1])
@pytest.mark.parametrize("q,dofc", [(9, 1), (11, 1), (12, 1), (12, 3), (14, 1), (16, 1)])
def test_semilag_in_situ_high_degree_matches_oracle(ctx, ora, q, dofc, bc, mode):
    """Degrees above 8 (each its own kernel instantiation; q = 14 is the
    headline degree, q = 16 the largest supported) on adaptive trees: a
    Taylor-Green velocity tree and a concentration tree refined around
    seeded Gaussians, two steps against the oracle.  dofc = 3 takes the
    general path (trajectory + bucketed functor + refit per dof)."""
    rng = np.random.default_rng(100 + q)
    av, dv = trees.adaptive_tree(fields.taylor_green(), 4, 3, 1e-2, 1, 2)
    blobs = fields.gaussian_blobs(rng, 3, (0.05, 0.1))
    ac, dc = trees.adaptive_tree(blobs, 4, 1, 1e-3, 1, 2)
    vc = trees.fit(fields.taylor_green(), av, dv, q, 3)
    cc = trees.fit(lambda p: np.repeat(blobs(p), dofc, axis=1) * (1 + np.arange(dofc)),
                   ac, dc, q, dofc)
    tv = tb.Tree(ctx, av, dv, q, 3, vc)
    tc = tb.Tree(ctx, ac, dc, q, dofc, cc)
    vel = tb.NodeFieldFunctor(tv, bc)
    ref_vel = dict(anchor=av, depth=dv, q=q, dof=3, coeff=vc)
    ref_con = dict(anchor=ac, depth=dc, q=q, dof=dofc, coeff=cc.copy())
    dt = 1.0 / (2.0 ** int(max(dv.max(), dc.max())) * q * q)  # Chebyshev CFL 1
    with ctx.sums_mode(MODES[mode]):
        for step in (1, 2):
            tb.solve_semilag_in_situ(vel, tc, step, dt, 1)
            ref_con["coeff"] = ora.semilag_in_situ(ref_vel, ref_con, step, dt, 1,
                                                   periodic=bool(bc))
            assert rel_err(tc.get_coeffs(), ref_con["coeff"]) <= TOL, step


@pytest.mark.parametrize("mode", ["fp64", "df"])
def test_headline_shape_reduced_matches_oracle(ctx, ora, mode):
    """The headline configuration's shape at a size the oracle finishes in
    seconds: q = 14, a Taylor-Green velocity tree and a concentration tree
    of 4 seeded Gaussians (sigma 0.03-0.08, centres U[0.2,0.8]^3), both
    refined by the coefficient-tail rule (tolerance 1e-3, depths 2..3 instead
    of 1e-6 and 3..8), FreeSpace, dt for Chebyshev CFL 1 on the finest leaf;
    two steps against the oracle."""
    from tbslas_gb300 import workloads
    wl = workloads.tree_adaptive_q14(tol=1e-3, depths=(2, 3))
    assert wl.q == 14 and wl.bc == 0 and int(wl.cd.max()) > int(wl.cd.min())
    tv = tb.Tree(ctx, wl.va, wl.vd, wl.q, 3, wl.vc)
    tc = tb.Tree(ctx, wl.ca, wl.cd, wl.q, 1, wl.cc)
    vel = tb.NodeFieldFunctor(tv, wl.bc)
    ref_vel = dict(anchor=wl.va, depth=wl.vd, q=wl.q, dof=3, coeff=wl.vc)
    ref_con = dict(anchor=wl.ca, depth=wl.cd, q=wl.q, dof=1, coeff=wl.cc.copy())
    with ctx.sums_mode(MODES[mode]):
        for step in (1, 2):
            tb.solve_semilag_in_situ(vel, tc, step, wl.dt, 1)
            ref_con["coeff"] = ora.semilag_in_situ(ref_vel, ref_con, step, wl.dt, 1)
            got = tc.get_coeffs()
            assert rel_err(got, ref_con["coeff"]) <= TOL, step
            if mode == "fp64" and step == 1:
                # the FP64 mode's node values are the oracle's bit for bit; the
                # coefficients differ only by the refit's summation order
                assert rel_err(got, ref_con["coeff"]) <= 1e-14


@pytest.mark.parametrize("mode", ["fp64", "df"])
def test_semilag_in_situ_stagnation_on_faces(ctx, ora, mode):
    """Taylor-Green's velocity vanishes on planes that are leaf faces; at q=6
    the fit's error moves the nodes there off the face (at q=14 it does not,
    and those nodes make most of the near-face targets of that workload)."""
    q = 6
    anchor, depth = trees.uniform_tree(3)
    vc = trees.fit(fields.taylor_green(), anchor, depth, q, 3)
    cc = trees.fit(fields.gaussian_blobs(np.random.default_rng(9), 3, (0.06, 0.1)), anchor, depth,
                   q, 1)
    tv = tb.Tree(ctx, anchor, depth, q, 3, vc)
    tc = tb.Tree(ctx, anchor, depth, q, 1, cc)
    ref = dict(anchor=anchor, depth=depth, q=q, dof=1, coeff=cc)
    vel = dict(anchor=anchor, depth=depth, q=q, dof=3, coeff=vc)
    with ctx.sums_mode(MODES[mode]):
        for step in (1, 2, 3):
            tb.solve_semilag_in_situ(tb.NodeFieldFunctor(tv), tc, step, 0.004)
            ref["coeff"] = ora.semilag_in_situ(vel, ref, step, 0.004)
    assert rel_err(tc.get_coeffs(), ref["coeff"]) <= TOL


@pytest.mark.parametrize("flow,bc", [("centre", 0), ("centre", 1), ("corner", 0)])
def test_semilag_in_situ_strain_flow_near_face(ctx, ora, flow, bc):
    """A linear strain flow (fitted exactly) whose normal velocity vanishes
    on leaf faces -- the planes x = 1/2 and y = 1/2 ("centre"), or the domain
    faces x = 0 and y = 0 ("corner") -- keeps the nodes there on the face
    in both paths, where the double-float bound cannot prove it: those
    targets go to the FP64 near-face pass, and the result matches the
    oracle (leaf choices are the FP64 path's)."""
    q, w = 6, 3.0
    o = 0.5 if flow == "centre" else 0.0
    anchor, depth = trees.uniform_tree(3)

    def strain(p):
        return np.stack([w * (p[:, 0] - o), w * (o - p[:, 1]), 0.0 * p[:, 2]], axis=1)
    vc = trees.fit(strain, anchor, depth, q, 3)
    cc = trees.fit(fields.gaussian_blobs(np.random.default_rng(11), 3, (0.06, 0.1)), anchor,
                   depth, q, 1)
    tv = tb.Tree(ctx, anchor, depth, q, 3, vc)
    tc = tb.Tree(ctx, anchor, depth, q, 1, cc)
    ref = dict(anchor=anchor, depth=depth, q=q, dof=1, coeff=cc)
    vel = dict(anchor=anchor, depth=depth, q=q, dof=3, coeff=vc)
    counts = []
    with ctx.sums_mode(tb.SUMS_DOUBLE_FLOAT):
        for step in (1, 2):
            tb.solve_semilag_in_situ(tb.NodeFieldFunctor(tv, bc), tc, step, 0.01)
            ref["coeff"] = ora.semilag_in_situ(vel, ref, step, 0.01, periodic=bool(bc))
            counts.append(ctx.last_fp64_targets())
            assert rel_err(tc.get_coeffs(), ref["coeff"]) <= TOL, (step, counts)
    assert all(n > 0 for n in counts), counts


def test_semilag_in_situ_host_equals_device(ctx):
    rng = np.random.default_rng(5)
    (av, dv, vc), (ac, dc, cc) = _sl_case("uniform", 6, 6, 1, rng)
    tv = tb.Tree(ctx, av, dv, 6, 3, vc)
    tc = tb.Tree(ctx, ac, dc, 6, 1, cc)
    vel = tb.NodeFieldFunctor(tv)
    tb.solve_semilag_in_situ(vel, tc, 1, 0.01)
    dev = tc.get_coeffs()
    host = cc.copy()
    tb.solve_semilag_in_situ(vel, tc, 1, 0.01, coeff_host=host)
    assert np.array_equal(host, dev)


@pytest.mark.parametrize("mode", ["fp64", "df"])
def test_config1_full_size_one_step_matches_oracle(ctx, ora, mode):
    """Depth-4 uniform tree (4096 leaves), q=8, rotation omega=2pi, Gaussian
    sigma=0.05 at (0.7,0.5,0.5), dt=0.01: one full SL step (2,985,984
    departure points) against the oracle."""
    q = 8
    anchor, depth = trees.uniform_tree(4)
    vc = trees.fit(fields.rotation(2 * math.pi), anchor, depth, q, 3)
    cc = trees.fit(fields.gaussian((0.7, 0.5, 0.5), 0.05), anchor, depth, q, 1)
    tv = tb.Tree(ctx, anchor, depth, q, 3, vc)
    tc = tb.Tree(ctx, anchor, depth, q, 1, cc)
    with ctx.sums_mode(MODES[mode]):
        tb.solve_semilag_in_situ(tb.NodeFieldFunctor(tv), tc, 1, 0.01)
    ref = ora.semilag_in_situ(dict(anchor=anchor, depth=depth, q=q, dof=3, coeff=vc),
                              dict(anchor=anchor, depth=depth, q=q, dof=1, coeff=cc), 1, 0.01)
    assert rel_err(tc.get_coeffs(), ref) <= TOL


def test_config1_full_size_translation_exact(ctx):
    """Size-independent property at full size: constant velocity and a
    polynomial of total degree <= q are advected exactly wherever the
    departure points stay inside the domain."""
    q = 8
    anchor, depth = trees.uniform_tree(4)
    v = np.array([0.4, -0.3, 0.2])
    dt = 0.03
    poly = lambda p: (1 + p[:, 0] ** 3 * p[:, 1] ** 2 - 2 * p[:, 2] ** 8 + p[:, 0] * p[:, 1] * p[:, 2] ** 6)[:, None]
    tv = tb.Tree(ctx, anchor, depth, q, 3, trees.fit(lambda p: np.tile(v, (len(p), 1)), anchor, depth, q, 3))
    tc = tb.Tree(ctx, anchor, depth, q, 1, trees.fit(poly, anchor, depth, q, 1))
    tb.solve_semilag_in_situ(tb.NodeFieldFunctor(tv), tc, 1, dt)
    exact = trees.fit(lambda p: poly(p - dt * v), anchor, depth, q, 1)
    h = 1.0 / 16
    safe = np.all((anchor - dt * v >= 0) & (anchor + h - dt * v <= 1), axis=1)
    got = tc.get_coeffs()
    assert safe.sum() > 3000
    assert rel_err(got[safe], exact[safe]) <= 1e-11

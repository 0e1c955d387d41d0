"""The oracle pinned to the reference's own code.

tests/golden/ref_pin.npz and ref_next.npz hold outputs of the reference's
SL-path sources (tree_functor.h, traj.inc, semilag.inc, tree_utils.h,
tree_semilag.h, tree_set_functor.h, tree_extrap_functor.h, cheb.h, cubic.h)
compiled here against stand-ins for PVFMM and MPI (oracle/_ref, recipe
oracle/build_ref.py, generator tests/golden/make_ref_golden.py).
The oracle must reproduce them bit for bit wherever its arithmetic is the
reference's (Chebyshev nodes, grid points, tree evaluation, trajectories,
the tricubic interpolant); the in-situ step, also through the
time-dependent velocity functors, and the advection-diffusion driver's BDF2
step (composed from the reference's functions in the driver's order) differ
only by the pseudo-inverse's and the refit GEMM's summation order (PVFMM's,
restated on both sides).  Where the reference's sources are present the same checks also
run live on fresh seeded cases.  The GPU tests compare the CUDA path with
the same vectors."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
G = np.load(os.path.join(HERE, "golden", "ref_pin.npz"))
STEP_TOL = 1e-13  # refit summation order (pinv, GEMM): observed ~5e-15


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(b).max()


def _eval_cases():
    for q, dof in ((5, 1), (8, 3), (14, 1)):
        a, d = ((G["tree_anchor"], G["tree_depth"]) if q < 14
                else (G["tree1_anchor"], G["tree1_depth"]))
        for bc in (0, 1):
            yield (q, dof, bc, a, d, G["eval_q%d_coeff" % q], G["eval_q%d_bc%d_pts" % (q, bc)],
                   G["eval_q%d_bc%d_out" % (q, bc)])


def _step_trees():
    vel = dict(anchor=G["step_va"], depth=G["step_vd"], q=6, dof=3, coeff=G["step_vc"])
    con = dict(anchor=G["step_ca"], depth=G["step_cd"], q=6, dof=1, coeff=G["step_cc"])
    return vel, con


def test_oracle_nodes_and_grid_points_equal_the_reference(ora):
    for q in (6, 8, 14):
        got = ora.collect_grid_points(np.zeros((1, 3)), np.zeros(1, dtype=np.int32), q)
        assert np.array_equal(got, G["nodes_q%d" % q]), q
    got = ora.collect_grid_points(G["tree_anchor"], G["tree_depth"], 3)
    assert np.array_equal(got, G["collect_q3"])


def test_oracle_tree_evaluation_equals_the_reference(ora):
    for q, dof, bc, a, d, c, p, ref in _eval_cases():
        got = ora.eval_tree(a, d, q, dof, c, p, periodic=bool(bc))
        assert np.array_equal(got, ref), (q, dof, bc, np.abs(got - ref).max())


def test_oracle_trajectories_equal_the_reference(ora):
    for bc, nrk in ((0, 1), (1, 1), (0, 3)):
        got = ora.traj_rk2(G["traj_anchor"], G["traj_depth"], 8, G["traj_vc"], G["traj_pts"],
                           0.3, 0.25, nrk, periodic=bool(bc))
        assert np.array_equal(got, G["traj_bc%d_nrk%d" % (bc, nrk)]), (bc, nrk)


def test_oracle_tricubic_interpolant_equals_the_reference(ora):
    got = ora.fast_interp(G["interp_grid"].ravel(), 3, 12, G["interp_pts"], periodic=False)
    assert np.array_equal(got, G["interp_out"])


def test_oracle_in_situ_step_matches_the_reference(ora):
    vel, con = _step_trees()
    for bc in (0, 1):
        got = ora.semilag_in_situ(vel, con, 2, 0.02, 1, bool(bc))
        assert _rel(got, G["step_bc%d_out" % bc]) <= STEP_TOL, bc


NEXT = np.load(os.path.join(HERE, "golden", "ref_next.npz"))


def _tv_case(i):
    pre = "case%d_" % i
    nv = 4 if int(NEXT[pre + "set"]) else 2
    q = int(NEXT["q"])
    vels = [dict(anchor=NEXT[pre + "v%d_anchor" % k], depth=NEXT[pre + "v%d_depth" % k], q=q,
                 dof=3, coeff=NEXT[pre + "v%d_coeff" % k]) for k in range(nv)]
    con = dict(anchor=NEXT["con_anchor"], depth=NEXT["con_depth"], q=q, dof=1,
               coeff=NEXT["con_coeff"])
    times = NEXT["times"] if nv == 4 else None
    return vels, con, bool(int(NEXT[pre + "periodic"])), times, NEXT[pre + "out"]


def test_oracle_time_dependent_step_matches_the_reference(ora):
    """The in-situ step through the reference's FieldSetFunctor (four trees,
    cubic in time) and its two-functor form with FieldExtrapFunctor, on trees
    of one and of different leaf structures, free space and periodic: the
    oracle's composition to the refit's summation order."""
    for i in range(int(NEXT["n_cases"])):
        vels, con, periodic, times, want = _tv_case(i)
        got = ora.semilag_in_situ_tv(vels, con, int(NEXT["timestep"]), float(NEXT["dt"]), 1,
                                     periodic, times=times)
        assert _rel(got, want) <= STEP_TOL, i


def test_oracle_bdf2_step_matches_the_reference(ora):
    """The driver's BDF2 step (src/applications/src/advdiff-ss.cpp:485-521:
    two in-place ComputeTrajRK2 backtraces, c_n at X1, c_{n-1} at X2, 4/3 and
    1/3, SetTreeGridValues) on three trees of different leaves."""
    q = int(NEXT["q"])
    prev = dict(anchor=NEXT["bdf2_pa"], depth=NEXT["bdf2_pd"], q=q, dof=1, coeff=NEXT["bdf2_pc"])
    cur = dict(anchor=NEXT["bdf2_ca"], depth=NEXT["bdf2_cd"], q=q, dof=1, coeff=NEXT["bdf2_cc"])
    nxt = dict(anchor=NEXT["bdf2_na"], depth=NEXT["bdf2_nd"], q=q, dof=1)
    from tbslas_gb300 import trees
    va, vd = trees.uniform_tree(1)
    for bc in (0, 1):
        vel = dict(anchor=va, depth=vd, q=q, dof=3, coeff=NEXT["bdf2_bc%d_vc" % bc])
        got = ora.semilag_bdf2(vel, prev, cur, nxt, 0.3, 0.02, 1, bool(bc))
        want = NEXT["bdf2_bc%d_out" % bc]
        assert _rel(np.reshape(got, want.shape), want) <= STEP_TOL, bc


def test_oracle_interp_cubic_1d_matches_the_reference(ora):
    """CubicInterpPolicy::InterpCubic1D (src/utils/cubic.h:42-56): the oracle's
    restatement to the rounding of the reference's contracted build."""
    x, xx, pp, want = NEXT["cubic_x"], NEXT["cubic_xx"], NEXT["cubic_pp"], NEXT["cubic_out"]
    got = np.array([ora.interp_cubic_1d(x[i], xx[i], pp[i]) for i in range(len(x))])
    assert np.all(np.abs(got - want) <= 1e-13 * (1.0 + np.abs(want)))


@pytest.fixture(scope="module")
def ref():
    from oracle import ref as r
    if r.lib() is None:
        pytest.skip("the reference's sources are not present on this machine")
    return r


@pytest.mark.parametrize("seed", [1, 2])
def test_live_oracle_equals_the_reference(ora, ref, seed):
    """Fresh seeded cases through the reference built here: evaluation and
    trajectories on adaptive trees bit for bit; the point-to-coefficient
    matrix to the two pseudo-inverses' rounding; the in-situ step."""
    from tbslas_gb300 import fields, trees
    rng = np.random.default_rng(seed)
    with trees.host_math(trees.HostMath(
            nodes=lambda q: ora.collect_grid_points(np.zeros((1, 3)),
                                                    np.zeros(1, dtype=np.int32), q),
            pt2coeff=ora.pt2coeff)):
        blob = fields.gaussian(tuple(rng.uniform(0.3, 0.7, 3)), 0.08)
        a, d = trees.adaptive_tree(blob, 4, 1, 1e-3, 1, 3)
        for q, dof in ((4, 1), (7, 3), (11, 1)):
            c = rng.standard_normal((len(d), dof, ref.nc(q)))
            for bc in (0, 1):
                p = rng.uniform(0.0, 1.0, (4000, 3)) if bc == 0 else rng.uniform(-0.1, 1.1,
                                                                                 (4000, 3))
                assert np.array_equal(ora.eval_tree(a, d, q, dof, c, p, bool(bc)),
                                      ref.eval_tree(a, d, q, dof, c, p, bc)), (q, bc)
        vc = trees.fit(fields.taylor_green(), a, d, 7, 3)
        x = rng.uniform(0, 1, (4000, 3))
        for bc, nrk in ((0, 1), (1, 2)):
            assert np.array_equal(ora.traj_rk2(a, d, 7, vc, x, 0.4, 0.37, nrk, bool(bc)),
                                  ref.traj_rk2(a, d, 7, vc, x, 0.4, 0.37, nrk, bc))
        for q in (3, 8, 14):
            M = ref.pt2coeff(q)
            assert _rel(ora.pt2coeff(q), M) <= 1e-12, q  # SVD vs QR pseudo-inverse
        cc = trees.fit(blob, a, d, 7, 1)
        vel = dict(anchor=a, depth=d, q=7, dof=3, coeff=vc)
        con = dict(anchor=a, depth=d, q=7, dof=1, coeff=cc)
        assert _rel(ora.semilag_in_situ(vel, con, 3, 0.01, 1, False),
                    ref.semilag_in_situ(vel, con, 3, 0.01, 1, False)) <= STEP_TOL


def test_live_reference_refits_multi_dof_values_in_the_wrong_layout(ora, ref):
    """A documented difference, shown on the reference's own code: its
    in-situ step hands EvalTree's point-major values [node][dof] to
    SetTreeGridValues, which reads each leaf's block as dof-major
    [dof][node] (src/tree/tree_semilag.h:120-133, src/tree/tree_utils.h:
    500-552).  For dof = 1 the layouts coincide; for dof > 1 the reference's
    result is the fit of the transposed block, while this library and the
    oracle fit each dof's own values."""
    from tbslas_gb300 import fields, trees
    q, dof = 4, 2
    a, d = trees.uniform_tree(1)
    blob = fields.gaussian((0.45, 0.5, 0.55), 0.15)
    M = ora.pt2coeff(q)
    with trees.host_math(trees.HostMath(
            nodes=lambda qq: ora.collect_grid_points(np.zeros((1, 3)),
                                                     np.zeros(1, dtype=np.int32), qq),
            pt2coeff=ora.pt2coeff)):
        vc = trees.fit(fields.taylor_green(), a, d, q, 3)
        cc = trees.fit(lambda p: np.concatenate([blob(p), 2 * blob(p) + p[:, :1]], axis=1),
                       a, d, q, dof)
    vel = dict(anchor=a, depth=d, q=q, dof=3, coeff=vc)
    con = dict(anchor=a, depth=d, q=q, dof=dof, coeff=cc)
    got_ref = ref.semilag_in_situ(vel, con, 1, 0.02, 1, False)
    # the reference's result from its own parts: departure points, values
    # point-major, each leaf's block read dof-major, fitted
    pts = ref.collect_grid_points(a, d, q)
    dep = ref.traj_rk2(a, d, q, vc, pts, 0.02, 0.0, 1, False)
    vals = ref.eval_tree(a, d, q, dof, cc, dep, 0)           # [L*Np][dof]
    L, Np = len(d), (q + 1) ** 3
    misread = vals.reshape(L, Np * dof).reshape(L * dof, Np)  # the leaf block read [dof][Np]
    assert _rel(got_ref, (misread @ M).reshape(L, dof, -1)) <= STEP_TOL
    ours = ora.semilag_in_situ(vel, con, 1, 0.02, 1, False)
    assert _rel(ours, got_ref) > 1e-3


# ---------------------------------------------------------------------------
# the CUDA path against the reference's vectors

def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.mark.gpu
def test_device_functor_and_trajectories_equal_the_reference(ctx):
    import tbslas_gb300 as tb
    for q, dof, bc, a, d, c, p, ref in _eval_cases():
        t = tb.Tree(ctx, a, d, q, dof, c)
        got = tb.NodeFieldFunctor(t, bc)(_dev(p)).cpu().numpy()
        assert np.array_equal(got, ref), (q, dof, bc)
        t.close()
    tv = tb.Tree(ctx, G["traj_anchor"], G["traj_depth"], 8, 3, G["traj_vc"])
    for bc, nrk in ((0, 1), (1, 1), (0, 3)):
        got = tb.compute_traj_rk2(tb.NodeFieldFunctor(tv, bc), _dev(G["traj_pts"]), 0.3, 0.25,
                                  nrk).cpu().numpy()
        assert np.array_equal(got, G["traj_bc%d_nrk%d" % (bc, nrk)]), (bc, nrk)
    tv.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "df"])
def test_device_in_situ_step_matches_the_reference(ctx, mode):
    import tbslas_gb300 as tb
    vel, con = _step_trees()
    tv = tb.Tree(ctx, vel["anchor"], vel["depth"], 6, 3, vel["coeff"])
    sums = tb.SUMS_FP64 if mode == "fp64" else tb.SUMS_DOUBLE_FLOAT
    for bc in (0, 1):
        tc = tb.Tree(ctx, con["anchor"], con["depth"], 6, 1, con["coeff"])
        with ctx.sums_mode(sums):
            tb.solve_semilag_in_situ(tb.NodeFieldFunctor(tv, bc), tc, 2, 0.02, 1)
        assert _rel(tc.get_coeffs(), G["step_bc%d_out" % bc]) <= 1e-12, bc
        tc.close()
    tv.close()


@pytest.mark.gpu
def test_device_tricubic_interpolant_matches_the_reference(ctx):
    import tbslas_gb300 as tb
    got = tb.fast_interp(ctx, _dev(G["interp_grid"]), 3, 12, _dev(G["interp_pts"]),
                         tb.FreeSpace).cpu().numpy()
    assert _rel(got, G["interp_out"]) <= 1e-12


def test_live_time_dependent_step_matches_the_reference(ora, ref):
    """A fresh case through the reference's time-dependent functors built
    here: q = 6, periodic Fourier velocities of different leaf structures."""
    from tbslas_gb300 import fields, trees
    rng = np.random.default_rng(5)
    with trees.host_math(trees.HostMath(
            nodes=lambda q: ora.collect_grid_points(np.zeros((1, 3)),
                                                    np.zeros(1, dtype=np.int32), q),
            pt2coeff=ora.pt2coeff)):
        q = 6
        vels = []
        for k in range(4):
            base = fields.fourier_velocity(np.random.default_rng(40 + k))
            g = fields.gaussian(tuple(rng.uniform(0.3, 0.7, 3)), 0.1)
            a, d = trees.adaptive_tree(g, q, 1, 1e-3, 1, 2)
            vels.append(dict(anchor=a, depth=d, q=q, dof=3,
                             coeff=trees.fit(lambda p: 0.3 * base(p), a, d, q, 3)))
        blob = fields.gaussian((0.4, 0.55, 0.5), 0.1)
        ca, cd = trees.adaptive_tree(blob, q, 1, 1e-3, 1, 2)
        con = dict(anchor=ca, depth=cd, q=q, dof=1, coeff=trees.fit(blob, ca, cd, q, 1))
        times = [0.0, 0.015, 0.03, 0.05]
        for vs, t in ((vels, times), (vels[:2], None)):
            want = ref.semilag_in_situ_tv(vs, con, 2, 0.015, 2, True, times=t)
            got = ora.semilag_in_situ_tv(vs, con, 2, 0.015, 2, True, times=t)
            assert _rel(got, want) <= STEP_TOL

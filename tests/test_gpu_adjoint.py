"""Adjoint of the in-situ SL step: the checkpointed forward is the in-situ
step storing its points (the oracle's departure points bit for bit in the
FP64 mode, the same leaves in the double-float mode); dJ/dc0 and dJ/dV from
the hand-written adjoint (behind torch.autograd) match central finite
differences (eps = 1e-6) along seeded random directions to 1e-6 relative and
forward-mode dual numbers through the oracle to 1e-10; checkpointing and
recomputation give the same gradients."""
import numpy as np
import pytest

import tbslas_gb300 as tb
from tbslas_gb300 import adjoint, fields, trees

pytestmark = pytest.mark.gpu


def _problem(ctx, q=5, depth=2, seed=3):
    rng = np.random.default_rng(seed)
    a, d = trees.uniform_tree(depth)
    vel_fn = fields.fourier_velocity(rng)
    vc = trees.fit(lambda p: 0.5 * vel_fn(p), a, d, q, 3)
    c0 = trees.fit(fields.gaussian((0.5, 0.45, 0.55), 0.12), a, d, q, 1)
    cobs = trees.fit(fields.gaussian((0.52, 0.47, 0.5), 0.11), a, d, q, 1)
    tv = tb.Tree(ctx, a, d, q, 3, vc)
    tc = tb.Tree(ctx, a, d, q, 1, c0)
    return a, d, q, vc, c0, cobs, tv, tc


def test_ckpt_step_matches_plain_step_and_oracle(ctx, ora):
    """The checkpointed step is the in-situ step of the context's sum mode
    (same coefficients, bit for bit) storing its points.  FP64 mode: the
    departure points are the oracle's bit for bit.  Double-float mode: they are
    within 1e-13 of the oracle's (the velocity sums' rounding times tau) and in
    the same leaves (targets near a face are recomputed in FP64)."""
    import torch
    a, d, q, vc, c0, _, tv, tc = _problem(ctx)
    vf = tb.NodeFieldFunctor(tv, tb.Periodic)
    n = len(d) * (q + 1) ** 3
    pts = ora.collect_grid_points(a, d, q)
    ref = ora.traj_rk2(a, d, q, vc, pts, 0.03, 0.0, 1, periodic=True)
    xw = np.mod(pts, 1.0)
    ref_mid = xw + (-0.015) * ora.eval_tree(a, d, q, 3, vc, xw, periodic=True)
    cells = 2 ** int(d.max())

    def leaf_of(x):
        return np.floor(np.mod(x, 1.0) * cells)

    try:
        for mode in (tb.SUMS_FP64, tb.SUMS_DOUBLE_FLOAT):
            ctx.sums = mode
            xm = torch.full((n, 3), np.nan, dtype=torch.float64, device="cuda")
            xd = torch.full_like(xm, np.nan)
            tc.set_coeffs(c0)
            adjoint.step_ckpt(vf, tc, 1, 0.03, xm, xd)
            got = tc.get_coeffs()
            tc.set_coeffs(c0)
            tb.solve_semilag_in_situ(vf, tc, 1, 0.03)
            assert np.array_equal(got, tc.get_coeffs())
            xd, xm = xd.cpu().numpy(), xm.cpu().numpy()
            assert np.abs(xm - ref_mid).max() <= 1e-15
            assert np.array_equal(leaf_of(xm), leaf_of(ref_mid))
            if mode == tb.SUMS_FP64:
                assert np.array_equal(xd, ref)
            else:
                assert np.abs(xd - ref).max() <= 1e-13
                assert np.array_equal(leaf_of(xd), leaf_of(ref))
    finally:
        ctx.sums = tb.SUMS_FP64  # the library default


def _J(c, V, cobs):
    import torch
    vals = torch.einsum("ln,pn->lp", c[:, 0, :], V)
    ovals = torch.einsum("ln,pn->lp", cobs[:, 0, :], V)
    return 0.5 * ((vals - ovals) ** 2).sum()


@pytest.mark.parametrize("checkpoint", [True, False, "jacobian"])
def test_adjoint_matches_central_differences(ctx, checkpoint):
    """Central differences, eps = 1e-6, along seeded random directions: N(0,1)
    coefficients for c0 (J is quadratic in c0), smooth random velocity fields
    for V.  J is only piecewise smooth in V: the per-leaf fits differ across a
    leaf face, so a departure point that the eps-perturbation pushes across a
    face makes the quotient jump.  At q = 4 on this seeded problem no point
    lies within that distance of a face (the quotients at eps = 1e-4 .. 1e-7
    agree to 1e-8); at q = 5 some do, and there the exact check is the
    dual-number test below, which holds leaf choices fixed."""
    import torch
    a, d, q, vc, c0, cobs, tv, tc = _problem(ctx, q=4)
    V = torch.from_numpy(adjoint.basis_at_nodes(q)).cuda()
    co = torch.from_numpy(cobs).cuda()
    c0t = torch.from_numpy(c0).cuda().requires_grad_(True)
    vct = torch.from_numpy(vc).cuda().requires_grad_(True)
    dt, steps = 0.03, 3
    cT = adjoint.advect(c0t, vct, tv, tc, dt, 1, steps, tb.Periodic, checkpoint)
    _J(cT, V, co).backward()
    gc, gv = c0t.grad.clone(), vct.grad.clone()

    def J_at(c, v):
        with torch.no_grad():
            return _J(adjoint.advect(c, v, tv, tc, dt, 1, steps, tb.Periodic, False), V, co).item()

    rng = np.random.default_rng(11)
    eps = 1e-6
    for _ in range(4):
        dc = torch.from_numpy(rng.standard_normal(c0.shape)).cuda()
        fd = (J_at(c0t.detach() + eps * dc, vct.detach()) -
              J_at(c0t.detach() - eps * dc, vct.detach())) / (2 * eps)
        an = (gc * dc).sum().item()
        assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)
        fv = fields.fourier_velocity(rng)
        dv = torch.from_numpy(trees.fit(fv, a, d, q, 3)).cuda()
        fd = (J_at(c0t.detach(), vct.detach() + eps * dv) -
              J_at(c0t.detach(), vct.detach() - eps * dv)) / (2 * eps)
        an = (gv * dv).sum().item()
        assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)


def test_adjoint_checkpoint_equals_recompute(ctx):
    import torch
    a, d, q, vc, c0, cobs, tv, tc = _problem(ctx, q=4, seed=5)
    V = torch.from_numpy(adjoint.basis_at_nodes(q)).cuda()
    co = torch.from_numpy(cobs).cuda()
    grads = []
    for ck in (True, "departure", False, "jacobian"):
        c0t = torch.from_numpy(c0).cuda().requires_grad_(True)
        vct = torch.from_numpy(vc).cuda().requires_grad_(True)
        _J(adjoint.advect(c0t, vct, tv, tc, 0.02, 1, 4, tb.Periodic, ck), V, co).backward()
        grads.append((c0t.grad.cpu().numpy(), vct.grad.cpu().numpy()))
    # departure-only checkpoints rebuild the forward's midpoints exactly (the
    # gradients differ only by the order of the FP64 atomics)
    for x, y in zip(grads[0], grads[1]):
        assert np.abs(x - y).max() <= 1e-14 * np.abs(y).max()
    for x, y in zip(grads[0], grads[2]):
        assert np.abs(x - y).max() <= 1e-12 * np.abs(y).max()
    # the Jacobian checkpoint forms J_v(X*)^T g from the stored Jacobian
    # (rounding of a different order than the coefficient-level sum)
    for x, y in zip(grads[3], grads[0]):
        assert np.abs(x - y).max() <= 1e-12 * np.abs(y).max()


@pytest.mark.parametrize("bc", [tb.FreeSpace, tb.Periodic])
def test_ckpt_jac_step_equals_ckpt_step_and_linear_jacobian(ctx, bc):
    """The Jacobian checkpoint's forward is the checkpointed step bit for bit
    (coefficients, midpoints, departure points).  On a linear velocity
    (represented exactly by the fit) the stored Jacobian is its matrix at
    every midpoint inside the domain, to the fit's rounding, and zero
    outside."""
    import torch
    q, A = 5, np.array([[0.3, -1.1, 0.2], [0.9, -0.4, 0.5], [-0.2, 0.7, 0.1]])
    a, d = trees.uniform_tree(2)
    vc = trees.fit(lambda p: (p - 0.5) @ A.T + 0.05, a, d, q, 3)
    c0 = trees.fit(fields.gaussian((0.5, 0.45, 0.55), 0.12), a, d, q, 1)
    tv = tb.Tree(ctx, a, d, q, 3, vc)
    tc = tb.Tree(ctx, a, d, q, 1, c0)
    vf = tb.NodeFieldFunctor(tv, bc)
    n = len(d) * (q + 1) ** 3
    out = []
    for jac in (False, True):
        tc.set_coeffs(c0)
        xm = torch.full((n, 3), np.nan, dtype=torch.float64, device="cuda")
        xd = torch.full_like(xm, np.nan)
        if jac:
            J = torch.full((n, 9), np.nan, dtype=torch.float64, device="cuda")
            adjoint.step_ckpt_jac(vf, tc, 1, 0.05, xm, xd, J)
        else:
            adjoint.step_ckpt(vf, tc, 1, 0.05, xm, xd)
        out.append((tc.get_coeffs(), xm.cpu().numpy(), xd.cpu().numpy()))
    for x, y in zip(out[0], out[1]):
        assert np.array_equal(x, y)
    J = J.cpu().numpy().reshape(n, 3, 3)
    xm = out[1][1]
    inside = np.all((xm >= 0.0) & (xm <= 1.0), axis=1) if bc == tb.FreeSpace else np.ones(n, bool)
    assert inside.any()
    assert np.abs(J[inside] - A[None]).max() <= 1e-12
    assert np.all(J[~inside] == 0.0)


def test_ckpt_jac_needs_fp64_sums(ctx):
    import torch
    a, d, q, vc, c0, cobs, tv, tc = _problem(ctx, q=3)
    vf = tb.NodeFieldFunctor(tv, tb.Periodic)
    n = len(d) * (q + 1) ** 3
    xm = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    J = torch.zeros((n, 9), dtype=torch.float64, device="cuda")
    try:
        ctx.sums = tb.SUMS_DOUBLE_FLOAT
        with pytest.raises(tb.capi.TbslasError):
            adjoint.step_ckpt_jac(vf, tc, 1, 0.05, xm, xm.clone(), J)
    finally:
        ctx.sums = tb.SUMS_FP64


@pytest.mark.parametrize("vel_kind,q", [("fourier", 4), ("taylor_green", 4), ("fourier", 5),
                                        ("fourier", 7)])
def test_adjoint_matches_dual_number_oracle(ctx, ora, vel_kind, q):
    """Exact directional derivative of the discrete T-step map (forward-mode
    dual numbers through the oracle, leaf choices held fixed) against the
    adjoint's gradient."""
    import torch
    steps, dt = 3, 0.03
    a, d = trees.uniform_tree(2)
    if vel_kind == "fourier":
        fn = fields.fourier_velocity(np.random.default_rng(3))
        vc = trees.fit(lambda p: 0.5 * fn(p), a, d, q, 3)
        bc = tb.Periodic
    else:
        vc = trees.fit(fields.taylor_green(), a, d, q, 3)
        bc = tb.FreeSpace
    c0 = trees.fit(fields.gaussian((0.5, 0.45, 0.55), 0.12), a, d, q, 1)
    cobs = trees.fit(fields.gaussian((0.52, 0.47, 0.5), 0.11), a, d, q, 1)
    tv = tb.Tree(ctx, a, d, q, 3, vc)
    tc = tb.Tree(ctx, a, d, q, 1, c0)
    Vb = adjoint.basis_at_nodes(q)
    c0t = torch.from_numpy(c0).cuda().requires_grad_(True)
    vct = torch.from_numpy(vc).cuda().requires_grad_(True)
    J = _J(adjoint.advect(c0t, vct, tv, tc, dt, 1, steps, bc, True),
           torch.from_numpy(Vb).cuda(), torch.from_numpy(cobs).cuda())
    J.backward()
    gc, gv = c0t.grad.cpu().numpy(), vct.grad.cpu().numpy()
    rng = np.random.default_rng(17)
    for _ in range(3):
        dc0, dvc = rng.standard_normal(c0.shape), rng.standard_normal(vc.shape)
        vel = dict(anchor=a, depth=d, q=q, dof=3, coeff=vc)
        c, dcur = c0, dc0
        for s in range(1, steps + 1):
            c, dcur = ora.semilag_in_situ_dual(vel, dvc, dict(anchor=a, depth=d, q=q, dof=1, coeff=c),
                                               dcur, s, dt, 1, bc == tb.Periodic)
        resid = c[:, 0, :] @ Vb.T - cobs[:, 0, :] @ Vb.T
        dJ = float((resid * (dcur[:, 0, :] @ Vb.T)).sum())
        an = float((gc * dc0).sum() + (gv * dvc).sum())
        assert abs(dJ - an) <= 1e-10 * abs(dJ), (dJ, an)


@pytest.mark.parametrize("checkpoint", [True, False])
def test_adjoint_fp64_sums_matches_double_float(ctx, checkpoint):
    """The all-FP64 adjoint kernel (TBSLAS_SUMS_FP64, the default) and the
    double-float one give the same gradients to 1e-12."""
    import torch
    a, d, q, vc, c0, cobs, tv, tc = _problem(ctx, q=6, seed=9)
    V = torch.from_numpy(adjoint.basis_at_nodes(q)).cuda()
    co = torch.from_numpy(cobs).cuda()
    grads = []
    try:
        for mode in (tb.SUMS_DOUBLE_FLOAT, tb.SUMS_FP64):
            ctx.sums = mode
            c0t = torch.from_numpy(c0).cuda().requires_grad_(True)
            vct = torch.from_numpy(vc).cuda().requires_grad_(True)
            _J(adjoint.advect(c0t, vct, tv, tc, 0.02, 1, 3, tb.Periodic, checkpoint), V,
               co).backward()
            grads.append((c0t.grad.cpu().numpy(), vct.grad.cpu().numpy()))
    finally:
        ctx.sums = tb.SUMS_FP64  # the library default
    for x, y in zip(grads[0], grads[1]):
        assert np.abs(x - y).max() <= 1e-12 * np.abs(y).max()


@pytest.mark.parametrize("mode", ["fp64", "double_float"])
@pytest.mark.parametrize("checkpoint", [True, "departure", False])
def test_adjoint_sequence_equals_per_step_scatters(ctx, checkpoint, mode):
    """The backward pass sums the node term's weights over the steps and
    scatters them once (tbslas_semilag_adjoint_seq + _node_term), with the
    velocity at the nodes evaluated once where the points are rebuilt.  It
    equals a loop of tbslas_semilag_adjoint calls, each scattering its own
    node term, up to the order of the FP64 additions: the scatters' atomics
    add in no fixed order (observed up to 2.5e-14 relative in the
    double-float mode), so the gate is the suite's 1e-12; a missing or
    doubled node term would be off by O(1)."""
    import torch
    a, d, q, vc, c0, cobs, tv, tc = _problem(ctx, q=5, seed=7)
    V = torch.from_numpy(adjoint.basis_at_nodes(q)).cuda()
    co = torch.from_numpy(cobs).cuda()
    dt, steps, n = 0.02, 4, len(d) * (q + 1) ** 3
    try:
        ctx.sums = tb.SUMS_FP64 if mode == "fp64" else tb.SUMS_DOUBLE_FLOAT
        c0t = torch.from_numpy(c0).cuda().requires_grad_(True)
        vct = torch.from_numpy(vc).cuda().requires_grad_(True)
        cT = adjoint.advect(c0t, vct, tv, tc, dt, 1, steps, tb.Periodic, checkpoint)
        _J(cT, V, co).backward()
        # per-step reference: forward states and points, then one
        # tbslas_semilag_adjoint per step
        vf = tb.NodeFieldFunctor(tv, tb.Periodic)
        tv.set_coeffs(vc)
        tc.set_coeffs(c0)
        states, pts = [], []
        for k in range(steps):
            states.append(tc.get_coeffs(torch.empty_like(c0t)))
            xd = torch.empty((n, 3), dtype=torch.float64, device="cuda")
            xm = torch.empty_like(xd)
            adjoint.step_ckpt(vf, tc, 1 + k, dt, xm, xd)
            pts.append((xm if checkpoint is True else None, xd if checkpoint else None))
        cT2 = tc.get_coeffs(torch.empty_like(c0t))
        assert torch.equal(cT2, cT.detach())
        cT2.requires_grad_(True)
        _J(cT2, V, co).backward()
        lam = cT2.grad.contiguous().clone()
        gv = torch.zeros_like(vct)
        for k in reversed(range(steps)):
            lam_k = torch.empty_like(lam)
            adjoint.step_adjoint(vf, tc, states[k], 1 + k, dt, lam, lam_k, gv, *pts[k])
            lam = lam_k
    finally:
        ctx.sums = tb.SUMS_FP64  # the library default
    assert np.abs((c0t.grad - lam).cpu().numpy()).max() <= 1e-12 * lam.abs().max().item()
    assert np.abs((vct.grad - gv).cpu().numpy()).max() <= 1e-12 * gv.abs().max().item()

"""GPU parity of the tricubic regular-grid path against the oracle.

Tolerance: max |gpu - oracle| <= 1e-12 * max |oracle| (FP64)."""
import numpy as np
import pytest

import tbslas_gb300 as tb
from tbslas_gb300 import fields

pytestmark = pytest.mark.gpu
TOL = 1e-12


def rel_err(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.mark.parametrize("bc", [0, 1])
@pytest.mark.parametrize("dof", [1, 3])
def test_fast_interp_matches_oracle(ctx, ora, bc, dof):
    rng = np.random.default_rng(dof + 2 * bc)
    N = 20
    grid = rng.standard_normal((dof, N, N, N))
    pts = rng.uniform(-0.1, 1.1, size=(30000, 3))
    pts[:6] = [[1.0, 1.0, 1.0], [0.0, 0.0, 0.0], [np.nan, 0.1, 0.1], [0.5, 1.0, 0.0],
               [1 - 1e-17, 0.3, 0.3], [-1e-300, 0.2, 0.2]]
    out = tb.fast_interp(ctx, _dev(grid), dof, N, _dev(pts), bc).cpu().numpy()
    ref = ora.fast_interp(grid.ravel(), dof, N, pts, periodic=bool(bc))
    assert rel_err(out, ref) <= TOL
    assert np.array_equal(out == 0, ref == 0)


@pytest.mark.parametrize("bc,nrk,N", [(1, 1, 32), (1, 2, 24), (0, 1, 32), (0, 2, 17)])
def test_semilag_grid_matches_oracle(ctx, ora, bc, nrk, N):
    rng = np.random.default_rng(N)
    if bc:
        vel = fields.fourier_velocity_grid(rng, N)
        con = fields.periodic_blob_grid(N, (0.4, 0.55, 0.5), 0.12)
    else:
        vel = rng.standard_normal((3, N, N, N)) * 0.3
        con = rng.standard_normal((N, N, N))
    dt = 1.5 / N
    out = tb.semilag_grid(ctx, _dev(vel), _dev(con), N, dt, nrk, bc).cpu().numpy()
    ref = ora.semilag_grid(vel, con, N, dt, nrk, periodic=bool(bc)).reshape(N, N, N)
    assert rel_err(out, ref) <= TOL
    host = tb.semilag_grid(ctx, vel, con, N, dt, nrk, bc)
    assert np.array_equal(host, out)


def test_semilag_grid_full_size_shift_and_sample(ctx, ora):
    """256^3 periodic: (1) a velocity that moves every departure point one
    node reproduces the shifted field -- exactly with FP64 stencil sums (the
    default), to the double-float split (2^-48 relative per value) with
    double-float sums; (2) one step of the config's random Fourier field matches the
    oracle on a sample of nodes."""
    import torch
    N = 256
    rng = np.random.default_rng(11)
    con = fields.periodic_blob_grid(N, (0.45, 0.5, 0.55), 0.1)
    vel = np.zeros((3, N, N, N))
    vel[1] = -0.5
    shifted = np.roll(con, -1, axis=1)
    with ctx.sums_mode(tb.SUMS_FP64):
        out = tb.semilag_grid(ctx, _dev(vel), _dev(con), N, 2.0 / N, 1, 1).cpu().numpy()
    assert np.array_equal(out, shifted)
    with ctx.sums_mode(tb.SUMS_DOUBLE_FLOAT):
        out = tb.semilag_grid(ctx, _dev(vel), _dev(con), N, 2.0 / N, 1, 1).cpu().numpy()
    assert np.all(np.abs(out - shifted) <= 2.0 ** -47 * np.abs(shifted))
    vel = fields.fourier_velocity_grid(rng, N)
    dt = 2.0 / N / np.abs(vel).max()
    out = tb.semilag_grid(ctx, _dev(vel), _dev(con), N, dt, 1, 1).cpu().numpy().ravel()
    for lo in (0, N ** 3 // 2 + 12345, N ** 3 - 40000):
        ref = ora.semilag_grid(vel, con, N, dt, 1, True, lo, lo + 40000)
        assert rel_err(out[lo:lo + 40000], ref) <= TOL
    del torch


@pytest.mark.parametrize("N", [16, 24])
def test_semilag_grid_nan_velocity_matches_fp64_sums(ctx, N):
    """A non-finite velocity value (NaN, inf) gives the FP64 path's result in
    the double-float path too: the point it moves is 'outside' (value 0, no
    stencil read), exactly as make_stencil treats it."""
    rng = np.random.default_rng(N)
    vel = fields.fourier_velocity_grid(rng, N)
    con = fields.periodic_blob_grid(N, (0.4, 0.55, 0.5), 0.12)
    vel[0, 3, 4, 5] = np.nan
    vel[2, 1, 7, 2] = np.inf
    dt = 1.5 / N
    with ctx.sums_mode(tb.SUMS_DOUBLE_FLOAT):
        out = tb.semilag_grid(ctx, _dev(vel), _dev(con), N, dt, 1, 1).cpu().numpy()
    with ctx.sums_mode(tb.SUMS_FP64):
        ref = tb.semilag_grid(ctx, _dev(vel), _dev(con), N, dt, 1, 1).cpu().numpy()
    assert np.array_equal(np.isnan(out), np.isnan(ref))
    ok = ~np.isnan(ref)
    assert np.abs(out[ok] - ref[ok]).max() <= 1e-13 * np.abs(ref[ok]).max()
    # the double-float split reported the non-finite values (kErrDfRange)
    with pytest.raises(tb.capi.TbslasError) as e:
        ctx.check()
    assert e.value.status == 7  # TBSLAS_ERR_DEVICE


@pytest.mark.parametrize("mode", ["fp64", "df"])
@pytest.mark.parametrize("bc,N", [(1, 32), (1, 20), (0, 24)])
def test_grid_steps_equal_repeated_single_steps(ctx, mode, bc, N):
    """tbslas_semilag_grid_steps (one stationary velocity, split once in the
    double-float mode) equals the same number of single steps bit for bit."""
    import torch
    rng = np.random.default_rng(N + bc)
    vel = fields.fourier_velocity_grid(rng, N) if bc else rng.standard_normal((3, N, N, N)) * 0.3
    con = (fields.periodic_blob_grid(N, (0.4, 0.55, 0.5), 0.12) if bc
           else rng.standard_normal((N, N, N)))
    dt = 1.5 / N
    v, c0 = _dev(vel), _dev(con)
    with ctx.sums_mode(tb.SUMS_FP64 if mode == "fp64" else tb.SUMS_DOUBLE_FLOAT):
        a, b = c0.clone(), torch.empty_like(c0)
        for k in range(5):
            tb.semilag_grid(ctx, v, a, N, dt, 1, bc, out=b)
            a, b = b, a
        many = tb.semilag_grid_steps(ctx, v, c0, N, dt, 5, 1, bc)
        one = tb.semilag_grid_steps(ctx, v, c0, N, dt, 1, 1, bc)
        single = tb.semilag_grid(ctx, v, c0, N, dt, 1, bc)
    assert torch.equal(many, a)
    assert torch.equal(one, single)
    assert np.abs(many.cpu().numpy()).max() > 0

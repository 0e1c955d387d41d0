"""CPU-side checks of the product library: it builds, loads and exports every
entry point include/tbslas_gb300.h declares; its host-side Chebyshev helpers
agree with the oracle; the host tree utilities build valid trees.  No
compute call here needs a GPU."""
import os
import re

import numpy as np
import pytest

import tbslas_gb300 as tb
from tbslas_gb300 import capi, fields, trees

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "tbslas_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(tbslas_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol(built):
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(built, n), n
    assert set(names) == set(capi.SIGNATURES), set(names) ^ set(capi.SIGNATURES)


def test_status_strings(built):
    assert capi.status_string(0) == "ok"
    assert capi.status_string(2) == "invalid tree"
    assert tb.capi.lib().tbslas_version() >= 1


def test_cheb_nodes_match_oracle(built, ora):
    for q in (1, 5, 8, 14, 16):
        assert np.array_equal(tb.new_nodes(q), ora.new_nodes(q))


@pytest.mark.parametrize("q", [2, 5, 8])
def test_pt2coeff_matches_oracle_pinv(built, ora, q):
    M = tb.get_pt2coeff_matrix(q)
    Mo = ora.pt2coeff(q)
    assert M.shape == Mo.shape
    assert np.abs(M - Mo).max() < 1e-13 * np.abs(Mo).max() * 100


def test_host_argument_errors(built):
    with pytest.raises(capi.TbslasError) as e:
        tb.get_pt2coeff_matrix(99)
    assert e.value.status == 4
    L = capi.lib()
    assert L.tbslas_cheb_nodes(3, None) == 1
    assert "null" in capi.last_error()


def test_uniform_tree_is_morton_sorted_and_complete():
    for d in (0, 1, 3):
        a, dep = trees.uniform_tree(d)
        k = trees.morton_keys(a)
        assert np.all(np.diff(k.astype(np.float64)) > 0)
        assert np.isclose(np.sum(np.ldexp(1.0, -3 * dep)), 1.0)


def test_adaptive_tree_balanced_and_complete(built):
    rng = np.random.default_rng(0)
    fn = fields.gaussian_blobs(rng, 2)
    a, d = trees.adaptive_tree(fn, 4, 1, 1e-4, 1, 5)
    assert d.min() >= 1 and d.max() <= 5 and len(set(d)) >= 3
    assert np.isclose(np.sum(np.ldexp(1.0, -3 * d.astype(np.int64))), 1.0)
    k = trees.morton_keys(a)
    assert np.all(np.diff(k.astype(np.float64)) > 0)
    a2, d2 = trees.balance21(a, d)
    assert len(d2) == len(d)  # already balanced


def test_fourier_grid_matches_point_function():
    n = 12
    g = fields.fourier_velocity_grid(np.random.default_rng(7), n)
    f = fields.fourier_velocity(np.random.default_rng(7))
    x = np.arange(n) / n
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    v = f(np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1))
    assert np.abs(g.reshape(3, -1).T - v).max() < 1e-12 * np.abs(v).max()
    # divergence-free: spectral divergence of the sampled field vanishes
    k = np.fft.fftfreq(n, 1.0 / n)
    KZ, KY, KX = np.meshgrid(k, k, k, indexing="ij")
    div = KX * np.fft.fftn(g[0]) + KY * np.fft.fftn(g[1]) + KZ * np.fft.fftn(g[2])
    assert np.abs(div).max() < 1e-9 * n ** 3


def test_cubic_time_weights_match_interp_cubic_1d(built, ora):
    """tbslas_cubic_time_weights: w . p equals CubicInterpPolicy::InterpCubic1D
    (src/utils/cubic.h:42-56, the oracle's restatement) for any values p,
    inside and outside the middle interval; non-increasing or non-finite
    times are refused."""
    rng = np.random.default_rng(7)
    for _ in range(200):
        times = np.sort(rng.uniform(-1.0, 1.0, 4))
        if np.any(np.diff(times) <= 1e-3):
            continue
        t = rng.uniform(times[0] - 0.2, times[3] + 0.2)
        w = tb.cubic_time_weights(times, t)
        p = rng.normal(size=(4, 5))
        ref = ora.interp_cubic_1d(t, times, list(p))
        got = w @ p
        assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
    with pytest.raises(capi.TbslasError):
        tb.cubic_time_weights([0.0, 0.1, 0.1, 0.2], 0.05)
    with pytest.raises(capi.TbslasError):
        tb.cubic_time_weights([0.0, 0.1, 0.2, np.inf], 0.05)


def test_field_set_stage_weights_follow_integrate_rk2(built, ora):
    """FieldSetFunctor's per-stage weights are the cubic weights at the times
    IntegrateRK2 queries (tinit and tinit + tau/2 of each sub-step,
    src/semilag/traj.inc:20-45): two weight rows per sub-step."""
    times = [0.0, 0.02, 0.04, 0.06]
    f = tb.FieldSetFunctor([None] * 4, times)
    for timestep, dt, nrk in ((3, 0.02, 1), (2, 0.03, 2), (5, 0.01, 3)):
        _, w = f.stage_weights(timestep, dt, nrk)
        assert w.shape == (2 * nrk * 4,)
        tinit = timestep * dt
        tau = (tinit - dt - tinit) / nrk
        cur = tinit
        for s in range(nrk):
            np.testing.assert_array_equal(w[8 * s:8 * s + 4], tb.cubic_time_weights(times, cur))
            np.testing.assert_array_equal(w[8 * s + 4:8 * s + 8],
                                          tb.cubic_time_weights(times, cur + 0.5 * tau))
            cur = cur + tau

"""Argument checks of the re-meshing, construction, time-dependent and BDF2
entry points: bad arguments are rejected on the host with a status and a
message, before any launch, and leave the trees usable."""
import ctypes

import numpy as np
import pytest

import tbslas_gb300 as tb
from tbslas_gb300 import capi, fields, trees

pytestmark = pytest.mark.gpu


def _pair(ctx, q=4):
    a, d = trees.uniform_tree(1)
    tv = tb.Tree(ctx, a, d, q, 3, trees.fit(fields.rotation(1.0), a, d, q, 3))
    tc = tb.Tree(ctx, a, d, q, 1, trees.fit(fields.gaussian((0.5, 0.5, 0.5), 0.2), a, d, q, 1))
    return tv, tc


def test_remesh_rejects_bad_arguments(ctx):
    _, tc = _pair(ctx)
    before = tc.get_coeffs()
    for args in ((-1.0, 0, 3), (float("nan"), 0, 3), (1e-3, 3, 2), (1e-3, -1, 3), (1e-3, 0, 22)):
        with pytest.raises(capi.TbslasError):
            tc.remesh(*args)
    with pytest.raises(capi.TbslasError):
        tc.remesh(1e-3, 0, 3, bc=7)
    assert np.array_equal(tc.get_coeffs(), before)


def test_construct_rejects_bad_arguments(ctx):
    f = tb.Field.gaussians([(0.5, 0.5, 0.5)], [0.1])
    for q, tol, lo, hi in ((0, 1e-3, 1, 3), (17, 1e-3, 1, 3), (4, -1.0, 1, 3), (4, 1e-3, 7, 8),
                           (4, 1e-3, 3, 2)):
        with pytest.raises(capi.TbslasError):
            tb.construct_tree(ctx, f, q, tol, lo, hi)
    with pytest.raises(capi.TbslasError):
        tb.construct_tree(ctx, tb.Field(99), 4, 1e-3, 1, 2)
    with pytest.raises(capi.TbslasError):
        tb.construct_tree(ctx, tb.Field(tb.Field.GAUSSIANS, [0.5, 0.5, 0.5, 0.1, float("inf")], 1),
                          4, 1e-3, 1, 2)
    _, tc = _pair(ctx)
    with pytest.raises(capi.TbslasError):  # dof 3 field on a dof 1 tree
        tc.fit_field(tb.Field.taylor_green())


def test_velocity_set_and_bdf2_reject_bad_arguments(ctx):
    tv, tc = _pair(ctx)
    five = [tv] * 5

    class Five:
        bc = tb.FreeSpace

        def stage_weights(self, timestep, dt, nrk):
            return five, np.ones(2 * nrk * 5)
    with pytest.raises(capi.TbslasError):
        tb.solve_semilag_in_situ_tv(Five(), tc, 1, 0.01)

    class NaNw:
        bc = tb.FreeSpace

        def stage_weights(self, timestep, dt, nrk):
            return [tv], np.array([1.0, float("nan")])
    with pytest.raises(capi.TbslasError):
        tb.solve_semilag_in_situ_tv(NaNw(), tc, 1, 0.01)
    with pytest.raises(capi.TbslasError):
        tb.cubic_time_weights([0.0, 2.0, 1.0, 3.0], 1.5)
    tv5, tc5 = _pair(ctx, 5)
    with pytest.raises(capi.TbslasError):  # mixed degrees
        tb.solve_semilag_bdf2(tb.NodeFieldFunctor(tv), tc, tc5, tc, 0.02, 0.01)
    with pytest.raises(capi.TbslasError):
        tb.solve_semilag_bdf2(tb.NodeFieldFunctor(tv), tc, tc, tc, float("inf"), 0.01)
    # the trees still work
    tb.solve_semilag_bdf2(tb.NodeFieldFunctor(tv), tc, tc, tc, 0.02, 0.01)
    assert np.isfinite(tc.get_coeffs()).all()

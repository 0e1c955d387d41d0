"""Device tree construction and fitting (tbslas_tree_construct /
tbslas_tree_fit_field: the reference's ConstructTree / InitTree,
src/tree/tree_utils.h:83-178) against the oracle's restatement: the same
leaves and coefficients within 1e-12, for scalar and velocity fields of the
reference's src/utils/fields.h."""
import numpy as np
import pytest

import tbslas_gb300 as tb
from tbslas_gb300 import fields, trees

pytestmark = pytest.mark.gpu

FIELDS = {
    "gaussians": lambda: tb.Field.gaussians([(0.3, 0.5, 0.5), (0.65, 0.4, 0.55)], [0.06, 0.09],
                                            [1.0, 0.7]),
    "gaussian_3d": lambda: tb.Field(tb.Field.GAUSSIAN_3D, [0.8, 0.5, 0.5, 1.0, 0.06, 0.35, 0.35]),
    "exp_alpha": lambda: tb.Field(tb.Field.EXP_ALPHA, [0.5, 0.5, 0.5, 0.2, 4.0]),
    "taylor_green": tb.Field.taylor_green,
    "taylor_green_abc": lambda: tb.Field(tb.Field.TAYLOR_GREEN_ABC,
                                         [1, 1, 1, 2 * np.pi, 2 * np.pi, 2 * np.pi]),
    "hopf": lambda: tb.Field(tb.Field.HOPF, [0.5, 0.5, 0.5, 0.05, 0.1]),
    "rotation": lambda: tb.Field.rotation(1.0),
    "fourier": lambda: tb.Field.fourier(*fields.fourier_modes(np.random.default_rng(4), 2)),
}


@pytest.mark.parametrize("name", sorted(FIELDS))
def test_construct_matches_oracle(ctx, name):
    from oracle import construct as oc
    f = FIELDS[name]()
    q, tol = 5, 1e-3
    t = tb.construct_tree(ctx, f, q, tol, 1, 4)
    ga, gd = t.leaves()
    gc = t.get_coeffs()
    ra, rd, rc = oc.construct(f.kind, f.n, f.params, q, tol, 1, 4)
    assert np.array_equal(gd, rd) and np.array_equal(ga, ra)
    assert np.abs(gc - rc).max() <= 1e-12 * max(np.abs(rc).max(), 1e-300)
    t.close()


def test_construct_periodic_balance(ctx):
    from oracle import construct as oc
    f = tb.Field.gaussians([(0.02, 0.5, 0.5)], [0.03])
    t = tb.construct_tree(ctx, f, 4, 1e-4, 1, 5, tb.Periodic)
    ga, gd = t.leaves()
    ra, rd, rc = oc.construct(f.kind, f.n, f.params, 4, 1e-4, 1, 5, True)
    assert np.array_equal(gd, rd) and np.array_equal(ga, ra)
    assert np.abs(t.get_coeffs() - rc).max() <= 1e-12 * np.abs(rc).max()
    t.close()


def test_fit_field_matches_host_fit(ctx):
    """InitTree on the device equals the host fit of the same closed form."""
    q = 6
    a, d = trees.adaptive_tree(fields.gaussian((0.4, 0.5, 0.6), 0.08), q, 1, 1e-4, 1, 3)
    t = tb.Tree(ctx, a, d, q, 3)
    t.fit_field(tb.Field.taylor_green())
    ref = trees.fit(fields.taylor_green(), a, d, q, 3)
    assert np.abs(t.get_coeffs() - ref).max() <= 1e-12 * np.abs(ref).max()
    t.close()


def test_construct_profiled_launches(ctx):
    """The construction reports its kernels to the context's profiler: with
    nothing to refine or balance, the uniform tree, one fit and refinement
    check (4), one balance check (2) and the install (maximum depth, lookup
    table, split and norms of the coefficients) make 11."""
    ctx.profile(True)
    ctx.profile_reset()
    t = tb.construct_tree(ctx, tb.Field.taylor_green(), 4, float("inf"), 2, 4)
    prof = ctx.profile_totals()
    ctx.profile(False)
    assert t.n_leaves == 64
    assert prof["construct"][:2] == (1, 11)
    t.close()

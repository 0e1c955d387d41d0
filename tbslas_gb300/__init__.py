"""tbslas_gb300: the tbslas semi-Lagrangian advection step on GB300 (sm_103a).

The compute path is libtbslas_gb300.so (hand-written CUDA behind a C ABI,
include/tbslas_gb300.h); this package is its Python face.
"""
from . import capi  # noqa: F401
from .api import (  # noqa: F401
    DEVICE_ERR_WAIT_TIMEOUT, SUMS_DOUBLE_FLOAT, SUMS_FP64, WAIT_LIMIT_DEFAULT, Batch, Context, FieldExtrapFunctor, FieldSetFunctor, FreeSpace,
    Field, NodeFieldFunctor, Periodic, Tree, construct_tree, cubic_time_weights,
    collect_cheb_tree_grid_points,
    compute_traj_rk2, fast_interp, get_pt2coeff_matrix, n_coeff, n_points, new_nodes,
    semilag_grid, semilag_grid_steps, set_tree_grid_values, solve_semilag_bdf2, solve_semilag_in_situ,
    solve_semilag_in_situ_tv)

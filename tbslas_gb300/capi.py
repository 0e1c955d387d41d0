"""ctypes binding of libtbslas_gb300.so (declarations in include/tbslas_gb300.h).

The library is built in-tree by tbslas_gb300.build.  Loading fails loudly if
it is missing: there is no CPU fallback.
"""
import ctypes
import functools
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libtbslas_gb300.so")

OK = 0
ERR_DEVICE = 7  # TBSLAS_ERR_DEVICE: a kernel reported an error status
BC_FREESPACE = 0
BC_PERIODIC = 1
MAX_DEGREE = 16
MAX_DEPTH = 21
NOALLOC_MAX_POINTS = 1 << 18
NOALLOC_MAX_LEAVES = 1 << 15

_c = ctypes
_vp, _i64, _i32, _f64 = _c.c_void_p, _c.c_int64, _c.c_int, _c.c_double
_u32 = _c.c_uint32
_u32p = _c.POINTER(_c.c_uint32)
_i64p = _c.POINTER(_c.c_int64)
_i32p = _c.POINTER(_c.c_int)

# name -> (argtypes) ; every function returns int (a tbslas_status) unless listed in _RESTYPES
SIGNATURES = {
    "tbslas_status_string": [_i32],
    "tbslas_last_error": [],
    "tbslas_version": [],
    "tbslas_ctx_create": [_i32, _c.POINTER(_vp)],
    "tbslas_ctx_destroy": [_vp],
    "tbslas_ctx_check": [_vp, _u32p],
    "tbslas_profile_enable": [_vp, _i32],
    "tbslas_profile_reset": [_vp],
    "tbslas_profile_count": [_vp, _i32p],
    "tbslas_profile_get": [_vp, _i32, _c.POINTER(_c.c_char_p), _i64p, _i64p, _c.POINTER(_f64)],
    "tbslas_fp64_fma_peak": [_vp, _c.POINTER(_f64)],
    "tbslas_fp32_fma_peak": [_vp, _c.POINTER(_f64)],
    "tbslas_ctx_set_sums": [_vp, _i32],
    "tbslas_ctx_set_wait_limit": [_vp, _u32],
    "tbslas_ctx_get_sums": [_vp, _c.POINTER(_i32)],
    "tbslas_ctx_last_fp64_targets": [_vp, _c.POINTER(_i64)],
    "tbslas_cheb_nodes": [_i32, _vp],
    "tbslas_pt2coeff_matrix": [_i32, _vp],
    "tbslas_tree_create": [_vp, _i64, _vp, _vp, _i32, _i32, _c.POINTER(_vp)],
    "tbslas_tree_destroy": [_vp],
    "tbslas_tree_info": [_vp, _i64p, _i32p, _i32p, _i32p],
    "tbslas_tree_set_coeffs_host": [_vp, _vp],
    "tbslas_tree_get_coeffs_host": [_vp, _vp],
    "tbslas_tree_set_coeffs": [_vp, _vp, _vp],
    "tbslas_tree_get_coeffs": [_vp, _vp, _vp],
    "tbslas_tree_get_leaves": [_vp, _vp, _vp],
    "tbslas_tree_remesh": [_vp, _vp, _c.c_double, _i32, _i32, _i32, _vp],
    "tbslas_semilag_bdf2": [_vp, _vp, _vp, _vp, _vp, _c.c_double, _c.c_double, _i32, _i32, _vp],
    "tbslas_semilag_in_situ_tv": [_vp, _i32, _vp, _vp, _vp, _i32, _c.c_double, _i32, _i32, _vp],
    "tbslas_cubic_time_weights": [_vp, _c.c_double, _vp],
    "tbslas_tree_fit_field": [_vp, _vp, _vp, _vp],
    "tbslas_tree_construct": [_vp, _vp, _i32, _c.c_double, _i32, _i32, _i32, _c.POINTER(_vp)],
    "tbslas_collect_grid_points": [_vp, _vp, _vp, _vp],
    "tbslas_eval_tree": [_vp, _vp, _vp, _i64, _vp, _i32, _vp],
    "tbslas_eval_tree_host": [_vp, _vp, _vp, _i64, _vp, _i32],
    "tbslas_eval_tree_on_nodes": [_vp, _vp, _vp, _vp, _i32, _vp],
    "tbslas_eval_tree_noalloc": [_vp, _vp, _i64, _vp, _i32, _vp],
    "tbslas_traj_rk2": [_vp, _vp, _vp, _i64, _f64, _f64, _i32, _i32, _vp, _vp],
    "tbslas_traj_rk2_host": [_vp, _vp, _vp, _i64, _f64, _f64, _i32, _i32, _vp],
    "tbslas_set_tree_grid_values": [_vp, _vp, _vp, _vp],
    "tbslas_semilag_in_situ": [_vp, _vp, _vp, _i32, _f64, _i32, _i32, _vp],
    "tbslas_semilag_in_situ_host": [_vp, _vp, _vp, _vp, _i32, _f64, _i32, _i32],
    "tbslas_semilag_in_situ_ckpt": [_vp, _vp, _vp, _i32, _f64, _i32, _vp, _vp, _vp],
    "tbslas_semilag_in_situ_ckpt_jac": [_vp, _vp, _vp, _i32, _f64, _i32, _vp, _vp, _vp, _vp],
    "tbslas_semilag_adjoint_jac": [_vp, _vp, _vp, _vp, _i32, _f64, _i32, _vp, _vp, _vp, _vp,
                                   _vp, _vp, _vp, _vp],
    "tbslas_semilag_adjoint": [_vp, _vp, _vp, _vp, _i32, _f64, _i32, _vp, _vp, _vp, _vp, _vp,
                               _vp],
    "tbslas_semilag_adjoint_seq": [_vp, _vp, _vp, _vp, _i32, _f64, _i32, _vp, _vp, _vp, _vp,
                                   _vp, _vp, _vp, _vp],
    "tbslas_semilag_adjoint_node_term": [_vp, _vp, _vp, _i32, _vp, _vp, _vp],
    "tbslas_batch_create": [_vp, _i32, _vp, _vp, _vp, _i32, _i32, _c.POINTER(_vp)],
    "tbslas_batch_destroy": [_vp],
    "tbslas_batch_info": [_vp, _i64p, _i64p],
    "tbslas_batch_set_params": [_vp, _i32, _i32, _i32],
    "tbslas_batch_get_params": [_vp, _i32p, _i32p, _i32p],
    "tbslas_batch_autotune": [_vp, _i32p, _i32p, _i32p],
    "tbslas_batch_run": [_vp, _i32, _i32, _i32, _vp],
    "tbslas_fast_interp": [_vp, _vp, _i32, _i32, _vp, _i64, _vp, _i32, _vp],
    "tbslas_semilag_grid": [_vp, _vp, _vp, _vp, _i32, _f64, _i32, _i32, _vp],
    "tbslas_semilag_grid_host": [_vp, _vp, _vp, _vp, _i32, _f64, _i32, _i32],
    "tbslas_semilag_grid_steps": [_vp, _vp, _vp, _vp, _i32, _f64, _i32, _i32, _i32, _vp],
}
_RESTYPES = {"tbslas_status_string": _c.c_char_p, "tbslas_last_error": _c.c_char_p}


class TbslasError(RuntimeError):
    def __init__(self, status, what, msg):
        super().__init__("%s failed: %s (%s)" % (what, msg, status_string(status)))
        self.status = status


@functools.lru_cache(maxsize=1)
def lib():
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "libtbslas_gb300.so is not built (%s); run tbslas_gb300.build.build()" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, _i32)
    return L


def status_string(status):
    return lib().tbslas_status_string(int(status)).decode()


def last_error():
    return lib().tbslas_last_error().decode()


def check(status, what):
    if status != OK:
        raise TbslasError(status, what, last_error())
    return status


def call(name, *args):
    return check(getattr(lib(), name)(*args), name)

"""Python face of the oracle (test infrastructure only).

Thin ctypes wrappers around oracle/oracle.cpp (the CPU restatement of the
tbslas semi-Lagrangian path) plus the point-to-coefficient matrix, restated
from tbslas::GetPt2CoeffMatrix (src/utils/cheb.h:166-196) as
pinv(V)^T with an SVD-based pseudo-inverse (numpy/LAPACK), which is how
PVFMM's Matrix::pinv computes it.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.
"""
import ctypes
import functools
import os

import numpy as np

from . import build as _build

_f64p = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int)


@functools.lru_cache(maxsize=1)
def lib():
    path = _build.build()
    L = ctypes.CDLL(path)
    i64, i32, f64 = ctypes.c_long, ctypes.c_int, ctypes.c_double
    L.orc_num_threads.argtypes = [i32]
    L.orc_new_nodes.argtypes = [i32, _f64p]
    L.orc_cheb_poly.argtypes = [i32, _f64p, i32, _f64p]
    L.orc_cheb_basis.argtypes = [i32, _f64p, i64, _f64p]
    L.orc_collect_grid_points.argtypes = [i64, _f64p, _i32p, i32, _f64p]
    L.orc_eval_tree.argtypes = [i64, _f64p, _i32p, i32, i32, _f64p, i32, _f64p, i64, _f64p]
    L.orc_traj_rk2.argtypes = [i64, _f64p, _i32p, i32, _f64p, i32, _f64p, i64, f64, f64, i32,
                               _f64p]
    L.orc_set_tree_grid_values.argtypes = [i64, i32, i32, _f64p, _f64p, _f64p]
    L.orc_semilag_in_situ.argtypes = [i64, _f64p, _i32p, i32, _f64p,
                                      i64, _f64p, _i32p, i32, i32, _f64p,
                                      _f64p, i32, f64, i32, i32, i64, i64, _f64p]
    L.orc_semilag_in_situ_dual.argtypes = [i64, _f64p, _i32p, i32, _f64p, _f64p,
                                           i64, _f64p, _i32p, i32, _f64p, _f64p,
                                           _f64p, i32, f64, i32, i32, _f64p, _f64p]
    L.orc_fast_interp.argtypes = [_f64p, i32, i32, _f64p, i64, _f64p, i32]
    L.orc_semilag_grid.argtypes = [_f64p, _f64p, i32, f64, i32, i32, i64, i64, _f64p]
    return L


def _d(a):
    return a.ctypes.data_as(_f64p)


def _i(a):
    return a.ctypes.data_as(_i32p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def num_threads(n=0):
    return lib().orc_num_threads(int(n))


def n_coeff(q):
    return (q + 1) * (q + 2) * (q + 3) // 6


def new_nodes(q):
    out = np.empty(((q + 1) ** 3, 3))
    lib().orc_new_nodes(q, _d(out))
    return out


def cheb_poly(q, x):
    x = _f64(x)
    out = np.zeros((q + 1, x.size))
    lib().orc_cheb_poly(q, _d(x), x.size, _d(out))
    return out


def cheb_basis(q, pts):
    pts = _f64(pts).reshape(-1, 3)
    V = np.empty((pts.shape[0], n_coeff(q)))
    lib().orc_cheb_basis(q, _d(pts), pts.shape[0], _d(V))
    return V


@functools.lru_cache(maxsize=None)
def _pt2coeff_cached(q):
    V = cheb_basis(q, 2.0 * new_nodes(q) - 1.0)
    M = np.linalg.pinv(V).T.copy()
    M.setflags(write=False)
    return M


def pt2coeff(q):
    """M (Np x Nc) with coeff = vals @ M; restates GetPt2CoeffMatrix."""
    return _pt2coeff_cached(q)


def collect_grid_points(anchor, depth, q):
    anchor, depth = _f64(anchor), _i32(depth)
    out = np.empty((depth.size * (q + 1) ** 3, 3))
    lib().orc_collect_grid_points(depth.size, _d(anchor), _i(depth), q, _d(out))
    return out


def eval_tree(anchor, depth, q, dof, coeff, pos, periodic=False):
    anchor, depth, coeff, pos = _f64(anchor), _i32(depth), _f64(coeff), _f64(pos).reshape(-1, 3)
    out = np.empty((pos.shape[0], dof))
    lib().orc_eval_tree(depth.size, _d(anchor), _i(depth), q, dof, _d(coeff), int(periodic),
                        _d(pos), pos.shape[0], _d(out))
    return out


def traj_rk2(anchor, depth, q, coeff, x, tinit, tfinal, nrk, periodic=False):
    anchor, depth, coeff, x = _f64(anchor), _i32(depth), _f64(coeff), _f64(x).reshape(-1, 3)
    out = np.empty_like(x)
    lib().orc_traj_rk2(depth.size, _d(anchor), _i(depth), q, _d(coeff), int(periodic), _d(x),
                       x.shape[0], float(tinit), float(tfinal), int(nrk), _d(out))
    return out


def set_tree_grid_values(L, q, dof, vals, M=None):
    M = pt2coeff(q) if M is None else _f64(M)
    vals = _f64(vals)
    out = np.empty((L, dof, n_coeff(q)))
    lib().orc_set_tree_grid_values(L, q, dof, _d(M), _d(vals), _d(out))
    return out


def semilag_in_situ(vel, con, timestep, dt, nrk=1, periodic=False, M=None, leaf_begin=0,
                    leaf_end=0):
    """One in-situ SL step.  vel/con: dicts with anchor, depth, q, dof, coeff.

    With leaf_end > leaf_begin only those leaves' targets are advected and
    their new coefficients returned (a bounded sample of the step)."""
    qc = con["q"]
    M = pt2coeff(qc) if M is None else _f64(M)
    av, dv, cv = _f64(vel["anchor"]), _i32(vel["depth"]), _f64(vel["coeff"])
    ac, dc, cc = _f64(con["anchor"]), _i32(con["depth"]), _f64(con["coeff"])
    nl = dc.size if leaf_end <= leaf_begin else leaf_end - leaf_begin
    out = np.empty((nl, con["dof"], n_coeff(qc)))
    lib().orc_semilag_in_situ(dv.size, _d(av), _i(dv), vel["q"], _d(cv),
                              dc.size, _d(ac), _i(dc), qc, con["dof"], _d(cc),
                              _d(M), int(timestep), float(dt), int(nrk), int(periodic),
                              int(leaf_begin), int(leaf_end), _d(out))
    return out


def semilag_bdf2(vel, prev, cur, nxt, t, dt, nrk=1, periodic=False, M=None):
    """BDF2 two-backtrace step of the advection-diffusion driver
    (src/applications/src/advdiff-ss.cpp:485-521), composed from the oracle's
    ComputeTrajRK2 / EvalTree / SetTreeGridValues restatements: for every node
    X of nxt (anchor, depth, q), X1 = traj(X, t -> t - dt), X2 = traj(X1,
    t - dt -> t - 2 dt), value = 4/3 cur(X1) - 1/3 prev(X2); returns nxt's new
    coefficients.  vel / prev / cur: dicts with anchor, depth, q, dof, coeff."""
    q = nxt["q"]
    pts = collect_grid_points(nxt["anchor"], nxt["depth"], q)
    x1 = traj_rk2(vel["anchor"], vel["depth"], vel["q"], vel["coeff"], pts, t, t - dt, nrk,
                  periodic)
    a = eval_tree(cur["anchor"], cur["depth"], cur["q"], 1, cur["coeff"], x1, periodic)
    x2 = traj_rk2(vel["anchor"], vel["depth"], vel["q"], vel["coeff"], x1, t - dt, t - dt * 2,
                  nrk, periodic)
    b = eval_tree(prev["anchor"], prev["depth"], prev["q"], 1, prev["coeff"], x2, periodic)
    vals = (4.0 / 3) * a - (1.0 / 3) * b
    return set_tree_grid_values(len(nxt["depth"]), q, 1, vals.reshape(-1), M)


def interp_cubic_1d(x, xx, pp):
    """CubicInterpPolicy::InterpCubic1D (src/utils/cubic.h:42-56), elementwise
    over the value arrays pp[0..3]."""
    def tangent(tk_1, tk, tk1, pk_1, pk, pk1):
        return (pk1 - pk) * 0.5 / (tk1 - tk) + (pk - pk_1) * 0.5 / (tk - tk_1)
    mk = tangent(xx[0], xx[1], xx[2], pp[0], pp[1], pp[2])
    mk1 = tangent(xx[1], xx[2], xx[3], pp[1], pp[2], pp[3])
    t = (x - xx[1]) / (xx[2] - xx[1])
    h00 = 2 * t * t * t - 3 * t * t + 1
    h10 = t * t * t - 2 * t * t + t
    h01 = -2 * t * t * t + 3 * t * t
    h11 = t * t * t - t * t
    return h00 * pp[1] + h10 * (xx[2] - xx[1]) * mk + h01 * pp[2] + h11 * (xx[2] - xx[1]) * mk1


def semilag_in_situ_tv(vels, con, timestep, dt, nrk=1, periodic=False, times=None, M=None,
                       leaf_end=0):
    """In-situ step through a time-dependent velocity (SolveSemilagInSitu ->
    SolveSemilagRK2 -> ComputeTrajRK2 -> IntegrateRK2, src/tree/tree_semilag.h:
    92-180, src/semilag/semilag.inc:26-80, src/semilag/traj.inc:20-93):
    with `times`, vels are the four trees of a FieldSetFunctor
    (tree_set_functor.h:49-72: every tree evaluated, then InterpCubic1D at the
    stage's time); without, vels = [v_n, v_{n-1}] of the two-functor form
    (v_n at X, FieldExtrapFunctor's 1.5 v_n - 0.5 v_{n-1} at X*,
    tree_extrap_functor.h:47-78).  Each evaluation wraps the point array in
    place under periodic boundaries (EvalTree's aliasing).  With leaf_end,
    only the first leaf_end leaves' targets (a bounded sample)."""
    q = con["q"]
    nl = len(con["depth"]) if leaf_end <= 0 else leaf_end
    x = collect_grid_points(con["anchor"][:nl], con["depth"][:nl], q)
    tinit = timestep * dt
    tfinal = tinit - dt
    tau = (tfinal - tinit) / nrk

    def wrap(p):
        if periodic:
            p = np.where(p < 0.0, p + 1.0, p)
            p = np.where(p >= 1.0, p - 1.0, p)
        return p

    def ev(tr, p):
        return eval_tree(tr["anchor"], tr["depth"], tr["q"], 3, tr["coeff"], p, periodic)

    cur = tinit
    for _ in range(nrk):
        x = wrap(x)
        if times is not None:
            v = interp_cubic_1d(cur, times, [ev(tr, x) for tr in vels])
        else:
            v = ev(vels[0], x)
        xt = x + 0.5 * tau * v
        xt = wrap(xt)
        if times is not None:
            v = interp_cubic_1d(cur + 0.5 * tau, times, [ev(tr, xt) for tr in vels])
        else:
            v = 1.5 * ev(vels[0], xt) - 0.5 * ev(vels[1], xt)
        x = x + tau * v
        cur = cur + tau
    c = eval_tree(con["anchor"], con["depth"], q, 1, con["coeff"], x, periodic)
    return set_tree_grid_values(nl, q, 1, c.reshape(-1), M)


def semilag_in_situ_dual(vel, vel_d, con, con_d, timestep, dt, nrk=1, periodic=False, M=None):
    """One SL step on forward-mode dual numbers: returns (new coefficients,
    their derivative along the input direction (vel_d, con_d))."""
    qc = con["q"]
    M = pt2coeff(qc) if M is None else _f64(M)
    av, dv, cv, cvd = (_f64(vel["anchor"]), _i32(vel["depth"]), _f64(vel["coeff"]), _f64(vel_d))
    ac, dc, cc, ccd = (_f64(con["anchor"]), _i32(con["depth"]), _f64(con["coeff"]), _f64(con_d))
    out = np.empty((dc.size, 1, n_coeff(qc)))
    outd = np.empty_like(out)
    lib().orc_semilag_in_situ_dual(dv.size, _d(av), _i(dv), vel["q"], _d(cv), _d(cvd),
                                   dc.size, _d(ac), _i(dc), qc, _d(cc), _d(ccd), _d(M),
                                   int(timestep), float(dt), int(nrk), int(periodic), _d(out),
                                   _d(outd))
    return out, outd


def fast_interp(grid, dof, nreg, pts, periodic=False):
    grid, pts = _f64(grid), _f64(pts).reshape(-1, 3)
    out = np.empty((pts.shape[0], dof))
    lib().orc_fast_interp(_d(grid), dof, nreg, _d(pts), pts.shape[0], _d(out), int(periodic))
    return out


def semilag_grid(vel, con, nreg, dt, nrk=1, periodic=True, node_begin=0, node_end=0):
    vel, con = _f64(vel), _f64(con)
    n = nreg ** 3 if node_end <= node_begin else node_end - node_begin
    out = np.empty(n)
    lib().orc_semilag_grid(_d(vel), _d(con), nreg, float(dt), int(nrk), int(periodic),
                           int(node_begin), int(node_end), _d(out))
    return out

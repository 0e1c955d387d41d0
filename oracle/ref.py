"""ctypes wrapper of oracle/_ref/libref.so: the reference's own SL-path code
built from its sources (oracle/ref_pin.cpp, recipe oracle/build_ref.py).

TEST INFRASTRUCTURE ONLY: the fixture generator tests/golden/
make_ref_golden.py and tests/test_ref_pin.py use it to pin the oracle.  It
exists only where the reference's sources are present (lib() returns None
elsewhere); nothing in the product loads it."""
import ctypes
import functools

import numpy as np

from . import build_ref

_d = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
_L, _F = ctypes.c_long, ctypes.c_double


@functools.lru_cache(maxsize=1)
def lib():
    path = build_ref.build()
    if path is None:
        return None
    L = ctypes.CDLL(path)
    for name in ("ref_new_nodes", "ref_vec_eval", "ref_fast_interp", "ref_collect_grid_points",
                 "ref_eval_tree", "ref_traj_rk2", "ref_pt2coeff", "ref_semilag_in_situ",
                 "ref_semilag_in_situ_set", "ref_semilag_in_situ_extrap",
                 "ref_semilag_bdf2", "ref_interp_cubic_1d"):
        getattr(L, name).restype = None
    return L


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def nc(q):
    return (q + 1) * (q + 2) * (q + 3) // 6


def new_nodes(q):
    out = np.empty(((q + 1) ** 3, 3))
    lib().ref_new_nodes(q, _d(out))
    return out


def collect_grid_points(anchor, depth, q):
    anchor, depth = _f64(anchor), _i32(depth)
    out = np.empty((len(depth) * (q + 1) ** 3, 3))
    lib().ref_collect_grid_points(_L(len(depth)), _d(anchor), _d(depth), q, _d(out))
    return out


def eval_tree(anchor, depth, q, dof, coeff, pos, periodic=False):
    anchor, depth, coeff, pos = _f64(anchor), _i32(depth), _f64(coeff), _f64(pos).reshape(-1, 3)
    out = np.empty((len(pos), dof))
    lib().ref_eval_tree(_L(len(depth)), _d(anchor), _d(depth), q, dof, _d(coeff), int(periodic),
                        _d(pos), _L(len(pos)), _d(out))
    return out


def traj_rk2(anchor, depth, q, coeff, x, tinit, tfinal, nrk, periodic=False):
    anchor, depth, coeff, x = _f64(anchor), _i32(depth), _f64(coeff), _f64(x).reshape(-1, 3)
    out = np.empty_like(x)
    lib().ref_traj_rk2(_L(len(depth)), _d(anchor), _d(depth), q, _d(coeff), int(periodic),
                       _d(x), _L(len(x)), _F(tinit), _F(tfinal), int(nrk), _d(out))
    return out


def fast_interp(grid, dof, n_reg, pts):
    grid, pts = _f64(grid), _f64(pts).reshape(-1, 3)
    out = np.empty((len(pts), dof))
    lib().ref_fast_interp(_d(grid), dof, n_reg, _d(pts), _L(len(pts)), _d(out))
    return out


def pt2coeff(q):
    out = np.empty(((q + 1) ** 3, nc(q)))
    lib().ref_pt2coeff(q, _d(out))
    return out


def semilag_in_situ(vel, con, timestep, dt, nrk=1, periodic=False):
    """vel / con: dicts anchor, depth, q, dof, coeff (as the oracle takes
    them); returns the concentration's coefficients after one step."""
    av, dv, vc = _f64(vel["anchor"]), _i32(vel["depth"]), _f64(vel["coeff"])
    ac, dc, cc = _f64(con["anchor"]), _i32(con["depth"]), _f64(con["coeff"])
    out = np.empty_like(cc)
    lib().ref_semilag_in_situ(_L(len(dv)), _d(av), _d(dv), _d(vc), _L(len(dc)), _d(ac), _d(dc),
                              int(con["dof"]), _d(cc), int(con["q"]), int(timestep), _F(dt),
                              int(nrk), int(periodic), _d(out))
    return out


def _concat(trees):
    return (_f64(np.concatenate([t["anchor"] for t in trees])),
            _i32(np.concatenate([t["depth"] for t in trees])),
            _f64(np.concatenate([np.ravel(t["coeff"]) for t in trees])))


def semilag_in_situ_tv(vels, con, timestep, dt, nrk=1, periodic=False, times=None):
    """The oracle's semilag_in_situ_tv signature: with times, vels are a
    FieldSetFunctor's four trees; without, vels = [v_n, v_{n-1}] of the
    two-functor step.  Returns the concentration's coefficients."""
    av, dv, vc = _concat(vels)
    ac, dc, cc = _f64(con["anchor"]), _i32(con["depth"]), _f64(con["coeff"])
    out = np.empty_like(cc)
    q = int(con["q"])
    tail = (_L(len(dc)), _d(ac), _d(dc), _d(cc), q, int(timestep), _F(dt), int(nrk),
            int(periodic), _d(out))
    if times is not None:
        Lv = np.ascontiguousarray([len(t["depth"]) for t in vels], dtype=np.int64)
        tm = _f64(times)
        lib().ref_semilag_in_situ_set(_d(Lv), _d(av), _d(dv), _d(vc), _d(tm), *tail)
    else:
        lib().ref_semilag_in_situ_extrap(_L(len(vels[0]["depth"])), _L(len(vels[1]["depth"])),
                                         _d(av), _d(dv), _d(vc), *tail)
    return out


def interp_cubic_1d(x, xx, pp):
    """InterpCubic1D for n triples: x [n], xx [n][4], pp [n][4]."""
    x, xx, pp = _f64(x), _f64(xx), _f64(pp)
    out = np.empty(len(x))
    lib().ref_interp_cubic_1d(_L(len(x)), _d(x), _d(xx), _d(pp), _d(out))
    return out


def semilag_bdf2(vel, prev, cur, nxt, t, dt, nrk=1, periodic=False):
    """The oracle's semilag_bdf2 signature: nxt's new coefficients."""
    q = int(nxt["q"])
    keep, args = [], []
    for tr in (vel, prev, cur, nxt):
        arrays = [_f64(tr["anchor"]), _i32(tr["depth"])]
        if tr is not nxt:
            arrays.append(_f64(tr["coeff"]))
        keep += arrays
        args += [_L(len(arrays[1]))] + [_d(a) for a in arrays]
    out = np.empty((len(nxt["depth"]), 1, nc(q)))
    lib().ref_semilag_bdf2(*args, q, _F(t), _F(dt), int(nrk), int(periodic), _d(out))
    return out

"""Python mirror of the tbslas SL interface over the C ABI.

Names follow the reference: NodeFieldFunctor (src/tree/tree_functor.h:793-815),
compute_traj_rk2 (ComputeTrajRK2, src/semilag/traj.inc:48-68),
solve_semilag_in_situ (SolveSemilagInSitu, src/tree/tree_semilag.h:92-135),
collect_cheb_tree_grid_points / set_tree_grid_values
(src/tree/tree_utils.h:442-552), new_nodes / get_pt2coeff_matrix
(src/utils/cheb.h:41-196) and fast_interp (src/tree/tree_functor.h:89-153).

Device arrays are torch CUDA float64 tensors; host arrays are numpy float64
arrays (the *_host entry points).  Every call goes to the CUDA library; there
is no CPU path.
"""
import contextlib
import ctypes
import weakref

import numpy as np

from . import capi
from .capi import BC_FREESPACE, BC_PERIODIC, call

FreeSpace = BC_FREESPACE
Periodic = BC_PERIODIC
SUMS_DOUBLE_FLOAT, SUMS_FP64 = 0, 1
WAIT_LIMIT_DEFAULT = 1 << 22
DEVICE_ERR_WAIT_TIMEOUT = 1


def n_coeff(q):
    return (q + 1) * (q + 2) * (q + 3) // 6


def n_points(q):
    return (q + 1) ** 3


def _ptr(a):
    """Raw data pointer of a torch tensor or numpy array (must be contiguous f64)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if a.dtype != np.float64 or not a.flags.c_contiguous:
            raise TypeError("expected a C-contiguous float64 numpy array")
        return a.ctypes.data
    import torch
    if not isinstance(a, torch.Tensor):
        raise TypeError("expected a torch tensor or numpy array, got %r" % type(a))
    if a.dtype != torch.float64 or not a.is_contiguous() or not a.is_cuda:
        raise TypeError("expected a contiguous float64 CUDA tensor")
    return a.data_ptr()


def _stream(stream):
    if stream is not None:
        return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
    import torch
    return torch.cuda.current_stream().cuda_stream


def new_nodes(q):
    if not 0 <= q <= capi.MAX_DEGREE:
        call("tbslas_cheb_nodes", int(q), None)  # raises the library's error
    out = np.empty((n_points(q), 3))
    call("tbslas_cheb_nodes", q, out.ctypes.data)
    return out


def get_pt2coeff_matrix(q):
    if not 1 <= q <= capi.MAX_DEGREE:
        call("tbslas_pt2coeff_matrix", int(q), None)  # raises the library's error
    out = np.empty((n_points(q), n_coeff(q)))
    call("tbslas_pt2coeff_matrix", q, out.ctypes.data)
    return out


class Context:
    """One CUDA device plus the library's cached scratch buffers."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        call("tbslas_ctx_create", int(device), ctypes.byref(h))
        self.handle = h
        self.device = int(device)
        self._objects = weakref.WeakSet()  # trees and batches made on this context

    def close(self):
        """Closes the context's remaining batches, then its trees, then the
        context (the C ABI destroys a context only after its objects)."""
        if self.handle:
            objs = list(self._objects)
            for o in objs:
                if isinstance(o, Batch):
                    o.close()
            for o in objs:
                o.close()
            capi.lib().tbslas_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def profile(self, enable=True):
        call("tbslas_profile_enable", self.handle, int(bool(enable)))

    def profile_reset(self):
        call("tbslas_profile_reset", self.handle)

    def profile_totals(self):
        """{name: (launch groups, kernel launches, total ms)} of the profiled launches."""
        n = ctypes.c_int(0)
        call("tbslas_profile_count", self.handle, ctypes.byref(n))
        out = {}
        for i in range(n.value):
            name, cnt, ker, ms = (ctypes.c_char_p(), ctypes.c_int64(), ctypes.c_int64(),
                                  ctypes.c_double())
            call("tbslas_profile_get", self.handle, i, ctypes.byref(name), ctypes.byref(cnt),
                 ctypes.byref(ker), ctypes.byref(ms))
            out[name.value.decode()] = (cnt.value, ker.value, ms.value)
        return out

    def fp64_fma_peak(self):
        """Measured FP64 FMA throughput, FLOP/s."""
        f = ctypes.c_double(0)
        call("tbslas_fp64_fma_peak", self.handle, ctypes.byref(f))
        return f.value

    @property
    def sums(self):
        """Arithmetic of the SL steps' Chebyshev sums: SUMS_FP64 (default,
        the reference's FP64 arithmetic, bit-identical to the oracle) or
        SUMS_DOUBLE_FLOAT (opt-in: hi/lo float pairs on the FP32 pipe, within
        ~1e-14 of FP64, leaf choices equal to FP64's)."""
        m = ctypes.c_int(0)
        call("tbslas_ctx_get_sums", self.handle, ctypes.byref(m))
        return m.value

    @sums.setter
    def sums(self, mode):
        call("tbslas_ctx_set_sums", self.handle, int(mode))

    @contextlib.contextmanager
    def sums_mode(self, mode):
        """`with ctx.sums_mode(SUMS_DOUBLE_FLOAT): ...` -- the mode for the
        block, the previous one restored after it."""
        prev = self.sums
        self.sums = mode
        try:
            yield self
        finally:
            self.sums = prev

    def set_wait_limit(self, polls=WAIT_LIMIT_DEFAULT):
        """Polls of the bounded device-side waits before they give up (and
        set DEVICE_ERR_WAIT_TIMEOUT in the error word ctx.check reports)."""
        call("tbslas_ctx_set_wait_limit", self.handle, int(polls))

    def last_fp64_targets(self):
        """Targets of the last double-float in-situ step recomputed in FP64."""
        n = ctypes.c_int64(0)
        call("tbslas_ctx_last_fp64_targets", self.handle, ctypes.byref(n))
        return n.value

    def fp32_fma_peak(self):
        """Measured FP32 FMA throughput, FLOP/s."""
        f = ctypes.c_double(0)
        call("tbslas_fp32_fma_peak", self.handle, ctypes.byref(f))
        return f.value

    def check(self):
        """Synchronise and return the device error word (raises if non-zero)."""
        w = ctypes.c_uint32(0)
        st = capi.lib().tbslas_ctx_check(self.handle, ctypes.byref(w))
        capi.check(st, "tbslas_ctx_check")
        return w.value

    def take_device_error(self):
        """Synchronise, return the device error word and clear it, without
        raising (0 when clean; bit DEVICE_ERR_WAIT_TIMEOUT: a bounded wait
        ran out)."""
        w = ctypes.c_uint32(0)
        st = capi.lib().tbslas_ctx_check(self.handle, ctypes.byref(w))
        if st not in (0, capi.ERR_DEVICE):
            capi.check(st, "tbslas_ctx_check")
        return w.value


class Tree:
    """Complete linear octree (leaves in Morton order) + Chebyshev coefficients."""

    def __init__(self, ctx, anchor, depth, q, dof, coeff=None):
        anchor = np.ascontiguousarray(anchor, dtype=np.float64).reshape(-1, 3)
        depth = np.ascontiguousarray(depth, dtype=np.int32).reshape(-1)
        if anchor.shape[0] != depth.shape[0]:
            raise ValueError("anchor/depth length mismatch")
        h = ctypes.c_void_p()
        call("tbslas_tree_create", ctx.handle, depth.size, anchor.ctypes.data, depth.ctypes.data,
             int(q), int(dof), ctypes.byref(h))
        self.ctx, self.handle = ctx, h
        ctx._objects.add(self)
        self.anchor, self.depth, self.q, self.dof = anchor, depth, int(q), int(dof)
        self.n_leaves = depth.size
        if coeff is not None:
            self.set_coeffs(coeff)

    def close(self):
        if self.handle:
            capi.lib().tbslas_tree_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def coeff_shape(self):
        return (self.n_leaves, self.dof, n_coeff(self.q))

    def set_coeffs(self, coeff, stream=None):
        if isinstance(coeff, np.ndarray):
            c = np.ascontiguousarray(coeff, dtype=np.float64)
            if c.size != np.prod(self.coeff_shape):
                raise ValueError("coefficient array has %d values, tree needs %d"
                                 % (c.size, np.prod(self.coeff_shape)))
            call("tbslas_tree_set_coeffs_host", self.handle, c.ctypes.data)
        else:
            if coeff.numel() != np.prod(self.coeff_shape):
                raise ValueError("coefficient tensor has wrong size")
            call("tbslas_tree_set_coeffs", self.handle, _ptr(coeff), _stream(stream))

    def get_coeffs(self, out=None, stream=None):
        if out is None:
            out = np.empty(self.coeff_shape)
        if isinstance(out, np.ndarray):
            call("tbslas_tree_get_coeffs_host", self.handle, out.ctypes.data)
        else:
            call("tbslas_tree_get_coeffs", self.handle, _ptr(out), _stream(stream))
        return out

    def leaves(self):
        """(anchor [L,3], depth [L]) of the current leaves."""
        a = np.empty((self.n_leaves, 3))
        d = np.empty(self.n_leaves, dtype=np.int32)
        call("tbslas_tree_get_leaves", self.handle, a.ctypes.data, d.ctypes.data)
        return a, d

    def fit_field(self, field, stream=None):
        """InitTree on the device: the analytic field fitted on every leaf."""
        f = field._c()
        call("tbslas_tree_fit_field", self.ctx.handle, self.handle, ctypes.byref(f),
             _stream(stream))

    def remesh(self, tol, min_depth, max_depth, bc=0):
        """Adaptive re-meshing on the device (coarsen one level, refine,
        2:1 balance; tbslas_tree_remesh).  Returns {"leaves", "merged",
        "split", "balanced", "kernels"}; the tree's leaves and n_leaves
        change."""
        st = np.zeros(5, dtype=np.int64)
        call("tbslas_tree_remesh", self.ctx.handle, self.handle, float(tol), int(min_depth),
             int(max_depth), int(bc), st.ctypes.data)
        self.n_leaves = int(st[0])
        self.anchor, self.depth = self.leaves()
        return {"leaves": int(st[0]), "merged": int(st[1]), "split": int(st[2]),
                "balanced": int(st[3]), "kernels": int(st[4])}


class _CField(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("n", ctypes.c_int),
                ("p", ctypes.POINTER(ctypes.c_double))]


class Field:
    """An analytic input field evaluated on the device (tbslas_field; the
    closed forms of the reference's src/utils/fields.h)."""
    GAUSSIANS, GAUSSIAN_3D, EXP_ALPHA, ROTATION = 0, 1, 2, 3
    TAYLOR_GREEN, TAYLOR_GREEN_ABC, HOPF, FOURIER = 4, 5, 6, 7

    # parameters per kind (per term for the sums), as the C ABI reads them
    _NPARAM = {GAUSSIANS: 5, GAUSSIAN_3D: 7, EXP_ALPHA: 5, ROTATION: 1, TAYLOR_GREEN: 0,
               TAYLOR_GREEN_ABC: 6, HOPF: 5, FOURIER: 9}

    def __init__(self, kind, params=(), n=0):
        self.kind, self.n = int(kind), int(n)
        self.params = np.ascontiguousarray(params, dtype=np.float64).reshape(-1)
        per = Field._NPARAM.get(self.kind)  # unknown kinds: the C ABI rejects them
        want = per * self.n if self.kind in (Field.GAUSSIANS, Field.FOURIER) else per
        # the C ABI reads exactly `want` doubles from the array
        if per is not None and self.params.size != want:
            raise ValueError("field kind %d takes %d parameters, got %d"
                             % (self.kind, want, self.params.size))

    def _c(self):
        return _CField(self.kind, self.n,
                       self.params.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))

    @staticmethod
    def gaussians(centres, sigmas, amps=None):
        c = np.asarray(centres, dtype=np.float64).reshape(-1, 3)
        sg = np.broadcast_to(np.asarray(sigmas, dtype=np.float64), (len(c),))
        a = np.ones(len(c)) if amps is None else np.broadcast_to(np.asarray(amps, float), (len(c),))
        return Field(Field.GAUSSIANS, np.column_stack([c, sg, a]), len(c))

    @staticmethod
    def rotation(omega=1.0):
        return Field(Field.ROTATION, [omega])

    @staticmethod
    def taylor_green():
        return Field(Field.TAYLOR_GREEN)

    @staticmethod
    def fourier(ks, A, B):
        ks = np.asarray(ks, dtype=np.float64).reshape(-1, 3)
        return Field(Field.FOURIER, np.column_stack([ks, np.asarray(A).reshape(-1, 3),
                                                    np.asarray(B).reshape(-1, 3)]), len(ks))

    @property
    def dof(self):
        return 1 if self.kind in (Field.GAUSSIANS, Field.GAUSSIAN_3D, Field.EXP_ALPHA) else 3


def construct_tree(ctx, field, q, tol, min_depth, max_depth, bc=FreeSpace):
    """ConstructTree on the device (tbslas_tree_construct): an adaptive tree
    of the analytic field, fitted."""
    h = ctypes.c_void_p()
    f = field._c()
    call("tbslas_tree_construct", ctx.handle, ctypes.byref(f), int(q), float(tol), int(min_depth),
         int(max_depth), int(bc), ctypes.byref(h))
    t = Tree.__new__(Tree)
    t.ctx, t.handle, t.q, t.dof = ctx, h, int(q), field.dof
    ctx._objects.add(t)
    L = ctypes.c_int64()
    call("tbslas_tree_info", h, ctypes.byref(L), None, None, None)
    t.n_leaves = int(L.value)
    t.anchor, t.depth = t.leaves()
    return t


class NodeFieldFunctor:
    """Field functor of a tree: f(pos[n,3]) -> values[n,dof].

    Host numpy arrays go through the synchronous host entry point (the
    reference's calling convention); torch CUDA tensors stay on the device.
    Unlike the reference, the caller's coordinates are never modified.
    """

    def __init__(self, tree, bc=FreeSpace):
        self.tree, self.bc = tree, int(bc)

    def __call__(self, pos, out=None, stream=None):
        t = self.tree
        if isinstance(pos, np.ndarray):
            pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
            if out is None:
                out = np.empty((pos.shape[0], t.dof))
            call("tbslas_eval_tree_host", t.ctx.handle, t.handle, pos.ctypes.data, pos.shape[0],
                 out.ctypes.data, self.bc)
            return out
        import torch
        n = pos.numel() // 3
        if out is None:
            out = torch.empty((n, t.dof), dtype=torch.float64, device=pos.device)
        call("tbslas_eval_tree", t.ctx.handle, t.handle, _ptr(pos), n, _ptr(out), self.bc,
             _stream(stream))
        return out

    def at_nodes(self, dst_tree, out=None, stream=None):
        """The field at every Chebyshev node of dst_tree's leaves, [N, dof] in
        collect_cheb_tree_grid_points order (same values as calling the
        functor at those points, by sum factorisation)."""
        import torch
        t = self.tree
        if out is None:
            out = torch.empty((dst_tree.n_leaves * n_points(dst_tree.q), t.dof),
                              dtype=torch.float64, device="cuda:%d" % t.ctx.device)
        call("tbslas_eval_tree_on_nodes", t.ctx.handle, t.handle, dst_tree.handle, _ptr(out),
             self.bc, _stream(stream))
        return out


def compute_traj_rk2(vel_functor, xinit, tinit, tfinal, num_rk_step, xsol=None, stream=None):
    """RK2 departure points of xinit (CUDA tensor [n,3]) through a tree velocity."""
    import torch
    t = vel_functor.tree
    n = xinit.numel() // 3
    if xsol is None:
        xsol = torch.empty_like(xinit)
    call("tbslas_traj_rk2", t.ctx.handle, t.handle, _ptr(xinit), n, float(tinit), float(tfinal),
         int(num_rk_step), vel_functor.bc, _ptr(xsol), _stream(stream))
    return xsol


def collect_cheb_tree_grid_points(tree, out=None, stream=None):
    import torch
    if out is None:
        out = torch.empty((tree.n_leaves * n_points(tree.q), 3), dtype=torch.float64,
                          device="cuda:%d" % tree.ctx.device)
    call("tbslas_collect_grid_points", tree.ctx.handle, tree.handle, _ptr(out), _stream(stream))
    return out


def set_tree_grid_values(tree, vals, stream=None):
    """vals: CUDA tensor [L, dof, (q+1)^3] of node values -> tree coefficients."""
    call("tbslas_set_tree_grid_values", tree.ctx.handle, tree.handle, _ptr(vals), _stream(stream))


def solve_semilag_in_situ(vel_functor, tree, timestep, dt, num_rk_step=1, stream=None,
                          coeff_host=None):
    """One in-situ SL step of `tree` through the velocity functor's tree.

    With coeff_host (numpy [L,dof,Nc]) the coefficients are taken from and
    returned to host memory (synchronous); otherwise the step is enqueued on
    the stream and works on the tree's device coefficients.
    """
    v = vel_functor.tree
    if coeff_host is not None:
        if coeff_host.dtype != np.float64 or not coeff_host.flags.c_contiguous:
            raise TypeError("coeff_host must be C-contiguous float64")
        call("tbslas_semilag_in_situ_host", tree.ctx.handle, v.handle, tree.handle,
             coeff_host.ctypes.data, int(timestep), float(dt), int(num_rk_step), vel_functor.bc)
        return coeff_host
    call("tbslas_semilag_in_situ", tree.ctx.handle, v.handle, tree.handle, int(timestep),
         float(dt), int(num_rk_step), vel_functor.bc, _stream(stream))
    return None


def cubic_time_weights(times, t):
    """w[4] with CubicInterpPolicy::InterpCubic1D(t, times, p) = w . p."""
    tm = np.ascontiguousarray(times, dtype=np.float64)
    w = np.empty(4)
    call("tbslas_cubic_time_weights", tm.ctypes.data, float(t), w.ctypes.data)
    return w


def _stage_times(timestep, dt, nrk):
    """(time at X, time at X*) of each RK2 sub-step as ComputeTrajRK2 /
    IntegrateRK2 pass them (src/semilag/traj.inc:20-68)."""
    tinit = timestep * dt
    tfinal = tinit - dt
    tau = (tfinal - tinit) / nrk
    out, cur = [], tinit
    for _ in range(nrk):
        out.append((cur, cur + 0.5 * tau))
        cur = cur + tau
    return out


class FieldSetFunctor:
    """Velocity interpolated cubically in time between four trees
    (tbslas::FieldSetFunctor, src/tree/tree_set_functor.h:28-103)."""

    def __init__(self, trees, times, bc=FreeSpace):
        if len(trees) != 4 or len(times) != 4:
            raise ValueError("four trees and four times")
        self.trees, self.times, self.bc = list(trees), [float(x) for x in times], int(bc)

    def update(self, new_tree, time):
        """Drop the oldest tree, append new_tree at `time` (as the reference)."""
        self.trees = self.trees[1:] + [new_tree]
        self.times = self.times[1:] + [float(time)]

    def stage_weights(self, timestep, dt, nrk):
        w = []
        for t0, t1 in _stage_times(timestep, dt, nrk):
            w.extend(cubic_time_weights(self.times, t0))
            w.extend(cubic_time_weights(self.times, t1))
        return self.trees, np.asarray(w)


class FieldExtrapFunctor:
    """1.5 v_n - 0.5 v_{n-1} (tbslas::FieldExtrapFunctor,
    src/tree/tree_extrap_functor.h:27-95), used at the midpoint stage while
    the first stage takes v_n (the two-functor SolveSemilagInSitu)."""

    def __init__(self, tree_prev, tree_cur, bc=FreeSpace):
        self.tp, self.tc, self.bc = tree_prev, tree_cur, int(bc)

    def update(self, new_tree, time=None):
        self.tp, self.tc = self.tc, new_tree

    def stage_weights(self, timestep, dt, nrk):
        return [self.tc, self.tp], np.tile([1.0, 0.0, 1.5, -0.5], nrk)


def solve_semilag_in_situ_tv(vel_functor, tree, timestep, dt, num_rk_step=1, stream=None):
    """In-situ SL step through a FieldSetFunctor or FieldExtrapFunctor
    velocity (tbslas_semilag_in_situ_tv)."""
    trees, w = vel_functor.stage_weights(timestep, dt, int(num_rk_step))
    handles = (ctypes.c_void_p * len(trees))(*[t.handle.value for t in trees])
    w = np.ascontiguousarray(w, dtype=np.float64)
    call("tbslas_semilag_in_situ_tv", tree.ctx.handle, len(trees), ctypes.addressof(handles),
         w.ctypes.data, tree.handle, int(timestep), float(dt), int(num_rk_step), vel_functor.bc,
         _stream(stream))


def solve_semilag_bdf2(vel_functor, tree_prev, tree_cur, tree_next, t, dt, num_rk_step=1,
                       stream=None):
    """BDF2 two-backtrace SL step (the advection-diffusion driver's step,
    src/applications/src/advdiff-ss.cpp:485-521): tree_next's coefficients
    become the fit of 4/3 tree_cur(X1) - 1/3 tree_prev(X2) at its nodes, X1 /
    X2 the RK2 backtraces from t over one and two steps of dt."""
    call("tbslas_semilag_bdf2", tree_next.ctx.handle, vel_functor.tree.handle, tree_prev.handle,
         tree_cur.handle, tree_next.handle, float(t), float(dt), int(num_rk_step),
         vel_functor.bc, _stream(stream))


class Batch:
    """Many independent in-situ SL problems advanced by one kernel per step.

    problems: list of (velocity Tree, concentration Tree, dt)."""

    def __init__(self, ctx, problems, num_rk_step=1, bc=FreeSpace):
        n = len(problems)
        vel = (ctypes.c_void_p * n)(*[p[0].handle.value for p in problems])
        con = (ctypes.c_void_p * n)(*[p[1].handle.value for p in problems])
        dt = (ctypes.c_double * n)(*[float(p[2]) for p in problems])
        h = ctypes.c_void_p()
        call("tbslas_batch_create", ctx.handle, n, ctypes.cast(vel, ctypes.c_void_p),
             ctypes.cast(con, ctypes.c_void_p), ctypes.cast(dt, ctypes.c_void_p),
             int(num_rk_step), int(bc), ctypes.byref(h))
        self.ctx, self.handle, self.problems = ctx, h, list(problems)
        ctx._objects.add(self)

    def close(self):
        if self.handle:
            capi.lib().tbslas_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        t, w = ctypes.c_int64(), ctypes.c_int64()
        call("tbslas_batch_info", self.handle, ctypes.byref(t), ctypes.byref(w))
        return t.value, w.value

    def params(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        call("tbslas_batch_get_params", self.handle, ctypes.byref(a), ctypes.byref(b),
             ctypes.byref(c))
        return a.value, b.value, c.value

    def set_params(self, block, targets_per_item, ctas_per_sm):
        call("tbslas_batch_set_params", self.handle, int(block), int(targets_per_item),
             int(ctas_per_sm))

    def autotune(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        call("tbslas_batch_autotune", self.handle, ctypes.byref(a), ctypes.byref(b),
             ctypes.byref(c))
        return a.value, b.value, c.value

    def run(self, timestep0, nsteps, use_graph=True, stream=None):
        call("tbslas_batch_run", self.handle, int(timestep0), int(nsteps), int(bool(use_graph)),
             _stream(stream))


def fast_interp(ctx, grid, dof, n_reg, pts, bc=FreeSpace, out=None, stream=None):
    import torch
    n = pts.numel() // 3
    if out is None:
        out = torch.empty((n, dof), dtype=torch.float64, device=pts.device)
    call("tbslas_fast_interp", ctx.handle, _ptr(grid), int(dof), int(n_reg), _ptr(pts), n,
         _ptr(out), int(bc), _stream(stream))
    return out


def semilag_grid_steps(ctx, vel, con, n_reg, dt, nsteps, num_rk_step=1, bc=Periodic, out=None,
                       stream=None):
    """nsteps grid SL steps through one stationary velocity (CUDA tensors):
    the concentration after nsteps (out must not alias con)."""
    import torch
    if out is None:
        out = torch.empty_like(con)
    call("tbslas_semilag_grid_steps", ctx.handle, _ptr(vel), _ptr(con), _ptr(out), int(n_reg),
         float(dt), int(nsteps), int(num_rk_step), int(bc), _stream(stream))
    return out


def semilag_grid(ctx, vel, con, n_reg, dt, num_rk_step=1, bc=Periodic, out=None, stream=None):
    """One grid SL step.  vel [3,N,N,N], con [N,N,N] (CUDA tensors or numpy arrays)."""
    if isinstance(con, np.ndarray):
        if out is None:
            out = np.empty_like(con)
        call("tbslas_semilag_grid_host", ctx.handle, _ptr(vel), _ptr(con), _ptr(out),
             int(n_reg), float(dt), int(num_rk_step), int(bc))
        return out
    import torch
    if out is None:
        out = torch.empty_like(con)
    call("tbslas_semilag_grid", ctx.handle, _ptr(vel), _ptr(con), _ptr(out), int(n_reg),
         float(dt), int(num_rk_step), int(bc), _stream(stream))
    return out

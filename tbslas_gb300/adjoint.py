"""Differentiable T-step SL advection: torch.autograd.Function over the
in-situ SL step and the hand-written adjoint kernels.  The forward pass is
the production step (tbslas_semilag_in_situ, in the context's sum mode).  In
the double-float mode its leaf choices are the FP64 step's (targets near a
face are recomputed in FP64) and its values differ from the FP64 step's by
the sums' rounding (~1e-14), so the adjoint -- the derivative of that
piecewise-polynomial map with the leaf choices held fixed -- is its
derivative to the same accuracy.

    cT = advect(c0, vcoeff, vel_tree, con_tree, dt, timestep0, nsteps, bc, checkpoint)

c0 [L, 1, Nc] and vcoeff [Lv, 3, Nc] are CUDA float64 tensors (the
concentration and velocity Chebyshev coefficients); the result is the
concentration coefficients after nsteps in-situ SL steps (nrk = 1).  Backward
gives dJ/dc0 and dJ/dvcoeff.  checkpoint=True stores every step's RK2
midpoints and departure points (48 bytes per node per step); False
recomputes them in the backward pass; checkpoint="departure" stores the
departure points only (24 bytes per node per step) and rebuilds the
midpoints from the node-grid velocity in the backward pass;
checkpoint="jacobian" (FP64 sums) also stores the velocity Jacobian at every
midpoint (120 bytes per node per step), which the forward forms from the same
sums as the midpoint velocity and which takes the velocity-gradient term's
evaluation out of the backward pass.
"""
import numpy as np

from . import api
from .capi import call


def basis_at_nodes(q):
    """V[p][n] = T_i(z_p) T_j(y_p) T_k(x_p) at the leaf's nodes mapped to [-1,1]
    (the matrix whose pseudo-inverse is the point-to-coefficient matrix):
    node values of a leaf = coefficients @ V^T."""
    pts = 2.0 * api.new_nodes(q) - 1.0
    d = q + 1
    T = []
    for a in range(3):
        x = pts[:, a]
        t = [np.ones_like(x), x]
        for k in range(2, d):
            t.append(2 * x * t[-1] - t[-2])
        T.append(t[:d])
    cols = []
    for i in range(d):
        for j in range(d - i):
            for k in range(d - i - j):
                cols.append(T[2][i] * T[1][j] * T[0][k])
    return np.stack(cols, axis=1)


def step_ckpt(vel_functor, tree, timestep, dt, xmid, xdep, stream=None):
    call("tbslas_semilag_in_situ_ckpt", tree.ctx.handle, vel_functor.tree.handle, tree.handle,
         int(timestep), float(dt), vel_functor.bc, api._ptr(xmid), api._ptr(xdep),
         api._stream(stream))


def step_ckpt_jac(vel_functor, tree, timestep, dt, xmid, xdep, jac, stream=None):
    call("tbslas_semilag_in_situ_ckpt_jac", tree.ctx.handle, vel_functor.tree.handle,
         tree.handle, int(timestep), float(dt), vel_functor.bc, api._ptr(xmid), api._ptr(xdep),
         api._ptr(jac), api._stream(stream))


def step_adjoint_jac(vel_functor, tree, coeff_k, timestep, dt, lam_next, lam_k, grad_vel, xmid,
                     xdep, jac, node_w=None, stream=None):
    """One adjoint step from a Jacobian checkpoint; node_w as step_adjoint_seq
    (None: the step scatters its own node term)."""
    call("tbslas_semilag_adjoint_jac", tree.ctx.handle, vel_functor.tree.handle, tree.handle,
         api._ptr(coeff_k), int(timestep), float(dt), vel_functor.bc, api._ptr(lam_next),
         api._ptr(lam_k), api._ptr(grad_vel), api._ptr(xmid), api._ptr(xdep), api._ptr(jac),
         api._ptr(node_w), api._stream(stream))


def step_adjoint(vel_functor, tree, coeff_k, timestep, dt, lam_next, lam_k, grad_vel, xmid=None,
                 xdep=None, stream=None):
    call("tbslas_semilag_adjoint", tree.ctx.handle, vel_functor.tree.handle, tree.handle,
         api._ptr(coeff_k), int(timestep), float(dt), vel_functor.bc, api._ptr(lam_next),
         api._ptr(lam_k), api._ptr(grad_vel), api._ptr(xmid), api._ptr(xdep), api._stream(stream))


def step_adjoint_seq(vel_functor, tree, coeff_k, timestep, dt, lam_next, lam_k, grad_vel,
                     node_w, xmid=None, xdep=None, vel_at_nodes=None, stream=None):
    """One adjoint step of a sequence through one stationary velocity: the
    node term's weights are added to node_w ([N, 3], zeroed before the first
    step) for node_term to scatter once."""
    call("tbslas_semilag_adjoint_seq", tree.ctx.handle, vel_functor.tree.handle, tree.handle,
         api._ptr(coeff_k), int(timestep), float(dt), vel_functor.bc, api._ptr(lam_next),
         api._ptr(lam_k), api._ptr(grad_vel), api._ptr(xmid), api._ptr(xdep),
         api._ptr(vel_at_nodes), api._ptr(node_w), api._stream(stream))


def node_term(vel_functor, tree, node_w, grad_vel, stream=None):
    call("tbslas_semilag_adjoint_node_term", tree.ctx.handle, vel_functor.tree.handle,
         tree.handle, vel_functor.bc, api._ptr(node_w), api._ptr(grad_vel), api._stream(stream))


def _function():
    import torch

    class SemilagAdvect(torch.autograd.Function):
        @staticmethod
        def forward(ctx, c0, vcoeff, vel_tree, con_tree, dt, timestep0, nsteps, bc, checkpoint):
            vel_tree.set_coeffs(vcoeff.contiguous())
            con_tree.set_coeffs(c0.contiguous())
            vf = api.NodeFieldFunctor(vel_tree, bc)
            n = con_tree.n_leaves * api.n_points(con_tree.q)
            states, ckpts = [], []
            for k in range(nsteps):
                states.append(con_tree.get_coeffs(torch.empty_like(c0)))
                if checkpoint == "jacobian":
                    xd = torch.empty((n, 3), dtype=torch.float64, device=c0.device)
                    xm = torch.empty_like(xd)
                    jac = torch.empty((n, 9), dtype=torch.float64, device=c0.device)
                    step_ckpt_jac(vf, con_tree, timestep0 + k, dt, xm, xd, jac)
                    ckpts.append((xm, xd, jac))
                elif checkpoint:
                    xd = torch.empty((n, 3), dtype=torch.float64, device=c0.device)
                    xm = None if checkpoint == "departure" else torch.empty_like(xd)
                    step_ckpt(vf, con_tree, timestep0 + k, dt, xm, xd)
                    ckpts.append((xm, xd, None))
                else:
                    api.solve_semilag_in_situ(vf, con_tree, timestep0 + k, dt, 1)
            cT = con_tree.get_coeffs(torch.empty_like(c0))
            ctx.vel_tree, ctx.con_tree, ctx.dt, ctx.ts0, ctx.bc = vel_tree, con_tree, dt, timestep0, bc
            ctx.states, ctx.ckpts, ctx.vshape = states, ckpts, vcoeff.shape
            ctx.vcoeff = vcoeff
            return cT

        @staticmethod
        def backward(ctx, grad_cT):
            vel_tree, con_tree = ctx.vel_tree, ctx.con_tree
            vel_tree.set_coeffs(ctx.vcoeff.detach().contiguous())
            vf = api.NodeFieldFunctor(vel_tree, ctx.bc)
            lam = grad_cT.contiguous().clone()
            gv = torch.zeros(ctx.vshape, dtype=torch.float64, device=grad_cT.device)
            # The velocity is one parameter for every step and the tree shapes
            # stay fixed: the node term's weights are summed over the steps and
            # scattered once, and where the steps rebuild their points the
            # velocity at the nodes is evaluated once.
            n = con_tree.n_leaves * api.n_points(con_tree.q)
            node_w = torch.zeros((n, 3), dtype=torch.float64, device=grad_cT.device)
            rebuild = not ctx.ckpts or ctx.ckpts[0][0] is None
            vn = vf.at_nodes(con_tree) if rebuild and ctx.states else None
            for k in reversed(range(len(ctx.states))):
                lam_k = torch.empty_like(lam)
                xm, xd, jac = ctx.ckpts[k] if ctx.ckpts else (None, None, None)
                if jac is not None:
                    step_adjoint_jac(vf, con_tree, ctx.states[k], ctx.ts0 + k, ctx.dt, lam, lam_k,
                                     gv, xm, xd, jac, node_w)
                else:
                    step_adjoint_seq(vf, con_tree, ctx.states[k], ctx.ts0 + k, ctx.dt, lam,
                                     lam_k, gv, node_w, xm, xd, vn)
                lam = lam_k
            if ctx.states:
                node_term(vf, con_tree, node_w, gv)
            return lam, gv, None, None, None, None, None, None, None

    return SemilagAdvect


_FN = None


def advect(c0, vcoeff, vel_tree, con_tree, dt, timestep0=1, nsteps=1, bc=api.FreeSpace,
           checkpoint=True):
    global _FN
    if _FN is None:
        _FN = _function()
    if checkpoint not in (True, False, "departure", "jacobian"):
        raise ValueError("checkpoint must be True, False, 'departure' or 'jacobian'")
    return _FN.apply(c0, vcoeff, vel_tree, con_tree, float(dt), int(timestep0), int(nsteps),
                     int(bc), checkpoint)

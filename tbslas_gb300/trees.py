"""Host-side construction of linear octrees and their initial coefficients.

Set-up code, not on the SL path: it stands in for ConstructTree / InitTree
(src/tree/tree_utils.h:83-178), whose refinement lives in PVFMM
(Cheb_Node::RefineTree / SubdivCond, not vendored).  The refinement rule here
is this project's own coefficient-tail criterion: a leaf is split while the
sum of |c| over its total-degree-q coefficients (all dofs) exceeds `tol` and
it is shallower than `max_depth`; leaves are then 2:1 balanced across faces,
edges and corners.  Initial coefficients are the least-squares fit at the
leaf's Chebyshev nodes (the SetTreeGridValues operator).
"""
import contextlib

import numpy as np

from . import api

KEY_BITS = 21


class HostMath:
    """Where host-side set-up takes the Chebyshev nodes of degree q
    ((q+1)^3 x 3, new_nodes order) and the point-to-coefficient matrix M
    (GetPt2CoeffMatrix) from: by default this library's own host routines
    (tbslas_cheb_nodes / tbslas_pt2coeff_matrix)."""

    def __init__(self, nodes=None, pt2coeff=None):
        self.nodes = nodes or api.new_nodes
        self.pt2coeff = pt2coeff or api.get_pt2coeff_matrix


_math = HostMath()


@contextlib.contextmanager
def host_math(math):
    """Builds trees and fits with `math` (a HostMath) inside the block."""
    global _math
    prev, _math = _math, math
    try:
        yield math
    finally:
        _math = prev


def cheb_nodes(q):
    return _math.nodes(q)


def pt2coeff(q):
    return _math.pt2coeff(q)


def _spread3(v):
    v = v.astype(np.uint64) & np.uint64(0x1FFFFF)
    v = (v | (v << np.uint64(32))) & np.uint64(0x1F00000000FFFF)
    v = (v | (v << np.uint64(16))) & np.uint64(0x1F0000FF0000FF)
    v = (v | (v << np.uint64(8))) & np.uint64(0x100F00F00F00F00F)
    v = (v | (v << np.uint64(4))) & np.uint64(0x10C30C30C30C30C3)
    v = (v | (v << np.uint64(2))) & np.uint64(0x1249249249249249)
    return v


def morton_keys(anchor):
    """63-bit interleaved keys (z most significant in each level) of points in [0,1)^3."""
    a = np.asarray(anchor, dtype=np.float64).reshape(-1, 3)
    q = np.floor(a * float(1 << KEY_BITS)).astype(np.uint64)
    return _spread3(q[:, 0]) | (_spread3(q[:, 1]) << np.uint64(1)) | (_spread3(q[:, 2]) << np.uint64(2))


def sort_leaves(anchor, depth):
    k = morton_keys(anchor)
    o = np.argsort(k, kind="stable")
    return np.ascontiguousarray(anchor[o]), np.ascontiguousarray(depth[o])


def uniform_tree(depth):
    n = 1 << depth
    i = np.arange(n ** 3)
    anchor = np.stack([(i % n), (i // n) % n, i // (n * n)], axis=1).astype(np.float64) / n
    return sort_leaves(anchor, np.full(n ** 3, depth, dtype=np.int32))


def split(anchor, depth):
    """The 8 children of each leaf, in child order x + 2y + 4z."""
    h = np.ldexp(1.0, -(depth + 1))
    off = np.array([[(c >> 0) & 1, (c >> 1) & 1, (c >> 2) & 1] for c in range(8)], dtype=np.float64)
    ch = anchor[:, None, :] + h[:, None, None] * off[None, :, :]
    return ch.reshape(-1, 3), np.repeat(depth + 1, 8).astype(np.int32)


def leaf_nodes(anchor, depth, q):
    """Chebyshev nodes of every leaf [L*Np, 3] (CollectChebTreeGridPoints order)."""
    nodes = _math.nodes(q)
    h = np.ldexp(1.0, -depth.astype(np.int64))
    return (anchor[:, None, :] + h[:, None, None] * nodes[None, :, :]).reshape(-1, 3)


def fit(fn, anchor, depth, q, dof, M=None):
    """[L, dof, Nc] coefficients of fn (pts[n,3] -> vals[n,dof]) on every leaf."""
    M = _math.pt2coeff(q) if M is None else M
    L = depth.size
    np_ = (q + 1) ** 3
    vals = np.asarray(fn(leaf_nodes(anchor, depth, q)), dtype=np.float64).reshape(L, np_, dof)
    vals = np.ascontiguousarray(vals.transpose(0, 2, 1)).reshape(L * dof, np_)
    return (vals @ M).reshape(L, dof, -1)


def tail(coeff, q):
    """Sum over dofs of |c| over the total-degree-q coefficients of each leaf."""
    mask = []
    d = q + 1
    for i in range(d):
        for j in range(d - i):
            for k in range(d - i - j):
                mask.append(i + j + k == q)
    mask = np.array(mask)
    return np.abs(coeff[:, :, mask]).sum(axis=(1, 2))


def _containing_leaf(keys, pts):
    pk = morton_keys(pts)
    return np.searchsorted(keys, pk, side="right") - 1


def balance21(anchor, depth, periodic=False):
    """Refine until every leaf's face/edge/corner neighbours differ by <= 1 level."""
    dirs = np.array([(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)
                     if (a, b, c) != (0, 0, 0)], dtype=np.float64)
    while True:
        anchor, depth = sort_leaves(anchor, depth)
        keys = morton_keys(anchor)
        h = np.ldexp(1.0, -depth.astype(np.int64))
        delta = np.ldexp(1.0, -(KEY_BITS + 1))
        centre = anchor + 0.5 * h[:, None]
        probe = centre[:, None, :] + dirs[None, :, :] * (0.5 * h[:, None, None] + delta)
        probe = probe.reshape(-1, 3)
        src = np.repeat(np.arange(depth.size), len(dirs))
        if periodic:
            probe = probe - np.floor(probe)
            ok = np.ones(len(probe), dtype=bool)
        else:
            ok = np.all((probe >= 0.0) & (probe < 1.0), axis=1)
        nb = _containing_leaf(keys, probe[ok])
        coarse = depth[nb] < depth[src[ok]] - 1
        refine = np.zeros(depth.size, dtype=bool)
        refine[nb[coarse]] = True
        if not refine.any():
            return anchor, depth
        ca, cd = split(anchor[refine], depth[refine])
        anchor = np.concatenate([anchor[~refine], ca])
        depth = np.concatenate([depth[~refine], cd])


def adaptive_tree(fn, q, dof, tol, min_depth, max_depth, balance=True, periodic=False, M=None,
                  fitter=None):
    """Leaves refined by the coefficient-tail rule; returns (anchor, depth).

    fitter(anchor, depth) -> [L, dof, Nc] replaces fit(fn, ...) when given."""
    M = _math.pt2coeff(q) if M is None else M
    anchor, depth = uniform_tree(min_depth)
    while True:
        c = fitter(anchor, depth) if fitter is not None else fit(fn, anchor, depth, q, dof, M)
        refine = (tail(c, q) > tol) & (depth < max_depth)
        if not refine.any():
            break
        ca, cd = split(anchor[refine], depth[refine])
        anchor = np.concatenate([anchor[~refine], ca])
        depth = np.concatenate([depth[~refine], cd])
        anchor, depth = sort_leaves(anchor, depth)
    if balance:
        anchor, depth = balance21(anchor, depth, periodic)
    return sort_leaves(anchor, depth)

"""Re-meshing oracle (test infrastructure only).

CPU restatement of the adaptive re-meshing the reference runs after every SL
step: `tcon.RefineTree(); tcon.Balance21(bc);`
(src/applications/src/advection.cpp:305-311).  Both calls live in PVFMM
(MPI_Tree::RefineTree, Cheb_Node::SubdivCond / Subdivide / Truncate,
MPI_Tree::Balance21), which is not vendored, so the rule below is this
project's restatement of their published behaviour and its parity is
UNPINNED against the reference; the device path (tbslas_tree_remesh) is
checked against this file.

Rules, with tail(leaf) = sum over dofs of |c| over the coefficients of total
degree q (the Chebyshev truncation estimate of SubdivCond):
  1. coarsen, one level: every complete group of 8 sibling leaves of depth
     d > min_depth is replaced by its parent when the parent's tail <= tol;
     the parent's coefficients are the fit, at the parent's nodes, of the
     sibling whose closed half contains each node along every axis (node
     coordinate >= 0.5 of the parent: upper child);
  2. refine: while some leaf has tail > tol and depth < max_depth, split every
     such leaf into its 8 children, whose coefficients are the fit of the
     parent's expansion at the child's nodes (its exact restriction, up to
     rounding);
  3. balance 2:1: while some leaf has a face, edge or corner neighbour more
     than one level deeper (probed just outside its box; periodic images
     under a periodic boundary), split every such leaf as in 2.
Leaves that no rule touches keep their coefficients bit for bit.
"""
import numpy as np

from . import oracle as ora

KEY_BITS = 21


def _spread3(v):
    v = v.astype(np.uint64) & np.uint64(0x1FFFFF)
    for sh, m in ((32, 0x1F00000000FFFF), (16, 0x1F0000FF0000FF), (8, 0x100F00F00F00F00F),
                  (4, 0x10C30C30C30C30C3), (2, 0x1249249249249249)):
        v = (v | (v << np.uint64(sh))) & np.uint64(m)
    return v


def keys(pts):
    """Interleaved 21-bit keys, z most significant within a level; 1.0 maps to
    the last cell."""
    p = np.asarray(pts, dtype=np.float64).reshape(-1, 3)
    q = np.where(p >= 1.0, float((1 << KEY_BITS) - 1), np.floor(p * float(1 << KEY_BITS)))
    q = np.clip(np.nan_to_num(q), 0.0, float((1 << KEY_BITS) - 1)).astype(np.uint64)
    return _spread3(q[:, 0]) | (_spread3(q[:, 1]) << np.uint64(1)) | (_spread3(q[:, 2]) << np.uint64(2))


def tails(coeff, q):
    d = q + 1
    mask = np.array([i + j + k == q for i in range(d) for j in range(d - i) for k in range(d - i - j)])
    return np.abs(coeff[:, :, mask]).sum(axis=(1, 2))


def _nodes1(q):
    return ora.new_nodes(q)[: q + 1, 0].copy()


def _eval_leaf(c, q, xi):
    """Expansion c [dof, Nc] at local coordinates xi [n, 3] in [-1, 1]."""
    return ora.cheb_basis(q, xi) @ c.T


def _grid(a):
    """Tensor grid of per-axis coordinates a [3][D], x fastest: [D^3, 3]."""
    D = a.shape[1]
    i = np.arange(D ** 3)
    return np.stack([a[0][i % D], a[1][(i // D) % D], a[2][i // (D * D)]], axis=1)


def child_coeffs(cp, q, anchor, depth, child, M):
    """Restriction of the parent's expansion cp [dof, Nc] (leaf at anchor,
    depth) to child `child` (x + 2y + 4z)."""
    x1 = _nodes1(q)
    h = np.ldexp(1.0, -int(depth))
    hc = 0.5 * h
    w = np.ldexp(2.0, int(depth))
    bits = np.array([(child >> a) & 1 for a in range(3)], dtype=np.float64)
    ca = anchor + hc * bits
    X = np.stack([ca[a] + hc * x1 for a in range(3)])  # child node coordinates
    xi = np.stack([(X[a] - anchor[a]) * w - 1.0 for a in range(3)])
    vals = _eval_leaf(cp, q, _grid(xi))  # [Np, dof]
    return (vals.T @ M)


def parent_coeffs(cs, q, anchor, depth_p, M):
    """Fit of the 8 siblings cs [8][dof, Nc] at the nodes of their parent
    (anchor, depth_p); along each axis a node at >= 0.5 of the parent takes
    the upper child."""
    x1 = _nodes1(q)
    D = q + 1
    h = np.ldexp(1.0, -int(depth_p))
    hc = 0.5 * h
    wc = np.ldexp(2.0, int(depth_p) + 1)
    X = np.stack([anchor[a] + h * x1 for a in range(3)])
    up = x1 >= 0.5
    pts = _grid(X)
    i = np.arange(D ** 3)
    bits = np.stack([up[i % D], up[(i // D) % D], up[i // (D * D)]], axis=1).astype(np.int64)
    child = bits[:, 0] + 2 * bits[:, 1] + 4 * bits[:, 2]
    vals = np.zeros((D ** 3, cs.shape[1]))
    for c in range(8):
        sel = child == c
        if not sel.any():
            continue
        ca = anchor + hc * np.array([(c >> a) & 1 for a in range(3)], dtype=np.float64)
        xi = (pts[sel] - ca[None, :]) * wc - 1.0
        vals[sel] = _eval_leaf(cs[c], q, xi)
    return vals.T @ M


def _split(anchor, depth, coeff, origin, flag, q, M):
    out_a, out_d, out_c, out_o = [], [], [], []
    for i in range(depth.size):
        if not flag[i]:
            out_a.append(anchor[i][None])
            out_d.append(depth[i:i + 1])
            out_c.append(coeff[i][None])
            out_o.append(origin[i:i + 1])
            continue
        h = np.ldexp(1.0, -int(depth[i]) - 1)
        for c in range(8):
            out_a.append((anchor[i] + h * np.array([(c >> a) & 1 for a in range(3)], dtype=np.float64))[None])
            out_d.append(np.array([depth[i] + 1], dtype=np.int32))
            out_c.append(child_coeffs(coeff[i], q, anchor[i], depth[i], c, M)[None])
            out_o.append(np.array([-1]))
    return (np.concatenate(out_a), np.concatenate(out_d).astype(np.int32), np.concatenate(out_c),
            np.concatenate(out_o))


def sibling_groups(anchor, depth, min_depth):
    """First leaf of every complete group of 8 sibling leaves deeper than
    min_depth (leaves in Morton order)."""
    k = keys(anchor)
    L = depth.size
    out = []
    for i in range(L - 7):
        d = int(depth[i])
        if d <= min_depth:
            continue
        unit = np.uint64(1) << np.uint64(3 * (KEY_BITS - d))
        if k[i] % (unit * np.uint64(8)) != 0:
            continue
        if depth[i + 7] == d and k[i + 7] == k[i] + np.uint64(7) * unit:
            out.append(i)
    return out


def balance_flags(anchor, depth, periodic):
    dirs = np.array([(a, b, c) for c in (-1, 0, 1) for b in (-1, 0, 1) for a in (-1, 0, 1)
                     if (a, b, c) != (0, 0, 0)], dtype=np.float64)
    k = keys(anchor)
    h = np.ldexp(1.0, -depth.astype(np.int64))
    delta = np.ldexp(1.0, -(KEY_BITS + 1))
    centre = anchor + 0.5 * h[:, None]
    flag = np.zeros(depth.size, dtype=bool)
    for dv in dirs:
        p = centre + dv[None, :] * (0.5 * h[:, None] + delta)
        if periodic:
            p = np.where(p < 0.0, p + 1.0, p)
            p = np.where(p >= 1.0, p - 1.0, p)
            ok = np.ones(depth.size, dtype=bool)
        else:
            ok = np.all((p >= 0.0) & (p < 1.0), axis=1)
        nb = np.searchsorted(k, keys(p), side="right") - 1
        flag |= ok & (depth[nb] > depth + 1)
    return flag


def remesh(anchor, depth, q, coeff, tol, min_depth, max_depth, periodic=False, origin=False):
    """(anchor, depth, coeff) after the three rules; coeff [L, dof, Nc].
    With origin, also the index of the input leaf each output leaf is an
    untouched copy of (-1 for merged and split leaves)."""
    M = ora.pt2coeff(q)
    anchor = np.asarray(anchor, dtype=np.float64).copy()
    depth = np.asarray(depth, dtype=np.int32).copy()
    coeff = np.asarray(coeff, dtype=np.float64).copy()
    org = np.arange(depth.size)
    # 1. coarsen one level
    groups = sibling_groups(anchor, depth, min_depth)
    keep = np.ones(depth.size, dtype=bool)
    merged = {}
    for i in groups:
        pc = parent_coeffs(coeff[i:i + 8], q, anchor[i], depth[i] - 1, M)
        if tails(pc[None], q)[0] <= tol:
            merged[i] = pc
            keep[i + 1:i + 8] = False
    if merged:
        for i, pc in merged.items():
            coeff[i] = pc
            depth[i] -= 1
            org[i] = -1
        anchor, depth, coeff, org = anchor[keep], depth[keep], coeff[keep], org[keep]
    # 2. refine
    while True:
        flag = (tails(coeff, q) > tol) & (depth < max_depth)
        if not flag.any():
            break
        anchor, depth, coeff, org = _split(anchor, depth, coeff, org, flag, q, M)
    # 3. balance 2:1
    while True:
        flag = balance_flags(anchor, depth, periodic)
        if not flag.any():
            break
        anchor, depth, coeff, org = _split(anchor, depth, coeff, org, flag, q, M)
    return (anchor, depth, coeff, org) if origin else (anchor, depth, coeff)

"""Tree-construction oracle (test infrastructure only).

CPU restatement of the reference's ConstructTree / InitTree
(src/tree/tree_utils.h:83-178) as the device path (tbslas_tree_construct /
tbslas_tree_fit_field) states it: the analytic input fields of
src/utils/fields.h evaluated at every leaf's Chebyshev nodes and fitted
(SetTreeGridValues' operator); from the uniform tree of min_depth, leaves
whose fit has tail > tol below max_depth are split and refitted until none
is, then 2:1 balanced (oracle/remesh.py's rule) and fitted.  PVFMM's own
refinement (Initialize / RefineTree) is not vendored, so the tree shape's
parity against the reference is UNPINNED.
"""
import math

import numpy as np

from . import oracle as ora
from . import remesh as rm

TWO_PI = 2 * math.pi


def field_values(kind, n, p, pts):
    """[npts, dof] values of the field (kinds as tbslas_field)."""
    p = np.asarray(p, dtype=np.float64).reshape(-1)
    x, y, z = pts[:, 0], pts[:, 1], pts[:, 2]
    if kind == 0:  # sum of Gaussians
        s = np.zeros(len(pts))
        for i in range(n):
            cx, cy, cz, sg, amp = p[5 * i:5 * i + 5]
            s += amp * np.exp(-((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2) / (2.0 * sg * sg))
        return s[:, None]
    if kind == 1:  # get_gaussian_field_3d, fields.h:275-294
        return (p[3] * np.exp(-((x - p[0]) ** 2 / (2 * p[4] * p[4]) + (y - p[1]) ** 2
                                / (2 * p[5] * p[5]) + (z - p[2]) ** 2 / (2 * p[6] * p[6]))))[:, None]
    if kind == 2:  # get_exp_alpha_field, fields.h:28-42
        r = np.sqrt((x - p[0]) ** 2 + (y - p[1]) ** 2 + (z - p[2]) ** 2)
        return np.exp(-(r / p[3]) ** p[4])[:, None]
    if kind == 3:  # get_vorticity_field, fields.h:142-157
        return np.stack([p[0] * (0.5 - y), p[0] * (x - 0.5), np.zeros(len(pts))], axis=1)
    if kind == 4:
        return np.stack([np.sin(TWO_PI * x) * np.cos(TWO_PI * y) * np.cos(TWO_PI * z),
                         -np.cos(TWO_PI * x) * np.sin(TWO_PI * y) * np.cos(TWO_PI * z),
                         np.zeros(len(pts))], axis=1)
    if kind == 5:  # get_taylor_green_field, fields.h:51-80
        A, B, C, a, b, c = p[:6]
        return np.stack([A * np.cos(a * x) * np.sin(b * y) * np.sin(c * z),
                         B * np.sin(a * x) * np.cos(b * y) * np.sin(c * z),
                         C * np.sin(a * x) * np.sin(b * y) * np.cos(c * z)], axis=1)
    if kind == 6:  # get_hopf_field, fields.h:119-139
        dx, dy, dz, r = x - p[0], y - p[1], z - p[2], p[4]
        r2 = dx * dx + dy * dy + dz * dz
        c = p[3] / ((r * r + r2) * (r * r + r2))
        return np.stack([c * (2 * (-r * dy + dx * dz)), c * (2 * (r * dx + dy * dz)),
                         c * (r * r - dx * dx - dy * dy + dz * dz)], axis=1)
    if kind == 7:  # Fourier modes
        out = np.zeros((len(pts), 3))
        for i in range(n):
            m = p[9 * i:9 * i + 9]
            ph = TWO_PI * (m[0] * x + m[1] * y + m[2] * z)
            out += np.cos(ph)[:, None] * m[3:6][None, :] + np.sin(ph)[:, None] * m[6:9][None, :]
        return out
    raise ValueError("field kind %d" % kind)


def dof_of(kind):
    return 1 if kind in (0, 1, 2) else 3


def fit(kind, n, p, anchor, depth, q):
    """InitTree: [L, dof, Nc] fit of the field on every leaf."""
    pts = ora.collect_grid_points(anchor, depth, q)
    v = field_values(kind, n, p, pts)  # [L*Np, dof]
    L, npl, dof = len(depth), (q + 1) ** 3, v.shape[1]
    vals = v.reshape(L, npl, dof).transpose(0, 2, 1).reshape(-1)
    return ora.set_tree_grid_values(L, q, dof, vals)


def uniform(depth):
    n = 1 << depth
    i = np.arange(n ** 3)
    a = np.stack([i % n, (i // n) % n, i // (n * n)], axis=1).astype(np.float64) / n
    o = np.argsort(rm.keys(a), kind="stable")
    return a[o], np.full(n ** 3, depth, dtype=np.int32)


def _split_shape(anchor, depth, flag):
    out_a, out_d = [], []
    for i in range(depth.size):
        if not flag[i]:
            out_a.append(anchor[i][None])
            out_d.append(depth[i:i + 1])
            continue
        h = np.ldexp(1.0, -int(depth[i]) - 1)
        for c in range(8):
            out_a.append((anchor[i] + h * np.array([(c >> a) & 1 for a in range(3)], float))[None])
            out_d.append(np.array([depth[i] + 1], dtype=np.int32))
    return np.concatenate(out_a), np.concatenate(out_d).astype(np.int32)


def construct(kind, n, p, q, tol, min_depth, max_depth, periodic=False):
    """ConstructTree: (anchor, depth, coeff) of the adaptive tree."""
    anchor, depth = uniform(min_depth)
    while True:
        c = fit(kind, n, p, anchor, depth, q)
        flag = (rm.tails(c, q) > tol) & (depth < max_depth)
        if not flag.any():
            break
        anchor, depth = _split_shape(anchor, depth, flag)
    balanced = False
    while True:
        flag = rm.balance_flags(anchor, depth, periodic)
        if not flag.any():
            break
        balanced = True
        anchor, depth = _split_shape(anchor, depth, flag)
    if balanced:
        c = fit(kind, n, p, anchor, depth, q)
    return anchor, depth, c

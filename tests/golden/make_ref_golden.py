"""Writes tests/golden/ref_pin.npz and tests/golden/ref_next.npz: outputs of
the reference's own SL-path code (oracle/_ref, built from the reference's
sources by oracle/build_ref.py) on small seeded cases -- the step and its
parts; the step through the time-dependent velocity functors
(FieldSetFunctor, FieldExtrapFunctor, InterpCubic1D) and the driver's BDF2
step.  Run from the repository root where the reference's sources are
present:

    python tests/golden/make_ref_golden.py          # both files
    python tests/golden/make_ref_golden.py next     # ref_next.npz only

The inputs are built with the oracle's set-up math only (its Chebyshev nodes
and pseudo-inverse).  tests/test_ref_pin.py checks the oracle against these
vectors on every machine (bit for bit where the arithmetic is the same) and
the CUDA path against them on the GPU."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as ora  # noqa: E402
from oracle import ref  # noqa: E402
from tbslas_gb300 import fields, trees  # noqa: E402


def oracle_math():
    def nodes(q):
        return ora.collect_grid_points(np.zeros((1, 3)), np.zeros(1, dtype=np.int32), q)
    return trees.HostMath(nodes=nodes, pt2coeff=ora.pt2coeff)


def special_points(rng, n):
    """Points in [0,1]^3 with leaf faces, the domain faces and 1.0 among them."""
    p = rng.uniform(0.0, 1.0, size=(n, 3))
    p[:8] = [[1.0, 0.5, 0.5], [0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [0.5, 0.5, 0.5],
             [0.25, 0.75, 1.0], [0.125, 0.375, 0.0], [1.0 - 2 ** -53, 0.5, 0.25],
             [0.5, 0.0625, 0.9375]]
    return p


def main():
    if ref.lib() is None:
        raise SystemExit("the reference's sources are not present; nothing to generate")
    rng = np.random.default_rng(2024)
    out = {}
    with trees.host_math(oracle_math()):
        blob = fields.gaussian((0.35, 0.6, 0.45), 0.07)
        a, d = trees.adaptive_tree(blob, 4, 1, 1e-3, 1, 2)
        out["tree_anchor"], out["tree_depth"] = a, d
        out["collect_q3"] = ref.collect_grid_points(a, d, 3)
        for q in (6, 8, 14):
            out["nodes_q%d" % q] = ref.new_nodes(q)
        ua1, ud1 = trees.uniform_tree(1)
        out["tree1_anchor"], out["tree1_depth"] = ua1, ud1
        for q, dof in ((5, 1), (8, 3), (14, 1)):
            ta, td = (a, d) if q < 14 else (ua1, ud1)  # q = 14 on the 8-leaf tree
            c = rng.standard_normal((len(td), dof, ref.nc(q))) / (1 + np.arange(ref.nc(q)))
            out["eval_q%d_coeff" % q] = c
            for bc in (0, 1):
                p = (special_points(rng, 1000) if bc == 0
                     else rng.uniform(-0.05, 1.05, size=(1000, 3)))
                out["eval_q%d_bc%d_pts" % (q, bc)] = p
                out["eval_q%d_bc%d_out" % (q, bc)] = ref.eval_tree(ta, td, q, dof, c, p, bc)
        q = 8
        ua, ud = trees.uniform_tree(1)
        vt = trees.fit(fields.taylor_green(), ua, ud, q, 3)
        out["traj_anchor"], out["traj_depth"], out["traj_vc"] = ua, ud, vt
        x = special_points(rng, 1000)
        out["traj_pts"] = x
        for bc, nrk in ((0, 1), (1, 1), (0, 3)):
            out["traj_bc%d_nrk%d" % (bc, nrk)] = ref.traj_rk2(ua, ud, q, vt, x, 0.3, 0.25, nrk,
                                                                bc)
        N = 12
        g = rng.standard_normal((3, N, N, N))
        pg = rng.uniform(-0.1, 1.1, size=(2000, 3))
        pg[:4] = [[1.0, 1.0, 1.0], [0.0, 0.0, 0.0], [0.5, 1.0, 0.0], [1 - 1e-17, 0.3, 0.3]]
        out["interp_grid"], out["interp_pts"] = g, pg
        out["interp_out"] = ref.fast_interp(g, 3, N, pg)
        # one in-situ step (dof 1): Taylor-Green velocity tree, Gaussian blobs
        q = 6
        va, vd = trees.adaptive_tree(fields.taylor_green(), 4, 3, 1e-2, 1, 2)
        blobs = fields.gaussian_blobs(rng, 3, (0.05, 0.1))
        ca, cd = trees.adaptive_tree(blobs, 4, 1, 1e-3, 1, 2)
        vc = trees.fit(fields.taylor_green(), va, vd, q, 3)
        cc = trees.fit(blobs, ca, cd, q, 1)
        for k, v in (("va", va), ("vd", vd), ("vc", vc), ("ca", ca), ("cd", cd), ("cc", cc)):
            out["step_" + k] = v
        for bc in (0, 1):
            out["step_bc%d_out" % bc] = ref.semilag_in_situ(
                dict(anchor=va, depth=vd, q=q, dof=3, coeff=vc),
                dict(anchor=ca, depth=cd, q=q, dof=1, coeff=cc), 2, 0.02, 1, bc)
    path = os.path.join(HERE, "ref_pin.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


def tv_velocity(k, periodic):
    """Four related velocity fields of a time series (the ones
    tests/test_gpu_tv.py uses)."""
    if periodic:
        base = fields.fourier_velocity(np.random.default_rng(20 + k))
        return lambda p: 0.4 * base(p)
    tg, rot, s = fields.taylor_green(), fields.rotation(2 * np.pi), 0.2 * k
    return lambda p: (1.0 - s) * tg(p) + s * rot(p)


def main_next():
    if ref.lib() is None:
        raise SystemExit("the reference's sources are not present; nothing to generate")
    rng = np.random.default_rng(2025)
    out = {}
    q, timestep, dt = 4, 3, 0.02
    times = np.array([0.0, 0.02, 0.04, 0.06])
    out["times"] = times
    with trees.host_math(oracle_math()):
        blob = fields.gaussian((0.5, 0.45, 0.55), 0.1)
        ca, cd = trees.adaptive_tree(blob, q, 1, 1e-3, 1, 2)
        out["con_anchor"], out["con_depth"] = ca, cd
        out["con_coeff"] = trees.fit(blob, ca, cd, q, 1)
        con = dict(anchor=ca, depth=cd, q=q, dof=1, coeff=out["con_coeff"])
        i = 0
        for periodic, same in ((0, True), (0, False), (1, True)):
            vels = []
            for k in range(4):
                if same:
                    a, d = trees.uniform_tree(1)
                else:
                    g = fields.gaussian((0.3 + 0.1 * k, 0.5, 0.5), 0.1)
                    a, d = trees.adaptive_tree(g, q, 1, 1e-3, 1, 2)
                c = trees.fit(tv_velocity(k, periodic), a, d, q, 3)
                vels.append(dict(anchor=a, depth=d, q=q, dof=3, coeff=c))
            for kind in ("set", "extrap"):
                pre = "case%d_" % i
                vs = vels if kind == "set" else [vels[1], vels[0]]
                out[pre + "periodic"] = np.int32(periodic)
                out[pre + "set"] = np.int32(kind == "set")
                for k, v in enumerate(vs):
                    for f in ("anchor", "depth", "coeff"):
                        out[pre + "v%d_%s" % (k, f)] = v[f]
                out[pre + "out"] = ref.semilag_in_situ_tv(
                    vs, con, timestep, dt, 1, periodic, times=times if kind == "set" else None)
                i += 1
        out["n_cases"] = np.int32(i)
        out["timestep"], out["dt"], out["q"] = np.int32(timestep), np.float64(dt), np.int32(q)
        # InterpCubic1D on its own: increasing times, queries inside and
        # outside the middle interval
        xx = np.sort(rng.uniform(-1.0, 1.0, (500, 4)), axis=1) + np.arange(4) * 0.1
        x = xx[:, 0] - 0.1 + rng.uniform(0.0, 1.0, 500) * (xx[:, 3] - xx[:, 0] + 0.2)
        pp = rng.standard_normal((500, 4))
        out["cubic_x"], out["cubic_xx"], out["cubic_pp"] = x, xx, pp
        out["cubic_out"] = ref.interp_cubic_1d(x, xx, pp)
        # the BDF2 step: c_{n-1}, c_n and the target tree of different
        # leaves, free space and periodic
        b1, b2 = fields.gaussian((0.5, 0.45, 0.55), 0.1), fields.gaussian((0.52, 0.45, 0.55), 0.1)
        pa, pd = trees.adaptive_tree(b1, q, 1, 1e-3, 1, 2)
        ca2, cd2 = trees.adaptive_tree(b2, q, 1, 1e-3, 1, 3)
        na, nd = trees.adaptive_tree(b2, q, 1, 1e-4, 1, 2)
        for k, v in (("pa", pa), ("pd", pd), ("ca", ca2), ("cd", cd2), ("na", na), ("nd", nd)):
            out["bdf2_" + k] = v
        out["bdf2_pc"] = trees.fit(b1, pa, pd, q, 1)
        out["bdf2_cc"] = trees.fit(b2, ca2, cd2, q, 1)
        prev = dict(anchor=pa, depth=pd, q=q, dof=1, coeff=out["bdf2_pc"])
        cur = dict(anchor=ca2, depth=cd2, q=q, dof=1, coeff=out["bdf2_cc"])
        nxt = dict(anchor=na, depth=nd, q=q, dof=1)
        for periodic in (0, 1):
            va, vd = trees.uniform_tree(1)
            vc = trees.fit(tv_velocity(1, periodic), va, vd, q, 3)
            out["bdf2_bc%d_vc" % periodic] = vc
            vel = dict(anchor=va, depth=vd, q=q, dof=3, coeff=vc)
            out["bdf2_bc%d_out" % periodic] = ref.semilag_bdf2(vel, prev, cur, nxt, 0.3, 0.02, 1,
                                                               periodic)
    path = os.path.join(HERE, "ref_next.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    if sys.argv[1:] != ["next"]:
        main()
    main_next()

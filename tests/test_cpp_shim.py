"""The C++ drop-in layer (include/tbslas_gb300.hpp): it compiles against the
header and links against the library on any host; on the GPU a driver-shaped
program (tests/cpp/shim_demo.cpp) reproduces the oracle."""
import os
import subprocess

import numpy as np
import pytest

from tbslas_gb300 import fields, trees

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _compile(built, tmp_path, name="shim_demo"):
    exe = str(tmp_path / name)
    pkg = os.path.join(ROOT, "tbslas_gb300")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                           os.path.join(HERE, "cpp", name + ".cpp"), "-L" + pkg,
                           "-ltbslas_gb300", "-Wl,-rpath," + pkg, "-o", exe])
    return exe


@pytest.mark.parametrize("name", ["shim_demo", "shim_next"])
def test_shim_compiles_and_links(built, tmp_path, name):
    assert os.path.exists(_compile(built, tmp_path, name))


@pytest.mark.gpu
def test_shim_next_matches_oracle(built, ora, tmp_path):
    """FieldSetFunctor / the two-functor step / BDF2 / re-meshing through the
    C++ layer against the oracle's restatements."""
    from oracle import remesh as rm
    q, dt, tol, maxd = 4, 0.02, 1e-3, 3
    a, d = trees.uniform_tree(2)
    tg, rot = fields.taylor_green(), fields.rotation(2 * np.pi)
    vcs = [trees.fit(lambda p, s=0.2 * k: (1 - s) * tg(p) + s * rot(p), a, d, q, 3)
           for k in range(4)]
    cc = trees.fit(fields.gaussian((0.45, 0.5, 0.55), 0.08), a, d, q, 1)
    cp = trees.fit(fields.gaussian((0.46, 0.5, 0.54), 0.08), a, d, q, 1)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        for x in [np.array([len(d), q, dt, tol, maxd]), a, d.astype(np.float64)] + vcs + [cc, cp]:
            f.write(np.ascontiguousarray(x, dtype=np.float64).tobytes())
    out = tmp_path / "out.bin"
    subprocess.check_call([_compile(built, tmp_path, "shim_next"), str(inp), str(out)])
    res = np.fromfile(out, dtype=np.float64)
    n = cc.size
    vd = [dict(anchor=a, depth=d, q=q, dof=3, coeff=c) for c in vcs]
    con = dict(anchor=a, depth=d, q=q, dof=1, coeff=cc)

    def close(x, ref):
        assert np.abs(x - ref.ravel()).max() <= 1e-12 * np.abs(ref).max()
    close(res[:n], ora.semilag_in_situ_tv(vd, con, 2, dt, times=[0.0, dt, 2 * dt, 3 * dt]))
    close(res[n:2 * n], ora.semilag_in_situ_tv([vd[1], vd[0]], con, 2, dt))
    b2 = ora.semilag_bdf2(vd[0], dict(anchor=a, depth=d, q=q, dof=1, coeff=cp), con,
                          dict(anchor=a, depth=d, q=q), 2 * dt, dt)
    close(res[2 * n:3 * n], b2)
    nl = int(res[3 * n])
    ra, rd, rc = rm.remesh(a, d, q, b2, tol, 0, maxd)
    o = 3 * n + 1
    assert nl == len(rd)
    assert np.array_equal(res[o:o + 3 * nl], ra.ravel())
    assert np.array_equal(res[o + 3 * nl:o + 4 * nl], rd.astype(np.float64))
    close(res[o + 4 * nl:], rc)


@pytest.mark.gpu
def test_shim_program_matches_oracle(built, ora, tmp_path):
    q, dt, steps = 6, 0.02, 2
    anchor, depth = trees.uniform_tree(2)
    vc = trees.fit(fields.taylor_green(), anchor, depth, q, 3)
    cc = trees.fit(fields.gaussian((0.4, 0.55, 0.5), 0.1), anchor, depth, q, 1)
    rng = np.random.default_rng(0)
    pts = rng.uniform(0, 1, size=(777, 3))
    inp = tmp_path / "in.bin"
    hdr = np.array([len(depth), q, len(pts), dt, 0, steps], dtype=np.float64)
    with open(inp, "wb") as f:
        for a in (hdr, anchor, depth.astype(np.float64), vc, cc, pts):
            f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    out = tmp_path / "out.bin"
    subprocess.check_call([_compile(built, tmp_path), str(inp), str(out)])
    res = np.fromfile(out, dtype=np.float64)
    n = len(pts)
    v, xdep, coeff = res[:3 * n], res[3 * n:6 * n], res[6 * n:]
    assert np.array_equal(v, ora.eval_tree(anchor, depth, q, 3, vc, pts).ravel())
    assert np.array_equal(xdep, ora.traj_rk2(anchor, depth, q, vc, pts, 0.0, -dt, 1).ravel())
    con = dict(anchor=anchor, depth=depth, q=q, dof=1, coeff=cc)
    vel = dict(anchor=anchor, depth=depth, q=q, dof=3, coeff=vc)
    for s in range(1, steps + 1):
        con["coeff"] = ora.semilag_in_situ(vel, con, s, dt)
    ref = con["coeff"].ravel()
    assert np.abs(coeff - ref).max() <= 1e-12 * np.abs(ref).max()

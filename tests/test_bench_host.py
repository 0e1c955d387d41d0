"""Host-side logic of bench.py: FLOP/byte accounting and the multi-rank
aggregation (gloo, world size 2, on CPU: sum of points, max of times)."""
import os
import socket

import pytest

import bench


def test_flop_accounting_matches_reference_model():
    total, kernel = bench.flops_per_point_tree(14)
    # 2 velocity evaluations (dof 3) + 1 concentration evaluation + RK2 + refit
    assert kernel == 2 * (9 * 15 + 2 * 680 * 3) + 18 + (9 * 15 + 2 * 680)
    assert total == kernel + 2 * 680
    total8, _ = bench.flops_per_point_tree(8)
    assert total8 == 27 * 9 + 16 * 165 + 18


def test_fused_kernel_flop_accounting():
    """The fused step kernel's own work: one velocity evaluation after the
    node-grid first stage, one concentration evaluation and the RK2 updates."""
    d, nc = 15, 680
    assert bench.fused_flops_per_point_tree(14) == (9 * d + 2 * nc * 3) + 18 + (9 * d + 2 * nc)
    assert bench.fused_flops_per_point_tree(8, nrk=2) == 3 * (81 + 990) + 36 + (81 + 330)


def test_reference_arm_workload_loads_no_library_code():
    """The reference arm builds its inputs with the oracle's nodes and
    pseudo-inverse: the process never maps the library under test, and the
    trees are the same as the library-built workload's."""
    import subprocess
    import sys
    code = ("import bench, json; wl = bench.oracle_workload('tree_uniform_q8'); "
            "maps = open('/proc/self/maps').read(); "
            "print(json.dumps([wl.describe(), 'libtbslas_gb300' in maps]))")
    out = subprocess.run([sys.executable, "-c", code], cwd=os.path.dirname(bench.__file__),
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    import json
    desc, mapped = json.loads(out.stdout.strip().splitlines()[-1])
    assert mapped is False
    from tbslas_gb300 import workloads
    assert desc == json.loads(json.dumps(workloads.make("tree_uniform_q8").describe()))


def test_bubble_directions_vanish_on_leaf_faces(ora):
    """The velocity FD directions of the adjoint check vanish on every leaf
    face (evaluated through the oracle at points on the faces)."""
    import numpy as np
    from tbslas_gb300 import trees
    wl = type("W", (), {})()
    wl.q = 8
    wl.a, wl.d = trees.uniform_tree(2)
    dirs = bench.bubble_directions(wl, np.random.default_rng(0), 2)
    rng = np.random.default_rng(1)
    pts = rng.uniform(0, 1, size=(3000, 3))
    face = np.round(pts * 4) / 4  # snap one coordinate per point to a face of the 4^3 grid
    axis = rng.integers(0, 3, size=len(pts))
    pts[np.arange(len(pts)), axis] = face[np.arange(len(pts)), axis]
    inner = rng.uniform(0.05, 0.95, size=(3000, 3)) / 4 + np.floor(rng.uniform(0, 4, (3000, 3))) / 4
    for dv in dirs:
        on = ora.eval_tree(wl.a, wl.d, wl.q, 3, dv, pts)
        off = ora.eval_tree(wl.a, wl.d, wl.q, 3, dv, inner)
        assert np.abs(on).max() <= 1e-12 * np.abs(off).max()
        assert np.abs(off).max() > 0.1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pts, sec = bench.aggregate(1000 * (rank + 1), 0.5 + rank, world)
    q.put((rank, pts, sec))
    dist.barrier()
    dist.destroy_process_group()


def test_aggregate_two_ranks_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    ps = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, pts, sec in res:
        assert pts == 3000 and sec == 1.5


def _tiny_tree_workload():
    from tbslas_gb300 import fields, trees, workloads
    a, d = trees.uniform_tree(1)
    q = 3
    vc = trees.fit(fields.rotation(1.0), a, d, q, 3)
    cc = trees.fit(fields.gaussian((0.5, 0.5, 0.5), 0.2), a, d, q, 1)
    return workloads.TreeWorkload("tiny", (a, d, vc), (a, d, cc), q, 0.01, 0, "tiny")


class _Args:
    steps, warmup = 1, 0


def test_reference_arm_tree_and_adapters(capsys):
    """--impl reference on a tree workload prints the contract line; the
    batch and adjoint adapters hand cpu_baseline_tree the fields it reads."""
    import json
    wl = _tiny_tree_workload()
    bench.run_reference(_Args(), wl)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"
    batch = type("B", (), {})()
    batch.bc = 1
    batch.problems = [dict(va=wl.va, vd=wl.vd, vc=wl.vc, ca=wl.ca, cd=wl.cd, cc=wl.cc, q=wl.q,
                           dt=wl.dt)]
    t = bench._pick(batch, 3)
    assert t.q == wl.q and t.bc == 1 and t.cc is wl.cc
    assert bench._pick(wl, 0) is wl


def _tiny_next_row_workloads():
    """Tiny stand-ins of the re-meshing, BDF2, time-dependent velocity and
    construction workloads (q = 3, depth-1/2 trees)."""
    import numpy as np
    from tbslas_gb300 import fields, trees, workloads
    rm = _tiny_tree_workload()
    rm.name = "tiny_remesh"
    rm.remesh = (1e-3, 1, 2)
    bdf2 = workloads.Bdf2Workload(q=3, depth=1, name="tiny_bdf2")
    tv = workloads.TvWorkload(q=3, depth=1, name="tiny_tv")
    con = _tiny_tree_workload()
    con.name = "tiny_construct"
    con.blobs = fields.gaussian_blobs(np.random.default_rng(2), 2)
    con.construct = (1e-3, 1, 2)
    return [rm, bdf2, tv, con]


@pytest.mark.parametrize("i", range(4))
def test_reference_arm_next_rows(capsys, i):
    """--impl reference on the re-meshing, BDF2, time-dependent velocity and
    construction workloads: the oracle's own loop, one contract line each."""
    import json
    wl = _tiny_next_row_workloads()[i]
    bench.run_reference(_Args(), wl)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["config"]["workload"] == wl.name
    if hasattr(wl, "construct"):
        assert "construction" in line["unit"]


def test_clock_sampler_summary_parses_nvidia_smi_rows(tmp_path):
    """The clocks block of every bench line: median SM clock under load, the
    maximum, and the throttle reasons seen Active in any sample."""
    s = bench.ClockSampler(0)
    s.path = str(tmp_path / "clocks.csv")
    with open(s.path, "w") as f:
        f.write("0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active\n")
        f.write("0, 1995, 2070, 1390.5, 0x4, Not Active, Not Active, Not Active, Active\n")
        f.write("0, 2070, 2070, 1200.0, 0x0, Not Active, Not Active, Not Active, Not Active\n")
        f.write("[N/A]\n")
    out = s.summary()
    assert out == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"],
                   "samples": 3}
    empty = bench.ClockSampler(0)
    assert empty.summary()["reasons"] == ["unavailable"]

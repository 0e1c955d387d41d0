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

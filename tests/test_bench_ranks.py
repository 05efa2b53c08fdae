"""The replica aggregation of bench.py (N > 1 ranks, one GPU each, no data
exchange) on CPU: two gloo ranks report different elapsed times; both take
the slower one and count the nodes of both ranks."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms_total = 10.0 * (rank + 1)  # rank 1 is the slow one
        ms_step, value = bench.replica_rate(ms_total, 1000, 5, dist)
        e2e = bench.max_over_ranks(0.5 + rank, dist)
        out.put((rank, ms_step, value, e2e))
    finally:
        dist.destroy_process_group()


def test_replica_rate_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms_step, value, e2e in res:
        assert ms_step == pytest.approx(20.0 / 5)
        assert value == pytest.approx(2 * 1000 / (4.0e-3))
        assert e2e == pytest.approx(1.5)


def test_replica_rate_one_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_rate(12.0, 300, 4) == (3.0, pytest.approx(300 / 3e-3))

"""The multi-rank (torchrun) path of bench.py on CPU with gloo, world size 2: every rank must
see the slowest rank's time, and the whole-job rate counts all ranks' replicas."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys

    sys.path.insert(0, REPO)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = 1.0 + rank  # rank 1 is the slow one
        tmax = bench.max_over_ranks(t, dist, "cpu")
        rate = bench.whole_job_rate(100.0, world, tmax)
        q.put((rank, tmax, rate))
    finally:
        dist.destroy_process_group()


def test_two_ranks_use_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, tmax, rate in got:
        assert tmax == 2.0
        assert rate == pytest.approx(100.0 * 2 / 2.0)


def test_single_process_needs_no_group():
    import sys

    sys.path.insert(0, REPO)
    import bench

    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.whole_job_rate(10.0, 1, 2.0) == 5.0

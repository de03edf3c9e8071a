"""Multi-rank bench logic on CPU: two gloo ranks (replicas, no data exchange) reduce their timings
and particle counts the way bench.py does under torchrun."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        ms = [40.0, 55.0][rank]            # per-rank device time of K steps
        n = [1000, 3000][rank]             # per-rank particles (replicas of different sizes)
        mx = bench.over_ranks(dist, ms)
        tot = bench.over_ranks(dist, n, "sum")
        q.put((rank, mx, tot, bench.whole_job_rate(tot, 10, mx)))
    finally:
        dist.destroy_process_group()


def test_two_rank_reduction():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, tot, rate in out:
        assert mx == 55.0 and tot == 4000.0
        assert rate == pytest.approx(4000 * 10 / 0.055)


def test_single_process_is_identity():
    import bench
    assert bench.over_ranks(None, 3.5) == 3.5
    assert bench.whole_job_rate(100, 2, 1000.0) == 200.0

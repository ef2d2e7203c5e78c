"""bench.py's multi-rank path on CPU: two gloo ranks (one per GPU in a real run) aggregate
the whole job as the slowest rank's time and the sum of all ranks' events, and the
reference arm's other ranks exit without work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out = bench.aggregate_over_ranks(dist, secs=1.0 + rank, e2e_secs=2.0 - rank, events=100.0 * (rank + 1),
                                         e2e_events=10.0)
        q.put((rank, out))
    finally:
        dist.destroy_process_group()


def test_two_ranks_aggregate_whole_job():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        secs, e2e_secs, events, e2e_events = got[r]
        assert secs == 2.0 and e2e_secs == 2.0  # the slowest rank's time
        assert events == 300.0 and e2e_events == 20.0  # all ranks' work
    del torch


def test_single_rank_aggregate_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.aggregate_over_ranks(None, 1.5, 2.5, 7.0, 3.0) == (1.5, 2.5, 7.0, 3.0)


def test_reference_arm_other_ranks_exit_without_work(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    # rank 1 returns before importing the library or building anything
    assert bench.run_reference_arm(None) == 0

"""The benchmark's multi-rank host logic on two CPU processes (gloo): every
rank reports the slowest rank's time, and each rank steps its own replica."""

import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    sys.path.insert(0, REPO)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.0 + rank * 0.25, device="cpu")
        out.put((rank, t, bench.replica_seed(rank)))
    finally:
        dist.destroy_process_group()


def test_two_ranks_agree_on_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in procs)
    assert [g[1] for g in got] == [1.25, 1.25]
    assert got[0][2] != got[1][2]  # every rank its own replica


def test_one_process_needs_no_group():
    sys.path.insert(0, REPO)
    import bench

    assert bench.max_over_ranks(2.5, device="cpu") == 2.5
    assert bench.replica_seed(0) == 3

"""The benchmark's host logic, on the CPU.

On two gloo processes, every rank reports the slowest rank's time and the sum
of the ranks' bodies.  The ranks step disjoint shares of one global batch,
dealt out by body count.  The CPU baseline steps a constrained scene with its
joints and exclusions.
"""

import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PER_RANK = 48


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
        sc = bench.rank_scene(rank, world, per_rank=PER_RANK)
        total = bench.sum_over_ranks(sc.nbodies, device="cpu")
        out.put((rank, t, sc.nworlds, sc.nbodies, total, sc.gravity.tolist()))
    finally:
        dist.destroy_process_group()


def test_two_ranks_agree_on_time_and_bodies_and_share_one_batch():
    from resolve2d_gb300 import scenes

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
    assert [g[1] for g in got] == [1.25, 1.25]  # the slowest rank's time, everywhere
    full = scenes.config3(nworlds=2 * PER_RANK)
    assert got[0][4] == got[1][4] == full.nbodies  # the bodies of all ranks together
    assert got[0][2] + got[1][2] == full.nworlds
    assert abs(got[0][3] - got[1][3]) <= int(np.diff(full.body_off).max())  # balanced to one world
    # the two shares are disjoint: every world's gravity (a per-world draw) appears once
    g = sorted(got[0][5] + got[1][5])
    np.testing.assert_array_equal(g, np.sort(full.gravity))


def test_one_process_needs_no_group():
    sys.path.insert(0, REPO)
    import bench
    from resolve2d_gb300 import scenes

    assert bench.max_over_ranks(2.5, device="cpu") == 2.5
    assert bench.sum_over_ranks(7.0, device="cpu") == 7.0
    one = bench.rank_scene(0, 1, per_rank=PER_RANK)
    ref = scenes.config3(nworlds=PER_RANK)
    np.testing.assert_array_equal(one.opt, ref.opt)  # one process steps the headline batch itself


def test_the_cpu_baseline_steps_a_scene_with_its_joints():
    """A scene with joints and exclusions is settled (in the GPU's colour-major
    order, which the GPU reproduces bit for bit) and timed through a whole
    oracle solver, never by the body-only batch runner."""
    sys.path.insert(0, REPO)
    import bench
    from oracle import ORDER_COLOUR, Oracle
    from resolve2d_gb300 import scenes

    sc = scenes.config2(n_bodies=1200, n_chains=20, chain_links=10, n_motors=10, box_w=120.0, box_h=40.0)
    assert sc.jtype.size and sc.xpairs.size and bench._with_constraints(sc)
    got = bench.settle_scene(sc, 3)
    o = Oracle.from_scene(sc)
    for _ in range(3):
        assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
    np.testing.assert_array_equal(got, o.state())
    assert bench.oracle_time(sc, got, 1, 4) > 0.0


def test_bench_gpus_n_starts_n_ranks_itself():
    """`bench.py --gpus 2` without a launcher starts itself under
    torch.distributed.run with two local ranks; with --dry-run the ranks run
    the rank logic over gloo and rank 0 alone prints the totals."""
    import json
    import subprocess

    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--gpus", "2", "--dry-run",
                        "--dry-run-worlds", str(PER_RANK)], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    from resolve2d_gb300 import scenes

    full = scenes.config3(nworlds=2 * PER_RANK)
    assert lines[0]["n_gpus"] == 2 and lines[0]["worlds"] == full.nworlds and lines[0]["bodies"] == full.nbodies
    assert lines[0]["slowest_rank_time"] == 1.5


def test_bench_refuses_a_rank_count_other_than_gpus():
    import subprocess

    env = dict(os.environ, WORLD_SIZE="3", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--gpus", "2", "--dry-run"], env=env,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "--gpus 2" in (r.stdout + r.stderr)


def test_both_arms_print_one_config():
    sys.path.insert(0, REPO)
    import bench

    a = bench.headline_config(589_055, 4096, 1, 589_055)
    b = bench.headline_config(589_055, 4096, 1, 589_055)
    assert a == b and {"workload", "bodies", "worlds", "l2", "parallelism"} <= set(a)

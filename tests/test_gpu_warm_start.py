"""Warm starting (R2D_FLAG_WARM_START, an extension off in reference mode)
against the oracle's warm-start mode: bit-identical state, manifolds (with
their warm-started accumulators) and colourings, on both device paths, across
capacity replays (which re-lay out the warm tables) and across a world's move
from the fused kernel to the grid pipeline."""

import numpy as np
import pytest

from oracle import ORDER_COLOUR, Oracle
from parity import assert_manifolds_equal, assert_state_equal, run_pair
from resolve2d_gb300 import scenes
from resolve2d_gb300.engine import Batch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("grid", [False, True])
def test_config0_warm(grid):
    sc = scenes.config0()
    w, _ = run_pair(sc, steps=120, check_every=20, warm=True, grid=grid)
    # the mode is live: reference mode ends elsewhere
    ref = Oracle.from_scene(sc)
    for _ in range(120):
        assert ref.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
    assert not np.array_equal(w.read_state(), ref.state())


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("grid", [False, True])
def test_random_scenes_with_joints_warm(seed, grid):
    sc = scenes.random_scene(seed, n=40, joints=True)
    run_pair(sc, steps=40, check_every=5, warm=True, grid=grid)


def test_substeps_warm():
    sc = scenes.random_scene(11, n=30, joints=True)
    run_pair(sc, steps=20, check_every=4, sub_steps=4, iters=4, warm=True)


def test_batch_warm_with_capacity_replays():
    # 5 % buffers: every world overflows, is frozen and replayed with larger
    # capacities, which re-lays out the warm tables mid-run
    sc = scenes.batched_worlds("warm-tight", seed=8, nworlds=8, steps=16)
    b = Batch.from_scene(sc, capacity_scale=0.05, warm_start=True, debug=True)
    oracles = []
    for w in range(sc.nworlds):
        o = Oracle.from_scene(sc.world(w))
        o.set_warm_start(True)
        oracles.append(o)
    for s in range(sc.steps):
        b.process(sc.dt, 1, sc.iters)
        if s % 4 == 3:
            b.sync()
        for o in oracles:
            assert o.process(sc.dt, 1, sc.iters, ORDER_COLOUR) == 0
    b.sync()
    st = b.read_state()
    for w, o in enumerate(oracles):
        assert_state_equal(st[:, sc.body_off[w]:sc.body_off[w + 1]], o.state(), f"world {w}")
        gk, gd, gc = b.manifolds(w)
        ok, od = o.manifolds()
        oc, _ = o.colours()
        assert_manifolds_equal(gk, gd, gc, ok, od, oc)


def test_pile_moves_to_grid_pipeline_warm():
    # the world outgrows the fused kernel's shared memory on its first call
    # and continues on the grid pipeline, taking its warm table along
    b = scenes._Builder()
    b.rect(0.0, -0.5, 40.0, 1.0, 0.5, static=True)
    rng = np.random.default_rng(0)
    for pile in (-8.0, 8.0):
        for _ in range(60):
            b.disc(pile + rng.uniform(-0.05, 0.05), 3.0 + rng.uniform(-0.05, 0.05), 1.0, 0.5)
    ids, kind, opt = b.arrays()
    sc = scenes._concat("pile", [(ids, kind, opt)], [9.81], 1 / 60, 1, 8, 6)
    run_pair(sc, steps=6, check_every=1, warm=True)

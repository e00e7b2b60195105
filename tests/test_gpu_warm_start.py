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


# ---- compensated accumulation (R2D_FLAG_COMPENSATED, r2d_accum.h) ----

@pytest.mark.parametrize("warm", [False, True])
@pytest.mark.parametrize("grid", [False, True])
def test_config0_compensated(grid, warm):
    sc = scenes.config0()
    w, _ = run_pair(sc, steps=120, check_every=30, warm=warm, comp=True, grid=grid)
    # the mode is live: without compensation the run ends elsewhere
    ref = Oracle.from_scene(sc)
    ref.set_warm_start(warm)
    for _ in range(120):
        assert ref.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
    assert not np.array_equal(w.read_state(), ref.state())


@pytest.mark.parametrize("grid", [False, True])
def test_random_scenes_with_joints_compensated_warm(grid):
    for seed in (3, 4):
        sc = scenes.random_scene(seed, n=40, joints=True)
        run_pair(sc, steps=30, check_every=10, warm=True, comp=True, grid=grid)


def test_substeps_compensated_warm():
    sc = scenes.random_scene(11, n=30, joints=True)
    run_pair(sc, steps=20, check_every=5, sub_steps=4, iters=4, warm=True, comp=True)


def test_batch_compensated_warm_with_capacity_replays():
    sc = scenes.batched_worlds("comp-tight", seed=8, nworlds=8, steps=16)
    b = Batch.from_scene(sc, capacity_scale=0.05, warm_start=True, compensated=True)
    oracles = []
    for w in range(sc.nworlds):
        o = Oracle.from_scene(sc.world(w))
        o.set_warm_start(True)
        o.set_compensated(True)
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


def test_pile_moves_to_grid_pipeline_compensated_warm():
    b = scenes._Builder()
    b.rect(0.0, -0.5, 40.0, 1.0, 0.5, static=True)
    rng = np.random.default_rng(0)
    for pile in (-8.0, 8.0):
        for _ in range(60):
            b.disc(pile + rng.uniform(-0.05, 0.05), 3.0 + rng.uniform(-0.05, 0.05), 1.0, 0.5)
    ids, kind, opt = b.arrays()
    sc = scenes._concat("pile", [(ids, kind, opt)], [9.81], 1 / 60, 1, 8, 6)
    run_pair(sc, steps=6, check_every=1, warm=True, comp=True)


# ---- warm-start tables keyed by body ids, kept across body uploads ----

def _swap_remove_and_add(ids, kind, props, state, slot, new):
    """The store after swapRemove of `slot` (the last body takes its place,
    as AutoArrayHashMap.swapRemove, src/core/lib.zig:167-179) and one new body
    `new` = (id, kind, props[5], state[13]) appended."""
    ids, kind, props, state = ids.copy(), kind.copy(), props.copy(), state.copy()
    last = len(ids) - 1
    for a in (ids, kind):
        a[slot] = a[last]
    props[:, slot] = props[:, last]
    state[:, slot] = state[:, last]
    nid, nk, nprops, nstate = new
    ids = np.append(ids[:last], np.uint32(nid))
    kind = np.append(kind[:last], np.uint8(nk))
    props = np.concatenate([props[:, :last], np.asarray(nprops, np.float32).reshape(-1, 1)], axis=1)
    state = np.concatenate([state[:, :last], np.asarray(nstate, np.float32).reshape(-1, 1)], axis=1)
    return ids, kind, np.ascontiguousarray(props), np.ascontiguousarray(state)


@pytest.mark.parametrize("comp", [False, True])
@pytest.mark.parametrize("grid", [False, True])
def test_warm_impulses_survive_a_body_upload(grid, comp):
    from resolve2d_gb300.engine import World
    from resolve2d_gb300.scenes import derive_props_state

    sc = scenes.config0()
    w = World.from_scene(sc, warm_start=True, compensated=comp, grid=grid, debug=True)
    o = Oracle.from_scene(sc)
    o.set_warm_start(True)
    o.set_compensated(comp)
    for _ in range(90):  # the pile has landed: warm impulses everywhere
        w.process(sc.dt, 1, sc.iters)
        assert o.process(sc.dt, 1, sc.iters, ORDER_COLOUR) == 0
    w.sync()
    st = w.read_state()
    assert_state_equal(st, o.state(), "before the upload")
    props, _ = derive_props_state(sc.kind, sc.opt)
    # a new disc far from the pile (its first AABB as the engine computes it)
    probe = World.from_scene(sc)
    nprops = props[:, 1].copy()
    nstate = probe.read_state()[:, 1].copy()
    nstate[0] += 100.0
    nstate[9] += 100.0
    ids2, kind2, props2, st2 = _swap_remove_and_add(np.asarray(sc.ids, np.uint32), np.asarray(sc.kind & 3, np.uint8),
                                                    props, st, slot=57, new=(10_000, sc.kind[1] & 3, nprops, nstate))
    w.set_bodies(ids2, kind2, props2, st2, False)
    o2 = Oracle()
    o2.add_bodies_raw(ids2, kind2, props2, st2)
    o2.lib.r2o_add_gravity(o2.h, float(sc.gravity[0]))
    o2.set_warm_start(True)
    o2.set_compensated(comp)
    o2.take_warm(o)
    cold = Oracle()
    cold.add_bodies_raw(ids2, kind2, props2, st2)
    cold.lib.r2o_add_gravity(cold.h, float(sc.gravity[0]))
    cold.set_warm_start(True)
    cold.set_compensated(comp)
    for s in range(30):
        w.process(sc.dt, 1, sc.iters)
        assert o2.process(sc.dt, 1, sc.iters, ORDER_COLOUR) == 0
        assert cold.process(sc.dt, 1, sc.iters, ORDER_COLOUR) == 0
        if s in (0, 29):
            w.sync()
            assert_state_equal(w.read_state(), o2.state(), f"step {s + 1} after the upload")
    # the carried impulses mattered: a solver that lost them is elsewhere
    assert not np.array_equal(w.read_state(), cold.state())

"""GPU step vs the CPU oracle, through the C ABI.

The oracle replays the reference's per-constraint arithmetic in the GPU's
colour-major order (ORDER_COLOUR); the bar is bit-identical state, pair sets,
manifolds and colourings (see parity.py for the signed-zero note).
"""

import numpy as np
import pytest

from oracle import ORDER_COLOUR, Oracle
from parity import assert_manifolds_equal, assert_pairs_equal, assert_state_equal, run_pair
from resolve2d_gb300 import _native as N
from resolve2d_gb300 import scenes
from resolve2d_gb300.engine import Batch, World

pytestmark = pytest.mark.gpu


def test_config0_first_steps_bit_exact():
    run_pair(scenes.config0(), steps=5)


def test_config0_full_run_bit_exact():
    sc = scenes.config0()
    run_pair(sc, steps=sc.steps, check_every=50)


@pytest.mark.parametrize("seed", range(8))
def test_random_scenes_with_joints(seed):
    sc = scenes.random_scene(seed, n=40, joints=True)
    w, o = run_pair(sc, steps=40, check_every=5)
    if w is not None and sc.jtype.size:
        _, oj = o.colours()
        np.testing.assert_array_equal(w.joint_colours(len(sc.jtype)), oj)


@pytest.mark.parametrize("seed", [11, 12])
def test_substeps_and_iterations(seed):
    # the reference demos step with sub_steps = 4, iterations = 4 (demos/native/src/main.zig:16-20)
    sc = scenes.random_scene(seed, n=30, joints=True)
    run_pair(sc, steps=20, check_every=4, sub_steps=4, iters=4)


def test_batch_matches_oracle_per_world():
    sc = scenes.batched_worlds("batch-small", seed=3, nworlds=24, steps=40, lo=16, hi=512)
    b = Batch.from_scene(sc, debug=True)
    oracles = [Oracle.from_scene(sc.world(w)) for w in range(sc.nworlds)]
    for o in oracles:
        o.record_pairs()
    for s in range(sc.steps):
        b.process(sc.dt, sc.sub_steps, sc.iters)
        b.sync()
        for o in oracles:
            assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
    st = b.read_state()
    for w, o in enumerate(oracles):
        b0, b1 = sc.body_off[w], sc.body_off[w + 1]
        assert_state_equal(st[:, b0:b1], o.state(), f"world {w}")
        assert_pairs_equal(b.pairs(w), o.pairs(), f"world {w}")
        gk, gd, gc = b.manifolds(w)
        ok, od = o.manifolds()
        oc, _ = o.colours()
        assert_manifolds_equal(gk, gd, gc, ok, od, oc)


def test_batch_equals_single_world_path():
    sc = scenes.batched_worlds("batch-eq", seed=5, nworlds=6, steps=10)
    b = Batch.from_scene(sc)
    ws = [World.from_scene(sc.world(w)) for w in range(sc.nworlds)]
    for _ in range(sc.steps):
        b.process(sc.dt, 1, sc.iters)
        for w in ws:
            w.process(sc.dt, 1, sc.iters)
    b.sync()
    st = b.read_state()
    for k, w in enumerate(ws):
        w.sync()
        np.testing.assert_array_equal(st[:, sc.body_off[k]:sc.body_off[k + 1]], w.read_state())


def test_capacity_overflow_replays_bit_exact():
    # buffers at 5% of their normal size: every world overflows, is frozen on
    # the device, and is replayed with doubled capacities at sync
    sc = scenes.batched_worlds("tight", seed=8, nworlds=8, steps=12)
    b = Batch.from_scene(sc, capacity_scale=0.05)
    oracles = [Oracle.from_scene(sc.world(w)) for w in range(sc.nworlds)]
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


def test_determinism_run_twice():
    sc = scenes.batched_worlds("det", seed=9, nworlds=32, steps=30)
    out = []
    for _ in range(2):
        b = Batch.from_scene(sc)
        for _ in range(sc.steps):
            b.process(sc.dt, 1, sc.iters)
        b.sync()
        out.append(b.read_state())
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32))


def test_external_forces_and_torques():
    sc = scenes.random_scene(21, n=25, joints=True)
    w = World.from_scene(sc, debug=True)
    o = Oracle.from_scene(sc)
    st = o.state()
    rng = np.random.default_rng(0)
    st[6] = rng.normal(size=st.shape[1]).astype(np.float32) * 5
    st[7] = rng.normal(size=st.shape[1]).astype(np.float32) * 5
    st[8] = rng.normal(size=st.shape[1]).astype(np.float32)
    o.set_state(st)
    w.write_state(st)
    for s in range(6):
        w.process(sc.dt, 2, 6)
        w.sync()
        assert o.process(sc.dt, 2, 6, ORDER_COLOUR) == 0
        assert_state_equal(w.read_state(), o.state(), f"forces step {s}")


def test_exclusions_and_cell_boundaries():
    # bodies centred on multiples of the 4.0 cell and at negative coordinates,
    # touching pairs excluded by id (EntityFactory.excludeCollisionPair, lib.zig:124-129)
    b = scenes._Builder()
    b.rect(0.0, -0.5, 60.0, 1.0, 0.5, static=True)
    for i in range(-6, 7):
        b.disc(4.0 * i, 0.5, 0.5, 0.5)
        b.rect(4.0 * i + 0.95, 0.5, 1.0, 1.0, 0.5)
        b.disc(4.0 * i - 0.001, 4.0, 0.6, 0.5)
    ids, kind, opt = b.arrays()
    sc = scenes._concat("cells", [(ids, kind, opt)], [9.81], 1 / 60, 1, 8, 30,
                        excl=(np.zeros(3, np.uint32), np.array([[1, 2], [4, 5], [7, 8]], np.uint32)))
    run_pair(sc, steps=30, check_every=3)


def test_empty_single_and_static_worlds():
    for bodies in ([], [("disc", False)], [("rect", True), ("rect", True)]):
        b = scenes._Builder()
        for i, (t, st) in enumerate(bodies):
            if t == "disc":
                b.disc(0.0, 2.0 * i, 0.5, 0.5, static=st)
            else:
                b.rect(0.0, 2.0 * i, 1.0, 1.0, 0.5, static=st)
        if bodies:
            ids, kind, opt = b.arrays()
        else:
            ids, kind, opt = np.zeros(0, np.uint32), np.zeros(0, np.uint8), np.zeros((10, 0), np.float32)
        sc = scenes._concat("tiny", [(ids, kind, opt)], [9.81], 1 / 60, 1, 8, 5)
        if not bodies:
            w = World()
            w.process(sc.dt, 1, 8)
            w.sync()
            continue
        run_pair(sc, steps=5)


def test_world_above_fused_limit_takes_grid_pipeline():
    # 1,500 bodies exceed the largest fused class (520): the world steps
    # through the grid-wide pipeline and still matches the oracle bit for bit
    sc = scenes.batched_worlds("big", seed=1, nworlds=1, steps=6, lo=1500, hi=1500)
    run_pair(sc, steps=6, check_every=2)


def test_unknown_joint_body_id_is_an_error():
    sc = scenes.random_scene(3, n=10)
    w = World.from_scene(sc)
    w.set_joints(np.array([0], np.uint8), np.array([1], np.uint32), np.array([999], np.uint32),
                 np.array([[np.inf, -np.inf, 10, 1, 0, 0, 0, 0]], np.float32))
    before = w.read_state()
    with pytest.raises(N.R2DError) as e:
        w.process(sc.dt, 1, 8)
    assert e.value.code == -2
    np.testing.assert_array_equal(w.read_state(), before)


def test_tgs_live_depth_uses_full_layout():
    # Two discs of radius 3000 whose centres are 10 apart: the lower-id disc is
    # the reference, its contact depth is -5990, and approxEql(depth, depth,
    # 1e-4) fails at that magnitude, so updateTGSDepth rotates the lever arms
    # every substep (collision.zig:73-100).  The lean kernel hands such a world
    # to the full layout; the result must stay bit-identical.  A 1000-unit
    # cell keeps the spatial hash small (Solver.init's cell width argument).
    b = scenes._Builder()
    b.disc(0.0, 0.0, 3000.0, 0.5, vx=0.5)
    b.disc(10.0, 0.0, 3000.0, 0.5, vx=-0.5, omega=0.3)
    b.rect(0.0, 4000.0, 2.0, 1.0, 0.5)
    ids, kind, opt = b.arrays()
    sc = scenes._concat("tgs", [(ids, kind, opt)], [0.0], 1 / 60, 1, 8, 6)
    w = World.from_scene(sc, debug=True, cell=1000.0)
    o = Oracle.from_scene(sc)
    o.set_hash(1000.0, 2)
    for s in range(6):
        w.process(sc.dt, 2, 4)
        w.sync()
        assert o.process(sc.dt, 2, 4, ORDER_COLOUR) == 0
        assert_state_equal(w.read_state(), o.state(), f"tgs step {s}")
        gk, gd, gc = w.manifolds()
        ok, od = o.manifolds()
        oc, _ = o.colours()
        assert_manifolds_equal(gk, gd, gc, ok, od, oc)
    assert abs(od[0, 9 + 6]) > 2048


def _bucket(x, y, table):
    """The reference's bucket of cell (x, y) (SpatialHash.zig:78-81): i64
    wrapping products, xor, as u64, modulo the table size."""
    m = (1 << 64) - 1
    return (((x * 92837111) & m) ^ ((y * 689287499) & m)) % table


@pytest.mark.parametrize("grid", [False, True])
def test_pairs_across_cell_boundaries_with_and_without_bucket_collisions(grid):
    # Disc pairs whose AABBs are 0.005 apart across a 4.0 cell boundary: the
    # AABB test (margin 0.01) and SAT (margin 0.01) accept them, so the
    # reference makes a manifold exactly when the two cells' buckets
    # collide.  Half the pairs sit on rows where they do.  (With an even
    # table, side-by-side cells never collide -- both hash multipliers are
    # odd -- so this world uses table_mult 3 and an odd body count.)
    n_pairs, filler, mult = 10, 5, 3
    n = 2 * n_pairs + filler
    table = mult * n
    r, gap = 0.4, 0.005
    rows_hit, rows_miss = [], []
    for yc in range(-300, 300):
        for k in (1, 2, 3):
            same = _bucket(k - 1, yc, table) == _bucket(k, yc, table)
            (rows_hit if same else rows_miss).append((k, yc))
    picks = rows_hit[:n_pairs // 2] + rows_miss[:n_pairs - n_pairs // 2]
    assert len(picks) == n_pairs
    b = scenes._Builder()
    for k, yc in picks:
        y = 4.0 * yc + 2.0
        b.disc(4.0 * k - r - gap / 2, y, r, 0.5)
        b.disc(4.0 * k + r + gap / 2, y, r, 0.5)
    for f in range(filler):
        b.disc(5000.0 + 10.0 * f, 5000.0, r, 0.5)
    ids, kind, opt = b.arrays()
    assert len(ids) == n
    sc = scenes._concat("boundary", [(ids, kind, opt)], [0.0], 1 / 60, 1, 8, 2)
    w = World.from_scene(sc, debug=True, mult=mult, grid=grid)
    o = Oracle.from_scene(sc)
    o.set_hash(4.0, mult)
    o.record_pairs()
    for s in range(2):
        assert o.process(sc.dt, 1, 8, ORDER_COLOUR) == 0
        w.process(sc.dt, 1, 8)
        w.sync()
        assert_state_equal(w.read_state(), o.state(), f"boundary step {s + 1}")
        assert_pairs_equal(w.pairs(), o.pairs(), f"boundary step {s + 1}")
        gk, gd, gc = w.manifolds()
        ok, od = o.manifolds()
        oc, _ = o.colours()
        assert_manifolds_equal(gk, gd, gc, ok, od, oc)
    assert len(ok) == n_pairs // 2  # only the colliding rows pair up
    assert len(o.pairs()) == n_pairs // 2  # the other rows share no bucket: not even candidates


@pytest.mark.parametrize("grid", [False, True])
def test_candidate_pairs_include_aabb_overlaps_that_sat_rejects(grid):
    # Discs of radius 0.5 on a checkerboard of 0.8 spacing: every
    # diagonal neighbour's AABB overlaps (|dx| = 0.8 < 1.01) while the discs
    # are 1.13 apart, so SAT rejects them.  Those pairs reach the narrowphase
    # (lib.zig:282-284) without making a manifold; the tap must list them.
    # Two discs excluded from colliding and two static boxes that overlap
    # each other must not appear.
    b = scenes._Builder()
    for i in range(8):
        for j in range(8):
            if (i + j) % 2 == 0:  # a checkerboard: only diagonal neighbours' AABBs overlap
                b.disc(0.8 * i, 0.8 * j + 1.0, 0.5, 0.5)
    b.rect(2.0, -0.5, 20.0, 1.0, 0.5, static=True)
    b.rect(2.5, -0.5, 20.0, 1.0, 0.5, static=True)
    ids, kind, opt = b.arrays()
    sc = scenes._concat("diagonal", [(ids, kind, opt)], [0.0], 1 / 60, 1, 8, 1,
                        excl=(np.zeros(1, np.uint32), np.array([[ids[0], ids[4]]], np.uint32)))
    w, o = run_pair(sc, steps=1, grid=grid)
    pairs = set(map(tuple, w.pairs().tolist()))
    keys = {tuple(sorted(k)) for k in w.manifolds()[0].tolist()}
    assert keys < pairs and len(pairs - keys) >= 40
    assert (0, 4) not in pairs  # diagonal neighbours, excluded
    nb = len(ids)
    assert (nb - 2, nb - 1) not in pairs


@pytest.mark.parametrize("grid", [False, True])
def test_fp64_positions_integrate_in_double(grid):
    # Bodies in free flight (far apart, no contacts), under gravity, with
    # spin: momenta evolve in f32 exactly as in the f32 step; the pose is
    # integrated in double, x += p * (h / m), angle += L * h / I
    # (R2D_FLAG_FP64_POSITIONS).  Restated here in numpy float64.
    b = scenes._Builder()
    for k in range(6):
        b.disc(50.0 * k, 10.0 + k, 0.3 + 0.05 * k, 0.5, vx=0.37 * k, vy=1.3, omega=0.7 * k)
        b.rect(50.0 * k + 20.0, -5.0, 0.5 + 0.1 * k, 0.4, 0.5, vx=-0.21, omega=-1.1 + 0.3 * k)
    ids, kind, opt = b.arrays()
    g, dt, steps = 9.81, 1 / 60, 40
    sc = scenes._concat("flight", [(ids, kind, opt)], [g], dt, 1, 8, steps)
    w = World.from_scene(sc, fp64_positions=True, grid=grid)
    st0 = w.read_state()
    pose0 = w.read_positions_f64()
    np.testing.assert_array_equal(pose0, st0[:3].astype(np.float64))
    props, _ = scenes.derive_props_state(sc.kind, sc.opt)
    m, inertia = props[0].astype(np.float32), props[1].astype(np.float32)
    f32 = np.float32
    h = f32(f32(dt) / f32(1))
    my = st0[4].copy()
    mx, L = st0[3].copy(), st0[5].copy()
    x, y, a = pose0[0].copy(), pose0[1].copy(), pose0[2].copy()
    for _ in range(steps):
        fy = f32(0.0) + (f32(-g) * m)  # DownwardsGravity.apply on a zero force
        my = (my + fy * h).astype(np.float32)
        sm = np.float64(h) / m.astype(np.float64)
        x = x + mx.astype(np.float64) * sm
        y = y + my.astype(np.float64) * sm
        a = a + L.astype(np.float64) * np.float64(h) / inertia.astype(np.float64)
        w.process(dt, 1, 8)
    w.sync()
    pose = w.read_positions_f64()
    np.testing.assert_array_equal(pose, np.stack([x, y, a]))
    st = w.read_state()
    np.testing.assert_array_equal(st[:3], pose.astype(np.float32))
    np.testing.assert_array_equal(st[4], my)


def test_state_field_ranges_read_and_write():
    sc = scenes.random_scene(5, n=30)
    w = World.from_scene(sc)
    o = Oracle.from_scene(sc)
    full = w.read_state()
    np.testing.assert_array_equal(w.read_fields(0, 13), full)
    np.testing.assert_array_equal(w.read_fields(9, 4), full[9:13])
    # push the bodies: forces and torques in through the field-range entry point
    rng = np.random.default_rng(1)
    forces = (rng.normal(size=(3, full.shape[1])) * 4).astype(np.float32)
    w.write_fields(6, forces)
    st = o.state()
    st[6:9] = forces
    o.set_state(st)
    for _ in range(3):
        w.process(sc.dt, 1, sc.iters)
        w.sync()
        assert o.process(sc.dt, 1, sc.iters, ORDER_COLOUR) == 0
    assert_state_equal(w.read_fields(0, 13), o.state(), "after forces")
    with pytest.raises(N.R2DError):
        w.read_fields(10, 4)


def test_autotune_restores_state_and_keeps_results():
    # the autotuner times trial steps with other thread counts and restores
    # the state; the steps after it must still match the oracle bit for bit
    sc = scenes.batched_worlds("tune", seed=12, nworlds=40, steps=6, lo=16, hi=512)
    b = Batch.from_scene(sc)
    oracles = [Oracle.from_scene(sc.world(w)) for w in range(sc.nworlds)]

    def step(k):
        for _ in range(k):
            b.process(sc.dt, sc.sub_steps, sc.iters)
            for o in oracles:
                assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
        b.sync()

    step(2)
    before = b.read_state()
    b.autotune(sc.dt, sc.sub_steps, sc.iters, trial_steps=2)
    np.testing.assert_array_equal(b.read_state().view(np.uint32), before.view(np.uint32))
    step(4)
    st = b.read_state()
    for w, o in enumerate(oracles):
        assert_state_equal(st[:, sc.body_off[w]:sc.body_off[w + 1]], o.state(), f"world {w}")


def test_launch_paths_agree():
    # graph replay (the default), kernel-by-kernel launches (R2D_NO_GRAPH=1,
    # read when a batch is created) and the launch priorities left at the
    # default level (R2D_CLASS_PRIORITIES="") step a batch of every size
    # class to the same bits
    import os

    sc = scenes.batched_worlds("paths", seed=14, nworlds=48, steps=5, lo=16, hi=512)
    states = []
    for env in ({}, {"R2D_NO_GRAPH": "1"}, {"R2D_CLASS_PRIORITIES": ""}):
        old = {k: os.environ.get(k) for k in env}
        os.environ.update(env)
        try:
            b = Batch.from_scene(sc)
        finally:
            for k, v in old.items():
                if v is None:
                    del os.environ[k]
                else:
                    os.environ[k] = v
        for _ in range(sc.steps):
            b.process(sc.dt, sc.sub_steps, sc.iters)
        b.sync()
        states.append(b.read_state())
        b.close()
    for s in states[1:]:
        np.testing.assert_array_equal(s.view(np.uint32), states[0].view(np.uint32))

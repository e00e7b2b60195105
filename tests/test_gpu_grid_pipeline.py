"""The grid-wide pipeline against the oracle, through the C ABI.

Worlds above 520 bodies, worlds whose buffers do not fit one CTA's shared
memory, and every world under R2D_FLAG_GRID_PIPELINE step through the grid
pipeline over global scratch (r2d_large.cu): cluster-wide colouring, then
every substep in one resident cluster or one kernel per phase and colour.  It shares the
fused kernel's per-item device functions and its colouring, so the bar is the
same: bit-identical state, pair sets, manifolds and colourings.
"""

import numpy as np
import pytest

from oracle import ORDER_COLOUR, Oracle
from parity import assert_manifolds_equal, assert_state_equal, run_pair
from resolve2d_gb300 import _native as N
from resolve2d_gb300 import scenes
from resolve2d_gb300.engine import Batch, World

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", range(8))
def test_random_scenes_with_joints(seed):
    sc = scenes.random_scene(seed, n=40, joints=True)
    w, o = run_pair(sc, steps=40, check_every=5, grid=True)
    if w is not None and sc.jtype.size:
        _, oj = o.colours()
        np.testing.assert_array_equal(w.joint_colours(len(sc.jtype)), oj)


@pytest.mark.parametrize("seed", [11, 12])
def test_substeps_and_iterations(seed):
    sc = scenes.random_scene(seed, n=30, joints=True)
    run_pair(sc, steps=20, check_every=4, sub_steps=4, iters=4, grid=True)


def test_config0_first_steps():
    run_pair(scenes.config0(), steps=10, check_every=5, grid=True)


def test_exclusions_and_cell_boundaries():
    b = scenes._Builder()
    b.rect(0.0, -0.5, 60.0, 1.0, 0.5, static=True)
    for i in range(-6, 7):
        b.disc(4.0 * i, 0.5, 0.5, 0.5)
        b.rect(4.0 * i + 0.95, 0.5, 1.0, 1.0, 0.5)
        b.disc(4.0 * i - 0.001, 4.0, 0.6, 0.5)
    ids, kind, opt = b.arrays()
    sc = scenes._concat("cells", [(ids, kind, opt)], [9.81], 1 / 60, 1, 8, 30,
                        excl=(np.zeros(3, np.uint32), np.array([[1, 2], [4, 5], [7, 8]], np.uint32)))
    run_pair(sc, steps=30, check_every=3, grid=True)


def test_tgs_live_depth():
    # contact depth -5990: updateTGSDepth rotates the lever arms every substep
    # (collision.zig:73-100); the grid pipeline always keeps both lever arms
    b = scenes._Builder()
    b.disc(0.0, 0.0, 3000.0, 0.5, vx=0.5)
    b.disc(10.0, 0.0, 3000.0, 0.5, vx=-0.5, omega=0.3)
    b.rect(0.0, 4000.0, 2.0, 1.0, 0.5)
    ids, kind, opt = b.arrays()
    sc = scenes._concat("tgs", [(ids, kind, opt)], [0.0], 1 / 60, 1, 8, 6)
    w = World.from_scene(sc, debug=True, cell=1000.0, grid=True)
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


def test_many_cells_world_leaves_the_fused_kernel():
    # A 100,000-unit static ground covers 25,000 spatial-hash cells: more
    # entries than one CTA's shared memory holds, so the planner routes the
    # world to the grid pipeline without a flag.
    b = scenes._Builder()
    b.rect(0.0, -0.5, 100000.0, 1.0, 0.5, static=True)
    for i in range(40):
        b.disc(-20.0 + 1.1 * i, 0.5 + (i % 3) * 1.2, 0.5, 0.5)
        b.rect(-20.0 + 1.1 * i, 4.0, 0.8, 0.8, 0.5)
    ids, kind, opt = b.arrays()
    sc = scenes._concat("long-ground", [(ids, kind, opt)], [9.81], 1 / 60, 1, 8, 20)
    run_pair(sc, steps=20, check_every=5)


def test_world_above_fused_limit():
    sc = scenes.batched_worlds("big", seed=4, nworlds=1, steps=10, lo=2600, hi=2600)
    run_pair(sc, steps=10, check_every=5)


def test_mixed_batch_fused_and_grid_worlds():
    # worlds of 16..1200 bodies: the ones above 520 run on the grid pipeline
    # while the fused classes run on their own streams
    sc = scenes.batched_worlds("mixed", seed=6, nworlds=12, steps=15, lo=16, hi=1200)
    sizes = np.diff(sc.body_off)
    assert (sizes > 520).any() and (sizes <= 520).any()
    b = Batch.from_scene(sc, debug=True)
    oracles = [Oracle.from_scene(sc.world(w)) for w in range(sc.nworlds)]
    for _ in range(sc.steps):
        b.process(sc.dt, sc.sub_steps, sc.iters)
        for o in oracles:
            assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
    b.sync()
    st = b.read_state()
    for w, o in enumerate(oracles):
        assert_state_equal(st[:, sc.body_off[w]:sc.body_off[w + 1]], o.state(), f"world {w} ({sizes[w]} bodies)")
        gk, gd, gc = b.manifolds(w)
        ok, od = o.manifolds()
        oc, _ = o.colours()
        assert_manifolds_equal(gk, gd, gc, ok, od, oc)


def test_grid_batch_equals_fused_batch():
    sc = scenes.batched_worlds("eq", seed=7, nworlds=10, steps=12)
    fused = Batch.from_scene(sc)
    grid = Batch.from_scene(sc, grid=True)
    for _ in range(sc.steps):
        fused.process(sc.dt, 1, sc.iters)
        grid.process(sc.dt, 1, sc.iters)
    fused.sync()
    grid.sync()
    np.testing.assert_array_equal(fused.read_state().view(np.uint32), grid.read_state().view(np.uint32))


def test_nonfinite_world_is_reported_and_frozen():
    sc = scenes.batched_worlds("nan", seed=2, nworlds=3, steps=3, lo=40, hi=60)
    b = Batch.from_scene(sc, grid=True)
    st = b.read_state()
    w1 = sc.body_off[1]
    st[9, w1 + 2] = np.nan  # an AABB centre with no spatial-hash cell
    b.write_state(st)
    oracles = []
    for w in range(sc.nworlds):
        o = Oracle.from_scene(sc.world(w))
        o.set_state(st[:, sc.body_off[w]:sc.body_off[w + 1]])
        oracles.append(o)
    b.process(sc.dt, 1, sc.iters)
    with pytest.raises(N.R2DError) as e:
        b.sync()
    assert e.value.code == -7
    assert oracles[1].process(sc.dt, 1, sc.iters, ORDER_COLOUR) == -7
    for w in (0, 2):
        assert oracles[w].process(sc.dt, 1, sc.iters, ORDER_COLOUR) == 0
    got = b.read_state()
    for w, o in enumerate(oracles):
        assert_state_equal(got[:, sc.body_off[w]:sc.body_off[w + 1]], o.state(), f"world {w}")
    status = b.world_status()
    assert list(status) == [0, -7, 0]


def test_overflowing_pile_moves_to_grid_pipeline():
    # Two piles of 60 coincident discs: 3,540 manifolds, far beyond what the
    # 128-body class holds.  The fused replays grow the buffers until they
    # pass the shared-memory budget; then the world continues on the grid
    # pipeline from its failing call.  (60 discs per pile keep the colour
    # count below 128.)
    b = scenes._Builder()
    b.rect(0.0, -0.5, 40.0, 1.0, 0.5, static=True)
    rng = np.random.default_rng(0)
    for pile in (-8.0, 8.0):
        for _ in range(60):
            b.disc(pile + rng.uniform(-0.05, 0.05), 3.0 + rng.uniform(-0.05, 0.05), 1.0, 0.5)
    ids, kind, opt = b.arrays()
    sc = scenes._concat("pile", [(ids, kind, opt)], [9.81], 1 / 60, 1, 8, 4)
    run_pair(sc, steps=4, check_every=1)


def test_new_joints_midrun_are_recoloured():
    """A grid-pipeline world keeps its joint colouring from step to step; new
    joints (here the same joints in reverse insertion order, which changes their
    priorities) must be coloured and packed afresh: stepping on after
    set_joints equals a world that had those joints from the same state."""
    sc = scenes.random_scene(21, n=40, joints=True)
    rev = slice(None, None, -1)
    jt, j1, j2, jp = (np.ascontiguousarray(a[rev]) for a in (sc.jtype, sc.jid1, sc.jid2, sc.jprm))
    w1 = World.from_scene(sc, debug=True, grid=True)
    kept = World.from_scene(sc, grid=True)
    for _ in range(10):
        w1.process(sc.dt, sc.sub_steps, sc.iters)
        kept.process(sc.dt, sc.sub_steps, sc.iters)
    w1.sync()
    kept.sync()
    mid = w1.read_state()
    w1.set_joints(jt, j1, j2, jp)
    fresh = World.from_scene(sc, debug=True, grid=True)
    fresh.set_joints(jt, j1, j2, jp)
    fresh.write_state(mid)
    for _ in range(10):
        for w in (w1, fresh, kept):
            w.process(sc.dt, sc.sub_steps, sc.iters)
    for w in (w1, fresh, kept):
        w.sync()
    assert_state_equal(w1.read_state(), fresh.read_state(), "set_joints mid-run")
    np.testing.assert_array_equal(w1.joint_colours(len(jt)), fresh.joint_colours(len(jt)))
    # the order matters, so a stale colouring would have shown
    assert not np.array_equal(kept.read_state(), w1.read_state())


@pytest.mark.parametrize("mode", ["0", "2"])
def test_per_colour_launch_path(mode):
    """Small worlds take the resident cluster; R2D_RESIDENT (read once per
    process, hence a child process) forces the paths that large colours take:
    0 one launch per phase and colour, 2 per-colour joints with each
    iteration's contact colours in one cluster launch.  Against the oracle,
    with joints, substeps and warm starting."""
    import os
    import subprocess
    import sys

    here = os.path.dirname(os.path.abspath(__file__))
    code = (
        "import sys; sys.path[:0] = [%r, %r, %r]\n"
        "from parity import run_pair\n"
        "from resolve2d_gb300 import scenes\n"
        "for seed in (31, 32):\n"
        "    run_pair(scenes.random_scene(seed, n=40, joints=True), steps=20, check_every=5, grid=True)\n"
        "run_pair(scenes.random_scene(33, n=30, joints=True), steps=12, check_every=4, sub_steps=3, iters=4, grid=True)\n"
        "run_pair(scenes.random_scene(34, n=40, joints=True), steps=20, check_every=5, warm=True, grid=True)\n"
        "run_pair(scenes.config0(), steps=10, check_every=5, grid=True)\n"
        "print('per-colour path ok')\n" % (here, os.path.dirname(here), os.path.join(os.path.dirname(here), "oracle"))
    )
    env = dict(os.environ, R2D_RESIDENT=mode)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "per-colour path ok" in r.stdout

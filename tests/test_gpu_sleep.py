"""Sleeping (R2D_FLAG_SLEEP, r2d_sleep.h) against the oracle's same rule.

A world whose every non-static body ends 60 consecutive steps slower than
0.01 units/s and 0.01 rad/s is not stepped until the host writes to it.  Both
GPU paths and the oracle decide on the same f32 values, so the counters, the
frame a world falls asleep on, and every state stay identical.
"""

import numpy as np
import pytest

from oracle import ORDER_COLOUR, Oracle
from parity import assert_state_equal
from resolve2d_gb300 import scenes
from resolve2d_gb300.engine import Batch, World

pytestmark = pytest.mark.gpu

SLEEP_FRAMES = 60


def resting_builder(shift: float = 0.0):
    """Boxes on a static ground with discs on top of them, all starting at rest
    and in contact: the world settles and falls asleep."""
    b = scenes._Builder()
    b.rect(0.0, -0.5, 40.0, 1.0, 0.5, static=True)
    for i in range(8):
        x = -8.0 + 2.0 * i + shift
        b.rect(x, 0.5, 1.0, 1.0, 0.5)
        b.disc(x, 1.5, 0.5, 0.5)
    return b


def resting_scene(shift: float = 0.0):
    return scenes._concat("resting", [resting_builder(shift).arrays()], [9.81], 1 / 60, 1, 8, 200)


@pytest.mark.parametrize("grid", [False, True])
def test_resting_world_sleeps_and_wakes_like_the_oracle(grid):
    sc = resting_scene()
    w = World.from_scene(sc, sleep=True, grid=grid)
    o = Oracle.from_scene(sc)
    o.set_sleep(True)
    asleep_at = None
    for k in range(100):
        w.process(sc.dt, sc.sub_steps, sc.iters)
        assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
        assert w.sleep_frames() == o.sleep_frames(), f"step {k + 1}"
        if k % 10 == 9:
            assert_state_equal(w.read_state(), o.state(), f"step {k + 1}")
        if asleep_at is None and o.sleep_frames() >= SLEEP_FRAMES:
            asleep_at = k + 1
    assert asleep_at is not None, "the resting world never fell asleep"
    # asleep: stepping changes nothing
    before = w.read_state()
    for _ in range(5):
        w.process(sc.dt, sc.sub_steps, sc.iters)
    np.testing.assert_array_equal(w.read_state(), before)
    # a written force wakes the world on both sides
    st = o.state()
    st[scenes.S_FORCE_X, 3] = 400.0
    o.set_state(st)
    w.write_fields(scenes.S_FORCE_X, st[scenes.S_FORCE_X : scenes.S_FORCE_X + 1])
    assert w.sleep_frames() == 0 == o.sleep_frames()
    for k in range(20):
        w.process(sc.dt, sc.sub_steps, sc.iters)
        assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
        assert w.sleep_frames() == o.sleep_frames()
    assert_state_equal(w.read_state(), o.state(), "after waking")
    assert not np.array_equal(w.read_state(), before)


def test_off_by_default_and_counters_read_zero():
    sc = resting_scene()
    w = World.from_scene(sc)
    for _ in range(70):
        w.process(sc.dt, sc.sub_steps, sc.iters)
    assert w.sleep_frames() == 0
    o = Oracle.from_scene(sc)
    for _ in range(70):
        assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
    assert_state_equal(w.read_state(), o.state(), "sleeping off")


def test_batch_of_resting_and_moving_worlds():
    parts = [resting_builder(0.0).arrays(), resting_builder(0.5).arrays()]
    for seed in (5, 6):
        r = scenes.random_scene(seed, n=30)
        parts.append((r.ids, r.kind, r.opt))
    sc = scenes._concat("mixed", parts, [9.81, 9.81, 9.81, 9.81], 1 / 60, 1, 8, 90)
    b = Batch.from_scene(sc, sleep=True)
    oracles = []
    for k in range(sc.nworlds):
        o = Oracle.from_scene(sc.world(k))
        o.set_sleep(True)
        oracles.append(o)
    for step in range(90):
        b.process(sc.dt, sc.sub_steps, sc.iters)
        for o in oracles:
            assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
        if step % 15 == 14:
            frames = b.sleep_frames()
            np.testing.assert_array_equal(frames, [o.sleep_frames() for o in oracles])
            state = b.read_state()
            for k, o in enumerate(oracles):
                b0, b1 = sc.body_off[k], sc.body_off[k + 1]
                assert_state_equal(state[:, b0:b1], o.state(), f"world {k} step {step + 1}")
    assert (b.sleep_frames()[:2] >= SLEEP_FRAMES).all(), "the resting worlds should sleep"

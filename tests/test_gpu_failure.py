"""Failure detection through the C ABI, with no GPU fault.

The step's one bounded device loop is the grid pipeline's colouring: one
resident cluster runs Jones-Plassmann rounds until every constraint has a
colour.  Each round colours at least one constraint, so the loop ends by
itself; its bound only guards that argument.  The R2D_COLOUR_ROUND_LIMIT
test hook (read when a solver is created) lowers the bound so that the loop
runs out on an ordinary pile: the kernel stops, flags the colouring as stuck
and returns, the call reports R2D_ERR_TIMEOUT, and the world keeps the state
it had before the call, because the colouring runs before any substep.

A spatial-hash table whose bucket count (multiplier x bodies) would wrap 32
bits is refused at upload with R2D_ERR_CAPACITY, before anything reaches the
device.
"""

import os

import numpy as np
import pytest

from parity import assert_state_equal
from resolve2d_gb300 import _native as N
from resolve2d_gb300 import scenes
from resolve2d_gb300.engine import World
from resolve2d_gb300.scenes import derive_props_state

pytestmark = pytest.mark.gpu

TIMEOUT = -6
CAPACITY = -5


def _settled_config0(frames=60):
    sc = scenes.config0()
    w = World.from_scene(sc)
    for _ in range(frames):
        w.process(sc.dt, sc.sub_steps, sc.iters)
    w.sync()
    state = w.read_state()
    w.close()
    return sc, state


def test_colouring_round_limit_reports_timeout_and_leaves_the_state():
    sc, state = _settled_config0()
    os.environ["R2D_COLOUR_ROUND_LIMIT"] = "1"
    try:
        w = World.from_scene(sc, grid=True)
    finally:
        del os.environ["R2D_COLOUR_ROUND_LIMIT"]
    w.write_state(state)
    w.sync()
    w.process(sc.dt, sc.sub_steps, sc.iters)
    with pytest.raises(N.R2DError) as e:
        w.sync()
    assert e.value.code == TIMEOUT
    assert "round limit" in str(e.value)
    assert_state_equal(w.read_state(), state, "state after the timed-out call")
    # the context stays usable: a solver without the hook steps the same state
    w2 = World.from_scene(sc, grid=True)
    w2.write_state(state)
    w2.process(sc.dt, sc.sub_steps, sc.iters)
    w2.sync()
    assert not np.array_equal(w2.read_state(), state)
    w.close()
    w2.close()


def test_a_table_size_that_wraps_32_bits_is_refused_at_upload():
    sc = scenes.batched_worlds("w1024", seed=7, nworlds=1, steps=1, lo=1024, hi=1024)
    props, state = derive_props_state(sc.kind, sc.opt)
    w = World(mult=1 << 22)  # 1,024 x 2^22 = 2^32 buckets
    with pytest.raises(N.R2DError) as e:
        w.set_bodies(sc.ids, sc.kind & 3, props, state, True)
    assert e.value.code == CAPACITY
    assert "buckets exceeds" in str(e.value)
    w.close()

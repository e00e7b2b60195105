"""Parity at the benchmark's own sizes, through the C ABI, bit for bit
against the oracle replaying the GPU's colour-major constraint order.

- config 3, the timed batch: all 4,096 worlds (589,055 bodies) through the
  300 settling steps the benchmark runs before it times, then one more step
  with the debug taps, whose candidate pairs, manifolds and colours are
  compared on a sample of worlds;
- config 4, the long-horizon batch: all 16,384 worlds for their first 30 steps;
- config 1 (12,001 bodies, grid pipeline) for 300 steps;
- config 2 (200,004 bodies, 102,000 joints, grid pipeline) for 30 steps.

The oracle steps the batches on every host thread.
"""

import os

import numpy as np
import pytest

from oracle import ORDER_COLOUR, Oracle, batch_run
from parity import assert_manifolds_equal, assert_pairs_equal, assert_state_equal, run_pair
from resolve2d_gb300 import scenes
from resolve2d_gb300.engine import Batch

pytestmark = pytest.mark.gpu


def _threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def _batch_vs_oracle(sc, steps):
    b = Batch.from_scene(sc)
    for _ in range(steps):
        b.process(sc.dt, sc.sub_steps, sc.iters)
    b.sync()
    got = b.read_state()
    _, want, st = batch_run(sc, steps, _threads(), order=ORDER_COLOUR)
    assert st == 0
    want = want.reshape(13, sc.nbodies)
    bad = [w for w in range(sc.nworlds)
           if not np.array_equal(np.nan_to_num(got[:, sc.body_off[w]:sc.body_off[w + 1]], nan=1e30),
                                 np.nan_to_num(want[:, sc.body_off[w]:sc.body_off[w + 1]], nan=1e30))]
    if bad:
        w = bad[0]
        b0, b1 = sc.body_off[w], sc.body_off[w + 1]
        assert_state_equal(got[:, b0:b1], want[:, b0:b1], f"{sc.name}: {len(bad)} worlds differ, first world {w}")
    return b, got


def test_config3_whole_batch_through_the_settling_steps():
    sc = scenes.config3()
    assert sc.nworlds == 4096 and sc.nbodies == 589_055
    b, settled = _batch_vs_oracle(sc, 300)
    b.close()
    # one more step with the debug taps, from the settled state: pairs,
    # manifolds and colours of a sample of worlds, large ones included
    dbg = Batch.from_scene(sc, debug=True)
    dbg.write_state(settled)
    dbg.process(sc.dt, sc.sub_steps, sc.iters)
    dbg.sync()
    got = dbg.read_state()
    sizes = np.diff(sc.body_off)
    sample = sorted(set(np.argsort(sizes)[-24:].tolist()) | set(range(0, sc.nworlds, 97)))
    for w in sample:
        sw = sc.world(w)
        b0, b1 = sc.body_off[w], sc.body_off[w + 1]
        o = Oracle.from_scene(sw)
        o.set_state(np.ascontiguousarray(settled[:, b0:b1]))
        o.record_pairs()
        assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
        assert_state_equal(got[:, b0:b1], o.state(), f"world {w} step 301")
        assert_pairs_equal(dbg.pairs(w), o.pairs(), f"world {w} step 301")
        gk, gd, gc = dbg.manifolds(w)
        ok, od = o.manifolds()
        oc, _ = o.colours()
        assert_manifolds_equal(gk, gd, gc, ok, od, oc)
    dbg.close()


def test_config4_whole_batch_first_steps():
    sc = scenes.config4()
    assert sc.nworlds == 16384
    b, _ = _batch_vs_oracle(sc, 30)
    b.close()


def test_config1_pyramid_300_steps():
    run_pair(scenes.config1(), steps=300, check_every=100)


def test_config2_chains_and_motors_30_steps():
    sc = scenes.config2()
    w, o = run_pair(sc, steps=30, check_every=10)
    _, oj = o.colours()
    np.testing.assert_array_equal(w.joint_colours(len(sc.jtype)), oj)

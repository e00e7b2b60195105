"""Behaviour of the CPU oracle on hand-checked cases and on the seeded scenes.

The reference ships no physics tests, so beyond its two unit tests (see
test_oracle_reference_tests.py) the oracle is checked here against cases
whose answer follows from the reference's formulas by hand, and against
self-consistency properties (determinism, symmetry of solve orders).
"""

import math

import numpy as np

from oracle import ORDER_COLOUR, ORDER_REFERENCE, Oracle
from resolve2d_gb300 import scenes


def one_world(bodies, g=9.81):
    b = scenes._Builder()
    for spec in bodies:
        getattr(b, spec[0])(*spec[1:])
    ids, kind, opt = b.arrays()
    return scenes._concat("hand", [(ids, kind, opt)], [g], 1 / 60, 1, 8, 1)


def test_entity_factory_mirror_matches_oracle():
    # scenes.derive_props_state restates makeDiscBody / makeRectangleBody (lib.zig:73-93)
    for sc in (scenes.config0(), scenes.random_scene(4, n=60)):
        o = Oracle.from_scene(sc)
        props, state = scenes.derive_props_state(sc.kind, sc.opt)
        np.testing.assert_array_equal(o.props(), props)
        np.testing.assert_array_equal(o.state()[:9], state[:9])


def test_disc_resting_on_ground_contact():
    # A disc of radius 0.5 at y = 0.49 over a ground box whose top is y = 0:
    # the ground (id 0) is o1; its top edge normal (0,1) gives the smallest
    # overlap, so it is the reference body and the disc is incident
    # (collision.zig:299-320).  The contact point is c - n*r = (0,-0.01) with
    # depth dot(p - edge.a, n) = -0.01 (Rectangle.zig:202-206), stored at
    # p - n*depth/2 (collision.zig:38-51).
    sc = one_world([("rect", 0.0, -0.5, 10.0, 1.0, 0.5, 1.0, 0, 0, 0, 0, True), ("disc", 0.0, 0.49, 0.5, 0.5)])
    o = Oracle.from_scene(sc)
    assert o.update_manifolds() == 0
    k, d = o.manifolds()
    assert k.tolist() == [[0, 1]]
    np.testing.assert_allclose(d[0, :2], [0.0, 1.0], atol=1e-6)
    assert d[0, 5] == 1 and d[0, 6] == 0
    depth = d[0, 9 + 6]
    assert abs(depth - (-0.01)) < 1e-6
    ref_r = d[0, 9 + 2:9 + 4]
    np.testing.assert_allclose(ref_r, [0.0, 0.5 - 0.005], atol=1e-5)


def test_head_on_discs_exchange_momentum_along_normal():
    # Two equal discs moving toward each other, overlapping by 0.02, no gravity,
    # no friction: the normal impulse only changes momentum along the line of
    # centres, total momentum is conserved exactly up to rounding, and the
    # approach velocity is removed (pn = (dv.n + bias) * mass_n, collision.zig:164-176).
    sc = one_world([("disc", -0.49, 0.0, 0.5, 0.0, 1.0, 1.0, 0.0), ("disc", 0.49, 0.0, 0.5, 0.0, 1.0, -1.0, 0.0)], g=0.0)
    o = Oracle.from_scene(sc)
    p0 = o.state()[3:5].sum(axis=1)
    assert o.process(1 / 60, 1, 8, ORDER_REFERENCE) == 0
    st = o.state()
    np.testing.assert_allclose(st[3:5].sum(axis=1), p0, atol=1e-5)
    assert abs(st[4]).max() < 1e-6             # no momentum off the line of centres
    v1 = st[3, 0] / (math.pi * 0.25)
    v2 = st[3, 1] / (math.pi * 0.25)
    assert v2 - v1 >= -1e-4                    # no longer approaching


def test_distance_joint_at_rest_length_is_inert():
    # J = -(n.dv + beta*err/L) / (w1 + w2) = 0 when dv = 0 and err = 0 (DistanceJoint.zig:56-64)
    sc = one_world([("disc", 0.0, 10.0, 0.2, 0.5), ("disc", 2.0, 10.0, 0.2, 0.5)], g=0.0)
    sc.jworld = np.zeros(1, np.uint32)
    sc.jtype = np.array([scenes.JOINT_DISTANCE], np.uint8)
    sc.jid1 = np.array([0], np.uint32)
    sc.jid2 = np.array([1], np.uint32)
    sc.jprm = np.array([[np.inf, -np.inf, 10, 2.0, 0, 0, 0, 0]], np.float32)
    o = Oracle.from_scene(sc)
    before = o.state()
    assert o.process(1 / 60, 1, 8) == 0
    np.testing.assert_array_equal(o.state()[:6], before[:6])


def test_power_limit_clamps_joint_impulse():
    # With |n.dv| = 1 the clamp is J in [power_min, power_max] / max(|n.dv|, 1e-4)
    # (DistanceJoint.zig:66-70): a stretched joint with power_max = 0.5 can add
    # at most 0.5 units of momentum per solve.
    sc = one_world([("disc", 0.0, 10.0, 0.2, 0.5, 1.0, -1.0, 0.0), ("disc", 3.0, 10.0, 0.2, 0.5, 1.0, 0.0, 0.0)], g=0.0)
    sc.jworld = np.zeros(1, np.uint32)
    sc.jtype = np.array([scenes.JOINT_DISTANCE], np.uint8)
    sc.jid1 = np.array([0], np.uint32)
    sc.jid2 = np.array([1], np.uint32)
    sc.jprm = np.array([[0.5, -0.5, 10, 1.0, 0, 0, 0, 0]], np.float32)
    o = Oracle.from_scene(sc)
    m0 = o.state()[3, 0]
    assert o.process(1 / 60, 1, 1) == 0
    dm = o.state()[3, 0] - m0
    assert abs(dm) <= 0.5 + 1e-5
    assert abs(dm) > 0.4


def test_runs_are_deterministic():
    sc = scenes.random_scene(7, n=50, joints=True)
    outs = []
    for _ in range(2):
        o = Oracle.from_scene(sc)
        for _ in range(30):
            assert o.process(sc.dt, 1, 8, ORDER_COLOUR) == 0
        outs.append(o.state())
    assert np.array_equal(outs[0].view(np.uint32), outs[1].view(np.uint32))


def test_colour_order_only_reorders_constraints():
    # After one step from the same state, the reference order and the colour-major
    # order give the same manifold set and the same integrated positions up to the
    # order dependence of Gauss-Seidel (small, not zero).
    sc = scenes.config0()
    a, b = Oracle.from_scene(sc), Oracle.from_scene(sc)
    for _ in range(120):
        a.process(sc.dt, 1, 8, ORDER_REFERENCE)
    b.set_state(a.state())
    a.process(sc.dt, 1, 8, ORDER_REFERENCE)
    b.process(sc.dt, 1, 8, ORDER_COLOUR)
    ka, _ = a.manifolds()
    kb, _ = b.manifolds()
    assert sorted(map(tuple, ka.tolist())) == sorted(map(tuple, kb.tolist()))
    sa, sb = a.state(), b.state()
    assert np.abs(sa[:2] - sb[:2]).max() < 1e-2


def test_colouring_is_body_disjoint():
    sc = scenes.config0()
    o = Oracle.from_scene(sc)
    for _ in range(200):
        o.process(sc.dt, 1, 8, ORDER_COLOUR)
    k, _ = o.manifolds()
    c, _ = o.colours()
    static = (sc.kind & scenes.KIND_STATIC) != 0
    seen = set()
    for (a, b), col in zip(k.tolist(), c.tolist()):
        for x in (a, b):
            if static[x]:
                continue
            assert (x, col) not in seen
            seen.add((x, col))


def test_fp64_oracle_tracks_fp32_over_short_horizon():
    sc = scenes.random_scene(2, n=20, spin=False)
    a, b = Oracle.from_scene(sc, 32), Oracle.from_scene(sc, 64)
    for _ in range(10):
        a.process(sc.dt, 1, 8)
        b.process(sc.dt, 1, 8)
    assert np.abs(a.state()[:2] - b.state64()[:2]).max() < 1e-2


def _resting(shift=0.0):
    b = scenes._Builder()
    b.rect(0.0, -0.5, 40.0, 1.0, 0.5, static=True)
    for i in range(8):
        b.rect(-8.0 + 2.0 * i + shift, 0.5, 1.0, 1.0, 0.5)
        b.disc(-8.0 + 2.0 * i + shift, 1.5, 0.5, 0.5)
    return scenes._concat("resting", [b.arrays()], [9.81], 1 / 60, 1, 8, 100)


def test_sleeping_rule():
    """The sleeping extension (r2d_sleep.h): a world whose bodies stay still
    for 60 steps stops changing; writing its state wakes it; a moving world
    never sleeps; with sleeping off nothing is skipped."""
    sc = _resting()
    o = Oracle.from_scene(sc)
    o.set_sleep(True)
    frames = []
    for _ in range(80):
        assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
        frames.append(o.sleep_frames())
    assert max(frames) == 60 and frames[-1] == 60
    first = frames.index(60)
    assert frames[first - 59 : first + 1] == list(range(1, 61))  # 60 consecutive still frames
    asleep = o.state()
    assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
    np.testing.assert_array_equal(o.state(), asleep)
    asleep[scenes.S_MOM_X, 1] = 5.0  # a kick wakes it
    o.set_state(asleep)
    assert o.sleep_frames() == 0
    assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
    assert o.sleep_frames() == 0 and not np.array_equal(o.state(), asleep)
    # sleeping off: the same steps are all taken
    off = Oracle.from_scene(sc)
    for _ in range(80):
        assert off.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
    assert off.sleep_frames() == 0
    moving = Oracle.from_scene(scenes.config0())
    moving.set_sleep(True)
    for _ in range(80):
        assert moving.process(1 / 60, 1, 8, ORDER_COLOUR) == 0
    assert moving.sleep_frames() < 60


def test_phase_timing_measures_without_changing_results():
    from oracle import PHASES

    sc = scenes.random_scene(8, n=40, joints=True)
    timed, plain = Oracle.from_scene(sc), Oracle.from_scene(sc)
    timed.set_phase_timing(True)
    for _ in range(10):
        assert timed.process(1 / 60, 2, 8, ORDER_COLOUR) == 0
        assert plain.process(1 / 60, 2, 8, ORDER_COLOUR) == 0
    np.testing.assert_array_equal(timed.state(), plain.state())
    ph = timed.phase_seconds()
    assert ph.shape == (len(PHASES),) and (ph >= 0).all() and ph.sum() > 0
    assert ph[PHASES.index("solve")] > 0 and ph[PHASES.index("colouring")] > 0
    assert not plain.phase_seconds().any()  # off: nothing is read or added
    timed.set_phase_timing(False)
    assert not timed.phase_seconds().any()  # switching clears the sums


def test_the_batch_runner_refuses_what_it_would_drop():
    import pytest
    from oracle import batch_run

    with pytest.raises(ValueError, match="joints"):
        batch_run(scenes.random_scene(3, n=8, joints=True), 1, 1)

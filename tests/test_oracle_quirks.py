"""Quirks of the reference's step that the oracle (and so the GPU) must keep.

Each follows from a line of the reference and is checked here on the CPU:
- the stored AABB is one substep stale: updateAABB runs before integration
  (lib.zig:210 against lib.zig:238-249);
- static bodies get updateAABB too: the call comes before the static check
  (lib.zig:210-211);
- a point whose normal impulse is below 1e-4 is skipped whole, friction
  included (collision.zig:176), so a body too light to ever reach that
  impulse gets no support at all;
- the narrowphase runs once a frame, not once a substep (lib.zig:194);
- the TGS depth update writes no depth (collision.zig:73-100);
- both points of a manifold read the same start velocities (collision.zig:145-149).
"""

import math

import numpy as np

from oracle import ORDER_COLOUR, Oracle
from resolve2d_gb300 import scenes as S

DT = np.float32(1 / 60)


def world(bodies, g=9.81):
    b = S._Builder()
    for spec in bodies:
        getattr(b, spec[0])(*spec[1:])
    return Oracle.from_scene(S._concat("quirks", [b.arrays()], [g], float(DT), 1, 8, 1))


def test_the_stored_aabb_is_one_substep_stale():
    falling = [("disc", 0.0, 10.0, 0.5, 0.5, 1.0, 6.0, 1.0)]
    two = world(falling)
    assert two.process(float(DT), 2, 8, ORDER_COLOUR) == 0
    half = world(falling)  # one substep of dt/2: the pose after the first of the two
    assert half.process(float(DT / 2), 1, 8, ORDER_COLOUR) == 0
    st, ref = two.state(), half.state()
    assert st[S.S_AABB_X, 0] == ref[S.S_POS_X, 0] and st[S.S_AABB_Y, 0] == ref[S.S_POS_Y, 0]
    assert st[S.S_POS_X, 0] != st[S.S_AABB_X, 0]  # the body itself moved on
    one = world(falling)
    x0 = one.state()[S.S_POS_X, 0]
    assert one.process(float(DT), 1, 8, ORDER_COLOUR) == 0
    assert one.state()[S.S_AABB_X, 0] == x0  # one substep: the frame's starting pose


def test_a_static_body_gets_its_aabb_updated():
    # a static 2 x 1 box turned by 45 degrees through the state: its stored AABB
    # is still the unrotated one until a step runs updateAABB on it
    o = world([("rect", 0.0, 0.0, 2.0, 1.0, 0.5, 1.0, 0.0, 0.0, 0.0, 0.0, True)])
    st = o.state()
    assert st[S.S_AABB_HW, 0] == 1.0 and st[S.S_AABB_HH, 0] == 0.5
    st[S.S_ANGLE, 0] = math.pi / 4
    o.set_state(st)
    assert o.process(float(DT), 1, 8, ORDER_COLOUR) == 0
    turned = world([("rect", 0.0, 0.0, 2.0, 1.0, 0.5, 1.0, 0.0, 0.0, math.pi / 4, 0.0, True)])
    np.testing.assert_array_equal(o.state()[S.S_AABB_X:], turned.state()[S.S_AABB_X:])
    assert abs(o.state()[S.S_AABB_HW, 0] - 1.5 * math.sqrt(0.5)) < 1e-6
    assert o.state()[S.S_POS_X, 0] == 0.0 and o.state()[S.S_ANGLE, 0] == np.float32(math.pi / 4)


def test_a_body_too_light_for_the_impulse_threshold_sinks_through_the_ground():
    # A 1 x 1 box of mass 1e-4 resting on the ground: each point's normal impulse
    # is about (g*dt + bias) * m / 2, far below 1e-4, so every point is skipped and
    # gravity pulls it in until the Baumgarte bias alone lifts pn over the
    # threshold.  A box of mass 1 stays on top.
    ground = ("rect", 0.0, -0.5, 40.0, 1.0, 0.5, 1.0, 0.0, 0.0, 0.0, 0.0, True)
    light = world([ground, ("rect", 0.0, 0.495, 1.0, 1.0, 0.5, 1e-4)])
    heavy = world([ground, ("rect", 0.0, 0.495, 1.0, 1.0, 0.5, 1.0)])
    for _ in range(60):
        assert light.process(float(DT), 1, 8, ORDER_COLOUR) == 0
        assert heavy.process(float(DT), 1, 8, ORDER_COLOUR) == 0
    assert heavy.state()[S.S_POS_Y, 1] > 0.45  # resting on the top face at y = 0
    assert light.state()[S.S_POS_Y, 1] < 0.0  # sunk by more than half its height


def test_the_narrowphase_runs_once_a_frame():
    # A disc that only reaches the ground during a frame's later substeps makes no
    # manifold in that frame: contacts are found from the frame's starting pose.
    o = world([("rect", 0.0, -0.5, 40.0, 1.0, 0.5, 1.0, 0.0, 0.0, 0.0, 0.0, True),
               ("disc", 0.0, 0.52, 0.5, 0.5, 1.0, 0.0, -3.0)], g=0.0)
    assert o.process(float(DT), 4, 8, ORDER_COLOUR) == 0
    k, _ = o.manifolds()
    assert k.shape[0] == 0  # 0.02 apart at the start: beyond the 0.01 margin
    assert o.state()[S.S_POS_Y, 1] < 0.5  # yet it ended the frame overlapping the ground
    assert o.process(float(DT), 4, 8, ORDER_COLOUR) == 0
    k, _ = o.manifolds()
    assert k.shape[0] == 1  # found at the next frame's start


def test_the_tgs_depth_update_changes_no_depth():
    # updateTGSDepth skips a point whose depth still equals its original depth
    # (collision.zig:80), and that depth is only written after the check, so over
    # any number of substeps every point keeps the narrowphase's depth
    sc = S.random_scene(31, n=50)
    o = Oracle.from_scene(sc)
    for _ in range(20):
        assert o.process(sc.dt, 1, sc.iters, ORDER_COLOUR) == 0
    assert o.process(sc.dt, 4, sc.iters, ORDER_COLOUR) == 0
    _, d = o.manifolds()
    seen = 0
    for row in d:
        for p in range(2):
            if row[5 + p]:
                base = 9 + 12 * p
                assert row[base + 6] == row[base + 7]  # depth == original_depth
                seen += 1
    assert seen > 20


def test_both_points_of_a_manifold_read_the_same_start_velocities():
    # calculateImpulses reads the bodies' velocities once per manifold and applies
    # the summed impulses after its point loop (collision.zig:145-149, 208-217).
    # A flat box landing on the ground meets it with two mirror-image points:
    # one iteration gives them bit-identical normal impulses.  Read point by point,
    # point 0's impulse would start the box turning and change point 1's.
    o = world([("rect", 0.0, -0.5, 40.0, 1.0, 0.5, 1.0, 0.0, 0.0, 0.0, 0.0, True),
               ("rect", 0.0, 0.49, 1.0, 1.0, 0.5, 1.0, 0.0, -1.0)])
    assert o.process(float(DT), 1, 1, ORDER_COLOUR) == 0
    _, d = o.manifolds()
    assert d.shape[0] == 1 and d[0, 5] == 1 and d[0, 6] == 1
    pn0, pn1 = d[0, 9 + 10], d[0, 9 + 12 + 10]
    assert pn0 > 0.0 and pn0 == pn1
    assert o.state()[S.S_ANG_MOM, 1] == 0.0  # the pair's torques cancel exactly

"""The oracle's joints on cases whose answer follows from the reference's formulas.

MotorJoint.zig:38-64, FixedPositionJoint.zig:38-72 and OffsetDistanceJoint.zig
solve functions, worked by hand in float32: the first iteration exactly, then
where the iterations lead.  CPU only.
"""

import math

import numpy as np

from oracle import Oracle
from resolve2d_gb300 import scenes as S

F = np.float32
DT = 1 / 60


def world(bodies, joints, g=0.0):
    """bodies: ("disc"|"rect", args...) for scenes._Builder; joints: (type, a, b, params[8])."""
    b = S._Builder()
    for spec in bodies:
        getattr(b, spec[0])(*spec[1:])
    sc = S._concat("joints", [b.arrays()], [g], DT, 1, 8, 1)
    sc.jworld = np.zeros(len(joints), np.uint32)
    sc.jtype = np.array([j[0] for j in joints], np.uint8)
    sc.jid1 = np.array([j[1] for j in joints], np.uint32)
    sc.jid2 = np.array([j[2] for j in joints], np.uint32)
    sc.jprm = np.array([j[3] for j in joints], np.float32).reshape(-1, S.JOINT_PARAMS)
    return Oracle.from_scene(sc)


def omega(o, i=0):
    return float(o.state()[S.S_ANG_MOM, i] / o.props()[S.P_INERTIA, i])


INF = math.inf


def test_motor_first_iteration_is_exact():
    # omega = 0, C = 0 - 3, bias = 10 * C = -30, J = torque - bias = 30, unclamped
    # (den = 1 / max(|0 / I|, 1e-6)); L += J * dt
    o = world([("disc", 0.0, 0.0, 1.0, 0.5)], [(S.JOINT_MOTOR, 0, 0, [INF, -INF, 10.0, 3.0, 0, 0, 0, 0])])
    assert o.process(DT, 1, 1) == 0
    assert o.state()[S.S_ANG_MOM, 0] == F(30.0) * F(DT)


def test_motor_drives_the_spin_to_its_target():
    o = world([("disc", 0.0, 0.0, 1.0, 0.5)], [(S.JOINT_MOTOR, 0, 0, [INF, -INF, 10.0, 3.0, 0, 0, 0, 0])])
    for _ in range(30):
        assert o.process(DT, 1, 8) == 0
    assert abs(omega(o) - 3.0) < 1e-4
    np.testing.assert_array_equal(o.state()[S.S_MOM_X : S.S_MOM_Y + 1, 0], [0.0, 0.0])


def test_motor_power_limit_binds_with_an_applied_torque():
    # torque T: L += T*dt first (lib.zig:215); then J = T - beta*(omega - target)
    # is clamped to power_max / max(|T / I|, 1e-6) (MotorJoint.zig:57-61)
    o = world([("disc", 0.0, 0.0, 1.0, 0.5)], [(S.JOINT_MOTOR, 0, 0, [1.0, -1.0, 10.0, 3.0, 0, 0, 0, 0])])
    st = o.state()
    st[S.S_TORQUE, 0] = 2.0
    o.set_state(st)
    inertia = float(o.props()[S.P_INERTIA, 0])
    assert o.process(DT, 1, 1) == 0
    want = 2.0 * DT + (1.0 / (2.0 / inertia)) * DT
    assert abs(float(o.state()[S.S_ANG_MOM, 0]) - want) < 1e-6
    assert o.state()[S.S_TORQUE, 0] == 0.0  # cleared after integration (lib.zig:247-248)


def test_joints_leave_static_bodies_alone():
    o = world([("disc", 0.0, 0.0, 1.0, 0.5, 1.0, 0.0, 0.0, 0.0, 0.0, True)],
              [(S.JOINT_MOTOR, 0, 0, [INF, -INF, 10.0, 3.0, 0, 0, 0, 0]),
               (S.JOINT_FIXED_POSITION, 0, 0, [INF, -INF, 10.0, 5.0, 5.0, 0, 0, 0])], g=9.81)
    before = o.state()
    for _ in range(5):
        assert o.process(DT, 1, 8) == 0
    np.testing.assert_array_equal(o.state()[:9], before[:9])


def test_fixed_position_first_frame_moves_beta_times_distance():
    # v.n becomes beta * dist after the first iteration and stays there (J = 0 after),
    # so one frame moves the body beta * dist * dt toward the target
    o = world([("disc", 0.0, 0.0, 0.5, 0.5)], [(S.JOINT_FIXED_POSITION, 0, 0, [INF, -INF, 10.0, 3.0, 4.0, 0, 0, 0])])
    assert o.process(DT, 1, 8) == 0
    x, y = o.state()[S.S_POS_X, 0], o.state()[S.S_POS_Y, 0]
    step = 10.0 * 5.0 * DT
    assert abs(x - 0.6 * step) < 1e-5 and abs(y - 0.8 * step) < 1e-5


def test_fixed_position_converges_then_orbits_its_target():
    # The distance shrinks by (1 - beta*dt) = 5/6 a frame until float32 rounding
    # of the position turns the normal between frames.  The joint sets only the
    # velocity along the current normal (FixedPositionJoint.zig:62-71) and keeps
    # the tangential part, so the body settles into a small orbit around the
    # target instead of reaching it.
    o = world([("disc", 0.0, 0.0, 0.5, 0.5)], [(S.JOINT_FIXED_POSITION, 0, 0, [INF, -INF, 10.0, 3.0, 4.0, 0, 0, 0])])
    dist = []
    for _ in range(90):
        assert o.process(DT, 1, 8) == 0
        st = o.state()
        dist.append(math.hypot(st[S.S_POS_X, 0] - 3.0, st[S.S_POS_Y, 0] - 4.0))
    assert abs(dist[9] - 5.0 * (5 / 6) ** 10) < 1e-4  # still on the geometric decay
    assert max(dist[60:]) < 1e-3  # then within 1e-3 of the target for good
    st = o.state()
    speed = math.hypot(st[S.S_MOM_X, 0], st[S.S_MOM_Y, 0])
    assert 0.0 < speed < 0.05  # the residual orbit


def anchor_distance(o, r1, r2):
    st = o.state()

    def anchor(i, r):
        c, s = math.cos(st[S.S_ANGLE, i]), math.sin(st[S.S_ANGLE, i])
        return st[S.S_POS_X, i] + c * r[0] - s * r[1], st[S.S_POS_Y, i] + s * r[0] + c * r[1]

    (ax, ay), (bx, by) = anchor(0, r1), anchor(1, r2)
    return math.hypot(bx - ax, by - ay)


def test_offset_distance_joint_holds_a_pendulum_at_its_length():
    # a static pivot and a rectangle hung by an off-centre anchor, under gravity
    r1, r2, length = (0.0, 0.0), (-0.4, 0.0), 2.0
    o = world([("disc", 0.0, 10.0, 0.1, 0.5, 1.0, 0.0, 0.0, 0.0, 0.0, True),
               ("rect", 2.4, 10.0, 1.0, 0.3, 0.5)],
              [(S.JOINT_OFFSET_DISTANCE, 0, 1, [INF, -INF, 10.0, *r1, *r2, length])], g=9.81)
    assert abs(anchor_distance(o, r1, r2) - length) < 1e-6
    worst, lowest = 0.0, 10.0
    for _ in range(240):
        assert o.process(DT, 1, 8) == 0
        worst = max(worst, abs(anchor_distance(o, r1, r2) - length))
        lowest = min(lowest, float(o.state()[S.S_POS_Y, 1]))
    assert worst < 0.02 * length  # Baumgarte-held to within 2 %
    assert lowest < 8.5  # it swung down through the bottom of the arc
    assert o.state()[S.S_POS_X, 0] == 0.0 and o.state()[S.S_POS_Y, 0] == 10.0  # the pivot is static


def test_a_joint_on_an_unknown_body_is_invalid_rigid_body_id():
    # bodies.getEntry(id) orelse return error.InvalidRigidBodyId (DistanceJoint.zig:44-47)
    o = world([("disc", 0.0, 0.0, 0.5, 0.5)], [(S.JOINT_DISTANCE, 0, 7, [INF, -INF, 10.0, 1.0, 0, 0, 0, 0])])
    assert o.process(DT, 1, 8) == -2

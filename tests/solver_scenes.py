"""Scenes built two ways for the tests of the reference-style Solver
(resolve2d_gb300/solver.py): through its EntityFactory, and as the oracle's
arrays.  Shared by test_solver_api.py (CPU) and test_gpu_solver_api.py."""

import ctypes as C
import math

import numpy as np

from oracle import ORDER_COLOUR, Oracle, _p
from parity import assert_state_equal
from resolve2d_gb300 import _native as N
from resolve2d_gb300 import scenes as S
from resolve2d_gb300.solver import BodyOptions, Density, DiscOptions, Mass, Parameters, RectangleOptions


def body_specs(seed, n=36):
    """Bodies as the factory takes them: (shape, BodyOptions, geometry, static)."""
    rng = np.random.default_rng(seed)
    specs = [("rect", BodyOptions(pos=(0.0, -0.5), mass_prop=Density(5.0), mu=0.4), RectangleOptions(60.0, 1.0), True)]
    for _ in range(n):
        pos = (float(rng.uniform(-6, 6)), float(rng.uniform(0.2, 6)))
        mp = Density(float(rng.uniform(0.5, 3))) if rng.random() < 0.7 else Mass(float(rng.uniform(0.5, 4)))
        bo = BodyOptions(pos=pos, mass_prop=mp, vel=(float(rng.normal()), float(rng.normal())),
                         angle=float(rng.uniform(-math.pi, math.pi)), omega=float(rng.normal()),
                         mu=float(rng.uniform(0.1, 0.9)))
        static = bool(rng.random() < 0.08)
        if rng.random() < 0.5:
            specs.append(("rect", bo, RectangleOptions(float(rng.uniform(0.3, 1.6)), float(rng.uniform(0.3, 1.6))),
                          static))
        else:
            specs.append(("disc", bo, DiscOptions(float(rng.uniform(0.2, 0.8))), static))
    return specs


def spec_arrays(specs, first_id=0):
    """The same bodies as the oracle's (ids, kind, opt) arrays."""
    n = len(specs)
    ids = np.arange(first_id, first_id + n, dtype=np.uint32)
    kind = np.zeros(n, np.uint8)
    opt = np.zeros((S.NOPT, n), np.float32)
    for i, (shape, bo, go, static) in enumerate(specs):
        k = (S.KIND_RECT if shape == "rect" else 0) | (S.KIND_STATIC if static else 0)
        if isinstance(bo.mass_prop, Density):
            k |= S.KIND_DENSITY
            opt[S.MASS_PROP, i] = bo.mass_prop.density
        else:
            opt[S.MASS_PROP, i] = bo.mass_prop.mass
        kind[i] = k
        opt[S.POS_X, i], opt[S.POS_Y, i] = bo.pos
        opt[S.ANGLE, i], opt[S.OMEGA, i], opt[S.MU, i] = bo.angle, bo.omega, bo.mu
        opt[S.VEL_X, i], opt[S.VEL_Y, i] = bo.vel
        if shape == "rect":
            opt[S.DIM0, i], opt[S.DIM1, i] = go.width, go.height
        else:
            opt[S.DIM0, i] = go.radius
    return ids, kind, opt


def add_to_oracle(o, ids, kind, opt):
    o.lib.r2o_add_bodies(o.h, ids.shape[0], _p(ids, C.c_uint32), _p(kind, C.c_uint8),
                         _p(np.ascontiguousarray(opt), C.c_float))


def build(solver, specs):
    fac = solver.entityFactory()
    handles = []
    for shape, bo, go, static in specs:
        h = fac.makeRectangleBody(bo, go) if shape == "rect" else fac.makeDiscBody(bo, go)
        if static:
            h.body_unwrap().static = True
        handles.append(h)
    return handles


JOINTS = [  # (type, body a, body b, params, extra)
    (S.JOINT_DISTANCE, 3, 4, Parameters(beta=8.0), [1.5]),
    (S.JOINT_OFFSET_DISTANCE, 5, 6, Parameters(power_max=40.0, power_min=-40.0), [0.1, -0.2, 0.0, 0.15, 1.2]),
    (S.JOINT_FIXED_POSITION, 7, 7, Parameters(beta=4.0), [1.0, 3.0]),
    (S.JOINT_MOTOR, 8, 8, Parameters(power_max=25.0, power_min=-25.0), [3.0]),
]


def make_joints(fac, hs):
    for t, a, b, prm, extra in JOINTS:
        if t == S.JOINT_DISTANCE:
            fac.makeDistanceJoint(prm, hs[a], hs[b], extra[0])
        elif t == S.JOINT_OFFSET_DISTANCE:
            fac.makeOffsetDistanceJoint(prm, hs[a], hs[b], extra[0:2], extra[2:4], extra[4])
        elif t == S.JOINT_FIXED_POSITION:
            fac.makeFixedPositionJoint(prm, hs[a], extra)
        else:
            fac.makeMotorJoint(prm, hs[a], extra[0])


def add_joints_to_oracle(o):
    t = np.array([j[0] for j in JOINTS], np.uint8)
    a = np.array([j[1] for j in JOINTS], np.uint32)
    b = np.array([j[2] for j in JOINTS], np.uint32)
    prm = np.zeros((len(JOINTS), S.JOINT_PARAMS), np.float32)
    for i, (_, _, _, p, extra) in enumerate(JOINTS):
        prm[i, :3] = p.power_max, p.power_min, p.beta
        prm[i, 3 : 3 + len(extra)] = extra
    o.lib.r2o_add_joints(o.h, len(JOINTS), _p(t, C.c_uint8), _p(a, C.c_uint32), _p(b, C.c_uint32),
                         _p(prm, C.c_float))
    o.nj = len(JOINTS)


DT, SUB, ITERS = 1 / 60, 2, 8


def step_both(s, o, frames, what):
    for f in range(frames):
        s.process(DT, SUB, ITERS)
        assert o.process(DT, SUB, ITERS, ORDER_COLOUR) == 0
        if f % 5 == 4 or f == frames - 1:
            assert_state_equal(s.read_state(), o.state(), f"{what}, frame {f + 1}")


class OracleBackend:
    """engine.World's interface over the oracle, for host-only tests.  Every
    setter rebuilds the oracle from what it was given, carrying the current
    state across, and in warm-start mode last frame's impulses (keyed by body
    ids), as the engine keeps them across body uploads."""

    def __init__(self, warm_start=False, compensated=False, carry_warm=True):
        self.warm_start, self.compensated, self.carry_warm = warm_start, compensated, carry_warm
        self.o = None
        self.bodies = None
        self.g = []
        self.joints = (np.zeros(0, np.uint8), np.zeros(0, np.uint32), np.zeros(0, np.uint32),
                       np.zeros((0, S.JOINT_PARAMS), np.float32))
        self.x = np.zeros((0, 2), np.uint32)
        self.calls = []

    def _build(self, state, init_aabb):
        ids, kind, props = self.bodies
        n = ids.shape[0]
        opt = np.zeros((S.NOPT, n), np.float32)
        opt[S.POS_X], opt[S.POS_Y], opt[S.ANGLE] = state[S.S_POS_X], state[S.S_POS_Y], state[S.S_ANGLE]
        opt[S.MU], opt[S.MASS_PROP] = props[S.P_MU], props[S.P_MASS]
        opt[S.DIM0], opt[S.DIM1] = props[S.P_DIM0], props[S.P_DIM1]
        o = Oracle()
        k = np.ascontiguousarray(kind & 3, np.uint8)
        o.lib.r2o_add_bodies(o.h, n, _p(np.ascontiguousarray(ids, np.uint32), C.c_uint32), _p(k, C.c_uint8),
                             _p(opt, C.c_float))
        np.testing.assert_array_equal(o.props(), props)  # mass given: the oracle derives the same inertia
        st = o.state()
        if init_aabb:
            st[: S.S_AABB_X] = state[: S.S_AABB_X]
        else:
            st = np.array(state, np.float32)
        o.set_state(np.ascontiguousarray(st))
        for g in self.g:
            o.lib.r2o_add_gravity(o.h, g)
        t, a, b, prm = self.joints
        if t.size:
            o.lib.r2o_add_joints(o.h, t.shape[0], _p(t, C.c_uint8), _p(a, C.c_uint32), _p(b, C.c_uint32),
                                 _p(prm, C.c_float))
        o.nj = int(t.size)
        for x, y in self.x:
            o.lib.r2o_exclude_pair(o.h, int(x), int(y))
        o.set_warm_start(self.warm_start)
        o.set_compensated(self.compensated)
        if self.warm_start and self.carry_warm and self.o is not None:
            o.take_warm(self.o)
        self.o = o

    def _rebuild(self):
        if self.bodies is not None:
            self._build(self.o.state(), False)

    def set_bodies(self, ids, kind, props, state, init_aabb):
        self.calls.append(("set_bodies", int(ids.shape[0]), bool(init_aabb)))
        self.bodies = (np.array(ids, np.uint32), np.array(kind, np.uint8), np.array(props, np.float32))
        self._build(np.asarray(state, np.float32), init_aabb)

    def set_gravity(self, g):
        self.calls.append(("set_gravity", len(g)))
        self.g = [float(v) for v in g]
        self._rebuild()

    def set_joints(self, t, a, b, prm):
        self.calls.append(("set_joints", len(t)))
        self.joints = (np.array(t, np.uint8), np.array(a, np.uint32), np.array(b, np.uint32),
                       np.ascontiguousarray(prm, np.float32).reshape(-1, S.JOINT_PARAMS))
        self._rebuild()

    def set_exclusions(self, pairs):
        self.calls.append(("set_exclusions", len(pairs)))
        self.x = np.array(pairs, np.uint32).reshape(-1, 2)
        self._rebuild()

    def write_state(self, state):
        self.calls.append(("write_state",))
        self.o.set_state(np.ascontiguousarray(state, np.float32))

    def read_state(self):
        return self.o.state()

    def process(self, dt, sub, iters):
        self.calls.append(("process",))
        have = set(self.bodies[0].tolist())
        t, a, b, _ = self.joints
        two = (t == S.JOINT_DISTANCE) | (t == S.JOINT_OFFSET_DISTANCE)
        if any(x not in have for x in a.tolist()) or any(y not in have for y in b[two].tolist()):
            raise N.R2DError(-2, "r2d_solver_process", "a joint names an unknown body id")
        assert self.o.process(dt, sub, iters, ORDER_COLOUR) == 0

    def manifolds(self):
        k, d = self.o.manifolds()
        c, _ = self.o.colours()
        return k, d, c[: k.shape[0]]

    def sync(self):
        pass

    def close(self):
        self.o = None

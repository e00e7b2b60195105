"""The reference's scene-building API, ``Solver`` and ``EntityFactory``, over the GPU engine.

Mirrors src/core/lib.zig with the same names, argument meaning and errors, so
a scene written against the reference reads the same here:

- ``Solver.init``, ``deinit``, ``clear``, ``process``, ``bodyHandle``,
  ``removeRigidBody`` and ``entityFactory`` (lib.zig:131-314), and the
  ``bodies`` and ``manifolds`` fields (lib.zig:135-137) as a read-only map of
  body views and the last frame's manifolds keyed by id;
- ``EntityFactory.makeDiscBody``, ``makeRectangleBody``,
  ``makeDownwardsGravity``, ``makeOffsetDistanceJoint``, ``makeDistanceJoint``,
  ``makeFixedPositionJoint``, ``makeMotorJoint`` and ``excludeCollisionPair``
  (lib.zig:13-129);
- ``BodyHandle.body`` / ``body_unwrap``, which give a view of a body's
  ``RigidBody`` fields (``id``, ``static``, ``type``, ``props``, ``aabb``;
  RigidBody.zig:67-90).

``batch(solvers)`` steps many such scenes together, one world each, on the
batched engine (``engine.Batch``).

Bodies are kept on the host in the reference's map order: insertion order,
with ``swapRemove`` on removal (lib.zig:308-310).  They are handed to the
engine (``engine.World``, the C ABI's ``r2d_solver_*``) at the next
``process``.  The state then lives on the device and is read back when a body
is looked at or changed.

Deliberate differences from the reference:

- ids are u32 (``RigidBody.Id`` is u16, RigidBody.zig:15);
- ``init``'s spatial-hash arguments are honoured.  The reference ignores them
  and uses 4.0 and 2 (lib.zig:145,254-255); those are the defaults here;
- a joint that names a missing body fails the whole ``process`` call before
  anything is stepped.  The reference fails part-way through the first
  substep;
- ``clear`` also drops the collision exclusions.  The reference's ``clear``
  leaves that map deinitialised (lib.zig:159-187);
- at most four ``DownwardsGravity`` generators (the engine's limit);
- ``process`` on a solver without bodies does nothing.
"""

from __future__ import annotations

import dataclasses
import math
from collections.abc import Iterator, Mapping
from typing import Callable, NamedTuple, Sequence

import numpy as np

from . import _native as N
from .scenes import (
    DIM0, DIM1, JOINT_DISTANCE, JOINT_FIXED_POSITION, JOINT_MOTOR, JOINT_OFFSET_DISTANCE, JOINT_PARAMS,
    KIND_DENSITY, KIND_RECT, KIND_STATIC, MASS_PROP, NOPT, NPROP, NSTATE, P_DIM0, P_DIM1, P_INERTIA, P_MASS, P_MU,
    S_AABB_HH, S_AABB_HW, S_AABB_X, S_AABB_Y, S_ANG_MOM, S_ANGLE, S_FORCE_X, S_FORCE_Y, S_MOM_X, S_MOM_Y, S_POS_X,
    S_POS_Y, S_TORQUE, derive_props_state,
)
from .scenes import ANGLE as O_ANGLE
from .scenes import MU as O_MU
from .scenes import OMEGA as O_OMEGA
from .scenes import POS_X as O_POS_X
from .scenes import POS_Y as O_POS_Y
from .scenes import VEL_X as O_VEL_X
from .scenes import VEL_Y as O_VEL_Y

MAX_GRAVITY = 4
_F = np.float32


# ---------------------------------------------------------------------------
# options (lib.zig:35-60, Constraint.zig:27-31)
# ---------------------------------------------------------------------------
class Vector2(NamedTuple):
    x: float = 0.0
    y: float = 0.0


@dataclasses.dataclass
class Density:
    """``mass_prop = .{ .density = d }``: mass from the area, in kg / m^2."""

    density: float


@dataclasses.dataclass
class Mass:
    """``mass_prop = .{ .mass = m }``."""

    mass: float


@dataclasses.dataclass
class BodyOptions:
    pos: Sequence[float]
    mass_prop: Density | Mass
    vel: Sequence[float] = (0.0, 0.0)
    angle: float = 0.0
    omega: float = 0.0
    mu: float = 0.5


@dataclasses.dataclass
class DiscOptions:
    radius: float = 1.0


@dataclasses.dataclass
class RectangleOptions:
    width: float = 1.0
    height: float = 0.5


@dataclasses.dataclass
class Parameters:
    """Constraint.Parameters: the power limits and the position-correction gain."""

    power_max: float = math.inf
    power_min: float = -math.inf
    beta: float = 10.0


# ---------------------------------------------------------------------------
# errors
# ---------------------------------------------------------------------------
class InvalidRigidBodyId(N.R2DError):
    """error.InvalidRigidBodyId: a joint names a body that does not exist
    (DistanceJoint.zig:44-47 and the other joints' solve functions)."""


class NoSuchIdExists(KeyError):
    """error.NoSuchIdExists from ``removeRigidBody`` (lib.zig:308-310)."""


class AABB(NamedTuple):
    """The body's stored AABB (aabb.zig:6-8), as the last substep left it."""

    pos: Vector2
    half_width: float
    half_height: float


# ---------------------------------------------------------------------------
# views of one body
# ---------------------------------------------------------------------------
def _state_vec(fx: int, fy: int):
    def get(self) -> Vector2:
        st = self._solver._host_state()
        return Vector2(float(st[fx, self._slot]), float(st[fy, self._slot]))

    def set(self, v) -> None:
        st = self._solver._mutable_state()
        st[fx, self._slot] = _F(v[0])
        st[fy, self._slot] = _F(v[1])

    return property(get, set)


def _state_scalar(f: int):
    def get(self) -> float:
        return float(self._solver._host_state()[f, self._slot])

    def set(self, v) -> None:
        self._solver._mutable_state()[f, self._slot] = _F(v)

    return property(get, set)


def _prop_scalar(f: int):
    def get(self) -> float:
        return float(self._solver._props[f, self._slot])

    def set(self, v) -> None:
        self._solver._pull()
        self._solver._props[f, self._slot] = _F(v)
        self._solver._bodies_dirty = True

    return property(get, set)


class Props:
    """RigidBody.Props (RigidBody.zig:67-81) of one body, read from and
    written to the solver's state.  Values are float32, as the reference's.
    Reads see the last frame; writes reach the engine at the next ``process``,
    all of a frame's writes in one upload."""

    def __init__(self, solver: "Solver", slot: int):
        self._solver = solver
        self._slot = slot

    pos = _state_vec(S_POS_X, S_POS_Y)
    momentum = _state_vec(S_MOM_X, S_MOM_Y)
    force = _state_vec(S_FORCE_X, S_FORCE_Y)
    angle = _state_scalar(S_ANGLE)
    ang_momentum = _state_scalar(S_ANG_MOM)
    torque = _state_scalar(S_TORQUE)
    mass = _prop_scalar(P_MASS)
    inertia = _prop_scalar(P_INERTIA)
    mu = _prop_scalar(P_MU)


class RigidBody:
    """The fields of one ``RigidBody`` (RigidBody.zig:83-90).  Like the
    reference's pointer, a view is valid until the next body is added or removed."""

    def __init__(self, solver: "Solver", slot: int):
        self._solver = solver
        self._slot = slot

    @property
    def id(self) -> int:
        return int(self._solver._ids[self._slot])

    @property
    def type(self) -> str:
        return "rectangle" if self._solver._kind[self._slot] & KIND_RECT else "disc"

    @property
    def static(self) -> bool:
        return bool(self._solver._kind[self._slot] & KIND_STATIC)

    @static.setter
    def static(self, on: bool) -> None:
        s = self._solver
        s._pull()
        k = int(s._kind[self._slot])
        s._kind[self._slot] = (k | KIND_STATIC) if on else (k & ~KIND_STATIC)
        s._bodies_dirty = True

    @property
    def props(self) -> Props:
        return Props(self._solver, self._slot)

    @property
    def aabb(self) -> AABB:
        st = self._solver._host_state()
        i = self._slot
        return AABB(Vector2(float(st[S_AABB_X, i]), float(st[S_AABB_Y, i])),
                    float(st[S_AABB_HW, i]), float(st[S_AABB_HH, i]))

    @property
    def radius(self) -> float:
        """Disc.radius (Disc.zig:8)."""
        return float(self._solver._props[P_DIM0, self._slot])

    @property
    def width(self) -> float:
        """Rectangle.width (Rectangle.zig:17)."""
        return float(self._solver._props[P_DIM0, self._slot])

    @property
    def height(self) -> float:
        """Rectangle.height (Rectangle.zig:18)."""
        return float(self._solver._props[P_DIM1, self._slot])


@dataclasses.dataclass(frozen=True)
class BodyHandle:
    """EntityFactory.BodyHandle (lib.zig:15-31): a body id and its solver."""

    id: int
    solver: "Solver"

    def body(self) -> RigidBody | None:
        slot = self.solver._slot_of.get(self.id)
        return None if slot is None else RigidBody(self.solver, slot)

    def body_unwrap(self) -> RigidBody:
        b = self.body()
        if b is None:
            raise LookupError("Tried to unwrap a null *RigidBody")
        return b


class ContactPoint(NamedTuple):
    """CollisionPoint (collision.zig:22-51): lever arms from the two bodies'
    centres at the start of the frame, depths and accumulated impulses."""

    ref_r: Vector2
    inc_r: Vector2
    depth: float
    original_depth: float
    mass_n: float
    mass_t: float
    accumulated_pn: float
    accumulated_pt: float


class Manifold(NamedTuple):
    """CollisionManifold (collision.zig:53-69) of the last frame, keyed by body
    ids, with the colour its constraint was solved in."""

    ref_id: int
    inc_id: int
    normal: Vector2
    tangent: Vector2
    friction: float
    points: tuple[ContactPoint, ...]
    colour: int


_P0, _PF = 9, 12  # first float of point 0 in a manifold row, floats per point


def _manifold(ids: np.ndarray, key, row, colour) -> Manifold:
    pts = []
    for p in range(2):
        if row[5 + p]:
            b = _P0 + _PF * p
            pts.append(ContactPoint(Vector2(float(row[b + 2]), float(row[b + 3])),
                                    Vector2(float(row[b + 4]), float(row[b + 5])),
                                    *(float(v) for v in row[b + 6: b + 12])))
    return Manifold(int(ids[key[0]]), int(ids[key[1]]), Vector2(float(row[0]), float(row[1])),
                    Vector2(float(row[2]), float(row[3])), float(row[4]), tuple(pts), int(colour))


class BodyMap(Mapping):
    """Solver.bodies (lib.zig:135): id -> RigidBody view, in map order."""

    def __init__(self, solver: "Solver"):
        self._solver = solver

    def __getitem__(self, id) -> RigidBody:
        slot = self._solver._slot_of.get(int(id))
        if slot is None:
            raise KeyError(id)
        return RigidBody(self._solver, slot)

    def __iter__(self) -> Iterator[int]:
        return iter(self._solver._ids[: self._solver._n].tolist())

    def __len__(self) -> int:
        return self._solver._n

    def count(self) -> int:
        """AutoArrayHashMap.count."""
        return len(self)


def _id(h) -> int:
    return int(h.id) if isinstance(h, BodyHandle) else int(h)


# ---------------------------------------------------------------------------
# EntityFactory (lib.zig:13-129)
# ---------------------------------------------------------------------------
class EntityFactory:
    """Creates bodies, gravity, joints and exclusions in a solver."""

    def __init__(self, solver: "Solver"):
        self.solver = solver

    def makeDiscBody(self, bo: BodyOptions, go: DiscOptions | None = None) -> BodyHandle:
        """lib.zig:73-82: m = pi*r*r*density (or the given mass), I = m*r*r/2,
        momentum = vel*m, angular momentum = omega*I."""
        go = go or DiscOptions()
        return self.solver._append(0, bo, go.radius, 0.0)

    def makeRectangleBody(self, bo: BodyOptions, go: RectangleOptions | None = None) -> BodyHandle:
        """lib.zig:84-93: m = w*h*density (or the given mass), I = m*(w*w + h*h)/12."""
        go = go or RectangleOptions()
        return self.solver._append(KIND_RECT, bo, go.width, go.height)

    def makeDownwardsGravity(self, g: float) -> None:
        """lib.zig:95-98: force (0, -m*g) on every non-static body each substep."""
        s = self.solver
        if len(s._gravity) >= MAX_GRAVITY:
            raise ValueError(f"at most {MAX_GRAVITY} DownwardsGravity generators")
        s._gravity.append(float(g))
        s._gravity_dirty = True

    def _joint(self, jtype: int, params: Parameters, a: int, b: int, extra: Sequence[float]) -> int:
        s = self.solver
        prm = [params.power_max, params.power_min, params.beta, *extra]
        prm += [0.0] * (JOINT_PARAMS - len(prm))
        s._jtype.append(jtype)
        s._jid1.append(a)
        s._jid2.append(b)
        s._jprm.append(prm)
        s._joints_dirty = True
        return len(s._jtype) - 1

    def makeOffsetDistanceJoint(self, params: Parameters, h1, h2, r1: Sequence[float], r2: Sequence[float],
                                target_distance: float) -> int:
        """lib.zig:100-104 (OffsetDistanceJoint.zig): r1, r2 in each body's frame."""
        return self._joint(JOINT_OFFSET_DISTANCE, params, _id(h1), _id(h2),
                           [r1[0], r1[1], r2[0], r2[1], target_distance])

    def makeDistanceJoint(self, params: Parameters, h1, h2, target_distance: float) -> int:
        """lib.zig:106-110 (DistanceJoint.zig)."""
        return self._joint(JOINT_DISTANCE, params, _id(h1), _id(h2), [target_distance])

    def makeFixedPositionJoint(self, params: Parameters, h, target_position: Sequence[float]) -> int:
        """lib.zig:112-116 (FixedPositionJoint.zig)."""
        i = _id(h)
        return self._joint(JOINT_FIXED_POSITION, params, i, i, [target_position[0], target_position[1]])

    def makeMotorJoint(self, params: Parameters, h, target_omega: float) -> int:
        """lib.zig:118-122 (MotorJoint.zig)."""
        i = _id(h)
        return self._joint(JOINT_MOTOR, params, i, i, [target_omega])

    def excludeCollisionPair(self, h1, h2) -> None:
        """lib.zig:124-129: the two bodies never form a manifold, in either order."""
        a, b = _id(h1), _id(h2)
        self.solver._excl[(min(a, b), max(a, b))] = None
        self.solver._excl_dirty = True


# ---------------------------------------------------------------------------
# Solver (lib.zig:131-314)
# ---------------------------------------------------------------------------
class Solver:
    """A world stepped on the GPU, built the way the reference builds one.

    ``engine_options`` go to ``engine.World`` (``warm_start``, ``sleep``,
    ``fp64_positions``, ``grid``, ``debug``, ``stream``, ``capacity_scale``).
    ``backend`` replaces the engine factory: a callable returning an object
    with ``World``'s ``set_bodies``, ``set_gravity``, ``set_joints``,
    ``set_exclusions``, ``write_state``, ``read_state``, ``process``, ``sync``
    and ``close``.
    """

    def __init__(self, spatialhash_cell_width: float = 4.0, spatialhash_table_size_mult: int = 2, *,
                 backend: Callable[[], object] | None = None, **engine_options):
        self.spatialhash_cell_width = float(spatialhash_cell_width)
        self.spatialhash_table_size_mult = int(spatialhash_table_size_mult)
        if backend is None:
            from .engine import World

            cell, mult = self.spatialhash_cell_width, self.spatialhash_table_size_mult
            backend = lambda: World(cell, mult, **engine_options)  # noqa: E731
        self._factory = backend
        self._dev = None
        self.current_body_id = 0
        self._reset()

    @classmethod
    def init(cls, spatialhash_cell_width: float = 4.0, spatialhash_table_size_mult: int = 2, **kw) -> "Solver":
        """Solver.init (lib.zig:145-157)."""
        return cls(spatialhash_cell_width, spatialhash_table_size_mult, **kw)

    def _reset(self) -> None:
        cap = 64
        self._n = 0
        self._ids = np.zeros(cap, np.uint32)
        self._kind = np.zeros(cap, np.uint8)
        self._props = np.zeros((NPROP, cap), np.float32)
        self._state = np.zeros((NSTATE, cap), np.float32)
        self._fresh = np.zeros(cap, bool)
        self._slot_of: dict[int, int] = {}
        self._gravity: list[float] = []
        self._jtype: list[int] = []
        self._jid1: list[int] = []
        self._jid2: list[int] = []
        self._jprm: list[list[float]] = []
        self._excl: dict[tuple[int, int], None] = {}
        self._bodies_dirty = self._state_dirty = self._host_stale = False
        self._gravity_dirty = self._joints_dirty = self._excl_dirty = True
        self._frame_ids = None

    def deinit(self) -> None:
        """Solver.deinit (lib.zig:159-179): releases the device engine too."""
        if self._dev is not None and hasattr(self._dev, "close"):
            self._dev.close()
        self._dev = None
        self._reset()

    def clear(self) -> None:
        """Solver.clear (lib.zig:181-187): drops every body, force generator,
        constraint and exclusion; ids keep counting from ``current_body_id``."""
        self._reset()
        self._bodies_dirty = True

    def entityFactory(self) -> EntityFactory:
        return EntityFactory(self)

    def bodyHandle(self, id: int) -> BodyHandle:
        """lib.zig:301-306: a handle; whether the body exists is asked by ``body()``."""
        return BodyHandle(int(id), self)

    def removeRigidBody(self, id: int) -> None:
        """lib.zig:308-310: the last body moves into the removed body's slot."""
        if int(id) not in self._slot_of:
            raise NoSuchIdExists(int(id))
        self._pull()
        slot = self._slot_of.pop(int(id))
        last = self._n - 1
        if slot != last:
            moved = int(self._ids[last])
            self._ids[slot] = self._ids[last]
            self._kind[slot] = self._kind[last]
            self._props[:, slot] = self._props[:, last]
            self._state[:, slot] = self._state[:, last]
            self._fresh[slot] = self._fresh[last]
            self._slot_of[moved] = slot
        self._n = last
        self._bodies_dirty = True

    @property
    def num_bodies(self) -> int:
        return self._n

    @property
    def bodies(self) -> BodyMap:
        """The bodies by id, in map order (insertion order, ``swapRemove`` on removal)."""
        return BodyMap(self)

    def manifolds(self) -> list[Manifold]:
        """Solver.manifolds (lib.zig:137) of the last frame.  Needs the engine's
        debug taps: ``Solver(debug=True)``."""
        if self._dev is None or self._frame_ids is None:
            return []
        keys, data, colours = self._dev.manifolds()
        return [_manifold(self._frame_ids, keys[m], data[m], colours[m]) for m in range(keys.shape[0])]

    def ids(self) -> np.ndarray:
        """Body ids in map order."""
        return self._ids[: self._n].copy()

    def read_state(self) -> np.ndarray:
        """The state of every body in map order, float32 [13][n] (fields of include/r2d_gb300.h)."""
        return self._host_state().copy()

    def process(self, dt: float, sub_steps: int, collision_iters: int) -> None:
        """Solver.process (lib.zig:189-251): one frame.  Raises
        InvalidRigidBodyId, with nothing stepped, when a joint names a missing body."""
        if self._n == 0:
            return
        self._flush()
        try:
            self._dev.process(float(dt), int(sub_steps), int(collision_iters))
        except N.R2DError as e:
            if e.code == -2:
                raise InvalidRigidBodyId(e.code, "Solver.process", str(e)) from e
            raise
        self._host_stale = True
        self._frame_ids = self._ids[: self._n].copy()  # the order the frame's manifold keys index

    def sync(self) -> None:
        """Waits for the frames in flight and raises the first device-side error."""
        if self._dev is not None:
            self._dev.sync()

    # -- host copy of the bodies -------------------------------------------
    def _pull(self) -> None:
        if self._host_stale:
            self._state[:, : self._n] = self._dev.read_state()
            self._host_stale = False

    def _host_state(self) -> np.ndarray:
        self._pull()
        return self._state[:, : self._n]

    def _mutable_state(self) -> np.ndarray:
        self._pull()
        self._state_dirty = True
        return self._state

    def _grow(self) -> None:
        cap = 2 * self._ids.shape[0]
        self._ids = np.resize(self._ids, cap)
        self._kind = np.resize(self._kind, cap)
        self._fresh = np.resize(self._fresh, cap)
        for name in ("_props", "_state"):
            old = getattr(self, name)
            new = np.zeros((old.shape[0], cap), np.float32)
            new[:, : self._n] = old[:, : self._n]
            setattr(self, name, new)

    def _append(self, shape_kind: int, bo: BodyOptions, dim0: float, dim1: float) -> BodyHandle:
        self._pull()
        if self._n == self._ids.shape[0]:
            self._grow()
        kind = shape_kind
        if isinstance(bo.mass_prop, Density):
            kind |= KIND_DENSITY
            mass_prop = bo.mass_prop.density
        elif isinstance(bo.mass_prop, Mass):
            mass_prop = bo.mass_prop.mass
        else:
            raise TypeError("mass_prop must be Density(...) or Mass(...)")
        opt = np.zeros((NOPT, 1), np.float32)
        opt[O_POS_X, 0], opt[O_POS_Y, 0] = bo.pos[0], bo.pos[1]
        opt[O_ANGLE, 0] = bo.angle
        opt[O_VEL_X, 0], opt[O_VEL_Y, 0] = bo.vel[0], bo.vel[1]
        opt[O_OMEGA, 0] = bo.omega
        opt[O_MU, 0] = bo.mu
        opt[MASS_PROP, 0] = mass_prop
        opt[DIM0, 0], opt[DIM1, 0] = dim0, dim1
        props, state = derive_props_state(np.array([kind], np.uint8), opt)
        i, bid = self._n, self.current_body_id
        self._ids[i] = bid
        self._kind[i] = shape_kind
        self._props[:, i] = props[:, 0]
        self._state[:, i] = state[:, 0]
        self._fresh[i] = True
        self._slot_of[bid] = i
        self._n += 1
        self.current_body_id += 1
        self._bodies_dirty = True
        return BodyHandle(bid, self)

    def _flush(self) -> None:
        """Hands what changed since the last frame to the engine.  New bodies
        get their first AABB from the engine (RigidBody.updateAABB at creation);
        bodies that were there keep the AABB the last substep left them."""
        if self._dev is None:
            self._dev = self._factory()
            self._bodies_dirty = self._gravity_dirty = self._joints_dirty = self._excl_dirty = True
        d, n = self._dev, self._n
        if self._gravity_dirty:
            d.set_gravity(np.array(self._gravity, np.float32))
            self._gravity_dirty = False
        if self._bodies_dirty:
            ids = self._ids[:n].copy()
            kind = self._kind[:n].copy()
            props = np.ascontiguousarray(self._props[:, :n])
            st = np.ascontiguousarray(self._state[:, :n])
            fresh = self._fresh[:n].copy()
            if fresh.any():
                d.set_bodies(ids, kind, props, st, init_aabb=True)
                got = d.read_state()
                if not fresh.all():
                    for f in (S_AABB_X, S_AABB_Y, S_AABB_HW, S_AABB_HH):
                        got[f, ~fresh] = st[f, ~fresh]
                    d.write_state(got)
                self._state[:, :n] = got
            else:
                d.set_bodies(ids, kind, props, st, init_aabb=False)
            self._fresh[:n] = False
            self._bodies_dirty = self._state_dirty = False
        elif self._state_dirty:
            d.write_state(np.ascontiguousarray(self._state[:, :n]))
            self._state_dirty = False
        if self._joints_dirty:
            nj = len(self._jtype)
            d.set_joints(np.array(self._jtype, np.uint8), np.array(self._jid1, np.uint32),
                         np.array(self._jid2, np.uint32),
                         np.array(self._jprm, np.float32).reshape(nj, JOINT_PARAMS))
            self._joints_dirty = False
        if self._excl_dirty:
            d.set_exclusions(np.array(list(self._excl), np.uint32).reshape(-1, 2))
            self._excl_dirty = False


# ---------------------------------------------------------------------------
# many scenes at once
# ---------------------------------------------------------------------------
def batch_arrays(solvers: Sequence[Solver]):
    """The bodies of several solvers as one batch's arrays: (body_off, ids,
    kind, props, state, gravity).  Each solver becomes one world; worlds keep
    the solvers' order and their own ids.

    The batch entry points take one DownwardsGravity per world and no joints or
    exclusions, and they compute every first AABB or none.  So each solver must
    have at most one gravity generator, no joints and no exclusions, and either
    all the solvers have stepped or none has."""
    fresh = set()
    for s in solvers:
        if len(s._gravity) > 1 or s._jtype or s._excl:
            raise ValueError("a batched world has at most one gravity generator and no joints or exclusions")
        s._pull()
        if s._n:
            fresh.add(bool(s._fresh[: s._n].all()))
            if s._fresh[: s._n].any() and not s._fresh[: s._n].all():
                raise ValueError("a solver holds both new and stepped bodies; step it once first")
    if len(fresh) > 1:
        raise ValueError("either every solver has stepped or none has")
    counts = [s._n for s in solvers]
    body_off = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    ids = np.concatenate([s._ids[: s._n] for s in solvers]) if solvers else np.zeros(0, np.uint32)
    kind = np.concatenate([s._kind[: s._n] for s in solvers]) if solvers else np.zeros(0, np.uint8)
    props = np.concatenate([s._props[:, : s._n] for s in solvers], axis=1) if solvers else np.zeros((NPROP, 0))
    state = np.concatenate([s._state[:, : s._n] for s in solvers], axis=1) if solvers else np.zeros((NSTATE, 0))
    gravity = np.array([s._gravity[0] if s._gravity else 0.0 for s in solvers], np.float32)
    return (body_off, ids.astype(np.uint32), kind.astype(np.uint8), np.ascontiguousarray(props, np.float32),
            np.ascontiguousarray(state, np.float32), gravity, fresh == {True})


def batch(solvers: Sequence[Solver], **engine_options):
    """Independent worlds built with the reference's API, stepped together:
    an ``engine.Batch`` holding one world per solver (see ``batch_arrays``).
    The solvers themselves are not changed."""
    from .engine import Batch

    body_off, ids, kind, props, state, gravity, init_aabb = batch_arrays(solvers)
    b = Batch(**engine_options)
    b.set_worlds(body_off, ids, kind, props, state, gravity, init_aabb=init_aabb)
    return b

"""Seeded synthetic scenes for the benchmark configurations and the tests.

The reference ships no benchmark scenes, so the scenes are generated here
from fixed seeds with numpy's PCG64 generator (``numpy.random.default_rng``),
which gives the same stream on every platform.  Every body is described the
way the reference's ``EntityFactory`` takes it (``BodyOptions`` +
``DiscOptions`` / ``RectangleOptions``, src/core/lib.zig:35-60); mass,
inertia and momenta are then derived by :func:`derive_props_state`, a
restatement of ``makeDiscBody`` / ``makeRectangleBody`` (lib.zig:73-93,
Disc.zig:29-56, Rectangle.zig:33-64) in float32.

Decisions the configuration text leaves open are fixed here and recorded in
each builder's docstring.
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np

# body option fields, float32 field-major [NOPT][n]
POS_X, POS_Y, ANGLE, VEL_X, VEL_Y, OMEGA, MU, MASS_PROP, DIM0, DIM1 = range(10)
NOPT = 10
# kind bits (KIND_POLY: a convex polygon, whose vertices are Scene.poly_v;
# its opt MASS_PROP is its mass and DIM1 its inertia, DIM0 its bounding radius)
KIND_RECT, KIND_STATIC, KIND_DENSITY, KIND_POLY = 1, 2, 4, 8
MAX_POLY_VERTS = 8
# state / prop fields (include/r2d_gb300.h)
NSTATE, NPROP = 13, 5
S_POS_X, S_POS_Y, S_ANGLE, S_MOM_X, S_MOM_Y, S_ANG_MOM = range(6)
S_FORCE_X, S_FORCE_Y, S_TORQUE, S_AABB_X, S_AABB_Y, S_AABB_HW, S_AABB_HH = range(6, 13)
P_MASS, P_INERTIA, P_MU, P_DIM0, P_DIM1 = range(5)
# joint types (Constraint.Type, src/core/Constraints/Constraint.zig:15-20)
JOINT_DISTANCE, JOINT_OFFSET_DISTANCE, JOINT_FIXED_POSITION, JOINT_MOTOR = range(4)
JOINT_PARAMS = 8
INF = np.float32(np.inf)


@dataclasses.dataclass
class Scene:
    """Bodies of one or many worlds plus their forces and constraints."""

    name: str
    ids: np.ndarray        # u32 [n]  (ids restart at 0 in every world)
    kind: np.ndarray       # u8  [n]  KIND_* bits
    opt: np.ndarray        # f32 [NOPT][n]
    body_off: np.ndarray   # u32 [W+1]
    gravity: np.ndarray    # f32 [W]  one DownwardsGravity per world (0 = none)
    dt: float
    sub_steps: int
    iters: int
    steps: int
    jworld: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.uint32))
    jtype: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.uint8))
    jid1: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.uint32))
    jid2: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.uint32))
    jprm: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, JOINT_PARAMS), np.float32))
    xworld: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.uint32))
    xpairs: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 2), np.uint32))
    # convex polygons: vertex counts [n] (0 for other bodies) and local
    # vertices [n][MAX_POLY_VERTS][2], clockwise about the body's origin;
    # empty arrays when the scene has none
    poly_nv: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.uint8))
    poly_v: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, MAX_POLY_VERTS, 2), np.float32))

    @property
    def has_polygons(self) -> bool:
        return bool(self.poly_nv.size) and bool((self.poly_nv > 0).any())

    def _poly_rows(self, rows):
        if not self.poly_nv.size:
            return {}
        return {"poly_nv": self.poly_nv[rows].copy(), "poly_v": self.poly_v[rows].copy()}

    @property
    def nworlds(self) -> int:
        return len(self.body_off) - 1

    @property
    def nbodies(self) -> int:
        return int(self.body_off[-1])

    def world(self, w: int) -> "Scene":
        """The single world ``w`` as its own scene."""
        b0, b1 = int(self.body_off[w]), int(self.body_off[w + 1])
        jm = self.jworld == w
        xm = self.xworld == w
        return Scene(
            name=f"{self.name}[{w}]",
            ids=self.ids[b0:b1].copy(),
            kind=self.kind[b0:b1].copy(),
            opt=self.opt[:, b0:b1].copy(),
            body_off=np.array([0, b1 - b0], np.uint32),
            gravity=self.gravity[w : w + 1].copy(),
            dt=self.dt, sub_steps=self.sub_steps, iters=self.iters, steps=self.steps,
            jworld=np.zeros(int(jm.sum()), np.uint32), jtype=self.jtype[jm], jid1=self.jid1[jm],
            jid2=self.jid2[jm], jprm=self.jprm[jm],
            xworld=np.zeros(int(xm.sum()), np.uint32), xpairs=self.xpairs[xm],
            **self._poly_rows(slice(b0, b1)),
        )

    def worlds(self, w0: int, w1: int) -> "Scene":
        """Worlds ``w0 .. w1-1`` as their own (joint-free) scene."""
        if self.jtype.size or self.xpairs.size:
            raise ValueError("joint-free scenes only")
        b0, b1 = int(self.body_off[w0]), int(self.body_off[w1])
        return Scene(
            name=f"{self.name}[{w0}:{w1}]",
            ids=self.ids[b0:b1].copy(),
            kind=self.kind[b0:b1].copy(),
            opt=self.opt[:, b0:b1].copy(),
            body_off=(self.body_off[w0 : w1 + 1] - self.body_off[w0]).astype(np.uint32),
            gravity=self.gravity[w0:w1].copy(),
            dt=self.dt, sub_steps=self.sub_steps, iters=self.iters, steps=self.steps,
            **self._poly_rows(slice(b0, b1)),
        )

    def select(self, worlds) -> "Scene":
        """The worlds at the given indices, in that order, as their own
        (joint-free) scene."""
        if self.jtype.size or self.xpairs.size:
            raise ValueError("joint-free scenes only")
        worlds = np.asarray(worlds, np.int64)
        spans = [np.arange(self.body_off[w], self.body_off[w + 1]) for w in worlds]
        rows = np.concatenate(spans) if spans else np.zeros(0, np.int64)
        sizes = np.array([len(sp) for sp in spans], np.int64)
        return Scene(
            name=f"{self.name}[{len(worlds)} worlds]",
            ids=self.ids[rows].copy(),
            kind=self.kind[rows].copy(),
            opt=np.ascontiguousarray(self.opt[:, rows]),
            body_off=np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32),
            gravity=self.gravity[worlds].copy(),
            dt=self.dt, sub_steps=self.sub_steps, iters=self.iters, steps=self.steps,
            **self._poly_rows(rows),
        )

    def body_radius(self) -> np.ndarray:
        """Size of each body for error figures: a disc's radius, half the
        shorter side of a rectangle."""
        rect = (self.kind & KIND_RECT) != 0
        r = np.where(rect, 0.5 * np.minimum(self.opt[DIM0], self.opt[DIM1]), self.opt[DIM0]).astype(np.float64)
        if self.has_polygons:  # a polygon: its smallest vertex distance
            for i in np.flatnonzero(self.poly_nv):
                v = self.poly_v[i, : self.poly_nv[i]].astype(np.float64)
                r[i] = float(np.min(np.hypot(v[:, 0], v[:, 1])))
        return r


def derive_props_state(kind: np.ndarray, opt: np.ndarray):
    """Mass, inertia and initial momenta of new bodies, in float32.

    Restates EntityFactory.makeDiscBody / makeRectangleBody (lib.zig:73-93):
    disc m = pi*r*r*density, I = 0.5*m*r*r (Disc.zig:42); rectangle
    m = w*h*density, I = m*(w*w + h*h)/12 (Rectangle.zig:51); momentum =
    vel*m, angular momentum = omega*I.  Each product is evaluated left to
    right in float32, as Zig evaluates it.  Returns (props [5][n],
    state [13][n]) with zero force/torque and zero AABB (the AABB is computed
    by whoever creates the bodies, as RigidBody.updateAABB does at init).
    """
    f = np.float32
    n = kind.shape[0]
    poly = (kind & KIND_POLY) != 0
    rect = ((kind & KIND_RECT) != 0) & ~poly
    dens = (kind & KIND_DENSITY) != 0
    d0, d1, mp = opt[DIM0].astype(f), opt[DIM1].astype(f), opt[MASS_PROP].astype(f)
    pi32 = f(math.pi)
    disc_mass = ((pi32 * d0) * d0) * mp
    rect_mass = (d0 * d1) * mp
    mass = np.where(dens & ~poly, np.where(rect, rect_mass, disc_mass), mp).astype(f)
    disc_i = ((f(0.5) * mass) * d0) * d0
    rect_i = (mass * ((d0 * d0) + (d1 * d1))) / f(12)
    inertia = np.where(poly, d1, np.where(rect, rect_i, disc_i)).astype(f)
    props = np.zeros((NPROP, n), f)
    props[P_MASS] = mass
    props[P_INERTIA] = inertia
    props[P_MU] = opt[MU]
    props[P_DIM0] = d0
    props[P_DIM1] = np.where(rect | poly, d1, f(0))
    state = np.zeros((NSTATE, n), f)
    state[S_POS_X] = opt[POS_X]
    state[S_POS_Y] = opt[POS_Y]
    state[S_ANGLE] = opt[ANGLE]
    state[S_MOM_X] = opt[VEL_X] * mass
    state[S_MOM_Y] = opt[VEL_Y] * mass
    state[S_ANG_MOM] = opt[OMEGA] * inertia
    return props, state


class _Builder:
    """Appends bodies of one world in EntityFactory order (ids from 0)."""

    def __init__(self):
        self.rows: list[tuple] = []
        self.polys: dict[int, tuple] = {}

    def disc(self, x, y, r, mu, density=1.0, vx=0.0, vy=0.0, angle=0.0, omega=0.0, static=False):
        k = KIND_DENSITY | (KIND_STATIC if static else 0)
        self.rows.append((k, x, y, angle, vx, vy, omega, mu, density, r, 0.0))
        return len(self.rows) - 1

    def rect(self, x, y, w, h, mu, density=1.0, vx=0.0, vy=0.0, angle=0.0, omega=0.0, static=False):
        k = KIND_RECT | KIND_DENSITY | (KIND_STATIC if static else 0)
        self.rows.append((k, x, y, angle, vx, vy, omega, mu, density, w, h))
        return len(self.rows) - 1

    def polygon(self, x, y, verts, mu, density=1.0, vx=0.0, vy=0.0, angle=0.0, omega=0.0, static=False):
        """A convex polygon of uniform density: `verts` (k x 2, 3 <= k <= 8)
        about any point; they are shifted to the centroid, ordered
        clockwise, and the mass and inertia integrated over the shape
        (float64, then float32)."""
        v = np.asarray(verts, np.float64).reshape(-1, 2)
        k = v.shape[0]
        if not 3 <= k <= MAX_POLY_VERTS:
            raise ValueError(f"a polygon has 3 to {MAX_POLY_VERTS} vertices, not {k}")
        c = v.mean(axis=0)
        v = v[np.argsort(-np.arctan2(v[:, 1] - c[1], v[:, 0] - c[0]), kind="stable")]  # clockwise
        x0, y0, x1, y1 = v[:, 0], v[:, 1], np.roll(v[:, 0], -1), np.roll(v[:, 1], -1)
        cr = x0 * y1 - x1 * y0
        area = 0.5 * cr.sum()
        cx = ((x0 + x1) * cr).sum() / (6.0 * area)
        cy = ((y0 + y1) * cr).sum() / (6.0 * area)
        v = v - np.array([cx, cy])
        x0, y0, x1, y1 = v[:, 0], v[:, 1], np.roll(v[:, 0], -1), np.roll(v[:, 1], -1)
        cr = x0 * y1 - x1 * y0
        area = abs(0.5 * cr.sum())
        second = abs((cr * (x0 * x0 + x0 * x1 + x1 * x1 + y0 * y0 + y0 * y1 + y1 * y1)).sum()) / 12.0
        mass = density * area
        inertia = density * second
        bound = float(np.max(np.hypot(v[:, 0], v[:, 1])))
        kd = KIND_POLY | (KIND_STATIC if static else 0)
        self.rows.append((kd, x, y, angle, vx, vy, omega, mu, mass, bound, inertia))
        pv = np.zeros((MAX_POLY_VERTS, 2), np.float32)
        pv[:k] = v
        self.polys[len(self.rows) - 1] = (k, pv)
        return len(self.rows) - 1

    def polygon_arrays(self):
        """(poly_nv [n], poly_v [n][8][2]) of the bodies added so far."""
        n = len(self.rows)
        nv = np.zeros(n, np.uint8)
        pv = np.zeros((n, MAX_POLY_VERTS, 2), np.float32)
        for i, (k, v) in self.polys.items():
            nv[i] = k
            pv[i] = v
        return nv, pv

    def arrays(self):
        n = len(self.rows)
        kind = np.array([r[0] for r in self.rows], np.uint8).reshape(n)
        opt = np.array([r[1:] for r in self.rows], np.float64).reshape(n, NOPT).T.astype(np.float32)
        return np.arange(n, dtype=np.uint32), kind, np.ascontiguousarray(opt)


def _concat(name, worlds, gravity, dt, sub_steps, iters, steps, joints=None, excl=None, polys=None) -> Scene:
    ids, kinds, opts, off = [], [], [], [0]
    for (i, k, o) in worlds:
        ids.append(i)
        kinds.append(k)
        opts.append(o)
        off.append(off[-1] + len(i))
    sc = Scene(
        name=name,
        ids=np.concatenate(ids).astype(np.uint32),
        kind=np.concatenate(kinds).astype(np.uint8),
        opt=np.ascontiguousarray(np.concatenate(opts, axis=1).astype(np.float32)),
        body_off=np.array(off, np.uint32),
        gravity=np.asarray(gravity, np.float32),
        dt=float(dt), sub_steps=int(sub_steps), iters=int(iters), steps=int(steps),
    )
    if joints is not None:
        sc.jworld, sc.jtype, sc.jid1, sc.jid2, sc.jprm = joints
    if excl is not None:
        sc.xworld, sc.xpairs = excl
    if polys is not None:  # one (poly_nv, poly_v) per world
        sc.poly_nv = np.concatenate([p[0] for p in polys]).astype(np.uint8)
        sc.poly_v = np.ascontiguousarray(np.concatenate([p[1] for p in polys]).astype(np.float32))
    return sc


def _grid_world(rng, n, n_cols, disc_p, spacing, jitter, disc_r, rect_wh, mu, ground_w,
                types=None):
    """A static ground box (width ground_w, height 1, top at y = 0) and n bodies
    on a jittered grid: n_cols columns centred on x = 0, bottom row one
    spacing above the ground top, rows filled bottom-up, left to right."""
    b = _Builder()
    b.rect(0.0, -0.5, ground_w, 1.0, mu, static=True)
    if types is None:
        types = rng.random(n) < disc_p
    for k in range(n):
        row, col = divmod(k, n_cols)
        x = (col - (n_cols - 1) / 2.0) * spacing + rng.uniform(-jitter, jitter)
        y = spacing * (row + 1) + rng.uniform(-jitter, jitter)
        if types[k]:
            b.disc(x, y, rng.uniform(*disc_r), mu)
        else:
            b.rect(x, y, rng.uniform(*rect_wh), rng.uniform(*rect_wh), mu)
    return b.arrays()


def config0(seed: int = 0) -> Scene:
    """Plain, small: 150 discs (r ~ U[0.2,0.5]) + 50 rectangles (w,h ~ U[0.3,1.0]),
    density 1, mu 0.4, on a jittered 20x10 grid (spacing 1.2, jitter U[-0.1,0.1])
    above a static 40x1 ground box; g = 9.81, dt = 1/60, 8 iterations, 600 steps.
    Decisions: the ground is body 0 with its top at y = 0; disc/rectangle slots
    come from a seeded shuffle of the 200 slots; the bottom row is 1.2 above the
    ground top; angles and velocities start at 0."""
    rng = np.random.default_rng(seed)
    types = rng.permutation(np.array([True] * 150 + [False] * 50))
    w = _grid_world(rng, 200, 20, 0.75, 1.2, 0.1, (0.2, 0.5), (0.3, 1.0), 0.4, 40.0, types=types)
    return _concat("config0", [w], [9.81], 1 / 60, 1, 8, 600)


def config1(seed: int = 1) -> Scene:
    """Plain, dense stacking: 10,000 1x1 boxes in a pyramid + 2,000 discs
    (r ~ U[0.3,0.5]) over a static 120x1 ground; mu 0.5, g = 9.81, dt = 1/60,
    10 iterations, 1,000 steps.
    Decisions: a 100-wide pyramid of single rows holds 5,050 boxes, so rows have
    widths 100,100,99,99,... (each width twice), centred and touching, filled to
    exactly 10,000 (the last row is partial and centred); disc x ~ U over the
    base width; disc heights are U[60,120] above the pyramid's top so that no
    disc starts inside it."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    b.rect(0.0, -0.5, 120.0, 1.0, 0.5, static=True)
    placed, row, width = 0, 0, 100
    while placed < 10000:
        cnt = min(width, 10000 - placed)
        for c in range(cnt):
            b.rect((c - (cnt - 1) / 2.0) * 1.0, 0.5 + row, 1.0, 1.0, 0.5)
        placed += cnt
        row += 1
        if row % 2 == 0:
            width -= 1
    top = 0.5 + row
    for _ in range(2000):
        b.disc(rng.uniform(-50.0, 50.0), top + rng.uniform(60.0, 120.0), rng.uniform(0.3, 0.5), 0.5)
    return _concat("config1", [b.arrays()], [9.81], 1 / 60, 1, 10, 1000)


def config2(seed: int = 2, n_bodies: int = 200_000, n_chains: int = 5000, chain_links: int = 20,
            n_motors: int = 2000, box_w: float = 2000.0, box_h: float = 500.0) -> Scene:
    """Plain, large with constraints: 200,000 bodies (70% discs r ~ U[0.1,0.4],
    30% rectangles w,h ~ U[0.2,0.8]) uniform in a 2000x500 box with 4 static
    walls, v ~ N(0,1); 5,000 chains of 20 distance joints (rest 0.5), 2,000
    motors (power limit +-50, target omega ~ U[-5,5], beta 10); dt = 1/120,
    8 iterations, 300 steps.
    Decisions: walls are bodies 0-3; a chain is 21 consecutive-id discs laid on
    a line at spacing 0.5 from a uniform start in a uniform direction, with
    excludeCollisionPair between neighbours; chain discs come first, the other
    bodies follow in a seeded shuffle; motors drive distinct non-chain bodies;
    mu = 0.5 (the BodyOptions default), g = 9.81, density 1; overlaps at the
    start are allowed (the solver resolves them)."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    hw, hh = box_w / 2.0, box_h
    b.rect(0.0, -0.5, box_w + 2.0, 1.0, 0.5, static=True)
    b.rect(0.0, hh + 0.5, box_w + 2.0, 1.0, 0.5, static=True)
    b.rect(-hw - 0.5, hh / 2.0, 1.0, hh, 0.5, static=True)
    b.rect(hw + 0.5, hh / 2.0, 1.0, hh, 0.5, static=True)
    n_disc = int(round(0.7 * n_bodies))
    per_chain = chain_links + 1
    n_chain_discs = n_chains * per_chain
    jt, j1, j2, jp, xp = [], [], [], [], []
    for c in range(n_chains):
        th = rng.uniform(0, 2 * math.pi)
        dx, dy = math.cos(th) * 0.5, math.sin(th) * 0.5
        span = 0.5 * chain_links
        x0 = rng.uniform(-hw + span + 1, hw - span - 1)
        y0 = rng.uniform(span + 1, hh - span - 1)
        first = len(b.rows)
        for k in range(per_chain):
            b.disc(x0 + dx * k, y0 + dy * k, rng.uniform(0.1, 0.4), 0.5,
                   vx=rng.normal(), vy=rng.normal())
        for k in range(chain_links):
            jt.append(JOINT_DISTANCE)
            j1.append(first + k)
            j2.append(first + k + 1)
            jp.append([INF, -INF, 10.0, 0.5, 0, 0, 0, 0])
            xp.append((first + k, first + k + 1))
    rest_types = np.array([True] * (n_disc - n_chain_discs) + [False] * (n_bodies - n_disc))
    rest_types = rng.permutation(rest_types)
    rest_first = len(b.rows)
    for is_disc in rest_types:
        x = rng.uniform(-hw + 0.5, hw - 0.5)
        y = rng.uniform(0.5, hh - 0.5)
        if is_disc:
            b.disc(x, y, rng.uniform(0.1, 0.4), 0.5, vx=rng.normal(), vy=rng.normal())
        else:
            b.rect(x, y, rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8), 0.5, vx=rng.normal(), vy=rng.normal())
    motor_bodies = rng.choice(np.arange(rest_first, len(b.rows)), size=n_motors, replace=False)
    for mb in motor_bodies:
        jt.append(JOINT_MOTOR)
        j1.append(int(mb))
        j2.append(int(mb))
        jp.append([50.0, -50.0, 10.0, rng.uniform(-5, 5), 0, 0, 0, 0])
    joints = (np.zeros(len(jt), np.uint32), np.array(jt, np.uint8), np.array(j1, np.uint32),
              np.array(j2, np.uint32), np.array(jp, np.float32).reshape(-1, JOINT_PARAMS))
    excl = (np.zeros(len(xp), np.uint32), np.array(xp, np.uint32).reshape(-1, 2))
    return _concat("config2", [b.arrays()], [9.81], 1 / 120, 1, 8, 300, joints=joints, excl=excl)


def batched_worlds(name: str, seed: int, nworlds: int, steps: int, lo: int = 16, hi: int = 512) -> Scene:
    """Independent worlds: body counts log-uniform in [lo, hi] (rounded),
    60/40 disc/rectangle (per-body Bernoulli), sizes and grid as config 0
    (20 columns, rows = ceil(n/20)), each with its own 40x1 static ground and
    gravity g ~ U[5,15]; mu 0.4, dt = 1/60, 8 iterations.  The ground is not
    counted in n."""
    rng = np.random.default_rng(seed)
    counts = np.rint(np.exp(rng.uniform(math.log(lo), math.log(hi), nworlds))).astype(int)
    grav = rng.uniform(5.0, 15.0, nworlds)
    worlds = [_grid_world(rng, int(c), 20, 0.6, 1.2, 0.1, (0.2, 0.5), (0.3, 1.0), 0.4, 40.0) for c in counts]
    return _concat(name, worlds, grav, 1 / 60, 1, 8, steps)


def config3(seed: int = 3, nworlds: int = 4096) -> Scene:
    """Batched: 4,096 worlds (see batched_worlds), 600 steps."""
    return batched_worlds("config3", seed, nworlds, 600)


def config4(seed: int = 4, nworlds: int = 16384) -> Scene:
    """Precision study: 16,384 worlds of the config-3 distribution, 3,600 steps."""
    return batched_worlds("config4", seed, nworlds, 3600)


def random_scene(seed: int, n: int = 40, rect_p: float = 0.5, box: float = 8.0, static_p: float = 0.1,
                 spin: bool = True, joints: bool = False) -> Scene:
    """Small random world for property tests: overlapping discs/rectangles of
    mixed sizes with random angles and velocities, some static, optional joints."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    b.rect(0.0, -0.5, 3 * box, 1.0, 0.5, static=True)
    for _ in range(n):
        x, y = rng.uniform(-box, box), rng.uniform(0.0, box)
        st = rng.random() < static_p
        vx, vy = (0.0, 0.0) if st else (rng.normal(), rng.normal())
        ang = rng.uniform(-math.pi, math.pi) if spin else 0.0
        om = rng.normal() if spin else 0.0
        mu = rng.uniform(0.1, 0.9)
        if rng.random() < rect_p:
            b.rect(x, y, rng.uniform(0.3, 2.0), rng.uniform(0.3, 2.0), mu, vx=vx, vy=vy, angle=ang, omega=om, static=st)
        else:
            b.disc(x, y, rng.uniform(0.2, 1.0), mu, vx=vx, vy=vy, angle=ang, omega=om, static=st)
    js = None
    if joints:
        dyn = np.array([i for i, r in enumerate(b.rows) if not (r[0] & KIND_STATIC)])
        jt, j1, j2, jp = [], [], [], []
        for _ in range(max(1, n // 4)):
            a, c = rng.choice(dyn, 2, replace=False)
            t = int(rng.integers(0, 4))
            pmax = float(rng.choice([np.inf, rng.uniform(1, 50)]))
            prm = [pmax, -pmax, float(rng.uniform(1, 20)), 0, 0, 0, 0, 0]
            if t == JOINT_DISTANCE:
                prm[3] = float(rng.uniform(0.5, 3))
            elif t == JOINT_OFFSET_DISTANCE:
                prm[3:8] = [rng.uniform(-.3, .3), rng.uniform(-.3, .3), rng.uniform(-.3, .3),
                            rng.uniform(-.3, .3), rng.uniform(0.5, 3)]
            elif t == JOINT_FIXED_POSITION:
                prm[3:5] = [rng.uniform(-box, box), rng.uniform(0, box)]
            else:
                prm[3] = float(rng.uniform(-5, 5))
            jt.append(t)
            j1.append(int(a))
            j2.append(int(c))
            jp.append(prm)
        js = (np.zeros(len(jt), np.uint32), np.array(jt, np.uint8), np.array(j1, np.uint32),
              np.array(j2, np.uint32), np.array(jp, np.float32).reshape(-1, JOINT_PARAMS))
    return _concat(f"random{seed}", [b.arrays()], [9.81], 1 / 60, 1, 8, 60, joints=js)


def random_polygon(rng, r_lo=0.3, r_hi=1.0):
    """A random convex polygon of 3 to 8 vertices: points at jittered, evenly
    spaced angles on a circle (so every vertex is a corner of the hull)."""
    k = int(rng.integers(3, MAX_POLY_VERTS + 1))
    r = rng.uniform(r_lo, r_hi)
    a = (np.arange(k) + rng.uniform(-0.3, 0.3, k)) * (2.0 * math.pi / k)
    return np.stack([r * np.cos(a), r * np.sin(a)], axis=1)


def polygon_scene(seed: int, n: int = 40, box: float = 8.0, poly_p: float = 0.4, rect_p: float = 0.3,
                  static_p: float = 0.1, worlds: int = 1) -> Scene:
    """Random worlds mixing convex polygons (3-8 vertices) with discs and
    rectangles over a static ground, with random angles and velocities:
    every pair type (polygon-polygon, -rectangle, -disc) meets."""
    rng = np.random.default_rng(seed)
    parts, polys = [], []
    for _ in range(worlds):
        b = _Builder()
        b.rect(0.0, -0.5, 3 * box, 1.0, 0.5, static=True)
        for _ in range(n):
            x, y = rng.uniform(-box, box), rng.uniform(0.0, box)
            st = rng.random() < static_p
            vx, vy = (0.0, 0.0) if st else (rng.normal(), rng.normal())
            ang, om, mu = rng.uniform(-math.pi, math.pi), rng.normal(), rng.uniform(0.1, 0.9)
            u = rng.random()
            if u < poly_p:
                b.polygon(x, y, random_polygon(rng), mu, vx=vx, vy=vy, angle=ang, omega=om, static=st)
            elif u < poly_p + rect_p:
                b.rect(x, y, rng.uniform(0.3, 2.0), rng.uniform(0.3, 2.0), mu, vx=vx, vy=vy, angle=ang, omega=om,
                       static=st)
            else:
                b.disc(x, y, rng.uniform(0.2, 1.0), mu, vx=vx, vy=vy, angle=ang, omega=om, static=st)
        parts.append(b.arrays())
        polys.append(b.polygon_arrays())
    g = [9.81] * worlds
    return _concat(f"polygons{seed}", parts, g, 1 / 60, 1, 8, 60, polys=polys)


CONFIGS = {0: config0, 1: config1, 2: config2, 3: config3, 4: config4}

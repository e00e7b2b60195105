"""ctypes wrapper of the CPU oracle (r2d_oracle.hpp / oracle_capi.cpp).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py (its CPU baseline and --impl reference arm).  The product package
never imports it.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libr2d_oracle.so"
ORDER_REFERENCE, ORDER_COLOUR = 0, 1
NSTATE, NPROP, MF = 13, 5, 33

_u32p = C.POINTER(C.c_uint32)
_u8p = C.POINTER(C.c_uint8)
_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_i32p = C.POINTER(C.c_int)
_P = C.c_void_p

_SIG = {
    "r2o_create": ([C.c_int], _P),
    "r2o_destroy": ([_P], None),
    "r2o_add_bodies": ([_P, C.c_uint32, _u32p, _u8p, _f32p], C.c_int),
    "r2o_num_bodies": ([_P], C.c_uint32),
    "r2o_add_bodies_poly": ([_P, C.c_uint32, _u32p, _u8p, _f32p, _u8p, _f32p], C.c_int),
    "r2o_add_gravity": ([_P, C.c_float], None),
    "r2o_exclude_pair": ([_P, C.c_uint32, C.c_uint32], None),
    "r2o_add_joints": ([_P, C.c_uint32, _u8p, _u32p, _u32p, _f32p], None),
    "r2o_set_hash_config": ([_P, C.c_float, C.c_uint32], None),
    "r2o_set_warm_start": ([_P, C.c_int], None),
    "r2o_set_compensated": ([_P, C.c_int], None),
    "r2o_acc_sum": ([C.c_uint32, _f32p, C.c_float, C.c_float, C.c_float, _f32p], None),
    "r2o_copy_warm": ([_P, _P], C.c_int),
    "r2o_set_sleep": ([_P, C.c_int], None),
    "r2o_set_phase_timing": ([_P, C.c_int], None),
    "r2o_phase_seconds": ([_P, _f64p], None),
    "r2o_sleep_frames": ([_P], C.c_uint32),
    "r2o_get_state": ([_P, _f32p], None),
    "r2o_get_state_f64": ([_P, _f64p], None),
    "r2o_set_state": ([_P, _f32p], None),
    "r2o_get_props": ([_P, _f32p], None),
    "r2o_process": ([_P, C.c_float, C.c_uint32, C.c_uint32, C.c_int], C.c_int),
    "r2o_update_manifolds": ([_P, C.c_int], C.c_int),
    "r2o_num_manifolds": ([_P], C.c_uint32),
    "r2o_get_manifolds": ([_P, _u32p, _f32p], None),
    "r2o_get_colours": ([_P, C.c_uint32, _u32p, C.c_uint32, _u32p], C.c_uint32),
    "r2o_set_record_pairs": ([_P, C.c_int], None),
    "r2o_get_pairs": ([_P, C.c_uint32, _u32p], C.c_uint32),
    "r2o_batch_run_checkpoints": ([C.c_int, C.c_uint32, _u32p, _u32p, _u8p, _f32p, _f32p, C.c_float, C.c_uint32,
                                   C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_uint32, _u32p, _f64p], C.c_int),
    "r2o_nmath_kat": ([_f32p, _f32p, _f32p], None),
    "r2o_aabb_intersects": ([C.c_float] * 8, C.c_int),
    "r2o_sincosf": ([C.c_uint32, _f32p, _f32p, _f32p], None),
    "r2o_batch_run": ([C.c_int, C.c_uint32, _u32p, _u32p, _u8p, _f32p, _f32p, C.c_float, C.c_uint32,
                       C.c_uint32, C.c_uint32, C.c_int, C.c_int, _f32p, _f32p, _i32p], C.c_double),
}

_lib = None


# Phases of Solver::step, in r2o::Phase order (r2d_oracle.hpp)
PHASES = ("manifolds", "colouring", "forces", "prestep", "solve", "integrate")


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is not built (make -C oracle)")
        lib = C.CDLL(str(LIB_PATH))
        for k, (a, r) in _SIG.items():
            f = getattr(lib, k)
            f.argtypes = a
            f.restype = r
        _lib = lib
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Oracle:
    """One world of the CPU restatement (precision 32 = f32, 64 = FP64)."""

    def __init__(self, precision: int = 32):
        self.lib = load()
        self.h = self.lib.r2o_create(precision)
        self.precision = precision
        self.nj = 0

    def __del__(self):
        try:
            if self.h:
                self.lib.r2o_destroy(self.h)
                self.h = None
        except Exception:
            pass

    @classmethod
    def from_scene(cls, sc, precision: int = 32, world: int = 0) -> "Oracle":
        if sc.nworlds != 1:
            sc = sc.world(world)
        o = cls(precision)
        ids = np.ascontiguousarray(sc.ids, np.uint32)
        kind = np.ascontiguousarray(sc.kind, np.uint8)
        opt = np.ascontiguousarray(sc.opt, np.float32)
        if getattr(sc, "has_polygons", False):
            nv = np.ascontiguousarray(sc.poly_nv, np.uint8)
            pv = np.ascontiguousarray(sc.poly_v, np.float32)
            if o.lib.r2o_add_bodies_poly(o.h, ids.shape[0], _p(ids, C.c_uint32), _p(kind, C.c_uint8),
                                         _p(opt, C.c_float), _p(nv, C.c_uint8), _p(pv, C.c_float)) != 0:
                raise ValueError("a polygon needs 3 to 8 vertices")
        else:
            o.lib.r2o_add_bodies(o.h, ids.shape[0], _p(ids, C.c_uint32), _p(kind, C.c_uint8), _p(opt, C.c_float))
        for g in np.atleast_1d(sc.gravity):
            if g != 0:
                o.lib.r2o_add_gravity(o.h, float(g))
        if sc.jtype.size:
            t = np.ascontiguousarray(sc.jtype, np.uint8)
            a = np.ascontiguousarray(sc.jid1, np.uint32)
            b = np.ascontiguousarray(sc.jid2, np.uint32)
            p = np.ascontiguousarray(sc.jprm, np.float32)
            o.lib.r2o_add_joints(o.h, t.shape[0], _p(t, C.c_uint8), _p(a, C.c_uint32), _p(b, C.c_uint32),
                                 _p(p, C.c_float))
            o.nj = int(t.shape[0])
        for (x, y) in np.asarray(sc.xpairs).reshape(-1, 2):
            o.lib.r2o_exclude_pair(o.h, int(x), int(y))
        return o

    @property
    def n(self) -> int:
        return int(self.lib.r2o_num_bodies(self.h))

    def set_hash(self, cell: float, mult: int):
        self.lib.r2o_set_hash_config(self.h, cell, mult)

    def set_warm_start(self, on: bool = True):
        """Warm starting (off in reference mode): manifolds found again start
        from last frame's accumulated impulses."""
        self.lib.r2o_set_warm_start(self.h, int(bool(on)))

    def add_bodies_raw(self, ids, kind, props, state):
        """Appends bodies given as an engine takes them: ids, kind bits
        (rectangle 1, static 2), props [5][n] (mass, inertia, mu, dims) and a
        full state [13][n], AABBs included.  The oracle derives the inertia
        from the mass as EntityFactory does; it must equal props[1]."""
        ids = np.ascontiguousarray(ids, np.uint32)
        kind = np.ascontiguousarray(np.asarray(kind) & 3, np.uint8)
        props = np.asarray(props, np.float32)
        state = np.asarray(state, np.float32)
        n = ids.shape[0]
        first = int(self.lib.r2o_num_bodies(self.h))
        opt = np.zeros((10, n), np.float32)
        opt[0], opt[1], opt[2] = state[0], state[1], state[2]
        opt[6], opt[7] = props[2], props[0]
        opt[8], opt[9] = props[3], props[4]
        if self.lib.r2o_add_bodies(self.h, n, _p(ids, C.c_uint32), _p(kind, C.c_uint8), _p(opt, C.c_float)) != 0:
            raise ValueError("the oracle refused the bodies")
        st = self.state()
        if not np.array_equal(self.props()[:, first:], props):
            raise ValueError("the oracle derives other masses or inertias from these props")
        st[:, first:] = state
        self.set_state(np.ascontiguousarray(st))

    def set_compensated(self, on: bool = True):
        """Compensated (Kahan) accumulation of each point's impulses (off in
        reference mode; r2d_accum.h)."""
        self.lib.r2o_set_compensated(self.h, int(bool(on)))

    def take_warm(self, other: "Oracle"):
        """Carry `other`'s last-frame warm-start table (keyed by body ids)
        into this solver, as an engine keeps it across body uploads."""
        if self.lib.r2o_copy_warm(self.h, other.h) != 0:
            raise ValueError("the two oracles differ in precision")

    def set_sleep(self, on: bool = True):
        """Sleeping (r2d_sleep.h): a world still for R2D_SLEEP_FRAMES
        consecutive steps is not stepped until its state is written."""
        self.lib.r2o_set_sleep(self.h, int(bool(on)))

    def set_phase_timing(self, on: bool = True):
        """Time each phase of the step (PHASES order); clears the sums."""
        self.lib.r2o_set_phase_timing(self.h, int(bool(on)))

    def phase_seconds(self) -> np.ndarray:
        out = np.zeros(len(PHASES), np.float64)
        self.lib.r2o_phase_seconds(self.h, _p(out, C.c_double))
        return out

    def sleep_frames(self) -> int:
        return int(self.lib.r2o_sleep_frames(self.h))

    def state(self) -> np.ndarray:
        out = np.empty((NSTATE, self.n), np.float32)
        self.lib.r2o_get_state(self.h, _p(out, C.c_float))
        return out

    def state64(self) -> np.ndarray:
        out = np.empty((NSTATE, self.n), np.float64)
        self.lib.r2o_get_state_f64(self.h, _p(out, C.c_double))
        return out

    def set_state(self, st: np.ndarray):
        st = np.ascontiguousarray(st, np.float32)
        self.lib.r2o_set_state(self.h, _p(st, C.c_float))

    def props(self) -> np.ndarray:
        out = np.empty((NPROP, self.n), np.float32)
        self.lib.r2o_get_props(self.h, _p(out, C.c_float))
        return out

    def process(self, dt: float, sub_steps: int = 1, iters: int = 8, order: int = ORDER_COLOUR) -> int:
        return int(self.lib.r2o_process(self.h, float(dt), int(sub_steps), int(iters), int(order)))

    def update_manifolds(self, order: int = ORDER_COLOUR) -> int:
        return int(self.lib.r2o_update_manifolds(self.h, int(order)))

    def manifolds(self):
        m = int(self.lib.r2o_num_manifolds(self.h))
        k = np.zeros((m, 2), np.uint32)
        d = np.zeros((m, MF), np.float32)
        self.lib.r2o_get_manifolds(self.h, _p(k, C.c_uint32), _p(d, C.c_float))
        return k, d

    def record_pairs(self, on: bool = True):
        """Keep each narrowphase's candidate pairs (see pairs)."""
        self.lib.r2o_set_record_pairs(self.h, int(bool(on)))

    def pairs(self) -> np.ndarray:
        """The pairs the last narrowphase passed to performNarrowSAT
        (lib.zig:264-284): [k][2] (lower, higher) body indices, sorted."""
        n = int(self.lib.r2o_get_pairs(self.h, 0, None))
        out = np.zeros((n, 2), np.uint32)
        if n:
            self.lib.r2o_get_pairs(self.h, n, _p(out, C.c_uint32))
        return out

    def colours(self):
        m = int(self.lib.r2o_num_manifolds(self.h))
        c = np.zeros(max(m, 1), np.uint32)
        j = np.zeros(max(self.nj, 1), np.uint32)
        got = self.lib.r2o_get_colours(self.h, m, _p(c, C.c_uint32), self.nj, _p(j, C.c_uint32))
        return c[: min(m, got)], j[: self.nj]


def batch_run(sc, steps: int, nthreads: int, precision: int = 32, order: int = ORDER_COLOUR, state_in=None):
    """Step every world of a scene on host threads, optionally from a given
    state ([13][n] field-major over all worlds); returns (seconds, state
    [13][n], status).  The worlds are stepped with their bodies and gravity
    only, so a scene with joints or exclusions is refused: step it through
    Oracle.from_scene."""
    if sc.jtype.size or sc.xpairs.size:
        raise ValueError("batch_run steps bodies only; use Oracle.from_scene for joints or exclusions")
    lib = load()
    off = np.ascontiguousarray(sc.body_off, np.uint32)
    ids = np.ascontiguousarray(sc.ids, np.uint32)
    kind = np.ascontiguousarray(sc.kind, np.uint8)
    opt = np.ascontiguousarray(sc.opt, np.float32)
    grav = np.ascontiguousarray(sc.gravity, np.float32)
    state = np.zeros((NSTATE, sc.nbodies), np.float32)
    sin = None if state_in is None else np.ascontiguousarray(state_in, np.float32)
    status = C.c_int(0)
    secs = lib.r2o_batch_run(precision, sc.nworlds, _p(off, C.c_uint32), _p(ids, C.c_uint32), _p(kind, C.c_uint8),
                             _p(opt, C.c_float), _p(grav, C.c_float), float(sc.dt), sc.sub_steps, sc.iters,
                             int(steps), int(order), int(nthreads), None if sin is None else _p(sin, C.c_float),
                             _p(state, C.c_float), C.byref(status))
    return float(secs), state, int(status.value)


# modes of batch_checkpoints
BR_WARM, BR_COMPENSATED, BR_PERTURB_ULP, BR_PERTURB_F32_ULP = 1, 2, 4, 8


def batch_checkpoints(sc, checks, nthreads: int, precision: int = 64, order: int = ORDER_COLOUR, flags: int = 0):
    """Every world of a bodies-only scene stepped from its start on host
    threads in the mode `flags` (BR_*: warm starting, compensated sums, the
    dynamic bodies' x nudged up by one ulp of the precision or one f32 ulp);
    returns (f64 state [len(checks)][13][n] at each step count, status)."""
    if sc.jtype.size or sc.xpairs.size:
        raise ValueError("batch_checkpoints steps bodies only")
    lib = load()
    off = np.ascontiguousarray(sc.body_off, np.uint32)
    ids = np.ascontiguousarray(sc.ids, np.uint32)
    kind = np.ascontiguousarray(sc.kind, np.uint8)
    opt = np.ascontiguousarray(sc.opt, np.float32)
    grav = np.ascontiguousarray(sc.gravity, np.float32)
    ck = np.ascontiguousarray(sorted(int(c) for c in checks), np.uint32)
    out = np.zeros((ck.shape[0], NSTATE, sc.nbodies), np.float64)
    st = lib.r2o_batch_run_checkpoints(precision, sc.nworlds, _p(off, C.c_uint32), _p(ids, C.c_uint32),
                                       _p(kind, C.c_uint8), _p(opt, C.c_float), _p(grav, C.c_float), float(sc.dt),
                                       sc.sub_steps, sc.iters, int(order), int(nthreads), int(flags), ck.shape[0],
                                       _p(ck, C.c_uint32), _p(out, C.c_double))
    return out, int(st)


def nmath_kat(a, b) -> np.ndarray:
    """[add2 xy, sub2 xy, multelem2 xy, divelem2 xy, dot2, cross2, length2sq(a), length2(a)]"""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    out = np.zeros(12, np.float32)
    load().r2o_nmath_kat(_p(a, C.c_float), _p(b, C.c_float), _p(out, C.c_float))
    return out


def aabb_intersects(s1, s2) -> bool:
    return bool(load().r2o_aabb_intersects(*[float(v) for v in (*s1, *s2)]))


def sincosf(x) -> tuple[np.ndarray, np.ndarray]:
    x = np.ascontiguousarray(x, np.float32)
    s = np.empty_like(x)
    c = np.empty_like(x)
    load().r2o_sincosf(x.size, _p(x, C.c_float), _p(s, C.c_float), _p(c, C.c_float))
    return s, c


def acc_sum(x, s0: float = 0.0, lo: float = 0.0, hi: float | None = None):
    """Accumulates increments `x` from s0 with r2d_accum.h's clamped
    compensated update (lower bound lo; upper bound hi when given):
    returns (s, c, sum of the applied changes) as float32."""
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros(3, np.float32)
    load().r2o_acc_sum(x.shape[0], _p(x, C.c_float), float(s0), float(lo),
                       float("nan") if hi is None else float(hi), _p(out, C.c_float))
    return out

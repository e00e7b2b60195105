"""Thin Python handles over the C ABI: one world (``World``, the drop-in for
the reference's Solver) and many independent worlds (``Batch``).  Both own
device memory through the library; numpy arrays cross the boundary."""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .scenes import KIND_POLY, NSTATE, Scene, derive_props_state


def device_kind(kind) -> np.ndarray:
    """A scene's kind bits as the library takes them: rectangle 1, static 2,
    polygon 4 (the scene's mass-by-density bit stays on the host)."""
    k = np.asarray(kind).astype(np.uint8)
    return ((k & 3) | ((k & KIND_POLY) >> 1)).astype(np.uint8)


def _polygon_rows(sc: Scene):
    """(body indices, vertex counts, vertices [k][8][2]) of a scene's polygons."""
    idx = np.flatnonzero(sc.poly_nv).astype(np.uint32)
    return idx, np.ascontiguousarray(sc.poly_nv[idx], np.uint8), np.ascontiguousarray(sc.poly_v[idx], np.float32)


def _rows(a, k: int, n: int) -> np.ndarray:
    """`a` as the contiguous float32 [k][n] rows the library reads (no copy
    when it already is: a pinned buffer stays pinned)."""
    if isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous and a.shape == (k, n):
        return a
    return np.ascontiguousarray(np.asarray(a, np.float32).reshape(k, n))


def _out_rows(a: np.ndarray, k: int, n: int) -> np.ndarray:
    if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous and a.shape == (k, n)):
        raise ValueError(f"out must be a C-contiguous float32 array of shape ({k}, {n})")
    return a


def _config(cell: float, mult: int, debug: bool, stream, capacity_scale: float = 0.0,
            grid: bool = False, fp64_positions: bool = False, warm_start: bool = False,
            sleep: bool = False, compensated: bool = False) -> N.Config:
    cfg = N.Config()
    cfg.capacity_scale = float(capacity_scale)
    cfg.spatialhash_cell_width = float(cell)
    cfg.spatialhash_table_size_mult = int(mult)
    cfg.flags = ((N.FLAG_DEBUG_TAPS if debug else 0) | (N.FLAG_GRID_PIPELINE if grid else 0)
                 | (N.FLAG_FP64_POSITIONS if fp64_positions else 0) | (N.FLAG_WARM_START if warm_start else 0)
                 | (N.FLAG_SLEEP if sleep else 0) | (N.FLAG_COMPENSATED if compensated else 0))
    cfg.stream = int(stream) if stream else None
    return cfg


class World:
    """One world (r2d_solver_* entry points): the fused one-CTA kernel up to
    520 bodies, the grid-wide pipeline above that (or always, ``grid=True``)."""

    def __init__(self, cell: float = 0.0, mult: int = 0, debug: bool = False, stream=None, capacity_scale: float = 0.0,
                 grid: bool = False, fp64_positions: bool = False, warm_start: bool = False,
                 sleep: bool = False, compensated: bool = False):
        self._lib = N.load()
        self._h = C.c_void_p()
        cfg = _config(cell, mult, debug, stream, capacity_scale, grid, fp64_positions, warm_start, sleep,
                      compensated)
        N.check(self._lib.r2d_solver_create(C.byref(cfg), C.byref(self._h)), "r2d_solver_create")
        self.n = 0

    def close(self):
        if self._h:
            self._lib.r2d_solver_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_bodies(self, ids, kind, props, state, init_aabb: bool):
        ids, kind, props, state = N.u32(ids), N.u8(kind), N.f32(props), N.f32(state)
        self.n = int(ids.shape[0])
        N.check(self._lib.r2d_solver_set_bodies(self._h, self.n, N.ptr(ids, C.c_uint32), N.ptr(kind, C.c_uint8),
                                                N.ptr(props, C.c_float), N.ptr(state, C.c_float), int(init_aabb)),
                "r2d_solver_set_bodies")

    def set_polygons(self, body, nverts, verts):
        """Vertices of the polygon bodies at store indices `body`
        (r2d_solver_set_polygons): nverts [k], verts [k][8][2]."""
        body, nverts = N.u32(body), N.u8(nverts)
        verts = np.ascontiguousarray(np.asarray(verts, np.float32).reshape(-1, N.POLY_MAX_VERTS, 2))
        N.check(self._lib.r2d_solver_set_polygons(self._h, int(body.shape[0]), N.ptr(body, C.c_uint32),
                                                  N.ptr(nverts, C.c_uint8), N.ptr(verts, C.c_float)),
                "r2d_solver_set_polygons")

    def set_gravity(self, g):
        g = N.f32(np.atleast_1d(g))
        N.check(self._lib.r2d_solver_set_gravity(self._h, int(g.shape[0]), N.ptr(g, C.c_float)), "r2d_solver_set_gravity")

    def set_joints(self, jtype, id1, id2, prm):
        jtype, id1, id2, prm = N.u8(jtype), N.u32(id1), N.u32(id2), N.f32(prm)
        N.check(self._lib.r2d_solver_set_joints(self._h, int(jtype.shape[0]), N.ptr(jtype, C.c_uint8),
                                                N.ptr(id1, C.c_uint32), N.ptr(id2, C.c_uint32),
                                                N.ptr(prm, C.c_float)), "r2d_solver_set_joints")

    def set_exclusions(self, pairs):
        pairs = N.u32(np.asarray(pairs).reshape(-1, 2))
        N.check(self._lib.r2d_solver_set_exclusions(self._h, int(pairs.shape[0]), N.ptr(pairs, C.c_uint32)),
                "r2d_solver_set_exclusions")

    @classmethod
    def from_scene(cls, sc: Scene, debug: bool = False, stream=None, **kw) -> "World":
        if sc.nworlds != 1:
            raise ValueError(f"World.from_scene takes one world; this scene has {sc.nworlds} (use Batch)")
        w = cls(debug=debug, stream=stream, **kw)
        props, state = derive_props_state(sc.kind, sc.opt)
        w.set_gravity(sc.gravity[sc.gravity != 0] if sc.gravity.size else np.zeros(0, np.float32))
        w.set_bodies(sc.ids, device_kind(sc.kind), props, state, init_aabb=True)
        if sc.has_polygons:
            w.set_polygons(*_polygon_rows(sc))
        if sc.jtype.size:
            w.set_joints(sc.jtype, sc.jid1, sc.jid2, sc.jprm)
        if sc.xpairs.size:
            w.set_exclusions(sc.xpairs)
        return w

    def write_state(self, state):
        state = N.f32(state)
        N.check(self._lib.r2d_solver_write_state(self._h, N.ptr(state, C.c_float)), "r2d_solver_write_state")

    def read_state(self) -> np.ndarray:
        out = np.empty((NSTATE, self.n), np.float32)
        N.check(self._lib.r2d_solver_read_state(self._h, N.ptr(out, C.c_float)), "r2d_solver_read_state")
        return out

    def process(self, dt: float, sub_steps: int = 1, iters: int = 8):
        N.check(self._lib.r2d_solver_process(self._h, float(dt), int(sub_steps), int(iters)), "r2d_solver_process")

    def process_io(self, dt: float, sub_steps: int, iters: int, forces=None, out=None):
        """One frame: force/torque rows [3][n] in, step, pose and momentum rows
        [6][n] out (written into `out`, a C-contiguous float32 array; pinned
        buffers are accessed by the step directly)."""
        fp = N.ptr(_rows(forces, 3, self.n), C.c_float) if forces is not None else None
        op = N.ptr(_out_rows(out, 6, self.n), C.c_float) if out is not None else None
        N.check(self._lib.r2d_solver_process_io(self._h, float(dt), int(sub_steps), int(iters), fp, op),
                "r2d_solver_process_io")

    def sync(self):
        N.check(self._lib.r2d_solver_sync(self._h), "r2d_solver_sync")

    def launches_per_step(self) -> int:
        out = C.c_uint32()
        N.check(self._lib.r2d_solver_launches_per_step(self._h, C.byref(out)), "r2d_solver_launches_per_step")
        return int(out.value)

    def sleep_frames(self) -> int:
        """Consecutive still steps of the world (sleeping mode; it sleeps from 60)."""
        out = C.c_uint32()
        N.check(self._lib.r2d_solver_sleep_frames(self._h, C.byref(out)), "r2d_solver_sleep_frames")
        return int(out.value)

    def manifolds(self):
        m = C.c_uint32()
        N.check(self._lib.r2d_solver_num_manifolds(self._h, C.byref(m)), "r2d_solver_num_manifolds")
        k = np.zeros((m.value, 2), np.uint32)
        d = np.zeros((m.value, N.MANIFOLD_FLOATS), np.float32)
        c = np.zeros(m.value, np.uint32)
        N.check(self._lib.r2d_solver_get_manifolds(self._h, m.value, N.ptr(k, C.c_uint32), N.ptr(d, C.c_float),
                                                   N.ptr(c, C.c_uint32)), "r2d_solver_get_manifolds")
        return k, d, c

    def write_fields(self, first: int, rows):
        """State rows [first, first + len(rows)) (field-major)."""
        rows = N.f32(rows)
        N.check(self._lib.r2d_solver_write_state_fields(self._h, first, rows.shape[0], N.ptr(rows, C.c_float)),
                "r2d_solver_write_state_fields")

    def read_fields(self, first: int, count: int, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((count, self.n), np.float32)
        N.check(self._lib.r2d_solver_read_state_fields(self._h, first, count, N.ptr(out, C.c_float)),
                "r2d_solver_read_state_fields")
        return out

    def read_positions_f64(self) -> np.ndarray:
        out = np.empty((3, self.n), np.float64)
        N.check(self._lib.r2d_solver_read_positions_f64(self._h, out.ctypes.data_as(C.POINTER(C.c_double))),
                "r2d_solver_read_positions_f64")
        return out

    def pairs(self) -> np.ndarray:
        """The last frame's candidate pairs [k][2] (lower, higher body index),
        sorted: the pairs that reached the narrowphase."""
        m = C.c_uint32()
        N.check(self._lib.r2d_solver_num_pairs(self._h, C.byref(m)), "r2d_solver_num_pairs")
        out = np.zeros((m.value, 2), np.uint32)
        N.check(self._lib.r2d_solver_get_pairs(self._h, m.value, N.ptr(out, C.c_uint32)), "r2d_solver_get_pairs")
        return out

    def joint_colours(self, nj: int):
        c = np.zeros(nj, np.uint32)
        N.check(self._lib.r2d_solver_get_joint_colours(self._h, nj, N.ptr(c, C.c_uint32)), "r2d_solver_get_joint_colours")
        return c


class Batch:
    """Many independent worlds stepped together (r2d_batch_* entry points)."""

    def __init__(self, cell: float = 0.0, mult: int = 0, debug: bool = False, stream=None, capacity_scale: float = 0.0,
                 grid: bool = False, fp64_positions: bool = False, warm_start: bool = False,
                 sleep: bool = False, compensated: bool = False):
        self._lib = N.load()
        self._h = C.c_void_p()
        cfg = _config(cell, mult, debug, stream, capacity_scale, grid, fp64_positions, warm_start, sleep,
                      compensated)
        N.check(self._lib.r2d_batch_create(C.byref(cfg), C.byref(self._h)), "r2d_batch_create")
        self.n = 0
        self.nworlds = 0

    def close(self):
        if self._h:
            self._lib.r2d_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_worlds(self, body_off, ids, kind, props, state, gravity, init_aabb: bool):
        body_off, ids, kind = N.u32(body_off), N.u32(ids), N.u8(kind)
        props, state, gravity = N.f32(props), N.f32(state), N.f32(gravity)
        self.nworlds = int(body_off.shape[0] - 1)
        self.n = int(body_off[-1])
        N.check(self._lib.r2d_batch_set_worlds(self._h, self.nworlds, N.ptr(body_off, C.c_uint32),
                                               N.ptr(ids, C.c_uint32), N.ptr(kind, C.c_uint8),
                                               N.ptr(props, C.c_float), N.ptr(state, C.c_float),
                                               N.ptr(gravity, C.c_float), int(init_aabb)), "r2d_batch_set_worlds")

    def set_polygons(self, body, nverts, verts):
        """Vertices of the polygon bodies at indices `body` of the
        concatenated store (r2d_batch_set_polygons)."""
        body, nverts = N.u32(body), N.u8(nverts)
        verts = np.ascontiguousarray(np.asarray(verts, np.float32).reshape(-1, N.POLY_MAX_VERTS, 2))
        N.check(self._lib.r2d_batch_set_polygons(self._h, int(body.shape[0]), N.ptr(body, C.c_uint32),
                                                 N.ptr(nverts, C.c_uint8), N.ptr(verts, C.c_float)),
                "r2d_batch_set_polygons")

    @classmethod
    def from_scene(cls, sc: Scene, debug: bool = False, stream=None, **kw) -> "Batch":
        if sc.jtype.size or sc.xpairs.size:
            raise ValueError("the batch entry points take worlds without joints or exclusions (use World)")
        b = cls(debug=debug, stream=stream, **kw)
        props, state = derive_props_state(sc.kind, sc.opt)
        b.set_worlds(sc.body_off, sc.ids, device_kind(sc.kind), props, state, sc.gravity, init_aabb=True)
        if sc.has_polygons:
            b.set_polygons(*_polygon_rows(sc))
        return b

    def write_state(self, state):
        state = N.f32(state)
        N.check(self._lib.r2d_batch_write_state(self._h, N.ptr(state, C.c_float)), "r2d_batch_write_state")

    def read_state(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((NSTATE, self.n), np.float32)
        N.check(self._lib.r2d_batch_read_state(self._h, N.ptr(out, C.c_float)), "r2d_batch_read_state")
        return out

    def process(self, dt: float, sub_steps: int = 1, iters: int = 8):
        N.check(self._lib.r2d_batch_process(self._h, float(dt), int(sub_steps), int(iters)), "r2d_batch_process")

    def process_io(self, dt: float, sub_steps: int, iters: int, forces=None, out=None):
        """One frame over all worlds (see World.process_io)."""
        fp = N.ptr(_rows(forces, 3, self.n), C.c_float) if forces is not None else None
        op = N.ptr(_out_rows(out, 6, self.n), C.c_float) if out is not None else None
        N.check(self._lib.r2d_batch_process_io(self._h, float(dt), int(sub_steps), int(iters), fp, op),
                "r2d_batch_process_io")

    def sync(self):
        N.check(self._lib.r2d_batch_sync(self._h), "r2d_batch_sync")

    def write_fields(self, first: int, rows):
        """State rows [first, first + len(rows)) over all bodies (field-major)."""
        rows = N.f32(rows)
        N.check(self._lib.r2d_batch_write_state_fields(self._h, first, rows.shape[0], N.ptr(rows, C.c_float)),
                "r2d_batch_write_state_fields")

    def read_fields(self, first: int, count: int, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((count, self.n), np.float32)
        N.check(self._lib.r2d_batch_read_state_fields(self._h, first, count, N.ptr(out, C.c_float)),
                "r2d_batch_read_state_fields")
        return out

    def read_positions_f64(self) -> np.ndarray:
        out = np.empty((3, self.n), np.float64)
        N.check(self._lib.r2d_batch_read_positions_f64(self._h, out.ctypes.data_as(C.POINTER(C.c_double))),
                "r2d_batch_read_positions_f64")
        return out

    def autotune(self, dt: float, sub_steps: int = 1, iters: int = 8, trial_steps: int = 3):
        """Pick each size class's threads per CTA by timing (state restored)."""
        N.check(self._lib.r2d_batch_autotune(self._h, float(dt), int(sub_steps), int(iters), int(trial_steps)),
                "r2d_batch_autotune")

    def launches_per_step(self) -> int:
        out = C.c_uint32()
        N.check(self._lib.r2d_batch_launches_per_step(self._h, C.byref(out)), "r2d_batch_launches_per_step")
        return int(out.value)

    def sleep_frames(self) -> np.ndarray:
        """Consecutive still steps of every world (sleeping mode; a world sleeps from 60)."""
        out = np.zeros(self.nworlds, np.uint32)
        N.check(self._lib.r2d_batch_sleep_frames(self._h, N.ptr(out, C.c_uint32)), "r2d_batch_sleep_frames")
        return out

    def world_status(self) -> np.ndarray:
        out = np.zeros(self.nworlds, np.int32)
        N.check(self._lib.r2d_batch_world_status(self._h, N.ptr(out, C.c_int)), "r2d_batch_world_status")
        return out

    def manifolds(self, w: int):
        m = C.c_uint32()
        N.check(self._lib.r2d_batch_num_manifolds(self._h, w, C.byref(m)), "r2d_batch_num_manifolds")
        k = np.zeros((m.value, 2), np.uint32)
        d = np.zeros((m.value, N.MANIFOLD_FLOATS), np.float32)
        c = np.zeros(m.value, np.uint32)
        N.check(self._lib.r2d_batch_get_manifolds(self._h, w, m.value, N.ptr(k, C.c_uint32), N.ptr(d, C.c_float),
                                                  N.ptr(c, C.c_uint32)), "r2d_batch_get_manifolds")
        return k, d, c

    def pairs(self, w: int) -> np.ndarray:
        """World w's candidate pairs of the last frame (see World.pairs)."""
        m = C.c_uint32()
        N.check(self._lib.r2d_batch_num_pairs(self._h, w, C.byref(m)), "r2d_batch_num_pairs")
        out = np.zeros((m.value, 2), np.uint32)
        N.check(self._lib.r2d_batch_get_pairs(self._h, w, m.value, N.ptr(out, C.c_uint32)), "r2d_batch_get_pairs")
        return out

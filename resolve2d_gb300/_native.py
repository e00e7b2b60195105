"""ctypes binding of the C ABI in include/r2d_gb300.h.

The library is built in-tree (resolve2d_gb300/_build/libr2d_gb300.so).  There
is no CPU fallback: if the library is missing or a call fails, an exception
says so.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libr2d_gb300.so"
# A different build of the same library (for A/B timing); the default is the in-tree one.
if os.environ.get("R2D_LIB_PATH"):
    LIB_PATH = Path(os.environ["R2D_LIB_PATH"])

R2D_OK = 0
STATUS_NAMES = {
    0: "R2D_OK",
    -1: "R2D_ERR_INVALID_ARGUMENT",
    -2: "R2D_ERR_INVALID_BODY_ID",
    -3: "R2D_ERR_OUT_OF_MEMORY",
    -4: "R2D_ERR_CUDA",
    -5: "R2D_ERR_CAPACITY",
    -6: "R2D_ERR_TIMEOUT",
    -7: "R2D_ERR_NONFINITE",
    -8: "R2D_ERR_NO_DEVICE",
}
FLAG_DEBUG_TAPS = 1
FLAG_GRID_PIPELINE = 2
FLAG_FP64_POSITIONS = 4
FLAG_WARM_START = 8
FLAG_SLEEP = 16
FLAG_COMPENSATED = 32
KIND_POLYGON = 4
POLY_MAX_VERTS = 8
MANIFOLD_FLOATS = 33


class R2DError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str):
        super().__init__(f"{where}: {STATUS_NAMES.get(code, code)} ({detail})")
        self.code = code


class Config(C.Structure):
    _fields_ = [
        ("spatialhash_cell_width", C.c_float),
        ("spatialhash_table_size_mult", C.c_uint32),
        ("flags", C.c_uint32),
        ("stream", C.c_void_p),
        ("capacity_scale", C.c_float),
    ]


_P = C.c_void_p
_u32p = C.POINTER(C.c_uint32)
_u8p = C.POINTER(C.c_uint8)
_f32p = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int)

SIGNATURES = {
    "r2d_version": ([], C.c_int),
    "r2d_last_error_string": ([], C.c_char_p),
    "r2d_solver_create": ([C.POINTER(Config), C.POINTER(_P)], C.c_int),
    "r2d_solver_destroy": ([_P], C.c_int),
    "r2d_solver_set_bodies": ([_P, C.c_uint32, _u32p, _u8p, _f32p, _f32p, C.c_int], C.c_int),
    "r2d_solver_write_state": ([_P, _f32p], C.c_int),
    "r2d_solver_read_state": ([_P, _f32p], C.c_int),
    "r2d_solver_set_gravity": ([_P, C.c_uint32, _f32p], C.c_int),
    "r2d_solver_set_joints": ([_P, C.c_uint32, _u8p, _u32p, _u32p, _f32p], C.c_int),
    "r2d_solver_set_exclusions": ([_P, C.c_uint32, _u32p], C.c_int),
    "r2d_solver_process": ([_P, C.c_float, C.c_uint32, C.c_uint32], C.c_int),
    "r2d_solver_sync": ([_P], C.c_int),
    "r2d_solver_num_manifolds": ([_P, _u32p], C.c_int),
    "r2d_solver_launches_per_step": ([_P, _u32p], C.c_int),
    "r2d_solver_sleep_frames": ([_P, _u32p], C.c_int),
    "r2d_solver_process_io": ([_P, C.c_float, C.c_uint32, C.c_uint32, _f32p, _f32p], C.c_int),
    "r2d_batch_process_io": ([_P, C.c_float, C.c_uint32, C.c_uint32, _f32p, _f32p], C.c_int),
    "r2d_batch_sleep_frames": ([_P, _u32p], C.c_int),
    "r2d_solver_get_manifolds": ([_P, C.c_uint32, _u32p, _f32p, _u32p], C.c_int),
    "r2d_solver_get_joint_colours": ([_P, C.c_uint32, _u32p], C.c_int),
    "r2d_solver_set_polygons": ([_P, C.c_uint32, _u32p, _u8p, _f32p], C.c_int),
    "r2d_solver_num_pairs": ([_P, _u32p], C.c_int),
    "r2d_solver_get_pairs": ([_P, C.c_uint32, _u32p], C.c_int),
    "r2d_batch_create": ([C.POINTER(Config), C.POINTER(_P)], C.c_int),
    "r2d_batch_destroy": ([_P], C.c_int),
    "r2d_batch_set_worlds": ([_P, C.c_uint32, _u32p, _u32p, _u8p, _f32p, _f32p, _f32p, C.c_int], C.c_int),
    "r2d_batch_write_state": ([_P, _f32p], C.c_int),
    "r2d_batch_read_state": ([_P, _f32p], C.c_int),
    "r2d_batch_process": ([_P, C.c_float, C.c_uint32, C.c_uint32], C.c_int),
    "r2d_batch_sync": ([_P], C.c_int),
    "r2d_batch_launches_per_step": ([_P, _u32p], C.c_int),
    "r2d_batch_autotune": ([_P, C.c_float, C.c_uint32, C.c_uint32, C.c_uint32], C.c_int),
    "r2d_batch_world_status": ([_P, _i32p], C.c_int),
    "r2d_batch_num_manifolds": ([_P, C.c_uint32, _u32p], C.c_int),
    "r2d_batch_get_manifolds": ([_P, C.c_uint32, C.c_uint32, _u32p, _f32p, _u32p], C.c_int),
    "r2d_batch_set_polygons": ([_P, C.c_uint32, _u32p, _u8p, _f32p], C.c_int),
    "r2d_batch_num_pairs": ([_P, C.c_uint32, _u32p], C.c_int),
    "r2d_batch_get_pairs": ([_P, C.c_uint32, C.c_uint32, _u32p], C.c_int),
    "r2d_solver_write_state_fields": ([_P, C.c_uint32, C.c_uint32, _f32p], C.c_int),
    "r2d_solver_read_state_fields": ([_P, C.c_uint32, C.c_uint32, _f32p], C.c_int),
    "r2d_batch_write_state_fields": ([_P, C.c_uint32, C.c_uint32, _f32p], C.c_int),
    "r2d_batch_read_state_fields": ([_P, C.c_uint32, C.c_uint32, _f32p], C.c_int),
    "r2d_solver_read_positions_f64": ([_P, C.POINTER(C.c_double)], C.c_int),
    "r2d_batch_read_positions_f64": ([_P, C.POINTER(C.c_double)], C.c_int),
    "r2d_world_step_static": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, _f32p, C.c_uint32,
                               C.c_float, C.c_uint32, C.c_uint32, C.c_float, C.c_uint32, C.c_void_p], C.c_int),
}

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Load libr2d_gb300.so and declare every entry point's signature."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


def check(code: int, where: str) -> None:
    if code != R2D_OK:
        detail = load().r2d_last_error_string()
        raise R2DError(code, where, detail.decode() if detail else "")


def ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def u8(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint8)

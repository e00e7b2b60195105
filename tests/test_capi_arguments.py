"""Argument checks of the C ABI that return before any device work.

Every entry point that takes a solver or batch handle answers a NULL handle
with R2D_ERR_INVALID_ARGUMENT and a message, the creators refuse a NULL out
pointer, and the allocation-free step refuses NULL buffers, more than four
gravity generators and zero substeps.  None of these calls reaches the GPU,
so the file runs on any host.
"""

import ctypes as C

import pytest

from resolve2d_gb300 import _native as N

INVALID = -1


def zero_args(argtypes):
    out = []
    for t in argtypes:
        if t in (C.c_uint32, C.c_int):
            out.append(0)
        elif t is C.c_float:
            out.append(0.0)
        else:
            out.append(None)  # every pointer, the handle included
    return out


HANDLE_CALLS = sorted(
    name
    for name, (argtypes, _) in N.SIGNATURES.items()
    if argtypes and argtypes[0] is N._P and not name.endswith("_create") and name != "r2d_world_step_static"
)


def last_error(lib):
    return (lib.r2d_last_error_string() or b"").decode()


def test_every_handle_entry_point_is_covered():
    assert len(HANDLE_CALLS) >= 30
    assert "r2d_batch_process_io" in HANDLE_CALLS and "r2d_solver_destroy" in HANDLE_CALLS


@pytest.mark.parametrize("name", HANDLE_CALLS)
def test_null_handle_is_an_invalid_argument(name):
    lib = N.load()
    argtypes, _ = N.SIGNATURES[name]
    assert getattr(lib, name)(*zero_args(argtypes)) == INVALID
    assert last_error(lib), f"{name} gave no message"


@pytest.mark.parametrize("name", ["r2d_solver_create", "r2d_batch_create"])
def test_creators_refuse_a_null_out_pointer(name):
    lib = N.load()
    cfg = N.Config()
    assert getattr(lib, name)(C.byref(cfg), None) == INVALID
    assert "NULL" in last_error(lib)


def static_step(lib, n=1, bufs=True, ngrav=0, gravity=None, sub_steps=1):
    f = (C.c_float * 16)()
    u8 = (C.c_uint8 * 4)()
    u32 = (C.c_uint32 * 4)()
    ptr = (lambda a, t: C.cast(a, t)) if bufs else (lambda a, t: None)
    return lib.r2d_world_step_static(
        ptr(f, N._f32p), ptr(f, N._f32p), ptr(u8, N._u8p), ptr(u32, N._u32p), n,
        gravity, ngrav, 1.0 / 60.0, sub_steps, 8, 0.0, 0, None,
    )


def test_static_step_refuses_bad_arguments_before_launching():
    lib = N.load()
    assert static_step(lib, n=1, bufs=False) == INVALID
    assert "NULL" in last_error(lib)
    g = (C.c_float * 8)(*([9.81] * 8))
    assert static_step(lib, ngrav=5, gravity=C.cast(g, N._f32p)) == INVALID
    assert "gravity" in last_error(lib)
    assert static_step(lib, ngrav=1, gravity=None) == INVALID
    assert static_step(lib, sub_steps=0) == INVALID
    assert "sub_steps" in last_error(lib)


def test_static_step_refuses_a_table_size_that_wraps_32_bits():
    # 4,096 bodies x 2^20 = 2^32 buckets: 0 in 32-bit arithmetic.  The check
    # runs in 64 bits, before the device is touched (the buffers are never read).
    lib = N.load()
    f = (C.c_float * 16)()
    u8 = (C.c_uint8 * 4)()
    u32 = (C.c_uint32 * 4)()
    for mult in (1 << 20, (1 << 32) - 1, 3):
        rc = lib.r2d_world_step_static(C.cast(f, N._f32p), C.cast(f, N._f32p), C.cast(u8, N._u8p),
                                       C.cast(u32, N._u32p), 4096, None, 0, 1.0 / 60.0, 1, 8, 0.0, mult, None)
        assert rc == -5, mult
        assert "buckets exceeds" in last_error(lib)


def test_scene_shapes_the_handles_refuse_before_any_device_work():
    from resolve2d_gb300 import scenes
    from resolve2d_gb300.engine import Batch, World

    with pytest.raises(ValueError, match="one world"):
        World.from_scene(scenes.config3(nworlds=2))
    with pytest.raises(ValueError, match="without joints"):
        Batch.from_scene(scenes.random_scene(1, n=6, joints=True))

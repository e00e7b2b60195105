"""The allocation-free world step (r2d_world_step_static) against the
allocating one (r2d_solver_process + r2d_solver_read_state): the same world,
two calls in a row, the same bits (the tolerance of every parity test here).

It also checks that repeated calls leave the device's free memory unchanged,
and that each of the fixed maxima (bodies, spatial-hash cell entries,
candidate pairs) is refused with R2D_ERR_CAPACITY and the state untouched.

The file sorts last so that it also runs after every other test; it passes
alone in a fresh process as well.
"""

import ctypes as C

import numpy as np
import pytest

from parity import assert_state_equal
from resolve2d_gb300 import _native as N
from resolve2d_gb300 import scenes
from resolve2d_gb300.engine import World
from resolve2d_gb300.scenes import derive_props_state

pytestmark = pytest.mark.gpu


def _device_world(torch, sc, state):
    dev = torch.device("cuda:0")
    props, _ = derive_props_state(sc.kind, sc.opt)
    return (torch.from_numpy(np.ascontiguousarray(state, np.float32)).to(dev),
            torch.from_numpy(np.ascontiguousarray(props, np.float32)).to(dev),
            torch.from_numpy(np.ascontiguousarray(sc.kind & 3, np.uint8)).to(dev),
            torch.from_numpy(np.ascontiguousarray(sc.ids, np.uint32).view(np.int32)).to(dev))


def _static_step(lib, torch, bufs, n, g, dt, sub_steps, iters):
    state_d, props_d, kind_d, ids_d = bufs
    stream = torch.cuda.current_stream().cuda_stream
    return lib.r2d_world_step_static(state_d.data_ptr(), props_d.data_ptr(), kind_d.data_ptr(), ids_d.data_ptr(),
                                     n, N.ptr(g, C.c_float), int(g.shape[0]), float(dt), int(sub_steps), int(iters),
                                     0.0, 0, stream)


@pytest.mark.parametrize("which", ["config0", "world1500"])
def test_static_step_matches_solver_on_two_calls(which):
    torch = pytest.importorskip("torch")
    if which == "config0":
        sc = scenes.config0()
    else:  # above the fused kernel's 520 bodies: the solver takes the grid pipeline
        sc = scenes.batched_worlds("w1500", seed=5, nworlds=1, steps=2, lo=1500, hi=1500)
    w = World.from_scene(sc)
    start = w.read_state()  # AABBs initialised by the solver
    n = start.shape[1]
    bufs = _device_world(torch, sc, start)
    g = np.ascontiguousarray(sc.gravity[sc.gravity != 0], np.float32)
    lib = N.load()
    for call in range(2):
        N.check(_static_step(lib, torch, bufs, n, g, sc.dt, sc.sub_steps, sc.iters), "r2d_world_step_static")
        torch.cuda.synchronize()
        w.process(sc.dt, sc.sub_steps, sc.iters)
        w.sync()
        assert_state_equal(bufs[0].cpu().numpy(), w.read_state(), f"{which} call {call + 1}")


def test_static_step_leaves_device_memory_as_it_found_it():
    # The driver's free-memory count is unchanged across calls: the step
    # allocates nothing (no cudaMalloc, no pool growth).  The first call runs
    # before the count is taken, since it may load the library's kernels.
    torch = pytest.importorskip("torch")
    sc = scenes.config0()
    w = World.from_scene(sc)
    start = w.read_state()
    n = start.shape[1]
    bufs = _device_world(torch, sc, start)
    g = np.ascontiguousarray(sc.gravity[sc.gravity != 0], np.float32)
    lib = N.load()
    N.check(_static_step(lib, torch, bufs, n, g, sc.dt, sc.sub_steps, sc.iters), "r2d_world_step_static")
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        N.check(_static_step(lib, torch, bufs, n, g, sc.dt, sc.sub_steps, sc.iters), "r2d_world_step_static")
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def _refused_unchanged(torch, sc, what):
    """Steps `sc` once through the static step: it must refuse with
    R2D_ERR_CAPACITY naming `what`, and leave the state as it was."""
    w = World.from_scene(sc)
    start = w.read_state()
    bufs = _device_world(torch, sc, start)
    g = np.ascontiguousarray(sc.gravity[sc.gravity != 0], np.float32)
    lib = N.load()
    rc = _static_step(lib, torch, bufs, start.shape[1], g, sc.dt, sc.sub_steps, sc.iters)
    assert rc == -5
    assert what in lib.r2d_last_error_string()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(bufs[0].cpu().numpy(), start)


def test_static_step_refuses_too_many_cell_entries():
    # three static 1000 x 1000 slabs cover 251 x 251 cells of width 4 each:
    # ~189,000 entries against the maximum of 65,536
    torch = pytest.importorskip("torch")
    b = scenes._Builder()
    for k in range(3):
        b.rect(3000.0 * k, -500.0, 1000.0, 1000.0, 0.5, static=True)
    for k in range(20):
        b.disc(1.5 * k, 2.0, 0.5, 0.5)
    ids, kind, opt = b.arrays()
    sc = scenes._concat("slabs", [(ids, kind, opt)], [9.81], 1 / 60, 1, 8, 1)
    _refused_unchanged(torch, sc, b"cell entries")


def test_static_step_refuses_too_many_candidate_pairs():
    # 4,000 discs of radius 0.5 uniform in a 40 x 40 box: about 21,000
    # AABB-intersecting pairs against the maximum of 16,384 (and under the
    # 32,768 slots of the pair set, so its inserts stay short)
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(8)
    b = scenes._Builder()
    for x, y in rng.uniform(0.0, 40.0, size=(4000, 2)):
        b.disc(float(x), float(y), 0.5, 0.5)
    ids, kind, opt = b.arrays()
    sc = scenes._concat("dense", [(ids, kind, opt)], [9.81], 1 / 60, 1, 8, 1)
    _refused_unchanged(torch, sc, b"candidate pairs")


def test_static_step_refuses_polygon_bodies():
    # the allocation-free step takes no polygon vertices: a polygon body is
    # refused with R2D_ERR_INVALID_ARGUMENT, the state untouched
    torch = pytest.importorskip("torch")
    from resolve2d_gb300.engine import device_kind

    sc = scenes.polygon_scene(2, n=12)
    w = World.from_scene(sc)
    start = w.read_state()
    dev = torch.device("cuda:0")
    props, _ = derive_props_state(sc.kind, sc.opt)
    bufs = (torch.from_numpy(np.ascontiguousarray(start, np.float32)).to(dev),
            torch.from_numpy(np.ascontiguousarray(props, np.float32)).to(dev),
            torch.from_numpy(device_kind(sc.kind)).to(dev),
            torch.from_numpy(np.ascontiguousarray(sc.ids, np.uint32).view(np.int32)).to(dev))
    g = np.ascontiguousarray(sc.gravity[sc.gravity != 0], np.float32)
    lib = N.load()
    rc = _static_step(lib, torch, bufs, start.shape[1], g, sc.dt, sc.sub_steps, sc.iters)
    assert rc == -1
    assert b"polygon" in lib.r2d_last_error_string()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(bufs[0].cpu().numpy(), start)


def test_static_step_rejects_worlds_beyond_its_maximum():
    torch = pytest.importorskip("torch")
    sc = scenes.batched_worlds("w5000", seed=6, nworlds=1, steps=1, lo=5000, hi=5000)
    w = World.from_scene(sc)
    start = w.read_state()
    bufs = _device_world(torch, sc, start)
    g = np.ascontiguousarray(sc.gravity[sc.gravity != 0], np.float32)
    lib = N.load()
    rc = _static_step(lib, torch, bufs, start.shape[1], g, sc.dt, sc.sub_steps, sc.iters)
    assert rc == -5
    assert b"4096" in lib.r2d_last_error_string()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(bufs[0].cpu().numpy(), start)

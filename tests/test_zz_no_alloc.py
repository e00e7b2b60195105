"""The allocation-free world step (r2d_world_step_static) against the
allocating one (r2d_solver_process + r2d_solver_read_state): the same world,
two calls in a row, the same bits (the tolerance of every parity test here).

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

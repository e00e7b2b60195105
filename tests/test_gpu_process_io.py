"""One-call frames (r2d_*_process_io): forces in, step, pose and momenta out.

Pinned host rows are read and written by the step itself over the CPU-GPU
link; pageable ones and grid-pipeline worlds take the copy path.  Either way
the frame must equal writing the force rows, stepping and reading the rows
back, bit for bit, including worlds replayed with larger capacities inside
the call.
"""

import numpy as np
import pytest

from parity import assert_state_equal
from resolve2d_gb300 import scenes
from resolve2d_gb300.engine import Batch, World

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def pinned(shape):
    return torch.zeros(shape, dtype=torch.float32).pin_memory().numpy()


def frame_forces(n, k, seed):
    rng = np.random.default_rng(seed + k)
    f = np.zeros((3, n), np.float32)
    hit = rng.choice(n, size=max(1, n // 20), replace=False)
    f[0, hit] = rng.normal(0, 200, hit.size)
    f[1, hit] = rng.normal(0, 200, hit.size)
    f[2, hit] = rng.normal(0, 20, hit.size)
    return f


@pytest.mark.parametrize("capacity_scale", [0.0, 0.05])
@pytest.mark.parametrize("pin", [True, False])
def test_batch_frames_equal_the_copy_path(pin, capacity_scale):
    sc = scenes.batched_worlds("io", seed=12, nworlds=24, steps=12)
    kw = {"capacity_scale": capacity_scale} if capacity_scale else {}
    a = Batch.from_scene(sc, **kw)
    b = Batch.from_scene(sc, **kw)
    n = sc.nbodies
    fin = pinned((3, n)) if pin else np.zeros((3, n), np.float32)
    out = pinned((6, n)) if pin else np.zeros((6, n), np.float32)
    for k in range(12):
        f = frame_forces(n, k, 3)
        fin[...] = f
        a.process_io(sc.dt, sc.sub_steps, sc.iters, fin, out)
        b.write_fields(scenes.S_FORCE_X, f)
        b.process(sc.dt, sc.sub_steps, sc.iters)
        b.sync()
        want = b.read_state()
        assert_state_equal(out, want[:6], f"frame {k} rows")
        assert_state_equal(a.read_state(), want, f"frame {k} state")


def test_solver_frames_on_the_grid_pipeline_with_joints():
    sc = scenes.random_scene(41, n=40, joints=True)
    a = World.from_scene(sc, grid=True)
    b = World.from_scene(sc, grid=True)
    n = sc.nbodies
    fin, out = pinned((3, n)), pinned((6, n))
    for k in range(10):
        f = frame_forces(n, k, 9)
        fin[...] = f
        a.process_io(sc.dt, sc.sub_steps, sc.iters, fin, out)
        b.write_fields(scenes.S_FORCE_X, f)
        b.process(sc.dt, sc.sub_steps, sc.iters)
        b.sync()
        want = b.read_state()
        assert_state_equal(out, want[:6], f"frame {k} rows")
        assert_state_equal(a.read_state(), want, f"frame {k} state")


def test_plain_steps_after_frames_read_no_stale_forces():
    sc = scenes.batched_worlds("io2", seed=13, nworlds=8, steps=6)
    a = Batch.from_scene(sc)
    b = Batch.from_scene(sc)
    n = sc.nbodies
    fin, out = pinned((3, n)), pinned((6, n))
    fin[...] = frame_forces(n, 0, 5)
    a.process_io(sc.dt, sc.sub_steps, sc.iters, fin, out)
    b.write_fields(scenes.S_FORCE_X, np.array(fin))
    b.process(sc.dt, sc.sub_steps, sc.iters)
    fin[...] = 1000.0  # the host buffer changes; later plain steps must not read it
    for _ in range(5):
        a.process(sc.dt, sc.sub_steps, sc.iters)
        b.process(sc.dt, sc.sub_steps, sc.iters)
    a.sync()
    b.sync()
    assert_state_equal(a.read_state(), b.read_state(), "plain steps after a frame")

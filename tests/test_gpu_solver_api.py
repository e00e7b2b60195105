"""The reference-style ``Solver`` over the GPU engine, against the oracle.

The scene of ``solver_scenes.py`` is built through the factory: discs and
rectangles by density and by mass, a static ground set through
``body_unwrap().static``, gravity, all four joint types and an exclusion.  It
is stepped on the GPU through ``engine.World``, and every five frames it must
equal the same scene given to the oracle, bit for bit.
"""

import numpy as np
import pytest

from oracle import Oracle
from solver_scenes import add_joints_to_oracle, add_to_oracle, body_specs, build, make_joints, spec_arrays, step_both
from resolve2d_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def test_factory_scene_on_the_gpu_equals_the_oracle():
    specs = body_specs(11)
    s = Solver.init(4.0, 2)
    hs = build(s, specs)
    fac = s.entityFactory()
    fac.makeDownwardsGravity(9.81)
    make_joints(fac, hs)
    fac.excludeCollisionPair(hs[1], hs[2])
    o = Oracle()
    add_to_oracle(o, *spec_arrays(specs))
    o.lib.r2o_add_gravity(o.h, 9.81)
    add_joints_to_oracle(o)
    o.lib.r2o_exclude_pair(o.h, 1, 2)
    step_both(s, o, 30, "factory scene on the GPU")
    s.deinit()


def run_batched_reference_scenes():
    """Three reference-style scenes stepped as one batch (``solver.batch``),
    each world against its own oracle; returns nothing, asserts bit equality."""
    from oracle import ORDER_COLOUR
    from parity import assert_state_equal
    from resolve2d_gb300.solver import batch
    from solver_scenes import DT, ITERS

    groups = [body_specs(70 + k, n=6 + 9 * k) for k in range(3)]
    solvers, oracles = [], []
    for specs in groups:
        s = Solver.init(4.0, 2)  # its own engine is made at its first process, which never comes
        build(s, specs)
        s.entityFactory().makeDownwardsGravity(9.81)
        solvers.append(s)
        o = Oracle()
        add_to_oracle(o, *spec_arrays(specs))
        o.lib.r2o_add_gravity(o.h, 9.81)
        oracles.append(o)
    b = batch(solvers)
    off = [0]
    for specs in groups:
        off.append(off[-1] + len(specs))
    for _ in range(20):
        b.process(DT, 1, ITERS)
        for o in oracles:
            assert o.process(DT, 1, ITERS, ORDER_COLOUR) == 0
    st = b.read_state()
    for k, o in enumerate(oracles):
        assert_state_equal(st[:, off[k]: off[k + 1]], o.state(), f"batched world {k}")


def test_reference_scenes_batched_on_the_gpu_equal_the_oracle():
    run_batched_reference_scenes()


def test_warm_start_survives_an_addition_and_a_swap_remove():
    """Warm starting through the reference-style API: the engine keys last
    frame's impulses by body id, so a body added mid-run and a swapRemove
    (which moves the last body into the hole) keep every surviving pair's
    impulses.  The GPU equals the oracle stand-in that carries its table
    across the rebuild, and differs from one that drops it."""
    from solver_scenes import DT, ITERS, OracleBackend
    from resolve2d_gb300.solver import BodyOptions, Density, DiscOptions

    from parity import assert_state_equal

    specs = body_specs(12)
    gpu = Solver.init(4.0, 2, warm_start=True)
    ref = Solver(backend=lambda: OracleBackend(warm_start=True))
    cold = Solver(backend=lambda: OracleBackend(warm_start=True, carry_warm=False))
    solvers = (gpu, ref, cold)
    for s in solvers:
        build(s, specs)
        s.entityFactory().makeDownwardsGravity(9.81)
    for _ in range(60):
        for s in solvers:
            s.process(DT, 1, ITERS)
    assert_state_equal(gpu.read_state(), ref.read_state(), "before the changes")
    for s in solvers:
        s.entityFactory().makeDiscBody(BodyOptions(pos=(40.0, 5.0), mass_prop=Density(1.0)), DiscOptions(radius=0.5))
        s.removeRigidBody(5)
    assert gpu.ids().tolist() == ref.ids().tolist()
    for f in range(20):
        for s in solvers:
            s.process(DT, 1, ITERS)
        if f in (0, 19):
            assert_state_equal(gpu.read_state(), ref.read_state(), f"frame {f + 1} after the changes")
    assert not np.array_equal(gpu.read_state(), cold.read_state())
    for s in solvers:
        s.deinit()

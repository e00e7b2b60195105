"""The reference-style ``Solver`` / ``EntityFactory`` (resolve2d_gb300/solver.py).

Scenes are built through the factory exactly as the reference's examples build
them (src/examples/*.zig): options, handles, ``body_unwrap().static = true``,
joints by handle, exclusions.  They are compared with the same scene handed to
the oracle directly.  The engine is replaced here by ``OracleBackend``, a test
stand-in with ``engine.World``'s methods that steps the oracle.  These tests
therefore check the solver's own bookkeeping on any host: map order,
``swapRemove``, AABBs of new and old bodies, state write-back and errors.
``tests/test_gpu_solver_api.py`` runs the same scene on the GPU.
"""

import ctypes as C

import numpy as np
import pytest

from oracle import ORDER_COLOUR, Oracle, _p
from parity import assert_state_equal
from resolve2d_gb300 import _native as N
from resolve2d_gb300 import scenes as S
from resolve2d_gb300.solver import BodyOptions, DiscOptions, InvalidRigidBodyId, Mass, NoSuchIdExists, Parameters, Solver
from solver_scenes import (
    DT, ITERS, JOINTS, OracleBackend, add_joints_to_oracle, add_to_oracle, body_specs, build, make_joints, spec_arrays,
    step_both,
)


def test_factory_scene_steps_like_the_same_scene_given_to_the_oracle():
    specs = body_specs(11)
    s = Solver(backend=OracleBackend)
    hs = build(s, specs)
    fac = s.entityFactory()
    fac.makeDownwardsGravity(9.81)
    make_joints(fac, hs)
    fac.excludeCollisionPair(hs[1], hs[2])
    fac.excludeCollisionPair(hs[2], hs[1])  # the same pair
    o = Oracle()
    add_to_oracle(o, *spec_arrays(specs))
    o.lib.r2o_add_gravity(o.h, 9.81)
    add_joints_to_oracle(o)
    o.lib.r2o_exclude_pair(o.h, 1, 2)
    step_both(s, o, 30, "factory scene")
    assert s.ids().tolist() == list(range(len(specs)))
    assert s._dev.calls[:5] == [("set_gravity", 1), ("set_bodies", len(specs), True), ("set_joints", len(JOINTS)),
                                ("set_exclusions", 1), ("process",)]
    assert sum(c[0] == "set_bodies" for c in s._dev.calls) == 1  # nothing re-uploaded between frames


def test_handles_and_views_read_the_reference_fields():
    specs = body_specs(12, n=6)
    s = Solver(backend=OracleBackend)
    hs = build(s, specs)
    shape, bo, go, static = specs[3]
    b = hs[3].body_unwrap()
    assert b.id == 3 and b.type == ("rectangle" if shape == "rect" else "disc") and b.static == static
    m = np.float32(bo.mass_prop.mass) if isinstance(bo.mass_prop, Mass) else None
    if m is not None:
        assert b.props.mass == m
    assert b.props.pos == (np.float32(bo.pos[0]), np.float32(bo.pos[1]))
    assert b.props.momentum.x == np.float32(np.float32(bo.vel[0]) * np.float32(b.props.mass))
    assert b.props.ang_momentum == np.float32(np.float32(bo.omega) * np.float32(b.props.inertia))
    assert s.bodyHandle(999).body() is None
    with pytest.raises(LookupError):
        s.bodyHandle(999).body_unwrap()
    s.process(DT, 1, ITERS)  # the engine computes the first AABBs
    aabb = hs[0].body_unwrap().aabb
    assert aabb.half_width == np.float32(30.0) and aabb.half_height == np.float32(0.5)


def test_bodies_added_mid_run_get_a_first_aabb_and_the_others_keep_theirs():
    specs = body_specs(13)
    first, second = specs[:20], specs[20:]
    s = Solver(backend=OracleBackend)
    build(s, first)
    s.entityFactory().makeDownwardsGravity(9.81)
    o = Oracle()
    add_to_oracle(o, *spec_arrays(first))
    o.lib.r2o_add_gravity(o.h, 9.81)
    step_both(s, o, 10, "before the additions")
    build(s, second)
    add_to_oracle(o, *spec_arrays(second, first_id=len(first)))
    # the stored AABBs only feed the next broadphase, so compare them before stepping
    s._flush()
    assert_state_equal(s.read_state(), o.state(), "right after the additions")
    step_both(s, o, 15, "after the additions")
    assert ("set_bodies", len(specs), True) in s._dev.calls


def test_remove_rigid_body_moves_the_last_body_into_its_slot():
    specs = body_specs(14)
    n = len(specs)
    s = Solver(backend=OracleBackend)
    build(s, specs)
    s.entityFactory().makeDownwardsGravity(9.81)
    o = Oracle()
    ids, kind, opt = spec_arrays(specs)
    add_to_oracle(o, ids, kind, opt)
    o.lib.r2o_add_gravity(o.h, 9.81)
    step_both(s, o, 6, "before the removal")
    s.removeRigidBody(5)
    with pytest.raises(NoSuchIdExists):
        s.removeRigidBody(5)
    order = list(range(n))
    order[5] = n - 1
    order.pop()
    assert s.ids().tolist() == ids[order].tolist()
    st = o.state()[:, order]
    o2 = Oracle()
    add_to_oracle(o2, ids[order], kind[order], np.ascontiguousarray(opt[:, order]))
    o2.lib.r2o_add_gravity(o2.h, 9.81)
    o2.set_state(np.ascontiguousarray(st))
    assert_state_equal(s.read_state(), o2.state(), "right after the removal")
    step_both(s, o2, 10, "after the removal")
    assert ("set_bodies", n - 1, False) in s._dev.calls


def test_writes_through_a_view_reach_the_next_frame():
    specs = body_specs(15)
    s = Solver(backend=OracleBackend)
    hs = build(s, specs)
    s.entityFactory().makeDownwardsGravity(9.81)
    o = Oracle()
    add_to_oracle(o, *spec_arrays(specs))
    o.lib.r2o_add_gravity(o.h, 9.81)
    step_both(s, o, 5, "before the writes")
    p = hs[9].body_unwrap().props
    p.momentum = (3.0, -2.0)
    p.force = (10.0, 40.0)
    p.torque = -5.0
    st = o.state()
    st[S.S_MOM_X, 9], st[S.S_MOM_Y, 9] = 3.0, -2.0
    st[S.S_FORCE_X, 9], st[S.S_FORCE_Y, 9], st[S.S_TORQUE, 9] = 10.0, 40.0, -5.0
    o.set_state(st)
    assert ("write_state",) not in s._dev.calls  # written at the next frame, once
    step_both(s, o, 10, "after the writes")
    assert s._dev.calls.count(("write_state",)) == 1


def test_a_joint_to_a_removed_body_is_invalid_rigid_body_id():
    specs = body_specs(16, n=8)
    s = Solver(backend=OracleBackend)
    hs = build(s, specs)
    s.entityFactory().makeDistanceJoint(Parameters(), hs[3], hs[4], 1.0)
    s.process(DT, 1, ITERS)
    before = s.read_state()
    s.removeRigidBody(4)
    with pytest.raises(InvalidRigidBodyId):
        s.process(DT, 1, ITERS)
    assert np.array_equal(s.read_state()[:, :4], before[:, :4])


def test_clear_drops_everything_and_ids_keep_counting():
    s = Solver(backend=OracleBackend)
    hs = build(s, body_specs(17, n=5))
    fac = s.entityFactory()
    fac.makeDownwardsGravity(9.81)
    fac.makeMotorJoint(Parameters(), hs[2], 1.0)
    fac.excludeCollisionPair(hs[1], hs[2])
    s.process(DT, 1, ITERS)
    s.clear()
    assert s.num_bodies == 0 and s.current_body_id == 6
    s.process(DT, 1, ITERS)  # nothing to step
    h = fac.makeDiscBody(BodyOptions(pos=(0.0, 2.0), mass_prop=Mass(1.0)), DiscOptions(0.5))
    assert h.id == 6
    s.process(DT, 1, ITERS)
    tail = s._dev.calls[-5:]
    assert ("set_gravity", 0) in tail and ("set_joints", 0) in tail and ("set_exclusions", 0) in tail
    assert hs[0].body() is None and h.body_unwrap().props.pos.y < 2.0 + 1e-6


def test_without_bodies_no_engine_is_made_and_gravity_is_capped():
    made = []
    s = Solver(backend=lambda: made.append(1) or OracleBackend())
    s.process(DT, 1, ITERS)
    assert not made
    fac = s.entityFactory()
    for _ in range(4):
        fac.makeDownwardsGravity(9.81)
    with pytest.raises(ValueError):
        fac.makeDownwardsGravity(9.81)
    with pytest.raises(TypeError):
        fac.makeDiscBody(BodyOptions(pos=(0.0, 0.0), mass_prop=2.0))


def test_the_default_engine_is_the_gpu_library():
    """No stand-in: the solver drives the CUDA library, which reports a
    missing device instead of falling back to anything."""
    from conftest import gpu_available

    if gpu_available():
        pytest.skip("a GPU is present; tests/test_gpu_solver_api.py covers this path")
    s = Solver()
    build(s, body_specs(18, n=3))
    with pytest.raises(N.R2DError) as e:
        s.process(DT, 1, ITERS)
    assert e.value.code == -8


def test_the_solver_scene_example_runs(monkeypatch):
    """examples/solver_scene.py, a scene written against the reference's API,
    runs as written (engine replaced by the oracle stand-in), and the disc it
    follows falls onto the ground."""
    from pathlib import Path

    from conftest import REPO
    import resolve2d_gb300.solver as mod

    block = Path(REPO, "examples", "solver_scene.py").read_text()

    class OracleSolver(mod.Solver):
        def __init__(self, *a, **kw):
            super().__init__(*a, backend=OracleBackend, **kw)

    monkeypatch.setattr(mod, "Solver", OracleSolver)
    env = {"print": lambda *a: None}
    exec(block, env)
    a, solver = env["a"], env["solver"]
    assert solver.num_bodies == 2 and env["b"].body() is None
    y = a.body_unwrap().props.pos.y
    assert 0.0 < y < 4.0  # resting on the ground's top face (y = 0), below where it started


def test_bodies_map_and_last_frame_manifolds_are_keyed_by_id():
    specs = body_specs(19)
    n = len(specs)
    s = Solver(backend=OracleBackend)
    build(s, specs)
    s.entityFactory().makeDownwardsGravity(9.81)
    assert s.manifolds() == []  # nothing stepped yet
    for _ in range(3):
        s.process(DT, 1, ITERS)
    s.removeRigidBody(2)  # the last body takes slot 2: ids and slots now differ
    bodies = s.bodies
    assert len(bodies) == bodies.count() == n - 1 and 2 not in bodies
    assert list(bodies) == s.ids().tolist() and list(bodies)[2] == n - 1
    assert bodies[n - 1].id == n - 1
    with pytest.raises(KeyError):
        bodies[2]
    s.process(DT, 1, ITERS)
    ms = s.manifolds()
    k, d, c = s._dev.manifolds()
    assert len(ms) == k.shape[0] > 0
    ids = s.ids()
    for m, key, row, col in zip(ms, k, d, c):
        assert (m.ref_id, m.inc_id) == (ids[key[0]], ids[key[1]]) and m.colour == col
        assert len(m.points) == int(row[5]) + int(row[6])
        assert m.normal == (row[0], row[1]) and m.points[0].depth == row[9 + 6]
    # ids of manifolds name bodies that exist; the removed id never appears
    assert all(m.ref_id in bodies and m.inc_id in bodies for m in ms)
    s.removeRigidBody(5)
    assert {(m.ref_id, m.inc_id) for m in s.manifolds()} == {(m.ref_id, m.inc_id) for m in ms}


def test_batch_arrays_are_the_scene_arrays_a_batch_takes():
    from resolve2d_gb300.solver import batch_arrays

    groups = [body_specs(40 + k, n=5 + 7 * k) for k in range(3)]
    gravity = [9.81, 0.0, 4.5]
    solvers = []
    for specs, g in zip(groups, gravity):
        s = Solver(backend=OracleBackend)
        build(s, specs)
        if g:
            s.entityFactory().makeDownwardsGravity(g)
        solvers.append(s)
    body_off, ids, kind, props, state, grav, init_aabb = batch_arrays(solvers)
    sc = S._concat("three", [spec_arrays(specs) for specs in groups], gravity, DT, 1, ITERS, 1)
    want_props, want_state = S.derive_props_state(sc.kind, sc.opt)
    np.testing.assert_array_equal(body_off, sc.body_off)
    np.testing.assert_array_equal(ids, sc.ids)
    np.testing.assert_array_equal(kind, sc.kind & 3)
    np.testing.assert_array_equal(props, want_props)
    np.testing.assert_array_equal(state, want_state)
    np.testing.assert_array_equal(grav, np.float32(gravity))
    assert init_aabb  # nothing has stepped: the engine computes every first AABB


def test_batch_arrays_of_stepped_solvers_carry_their_states():
    from resolve2d_gb300.solver import batch_arrays

    solvers = []
    for k in range(2):
        s = Solver(backend=OracleBackend)
        build(s, body_specs(50 + k, n=8))
        s.entityFactory().makeDownwardsGravity(9.81)
        for _ in range(3):
            s.process(DT, 1, ITERS)
        solvers.append(s)
    body_off, _, _, _, state, _, init_aabb = batch_arrays(solvers)
    assert not init_aabb
    for k, s in enumerate(solvers):
        np.testing.assert_array_equal(state[:, body_off[k]: body_off[k + 1]], s.read_state())
    # a new body beside stepped ones: the batch cannot give only it a first AABB
    solvers[1].entityFactory().makeDiscBody(BodyOptions(pos=(0.0, 9.0), mass_prop=Mass(1.0)), DiscOptions(0.3))
    with pytest.raises(ValueError):
        batch_arrays(solvers)


def test_batch_arrays_refuse_what_a_batch_cannot_hold():
    from resolve2d_gb300.solver import batch_arrays

    s = Solver(backend=OracleBackend)
    hs = build(s, body_specs(60, n=4))
    s.entityFactory().makeDistanceJoint(Parameters(), hs[1], hs[2], 1.0)
    with pytest.raises(ValueError, match="joints"):
        batch_arrays([s])
    t = Solver(backend=OracleBackend)
    build(t, body_specs(61, n=4))
    t.entityFactory().makeDownwardsGravity(9.81)
    t.entityFactory().makeDownwardsGravity(1.0)
    with pytest.raises(ValueError, match="gravity"):
        batch_arrays([t])


def test_warm_table_carries_across_a_rebuild_on_the_cpu():
    """The oracle stand-in's warm carry (what the GPU test of the same name
    compares against) changes the trajectory: a body added and a swapRemove
    mid-run, with and without last frame's impulses."""
    from resolve2d_gb300.solver import BodyOptions, Density, DiscOptions

    specs = body_specs(12)
    runs = []
    for carry in (True, False):
        s = Solver(backend=lambda carry=carry: OracleBackend(warm_start=True, carry_warm=carry))
        build(s, specs)
        s.entityFactory().makeDownwardsGravity(9.81)
        for _ in range(60):
            s.process(DT, 1, ITERS)
        s.entityFactory().makeDiscBody(BodyOptions(pos=(40.0, 5.0), mass_prop=Density(1.0)), DiscOptions(radius=0.5))
        s.removeRigidBody(5)
        for _ in range(5):
            s.process(DT, 1, ITERS)
        runs.append(s.read_state())
    assert not np.array_equal(runs[0], runs[1])

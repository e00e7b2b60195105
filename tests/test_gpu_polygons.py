"""Convex polygons on the GPU against the oracle, through the C ABI.

A world holding a polygon (R2D_KIND_POLYGON, vertices from
r2d_*_set_polygons) steps on the grid pipeline, whose narrowphase then runs
the polygon-capable SAT and contact clipping (the rectangle's code over each
polygon's vertex ring).  The bar is the rest of the suite's: bit-identical
state, candidate pairs, manifolds and colourings against the oracle
replaying the GPU's colour-major order."""

import numpy as np
import pytest

from oracle import ORDER_COLOUR, Oracle
from parity import assert_manifolds_equal, assert_pairs_equal, assert_state_equal, run_pair
from resolve2d_gb300 import _native as N
from resolve2d_gb300 import scenes
from resolve2d_gb300.engine import Batch, World
from resolve2d_gb300.scenes import KIND_DENSITY, KIND_POLY, KIND_RECT, MASS_PROP, DIM0, DIM1, derive_props_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", range(4))
def test_polygon_scenes(seed):
    run_pair(scenes.polygon_scene(seed, n=40), steps=60, check_every=10)


def test_polygon_scene_substeps_and_warm_start():
    sc = scenes.polygon_scene(7, n=30)
    run_pair(sc, steps=30, check_every=10, sub_steps=4, iters=4)
    run_pair(sc, steps=40, check_every=10, warm=True, comp=True)


def test_four_vertex_polygon_world_equals_the_rectangle_world():
    # the rectangles of a world given as 4-vertex polygons with their own
    # vertex ring, mass and inertia: the same bits on the GPU as on the oracle
    sc = scenes.random_scene(5, n=40)
    props, _ = derive_props_state(sc.kind, sc.opt)
    pc = scenes.Scene(**{f: getattr(sc, f) for f in sc.__dataclass_fields__})
    pc.kind, pc.opt = sc.kind.copy(), sc.opt.copy()
    n = sc.nbodies
    pc.poly_nv = np.zeros(n, np.uint8)
    pc.poly_v = np.zeros((n, scenes.MAX_POLY_VERTS, 2), np.float32)
    for i in np.flatnonzero(sc.kind & KIND_RECT):
        w, h = np.float32(sc.opt[DIM0, i]) / np.float32(2), np.float32(sc.opt[DIM1, i]) / np.float32(2)
        pc.kind[i] = (int(sc.kind[i]) & ~(KIND_RECT | KIND_DENSITY) & 0xFF) | KIND_POLY
        pc.poly_nv[i] = 4
        pc.poly_v[i, :4] = [[-w, -h], [-w, h], [w, h], [w, -h]]
        pc.opt[MASS_PROP, i] = props[0, i]
        pc.opt[DIM1, i] = props[1, i]
    wr = World.from_scene(sc, grid=True)
    wp = World.from_scene(pc)
    for _ in range(40):
        wr.process(sc.dt, 1, 8)
        wp.process(sc.dt, 1, 8)
    wr.sync()
    wp.sync()
    np.testing.assert_array_equal(wp.read_state(), wr.read_state())


def test_batch_of_polygon_worlds_and_plain_worlds():
    poly = scenes.polygon_scene(3, n=25, worlds=3)
    plain = scenes.batched_worlds("plain", seed=4, nworlds=3, steps=1, lo=20, hi=60)
    parts = [poly.world(w) for w in range(3)] + [plain.world(w) for w in range(3)]
    sc = scenes._concat("mixed", [(p.ids, p.kind, p.opt) for p in parts], [9.81] * 6, 1 / 60, 1, 8, 30,
                        polys=[(p.poly_nv if p.poly_nv.size else np.zeros(p.nbodies, np.uint8),
                                p.poly_v if p.poly_v.size else np.zeros((p.nbodies, 8, 2), np.float32))
                               for p in parts])
    b = Batch.from_scene(sc, debug=True)
    oracles = [Oracle.from_scene(sc.world(w)) for w in range(sc.nworlds)]
    for o in oracles:
        o.record_pairs()
    for _ in range(30):
        b.process(sc.dt, 1, 8)
        for o in oracles:
            assert o.process(sc.dt, 1, 8, ORDER_COLOUR) == 0
    b.sync()
    st = b.read_state()
    for w, o in enumerate(oracles):
        b0, b1 = sc.body_off[w], sc.body_off[w + 1]
        assert_state_equal(st[:, b0:b1], o.state(), f"world {w}")
        assert_pairs_equal(b.pairs(w), o.pairs(), f"world {w}")
        gk, gd, gc = b.manifolds(w)
        ok, od = o.manifolds()
        oc, _ = o.colours()
        assert_manifolds_equal(gk, gd, gc, ok, od, oc)


def test_polygon_arguments_are_checked():
    sc = scenes.polygon_scene(1, n=10)
    props, state = derive_props_state(sc.kind, sc.opt)
    from resolve2d_gb300.engine import device_kind

    w = World()
    w.set_gravity(9.81)
    w.set_bodies(sc.ids, device_kind(sc.kind), props, state, True)
    with pytest.raises(N.R2DError) as e:  # vertices never given
        w.process(sc.dt, 1, 8)
    assert e.value.code == -1 and "no vertices" in str(e.value)
    disc = int(np.flatnonzero((sc.kind & (KIND_POLY | KIND_RECT)) == 0)[1])
    with pytest.raises(N.R2DError):  # not a polygon
        w.set_polygons([disc], [3], np.zeros((1, 8, 2), np.float32))
    poly = int(np.flatnonzero(sc.poly_nv)[0])
    with pytest.raises(N.R2DError):  # too many vertices
        w.set_polygons([poly], [9], np.zeros((1, 8, 2), np.float32))
    w.close()

"""Convex polygons in the oracle (the roadmap's next shape, README.md:64-67,
behind the RigidBody vtable, src/core/Bodies/RigidBody.zig:33-42): a polygon
runs the rectangle's code (Rectangle.zig:71-238) over its own vertex ring.

- A 4-vertex polygon with a rectangle's vertices, in the rectangle's order,
  mass and inertia steps bit for bit like that rectangle.
- A polygon's AABB is the largest rotated vertex in x and y
  (Rectangle.zig:71-86 over its vertices).
- A triangle and a hexagon dropped flat onto the ground come to rest on an
  edge, with two contact points along the ground's normal.
"""

import numpy as np

from oracle import ORDER_COLOUR, Oracle
from resolve2d_gb300 import scenes
from resolve2d_gb300.scenes import KIND_DENSITY, KIND_POLY, KIND_RECT, MASS_PROP, DIM0, DIM1, derive_props_state


def _as_polygons(sc):
    """The scene with every rectangle given as a 4-vertex polygon: the
    rectangle's own vertices (-w,-h), (-w,h), (w,h), (w,-h), its mass and
    inertia."""
    props, _ = derive_props_state(sc.kind, sc.opt)
    pc = scenes.Scene(**{f: getattr(sc, f) for f in sc.__dataclass_fields__})
    pc.kind = sc.kind.copy()
    pc.opt = sc.opt.copy()
    n = sc.nbodies
    pc.poly_nv = np.zeros(n, np.uint8)
    pc.poly_v = np.zeros((n, scenes.MAX_POLY_VERTS, 2), np.float32)
    for i in np.flatnonzero(sc.kind & KIND_RECT):
        w, h = np.float32(sc.opt[DIM0, i]) / np.float32(2), np.float32(sc.opt[DIM1, i]) / np.float32(2)
        pc.kind[i] = (int(sc.kind[i]) & ~(KIND_RECT | KIND_DENSITY) & 0xFF) | KIND_POLY
        pc.poly_nv[i] = 4
        pc.poly_v[i, :4] = [[-w, -h], [-w, h], [w, h], [w, -h]]
        pc.opt[MASS_PROP, i] = props[0, i]
        pc.opt[DIM0, i] = sc.opt[DIM0, i]
        pc.opt[DIM1, i] = props[1, i]  # a polygon's DIM1 holds its inertia
    return pc


def test_four_vertex_polygon_steps_like_the_rectangle():
    sc = scenes.random_scene(5, n=40)
    pc = _as_polygons(sc)
    a, b = Oracle.from_scene(sc), Oracle.from_scene(pc)
    pa = a.props()
    pb = b.props()
    np.testing.assert_array_equal(pa[:3], pb[:3])
    for step in range(60):
        assert a.process(sc.dt, 1, 8, ORDER_COLOUR) == 0
        assert b.process(sc.dt, 1, 8, ORDER_COLOUR) == 0
        np.testing.assert_array_equal(a.state(), b.state(), err_msg=f"step {step + 1}")
    ka, da = a.manifolds()
    kb, db = b.manifolds()
    np.testing.assert_array_equal(ka, kb)
    np.testing.assert_array_equal(np.nan_to_num(da), np.nan_to_num(db))


def test_polygon_aabb_is_its_largest_rotated_vertex():
    b = scenes._Builder()
    verts = [[0.0, 1.0], [0.9, 0.3], [0.6, -0.8], [-0.6, -0.8], [-0.9, 0.3]]
    b.polygon(2.0, 3.0, verts, 0.5, angle=0.7)
    ids, kind, opt = b.arrays()
    sc = scenes._concat("pentagon", [(ids, kind, opt)], [0.0], 1 / 60, 1, 8, 1, polys=[b.polygon_arrays()])
    o = Oracle.from_scene(sc)
    st = o.state()
    v = sc.poly_v[0, :5].astype(np.float64)
    c, s = np.cos(0.7), np.sin(0.7)
    rx, ry = v[:, 0] * c - v[:, 1] * s, v[:, 0] * s + v[:, 1] * c
    assert st[9, 0] == np.float32(2.0) and st[10, 0] == np.float32(3.0)
    assert abs(st[11, 0] - max(0.0, rx.max())) < 1e-6 and abs(st[12, 0] - max(0.0, ry.max())) < 1e-6


def _rest_on_ground(verts, frames=240):
    b = scenes._Builder()
    b.rect(0.0, -0.5, 20.0, 1.0, 0.5, static=True)
    b.polygon(0.0, 1.5, verts, 0.5)
    ids, kind, opt = b.arrays()
    sc = scenes._concat("rest", [(ids, kind, opt)], [9.81], 1 / 60, 1, 8, frames, polys=[b.polygon_arrays()])
    o = Oracle.from_scene(sc)
    for _ in range(frames):
        assert o.process(sc.dt, 1, 8, ORDER_COLOUR) == 0
    return sc, o


def test_triangle_comes_to_rest_on_its_edge():
    sc, o = _rest_on_ground([[-0.8, -0.4], [0.8, -0.4], [0.0, 0.9]])
    st = o.state()
    m = o.props()[0, 1]
    assert abs(st[3, 1] / m) < 1e-2 and abs(st[4, 1] / m) < 5e-2  # at rest
    assert abs(np.sin(st[2, 1])) < 1e-3  # still flat
    k, d = o.manifolds()
    assert len(k) == 1 and d[0, 5] == 1.0 and d[0, 6] == 1.0  # two contact points
    assert abs(abs(d[0, 1]) - 1.0) < 1e-6  # along the ground's normal
    # the lowest vertices sit on the ground's top face (y = 0) within the contact slop
    v = sc.poly_v[1, :3].astype(np.float64)
    y = st[1, 1] + v[:, 1]
    assert -0.02 < y.min() < 0.01


def test_hexagon_comes_to_rest_on_its_edge():
    a = np.arange(6) * np.pi / 3.0
    verts = np.stack([0.6 * np.cos(a), 0.6 * np.sin(a)], axis=1)  # flat top and bottom edges
    sc, o = _rest_on_ground(verts)
    y0 = o.state()[1, 1]
    for _ in range(80):  # resting: the pose holds (the solver leaves a frame's gravity in the momentum)
        assert o.process(sc.dt, 1, 8, ORDER_COLOUR) == 0
    st = o.state()
    assert abs(st[1, 1] - y0) < 1e-3 and abs(np.sin(st[2, 1])) < 1e-3
    assert abs(st[1, 1] - 0.5196) < 0.01  # the bottom edge (0.52 below the centre) on the ground
    k, d = o.manifolds()
    assert len(k) == 1 and d[0, 5] == 1.0 and d[0, 6] == 1.0
    assert abs(abs(d[0, 1]) - 1.0) < 1e-6

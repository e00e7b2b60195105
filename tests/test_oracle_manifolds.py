"""Rectangle manifolds of the oracle, worked by hand from the reference.

SAT runs over the lower id's normals, then the other body's
(collision.zig:299-320).  A box lying flat on the ground has a bottom normal
opposite to the ground's top normal.  The opposite-normal rule
(collision.zig:270-277) then hands the reference role to the box, because its
normal points toward the ground.  A box on its corner has no such normal, so
the ground stays the reference.  The incident edge is the other body's edge
most opposed to the normal (Rectangle.zig:219-236).  It is
clipped to the reference edge (clipLineToLine, collision.zig:330-363), and each
end deeper than COLLISION_MARGIN becomes a point (Rectangle.zig:171-209).  The
point is stored at p - n*depth/2 (collision.zig:38-51).  CPU only.
"""

import math

import numpy as np

from oracle import Oracle
from resolve2d_gb300 import scenes

P0 = 9  # first float of point 0 in a manifold row; 12 floats a point
POS, REF_R, INC_R, DEPTH = 0, 2, 4, 6


def world(bodies):
    b = scenes._Builder()
    for spec in bodies:
        getattr(b, spec[0])(*spec[1:])
    return Oracle.from_scene(scenes._concat("hand", [b.arrays()], [9.81], 1 / 60, 1, 8, 1))


def points(row):
    out = []
    for p in range(2):
        if row[5 + p]:
            base = P0 + 12 * p
            out.append({k: row[base + off: base + off + (1 if k == "depth" else 2)]
                        for k, off in (("pos", POS), ("ref_r", REF_R), ("inc_r", INC_R), ("depth", DEPTH))})
    return out


def ground(width=10.0):
    # static, top face at y = 0
    return ("rect", 0.0, -0.5, width, 1.0, 0.5, 1.0, 0.0, 0.0, 0.0, 0.0, True)


def test_box_resting_flat_gets_two_points_at_its_bottom_corners():
    # The box (id 1) is the reference, with normal (0, -1).  The ground's top edge
    # is clipped to the box's bottom edge: ends at x = -0.5 and 0.5, y = 0,
    # depth -0.01, stored 0.005 lower.
    o = world([ground(), ("rect", 0.0, 0.49, 1.0, 1.0, 0.5)])
    assert o.update_manifolds() == 0
    k, d = o.manifolds()
    assert k.tolist() == [[1, 0]]
    np.testing.assert_allclose(d[0, :2], [0.0, -1.0], atol=1e-6)
    pts = points(d[0])
    assert len(pts) == 2
    xs = sorted(float(p["pos"][0]) for p in pts)
    np.testing.assert_allclose(xs, [-0.5, 0.5], atol=1e-6)
    for p in pts:
        assert abs(p["depth"][0] + 0.01) < 1e-6
        assert abs(p["pos"][1] + 0.005) < 1e-6  # the middle of the overlap
        np.testing.assert_allclose(p["ref_r"], p["pos"] - np.array([0.0, 0.49], np.float32), atol=1e-6)
        np.testing.assert_allclose(p["inc_r"], p["pos"] - np.array([0.0, -0.5], np.float32), atol=1e-6)


def test_box_past_the_end_of_the_reference_edge_is_clipped_to_it():
    # A 1-wide ground (top edge x in [-0.5, 0.5]) and a box over x in [0.2, 1.2]:
    # the side overlaps are 0.3, the vertical ones 0.01, so the box's bottom edge
    # is the reference (the opposite-normal rule).  The ground's top edge is
    # clipped to it: its end at x = 0.5 lies inside and stays; the end at x = -0.5
    # lies outside and moves along the edge to x = 0.2, the nearer end of the
    # reference edge.
    o = world([ground(1.0), ("rect", 0.7, 0.49, 1.0, 1.0, 0.5)])
    assert o.update_manifolds() == 0
    k, d = o.manifolds()
    assert k.tolist() == [[1, 0]]
    np.testing.assert_allclose(d[0, :2], [0.0, -1.0], atol=1e-6)
    pts = points(d[0])
    assert len(pts) == 2
    xs = sorted(float(p["pos"][0]) for p in pts)
    np.testing.assert_allclose(xs, [0.2, 0.5], atol=1e-6)
    for p in pts:
        assert abs(p["depth"][0] + 0.01) < 1e-6


def test_box_on_its_corner_gets_one_point():
    # Rotated 45 degrees, its lowest corner 0.01 below the ground's top.  The
    # incident edge runs from that corner up to a neighbour 0.707 higher, which is
    # above COLLISION_MARGIN, so only the corner is a point.
    h = math.sqrt(0.5)
    o = world([ground(), ("rect", 0.0, h - 0.01, 1.0, 1.0, 0.5, 1.0, 0.0, 0.0, math.pi / 4, 0.0)])
    assert o.update_manifolds() == 0
    k, d = o.manifolds()
    assert k.tolist() == [[0, 1]]
    np.testing.assert_allclose(d[0, :2], [0.0, 1.0], atol=1e-6)
    pts = points(d[0])
    assert len(pts) == 1
    assert abs(pts[0]["depth"][0] + 0.01) < 1e-5
    np.testing.assert_allclose(pts[0]["pos"], [0.0, -0.005], atol=1e-5)


def test_boxes_apart_by_more_than_the_margin_make_no_manifold():
    # AABBs 0.02 apart: beyond the 0.01 overlap margin of aabb.zig, so no pair
    o = world([ground(), ("rect", 0.0, 0.52, 1.0, 1.0, 0.5)])
    assert o.update_manifolds() == 0
    k, _ = o.manifolds()
    assert k.shape[0] == 0


def test_disc_over_a_box_corner_becomes_the_reference():
    # Box 2x2 at the origin (id 0, static), disc r = 0.5 at (1.3, 1.3) (id 1).  The
    # box's faces overlap the disc by 0.2.  The disc's one axis runs from its
    # centre to the box's closest point, which for a rectangle is its nearest
    # vertex (1, 1) (Rectangle.zig:114-130).  Along that axis the overlap is
    # 0.5 - 0.3*sqrt(2) = 0.0757, smaller, so the disc is the reference
    # (collision.zig:281-286).  Its single point is that vertex, at depth
    # |c - v| - r (Disc.zig:99-123), stored half the depth along the normal.
    o = world([("rect", 0.0, 0.0, 2.0, 2.0, 0.5, 1.0, 0.0, 0.0, 0.0, 0.0, True), ("disc", 1.3, 1.3, 0.5, 0.5)])
    assert o.update_manifolds() == 0
    k, d = o.manifolds()
    assert k.tolist() == [[1, 0]]
    s = math.sqrt(0.5)
    np.testing.assert_allclose(d[0, :2], [-s, -s], atol=1e-6)
    pts = points(d[0])
    assert len(pts) == 1
    depth = 0.3 * math.sqrt(2.0) - 0.5
    assert abs(pts[0]["depth"][0] - depth) < 1e-6
    np.testing.assert_allclose(pts[0]["pos"], [1.0 + s * depth / 2, 1.0 + s * depth / 2], atol=1e-6)


def test_disc_beside_a_box_face_meets_the_face():
    # Disc r = 0.5 at (1.3, 0.0): the box's right face (overlap 0.2) beats the
    # disc's axis toward the vertex (1, 1), so the box is the reference.  The
    # disc's incident point is its centre minus r along the normal (Disc.zig:125-130):
    # (0.8, 0), depth -0.2, stored at (0.9, 0).
    o = world([("rect", 0.0, 0.0, 2.0, 2.0, 0.5, 1.0, 0.0, 0.0, 0.0, 0.0, True), ("disc", 1.3, 0.0, 0.5, 0.5)])
    assert o.update_manifolds() == 0
    k, d = o.manifolds()
    assert k.tolist() == [[0, 1]]
    np.testing.assert_allclose(d[0, :2], [1.0, 0.0], atol=1e-6)
    pts = points(d[0])
    assert len(pts) == 1
    assert abs(pts[0]["depth"][0] + 0.2) < 1e-6
    np.testing.assert_allclose(pts[0]["pos"], [0.9, 0.0], atol=1e-6)

"""The reference's own unit tests, run against the oracle's restatement.

src/core/nmath.zig:157-176 ("vector2") and src/core/aabb.zig:34-45
("sanity check aabb overlapping") are the only tests the reference holds for
the step's arithmetic; they are the oracle's known-answer pins.
"""

import numpy as np

import oracle as O


def test_vector2_known_answers():
    # nmath.zig:157-176
    a, b = (2, 3), (4, 5)
    out = O.nmath_kat(a, b)
    f = np.float32
    assert (out[0], out[1]) == (6, 8)                     # add2
    assert (out[2], out[3]) == (-2, -2)                   # sub2
    assert (out[4], out[5]) == (8, 15)                    # multelem2
    assert (out[6], out[7]) == (f(0.5), f(0.6))           # divelem2 (f32 literals)
    assert out[8] == 23                                   # dot2
    assert out[9] == -2                                   # cross2
    assert out[10] == 13                                  # length2sq(a)
    assert out[11] == np.sqrt(f(13))                      # length2(a) == @sqrt(13)
    out_b = O.nmath_kat(b, a)
    assert out_b[10] == 41 and out_b[11] == np.sqrt(f(41))


def test_aabb_overlap_known_answers():
    # aabb.zig:34-45
    s1 = [1, 1, 1.0, 0.5]
    s2 = [2, 3, 1.5, 3.0]
    assert O.aabb_intersects(s1, s2)
    s2[1] = 10
    assert not O.aabb_intersects(s1, s2)
    s1[1] = 10
    assert O.aabb_intersects(s1, s2)


def test_aabb_epsilon_boundary():
    # the +0.01 slack of AABB_EPS_OVERLAP (simulation_constants.zig:14, aabb.zig:12-19)
    f = np.float32
    hw = f(0.5)
    gap_in = f(1.0) + f(0.0099)
    gap_out = f(1.0) + f(0.0101)
    assert O.aabb_intersects([0, 0, hw, hw], [gap_in, 0, hw, hw])
    assert not O.aabb_intersects([0, 0, hw, hw], [gap_out, 0, hw, hw])

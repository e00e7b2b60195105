"""Compensated accumulation of a contact point's impulses (r2d_accum.h,
R2D_FLAG_COMPENSATED), through the oracle's copy of the shared header: the
accumulated impulse s + c tracks the exact sum of its increments where plain
f32 accumulation loses them, the clamps behave as the reference's
(collision.zig:182-190), and the bodies receive exactly the changes of s."""

import numpy as np

from oracle import acc_sum


def test_small_increments_onto_a_large_sum_are_kept():
    # 1e-5 is under half an ulp of 1000 (3.05e-5): plain f32 never moves
    x = np.full(100_000, 1e-5, np.float32)
    plain = np.float32(1000.0)
    for v in x[:1000]:
        plain = np.float32(plain + v)
    assert plain == np.float32(1000.0)
    s, c, applied = acc_sum(x, s0=1000.0)
    exact = 1000.0 + float(np.sum(x.astype(np.float64)))
    assert abs((float(s) + float(c)) - exact) < 1e-3 * 1e-5 * 100_000
    assert abs(float(s) - exact) <= float(np.spacing(np.float32(exact)))
    assert applied == np.float32(s) - np.float32(1000.0)


def test_the_lower_clamp_is_exact_and_clears_the_compensation():
    s, c, applied = acc_sum(np.array([1.0, -0.3, -5.0], np.float32), s0=0.0)
    assert s == 0.0 and c == 0.0
    assert applied == 0.0


def test_the_friction_clamp_bounds_the_sum():
    s, c, _ = acc_sum(np.full(10, 0.4, np.float32), s0=0.0, lo=-1.0, hi=1.0)
    assert s == np.float32(1.0) and c == 0.0
    s, c, _ = acc_sum(np.full(10, -0.4, np.float32), s0=0.0, lo=-1.0, hi=1.0)
    assert s == np.float32(-1.0) and c == 0.0


def test_a_nan_increment_clamps_to_the_bound():
    s, c, _ = acc_sum(np.array([0.5, np.nan], np.float32), s0=0.0)
    assert s == 0.0 and c == 0.0


def test_compensated_sums_track_float64_over_a_random_walk():
    rng = np.random.default_rng(0)
    x = rng.normal(1e-3, 1e-3, 200_000).astype(np.float32)
    s, c, _ = acc_sum(x, s0=50.0)
    exact = 50.0
    for v in x.astype(np.float64):
        exact = max(0.0, exact + v)
    plain = np.float32(50.0)
    for v in x:
        plain = max(np.float32(0.0), np.float32(plain + v))
    assert abs(float(s) + float(c) - exact) < 1e-5
    assert abs(float(plain) - exact) > 10 * abs(float(s) + float(c) - exact)

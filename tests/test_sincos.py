"""Accuracy of the shared f32 sin/cos (resolve2d_gb300/csrc/r2d_sincos.h).

The reference's rotate2 (src/core/nmath.zig:129-136) calls libm's f32 sin and
cos.  The project's stand-in must be a faithful sin/cos: every result within
one ulp of the exact value, and correctly rounded for almost all inputs.
"""

import mpmath
import numpy as np

import oracle as O


def _ulp_err(got: np.ndarray, exact: list) -> np.ndarray:
    out = np.empty(len(exact))
    for i, (g, e) in enumerate(zip(got.astype(np.float64), exact)):
        ulp = float(np.spacing(np.float32(abs(e)) if e != 0 else np.float32(1e-45)))
        out[i] = abs(g - e) / ulp
    return out


def test_sincos_accuracy_random():
    rng = np.random.default_rng(123)
    x = np.concatenate([
        rng.uniform(-4, 4, 3000),
        rng.uniform(-200, 200, 1500),
        rng.uniform(-1e4, 1e4, 500),
        np.array([0.0, -0.0, 1e-30, -1e-30, 1e-8, np.pi / 2, np.pi, 2 * np.pi, 1.0, -1.0]),
    ]).astype(np.float32)
    s, c = O.sincosf(x)
    mpmath.mp.prec = 120
    es = [float(mpmath.sin(mpmath.mpf(float(v)))) for v in x]
    ec = [float(mpmath.cos(mpmath.mpf(float(v)))) for v in x]
    ds, dc = _ulp_err(s, es), _ulp_err(c, ec)
    assert ds.max() <= 0.5 + 1e-6 or (ds > 0.5 + 1e-6).mean() < 1e-3
    assert dc.max() <= 0.5 + 1e-6 or (dc > 0.5 + 1e-6).mean() < 1e-3
    assert ds.max() < 1.0 and dc.max() < 1.0


def test_sincos_special_values():
    s, c = O.sincosf(np.array([0.0, -0.0, np.inf, -np.inf, np.nan], np.float32))
    assert s[0] == 0 and not np.signbit(s[0]) and c[0] == 1
    assert s[1] == 0 and np.signbit(s[1]) and c[1] == 1
    assert np.isnan(s[2:]).all() and np.isnan(c[2:]).all()

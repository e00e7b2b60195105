"""Helpers shared by the parity tests: run a scene on the GPU path and on the
oracle, and compare results bit for bit.

Float comparison is by value with NaN == NaN: the GPU path skips the +0 the
reference adds to a static body (collision.zig:208-212), which can only turn
a -0.0 into +0.0, so signed zeros are not distinguished.  Everything else must
be identical.
"""

from __future__ import annotations

import numpy as np
import pytest

FIELDS = ["pos_x", "pos_y", "angle", "mom_x", "mom_y", "ang_mom", "force_x", "force_y", "torque",
          "aabb_x", "aabb_y", "aabb_hw", "aabb_hh"]


def mismatch(got: np.ndarray, want: np.ndarray) -> np.ndarray:
    got = np.asarray(got)
    want = np.asarray(want)
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    return ~same


def assert_state_equal(got: np.ndarray, want: np.ndarray, what: str = "state"):
    assert got.shape == want.shape, (got.shape, want.shape)
    bad = mismatch(got, want)
    if bad.any():
        idx = np.argwhere(bad)
        lines = []
        for f, i in idx[:8]:
            lines.append(f"  {FIELDS[f] if got.shape[0] == 13 else f}[{i}]: gpu {got[f, i]!r} oracle {want[f, i]!r}")
        raise AssertionError(f"{what}: {len(idx)} entries differ\n" + "\n".join(lines))


def manifold_table(keys: np.ndarray, data: np.ndarray, colours: np.ndarray | None):
    """Manifolds keyed by (reference, incident), dropping the point positions
    (the GPU keeps ref_r / inc_r, not the contact position)."""
    out = {}
    for m in range(keys.shape[0]):
        d = data[m].copy()
        d[9:11] = 0.0   # point 0 pos
        d[21:23] = 0.0  # point 1 pos
        npts = int(d[5]) + int(d[6])
        if npts < 2:
            d[21:33] = 0.0
        if npts < 1:
            d[9:21] = 0.0
        out[(int(keys[m, 0]), int(keys[m, 1]))] = (d, None if colours is None else int(colours[m]))
    return out


def assert_manifolds_equal(gk, gd, gc, ok, od, oc):
    g = manifold_table(gk, gd, gc)
    o = manifold_table(ok, od, oc)
    assert set(g) == set(o), f"pair sets differ: gpu-only {sorted(set(g) - set(o))[:5]} oracle-only {sorted(set(o) - set(g))[:5]}"
    for k in o:
        dg, cg = g[k]
        do, co = o[k]
        bad = mismatch(dg, do)
        assert not bad.any(), f"manifold {k}: fields {np.flatnonzero(bad).tolist()} gpu {dg[bad]} oracle {do[bad]}"
        assert cg == co, f"manifold {k}: colour gpu {cg} oracle {co}"


def assert_pairs_equal(got: np.ndarray, want: np.ndarray, what: str = "pairs"):
    """Candidate pair sets (the pairs that reached the narrowphase), both
    sorted (lower, higher) index rows: identical, each pair once."""
    g = set(map(tuple, np.asarray(got).tolist()))
    o = set(map(tuple, np.asarray(want).tolist()))
    assert len(g) == len(got), f"{what}: the GPU reported a pair twice"
    assert g == o, f"{what}: gpu-only {sorted(g - o)[:5]} oracle-only {sorted(o - g)[:5]}"
    np.testing.assert_array_equal(np.asarray(got, np.uint32).reshape(-1, 2), np.asarray(want, np.uint32).reshape(-1, 2))


def run_pair(sc, steps, check_every=1, debug=True, sub_steps=None, iters=None, warm=False, comp=False, **world_kw):
    """Step scene `sc` on the GPU (one world through the C ABI) and on the
    oracle in colour-major order; compare state, manifolds and colours every
    `check_every` steps.  Returns (world, oracle), or (None, None) when the
    step fails on both with the same status."""
    from oracle import ORDER_COLOUR, Oracle
    from resolve2d_gb300 import _native as N
    from resolve2d_gb300.engine import World

    S = sc.sub_steps if sub_steps is None else sub_steps
    I = sc.iters if iters is None else iters
    w = World.from_scene(sc, debug=debug, warm_start=warm, compensated=comp, **world_kw)
    o = Oracle.from_scene(sc)
    o.set_warm_start(warm)
    o.set_compensated(comp)
    o.record_pairs(debug)
    assert_state_equal(w.read_state(), o.state(), "initial state")
    for s in range(steps):
        want = o.process(sc.dt, S, I, ORDER_COLOUR)
        if want != 0:
            # the reference's step fails here too (e.g. a non-finite AABB,
            # whose @intFromFloat is undefined); the GPU must report the same
            # error and leave the state of the last good step
            with pytest.raises(N.R2DError) as e:
                w.process(sc.dt, S, I)
                w.sync()
            assert e.value.code == want, (e.value.code, want)
            return None, None
        w.process(sc.dt, S, I)
        w.sync()
        if (s + 1) % check_every == 0 or s + 1 == steps:
            assert_state_equal(w.read_state(), o.state(), f"{sc.name} step {s + 1}")
            if debug:
                assert_pairs_equal(w.pairs(), o.pairs(), f"{sc.name} step {s + 1}")
                gk, gd, gc = w.manifolds()
                ok, od = o.manifolds()
                oc, _ = o.colours()
                assert_manifolds_equal(gk, gd, gc, ok, od, oc)
    return w, o

"""Golden fixtures (tests/golden/golden_*.npz, written by make_golden.py from
the oracle): the oracle must reproduce them on every machine, and the CUDA
path must reproduce the colour-order ones bit for bit (signed zeros aside,
see parity.py)."""

import glob
import os
import sys

import numpy as np
import pytest

from oracle import ORDER_COLOUR
from parity import assert_manifolds_equal, assert_state_equal

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "golden_*.npz")))
NAMES = [os.path.basename(p)[len("golden_"):-len(".npz")] for p in FIXTURES]


def test_every_case_has_a_fixture():
    assert sorted(NAMES) == sorted(make_golden.CASES)


def _load(name):
    return dict(np.load(os.path.join(HERE, "golden", f"golden_{name}.npz")))


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_fixture(name):
    want = _load(name)
    got = make_golden.run_case(name)
    for k in want:
        if k.startswith("state_") or k == "initial":
            assert_state_equal(got[k], want[k], f"{name} {k}")
    np.testing.assert_array_equal(got["keys"], want["keys"])
    np.testing.assert_array_equal(got["data"].view(np.uint32), want["data"].view(np.uint32))
    np.testing.assert_array_equal(got["contact_colours"], want["contact_colours"])
    np.testing.assert_array_equal(got["joint_colours"], want["joint_colours"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in NAMES if int(_load(n)["meta"][2]) == ORDER_COLOUR])
@pytest.mark.parametrize("grid", [False, True])
def test_gpu_reproduces_fixture(name, grid):
    from resolve2d_gb300.engine import World

    make, keep, _, _, _ = make_golden.CASES[name]
    sc = make()
    want = _load(name)
    S, I, _, last = (int(v) for v in want["meta"])
    w = World.from_scene(sc, debug=True, grid=grid)
    assert_state_equal(w.read_state(), want["initial"], f"{name} initial")
    for s in range(1, last + 1):
        w.process(sc.dt, S, I)
        w.sync()
        if f"state_{s}" in want:
            assert_state_equal(w.read_state(), want[f"state_{s}"], f"{name} step {s}")
    gk, gd, gc = w.manifolds()
    assert_manifolds_equal(gk, gd, gc, want["keys"], want["data"], want["contact_colours"])
    if sc.jtype.size:
        np.testing.assert_array_equal(w.joint_colours(len(sc.jtype)), want["joint_colours"])

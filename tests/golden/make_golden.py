"""Generate the golden fixtures in this folder from the oracle.

The reference ships no golden data (its only tests are the Vector2 and AABB
cases), so these vectors are the oracle's own outputs on seeded scenes,
committed so that (1) the oracle is checked against them on every machine it
runs on (x86 here, Arm beside the GPU), and (2) the CUDA path is compared with
fixed files as well as with a live oracle run.

    python tests/golden/make_golden.py        # rewrites golden_*.npz

Each fixture holds the scene's seed and generator name, the state (float32
[13][n], field-major) after the listed steps, the manifolds of the last step
(keys [m][2] and data [m][33], sorted by key) and the colourings.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [REPO, os.path.join(REPO, "oracle")]

from oracle import ORDER_COLOUR, ORDER_REFERENCE, Oracle  # noqa: E402
from resolve2d_gb300 import build, scenes  # noqa: E402

# name -> (scene factory, steps at which the state is kept, sub_steps, iters, solve order)
CASES = {
    "config0": (lambda: scenes.config0(), (1, 10, 100), None, None, ORDER_COLOUR),
    "config0_reference_order": (lambda: scenes.config0(), (10, 60), None, None, ORDER_REFERENCE),
    "random3_joints": (lambda: scenes.random_scene(3, n=40, joints=True), (1, 20), None, None, ORDER_COLOUR),
    "random11_substeps": (lambda: scenes.random_scene(11, n=30, joints=True), (5,), 4, 4, ORDER_COLOUR),
}


def run_case(name):
    make, keep, S, I, order = CASES[name]
    sc = make()
    S = sc.sub_steps if S is None else S
    I = sc.iters if I is None else I
    o = Oracle.from_scene(sc)
    out = {"initial": o.state()}
    for s in range(1, max(keep) + 1):
        st = o.process(sc.dt, S, I, order)
        assert st == 0, (name, s, st)
        if s in keep:
            out[f"state_{s}"] = o.state()
    keys, data = o.manifolds()
    cc, jc = o.colours()
    idx = np.lexsort((keys[:, 1], keys[:, 0])) if len(keys) else np.zeros(0, np.int64)
    out["keys"] = keys[idx].astype(np.uint32)
    out["data"] = data[idx].astype(np.float32)
    cc = np.asarray(cc)
    # the reference order computes no colouring
    out["contact_colours"] = cc[idx].astype(np.uint32) if cc.size == len(keys) else np.zeros(0, np.uint32)
    out["joint_colours"] = np.asarray(jc).astype(np.uint32)
    out["meta"] = np.array([S, I, order, max(keep)], np.int64)
    return out


def main():
    build.build_oracle()
    for name in CASES:
        out = run_case(name)
        path = os.path.join(HERE, f"golden_{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {os.path.getsize(path)} bytes, {len(out['keys'])} manifolds")


if __name__ == "__main__":
    main()

"""Precision study on the long-horizon workload (16,384 worlds of the
batched distribution, seed 4, 3,600 steps at dt 1/60).

    python tests/precision_study.py [--worlds 16384] [--steps 3600]
        [--checkpoints 1,10,60,120,300,600] [--oracle-worlds 256]
        [--out profiles/precision_config4.json]

Two GPU modes step every world from the same start: f32 throughout (the
reference's arithmetic, bit-identical to the f32 oracle) and f32 with the
pose integrated in f64 (R2D_FLAG_FP64_POSITIONS).  The first
`--oracle-worlds` worlds are also stepped by the FP64 oracle (the same
algorithm in double) on the host threads.  Reported, at the checkpoints:

* position error against the FP64 oracle, in body radii (a disc's radius,
  half the shorter side of a rectangle): max, p99, median;
* momentum and energy of each world against the FP64 oracle's: relative
  difference of the total linear momentum |sum p| and of the energy
  sum(|p|^2/2m + L^2/2I + m g y);
* energy drift of each mode over the run: (E(t) - E(0)) / |E(0)| per world;
* penetration depth percentiles (p50, p99, max) of the contact points of the
  oracle-compared worlds at the last step, from the debug taps.

Prints one JSON object and writes it to --out when given.
"""

from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path[:0] = [REPO, os.path.join(REPO, "oracle")]

import oracle as O  # noqa: E402
from resolve2d_gb300 import build, scenes  # noqa: E402
from resolve2d_gb300.engine import Batch  # noqa: E402
from resolve2d_gb300.scenes import DIM0, DIM1, KIND_RECT, KIND_STATIC, derive_props_state  # noqa: E402


def world_energy(sc, state, props, g_world):
    """Per-world linear momentum magnitude and energy (f64)."""
    st = state.astype(np.float64)
    m, inertia = props[0].astype(np.float64), props[1].astype(np.float64)
    dyn = (sc.kind & KIND_STATIC) == 0
    g = np.repeat(g_world.astype(np.float64), np.diff(sc.body_off))
    ke = np.where(dyn, (st[3] ** 2 + st[4] ** 2) / (2 * m) + st[5] ** 2 / (2 * inertia), 0.0)
    pe = np.where(dyn, m * g * st[1], 0.0)
    idx = np.repeat(np.arange(sc.nworlds), np.diff(sc.body_off))
    e = np.bincount(idx, weights=ke + pe, minlength=sc.nworlds)
    px = np.bincount(idx, weights=np.where(dyn, st[3], 0.0), minlength=sc.nworlds)
    py = np.bincount(idx, weights=np.where(dyn, st[4], 0.0), minlength=sc.nworlds)
    return np.hypot(px, py), e


def radii(sc):
    rect = (sc.kind & KIND_RECT) != 0
    return np.where(rect, 0.5 * np.minimum(sc.opt[DIM0], sc.opt[DIM1]), sc.opt[DIM0]).astype(np.float64)


def pos_error(sc, got, want):
    dyn = (sc.kind & KIND_STATIC) == 0
    err = np.hypot(got[0] - want[0], got[1] - want[1])[dyn] / radii(sc)[dyn]
    return {"max": float(err.max()), "p99": float(np.percentile(err, 99)), "median": float(np.median(err)),
            "frac_below_1e-3": float((err < 1e-3).mean())}


def rel(a, b):
    d = np.abs(a - b) / np.maximum(np.abs(b), 1e-12)
    return {"median": float(np.median(d)), "p99": float(np.percentile(d, 99)), "max": float(d.max())}


def penetration(batch, nworlds):
    depths = []
    for w in range(nworlds):
        _, d, _ = batch.manifolds(w)
        for p in range(2):
            has = d[:, 5 + p] > 0
            depths.append(-d[has, 9 + 12 * p + 6].astype(np.float64))
    x = np.concatenate(depths) if depths else np.zeros(1)
    x = np.maximum(x, 0.0)  # penetration = -depth where depth < 0
    return {"points": int(x.size), "p50": float(np.percentile(x, 50)), "p99": float(np.percentile(x, 99)),
            "max": float(x.max())}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--worlds", type=int, default=16384)
    ap.add_argument("--steps", type=int, default=3600)
    ap.add_argument("--checkpoints", default="1,10,60,120,300,600",
                    help="steps (besides the last) at which the errors are measured")
    ap.add_argument("--oracle-worlds", type=int, default=256)
    ap.add_argument("--threads", type=int, default=len(os.sched_getaffinity(0)))
    ap.add_argument("--out")
    a = ap.parse_args()
    build.build_library()
    build.build_oracle()
    sc = scenes.config4(nworlds=a.worlds)
    sub = sc.worlds(0, a.oracle_worlds)
    props, _ = derive_props_state(sc.kind, sc.opt)
    sprops, _ = derive_props_state(sub.kind, sub.opt)
    checks = sorted({min(int(c), a.steps) for c in a.checkpoints.split(",") if c.strip()} | {a.steps})
    res = {"workload": f"config4: {sc.nworlds} worlds, {sc.nbodies} bodies, seed 4, dt 1/60, {a.steps} steps",
           "oracle_worlds": a.oracle_worlds, "oracle_bodies": sub.nbodies, "checkpoints": {}}

    # FP64 oracle on the subset; each checkpoint is its own run from the
    # start (the oracle returns f32 state, which must not be fed back)
    t0 = time.time()
    ref = {}
    for c in checks:
        _, state, st = O.batch_run(sub, c, a.threads, precision=64)
        assert st == 0, st
        ref[c] = state
    res["oracle_seconds"] = time.time() - t0

    for mode, fp64 in (("f32", False), ("f32+f64 pose", True)):
        b = Batch.from_scene(sc, fp64_positions=fp64)
        bsub = Batch.from_scene(sub, fp64_positions=fp64, debug=True)
        s0 = b.read_state()
        _, e0 = world_energy(sc, s0, props, sc.gravity)
        done = 0
        t0 = time.time()
        for c in checks:
            for _ in range(c - done):
                b.process(sc.dt, sc.sub_steps, sc.iters)
                bsub.process(sc.dt, sc.sub_steps, sc.iters)
            b.sync()
            bsub.sync()
            done = c
            st = b.read_state()
            ss = bsub.read_state()
            if fp64:
                ss = ss.astype(np.float64)
                ss[:3] = bsub.read_positions_f64()
            p_all, e_all = world_energy(sc, st, props, sc.gravity)
            p_sub, e_sub = world_energy(sub, ss, sprops, sub.gravity)
            p_ref, e_ref = world_energy(sub, ref[c], sprops, sub.gravity)
            entry = res["checkpoints"].setdefault(str(c), {})
            entry[mode] = {
                "pos_error_vs_fp64_radii": pos_error(sub, ss, ref[c]),
                "momentum_vs_fp64_rel": rel(p_sub, p_ref),
                "energy_vs_fp64_rel": rel(e_sub, e_ref),
                "energy_drift_all_worlds": rel(e_all, e0),
            }
        res.setdefault("gpu_seconds", {})[mode] = time.time() - t0
        res.setdefault("penetration_last_step", {})[mode] = penetration(bsub, sub.nworlds)
        b.close()
        bsub.close()
    out = json.dumps(res)
    print(out)
    if a.out:
        with open(a.out, "w") as f:
            f.write(out + "\n")


if __name__ == "__main__":
    main()

"""Precision study on the long-horizon workload (16,384 worlds of the
batched distribution, seed 4, 3,600 steps at dt 1/60).

    python tests/precision_study.py [--worlds 16384] [--steps 3600]
        [--checkpoints 1,10,60,120,300,600] [--oracle-worlds 256]
        [--out profiles/precision_config4.json]

GPU modes step every world from the same start:

* f32: the reference's arithmetic, bit-identical to the f32 oracle;
* f32+f64 pose: the pose integrated in f64 (R2D_FLAG_FP64_POSITIONS);
* f32 warm: warm starting (R2D_FLAG_WARM_START);
* f32 warm+Kahan: warm starting with compensated impulse sums
  (R2D_FLAG_COMPENSATED);
* f32 warm+Kahan+f64 pose: all three.

The first `--oracle-worlds` worlds are also stepped by the FP64 oracle (the
same algorithm in double) on the host threads, in reference mode and in warm
mode; each GPU mode is compared with the FP64 run of its own algorithm.
The chaos floor: the FP64 oracle run again with every dynamic body's x
nudged up by one f64 ulp (and, separately, by one f32 ulp: the size of one
f32 rounding) at step 0, compared with the unperturbed FP64 run.  A
difference that small reaching the same error as f32 does means the error
is the scenes' sensitivity to any perturbation, not the f32 arithmetic.

Reported, at the checkpoints:

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

    # FP64 oracle runs of the subset, every checkpoint's state in f64
    t0 = time.time()
    ref = {}
    for name, flags in (("fp64", 0), ("fp64 warm", O.BR_WARM),
                        ("fp64 +1 ulp", O.BR_PERTURB_ULP), ("fp64 +1 f32 ulp", O.BR_PERTURB_F32_ULP),
                        ("fp64 warm +1 ulp", O.BR_WARM | O.BR_PERTURB_ULP)):
        out, st = O.batch_checkpoints(sub, checks, a.threads, precision=64, flags=flags)
        assert st == 0, (name, st)
        ref[name] = {c: out[k] for k, c in enumerate(checks)}
    res["oracle_seconds"] = time.time() - t0
    # the chaos floor: perturbed FP64 against FP64
    for name, base in (("fp64 +1 ulp", "fp64"), ("fp64 +1 f32 ulp", "fp64"), ("fp64 warm +1 ulp", "fp64 warm")):
        for c in checks:
            p_a, e_a = world_energy(sub, ref[name][c], sprops, sub.gravity)
            p_b, e_b = world_energy(sub, ref[base][c], sprops, sub.gravity)
            res["checkpoints"].setdefault(str(c), {})[name] = {
                "pos_error_vs_fp64_radii": pos_error(sub, ref[name][c], ref[base][c]),
                "momentum_vs_fp64_rel": rel(p_a, p_b),
                "energy_vs_fp64_rel": rel(e_a, e_b),
            }

    modes = (("f32", {}, "fp64"),
             ("f32+f64 pose", {"fp64_positions": True}, "fp64"),
             ("f32 warm", {"warm_start": True}, "fp64 warm"),
             ("f32 warm+Kahan", {"warm_start": True, "compensated": True}, "fp64 warm"),
             ("f32 warm+Kahan+f64 pose", {"warm_start": True, "compensated": True, "fp64_positions": True},
              "fp64 warm"))
    for mode, kw, base in modes:
        fp64 = kw.get("fp64_positions", False)
        b = Batch.from_scene(sc, **kw)
        bsub = Batch.from_scene(sub, debug=True, **kw)
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
            _, e_all = world_energy(sc, st, props, sc.gravity)
            p_sub, e_sub = world_energy(sub, ss, sprops, sub.gravity)
            p_ref, e_ref = world_energy(sub, ref[base][c], sprops, sub.gravity)
            entry = res["checkpoints"].setdefault(str(c), {})
            entry[mode] = {
                "against": base,
                "pos_error_vs_fp64_radii": pos_error(sub, ss, ref[base][c]),
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

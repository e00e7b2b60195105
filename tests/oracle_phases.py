"""Where the reference's step spends its CPU time, per phase, on the benchmark scenes.

The oracle steps each scene in the reference's own order (ORDER_REFERENCE: joints
then manifolds, in insertion and discovery order) with its per-phase timers on:
updateManifolds (broadphase and narrowphase), forces and velocities, TGS update
and preStep, the solver iterations, and integration.  The colour-major order adds
a colouring phase; it is timed beside as ORDER_COLOUR.  Each scene is settled
first, because the phase split of a pile that has landed differs from that of
bodies still in the air.  One host thread per world.  CPU only.

    python tests/oracle_phases.py [--threads 8]
"""

import argparse
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

from oracle import ORDER_COLOUR, ORDER_REFERENCE, PHASES, Oracle, batch_run  # noqa: E402
from resolve2d_gb300 import scenes as S  # noqa: E402

# (name, scene, settle steps, timed frames, worlds sampled)
CASES = [
    ("config0", lambda: S.config0(), 300, 60, None),
    ("config1", lambda: S.config1(), 120, 5, None),
    ("config2", lambda: S.config2(), 30, 3, None),
    ("config3", lambda: S.config3(), 300, 10, 256),
]


def settled_worlds(sc, settle, sample, threads):
    """(scene, state) of each world to time, after `settle` steps."""
    if sample is not None:
        sc = sc.select(np.random.default_rng(0).choice(sc.nworlds, sample, replace=False))
    if sc.jtype.size == 0:
        _, state, st = batch_run(sc, settle, threads)
        assert st == 0
        return [(sc.world(w), np.ascontiguousarray(state[:, sc.body_off[w]:sc.body_off[w + 1]]))
                for w in range(sc.nworlds)]
    o = Oracle.from_scene(sc)  # one world with joints
    for _ in range(settle):
        assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
    return [(sc, o.state())]


def time_phases(worlds, frames, order):
    total = np.zeros(len(PHASES))
    body_steps = 0
    for sc, state in worlds:
        o = Oracle.from_scene(sc)
        o.set_state(state)
        o.set_phase_timing(True)
        for _ in range(frames):
            assert o.process(sc.dt, sc.sub_steps, sc.iters, order) == 0
        total += o.phase_seconds()
        body_steps += sc.nbodies * frames
    return total, body_steps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=8)
    a = ap.parse_args()
    header = "| scene | order | body-steps/s (1 thread) | " + " | ".join(PHASES) + " |"
    print(header)
    print("|" + "---|" * (3 + len(PHASES)))
    for name, make, settle, frames, sample in CASES:
        t0 = time.time()
        worlds = settled_worlds(make(), settle, sample, a.threads)
        print(f"<!-- {name}: settled {settle} steps in {time.time() - t0:.0f} s -->", flush=True)
        for order, oname in ((ORDER_REFERENCE, "reference"), (ORDER_COLOUR, "colour-major")):
            secs, body_steps = time_phases(worlds, frames, order)
            shares = " | ".join(f"{100 * x / secs.sum():.1f} %" for x in secs)
            print(f"| {name} | {oname} | {body_steps / secs.sum():,.0f} | {shares} |", flush=True)


if __name__ == "__main__":
    main()

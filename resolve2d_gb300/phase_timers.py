"""Per-phase cycle counts of the fused world step on the benchmark worlds.

    python -m resolve2d_gb300.phase_timers [--settle 300] [--steps 3] [--autotune]

Builds libr2d_timers.so (the library with R2D_PHASE_TIMERS: each CTA reads
clock64() at its phase boundaries), steps the 4,096 benchmark worlds
(seed 3) `--settle` steps, then `--steps` more with the counters on, and the
library prints one line per size class to stderr: mean cycles per
world-step of load, broadphase (cells, bucket sort, candidates, pair list),
narrowphase, colouring (sort, walk), joint colouring, solve (of which the
forces and prestep passes), write-back, and
mean counts of entries, candidates, pairs, manifolds and colours.  Cycles are
wall-clock cycles of the SM the world ran on, so co-resident worlds inflate
them; they rank phases, they do not time the step (bench.py does).

It then prints the last step's CTA timeline (%globaltimer at each world's
start and end, and its SM): per size class the first start, last start, last
end and mean CTA time, and for the step the SMs' busy share, the spread of
the SMs' last ends and when 90 % and 99 % of the worlds had ended.  With
`--autotune` the size classes first get the benchmark's threads per CTA.
"""

from __future__ import annotations

import argparse

from . import _native as N
from . import build, scenes


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--settle", type=int, default=300)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--autotune", action="store_true")
    a = ap.parse_args()
    N._lib = N.load(build.build_library(timers=True))
    from .engine import Batch

    sc = scenes.config3()
    b = Batch.from_scene(sc)
    for _ in range(a.settle):
        b.process(sc.dt, sc.sub_steps, sc.iters)
    if a.autotune:
        b.autotune(sc.dt, sc.sub_steps, sc.iters, trial_steps=8)
    b.sync()  # prints (and clears) the counters of the settling steps
    print(f"settled {a.settle} steps; the lines below are {a.steps} more steps", flush=True)
    for _ in range(a.steps):
        b.process(sc.dt, sc.sub_steps, sc.iters)
    b.sync()


if __name__ == "__main__":
    main()

"""Frame-to-frame coherence of the settled 4,096-world batch, measured with the oracle.

Two reuses would skip work without changing any result:

(a) the colouring is a pure function of a world's manifold key set (first-fit
    greedy in a fixed priority order), so a world whose key set equals the
    previous frame's could keep its colours;
(b) candidate pairs found from AABBs grown by a margin delta stay a superset of
    the AABB-intersecting pairs until some body's AABB leaves its grown box, so
    the binning could be skipped until then and only the exact filter run.

This script measures how often each would apply: it settles the batch for 300
steps (the benchmark's settling), steps a seeded sample of worlds for a number
of frames, and prints (a) the fraction of world-frames whose key set is
unchanged (plain, weighted by body count, and by world size), and (b) per
delta, the fraction of world-frames that would rebuild and the candidate count
relative to the exact pair count.  CPU only.

    python tests/coherence_study.py [--worlds 256] [--frames 60] [--threads 8]
"""

import argparse
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

from oracle import ORDER_COLOUR, Oracle, batch_run  # noqa: E402
from resolve2d_gb300 import scenes as S  # noqa: E402

EPS = 0.01  # the AABB overlap margin (aabb.zig)
DELTAS = [0.0, 0.01, 0.02, 0.05, 0.1, 0.2]
SIZES = [(64, "<=64 bodies"), (192, "65-192 bodies"), (1 << 30, ">192 bodies")]


def overlapping(x0, x1, y0, y1, static):
    """Upper-triangular mask of box pairs that intersect within EPS, static-static pairs dropped."""
    ov = ((x0[:, None] <= x1[None, :] + EPS) & (x0[None, :] <= x1[:, None] + EPS)
          & (y0[:, None] <= y1[None, :] + EPS) & (y0[None, :] <= y1[:, None] + EPS))
    ov &= ~(static[:, None] & static[None, :])
    return np.triu(ov, 1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--worlds", type=int, default=256)
    ap.add_argument("--frames", type=int, default=60)
    ap.add_argument("--threads", type=int, default=8)
    ap.add_argument("--settle", type=int, default=300)
    a = ap.parse_args()

    sc = S.config3()
    t0 = time.time()
    _, state, status = batch_run(sc, a.settle, a.threads)
    assert status == 0
    print(f"settled {a.settle} steps in {time.time() - t0:.0f} s", flush=True)
    worlds = np.sort(np.random.default_rng(0).choice(sc.nworlds, a.worlds, replace=False))

    same = total = 0
    same_w = total_w = 0.0
    by_size = [[0, 0] for _ in SIZES]
    rebuilds = dict.fromkeys(DELTAS, 0)
    cands = dict.fromkeys(DELTAS, 0)
    exact = manifolds = 0
    for w in worlds:
        sub = sc.world(int(w))
        b0, b1 = int(sc.body_off[w]), int(sc.body_off[w + 1])
        n = b1 - b0
        o = Oracle.from_scene(sub)
        o.set_state(np.ascontiguousarray(state[:, b0:b1]))
        static = (sub.kind & S.KIND_STATIC) != 0
        prev, grown = None, dict.fromkeys(DELTAS)
        for _ in range(a.frames):
            s = o.state()
            x0, x1 = s[S.S_AABB_X] - s[S.S_AABB_HW], s[S.S_AABB_X] + s[S.S_AABB_HW]
            y0, y1 = s[S.S_AABB_Y] - s[S.S_AABB_HH], s[S.S_AABB_Y] + s[S.S_AABB_HH]
            exact += int(overlapping(x0, x1, y0, y1, static).sum())
            for d in DELTAS:
                g = grown[d]
                inside = g is not None and bool(
                    np.all(x0 >= g[0]) and np.all(x1 <= g[1]) and np.all(y0 >= g[2]) and np.all(y1 <= g[3]))
                if not inside:
                    rebuilds[d] += 1
                    box = (x0 - d, x1 + d, y0 - d, y1 + d)
                    grown[d] = (*box, int(overlapping(*box, static).sum()))
                cands[d] += grown[d][4]
            assert o.process(sub.dt, sub.sub_steps, sub.iters, ORDER_COLOUR) == 0
            k, _ = o.manifolds()
            manifolds += len(k)
            keys = set(map(tuple, np.sort(k, axis=1).tolist()))
            if prev is not None:
                hit = keys == prev
                same += hit
                total += 1
                same_w += n * hit
                total_w += n
                b = next(i for i, (top, _) in enumerate(SIZES) if n <= top)
                by_size[b][0] += hit
                by_size[b][1] += 1
            prev = keys

    frames = a.worlds * a.frames
    print(f"{a.worlds} worlds x {a.frames} frames: {manifolds / frames:.1f} manifolds and "
          f"{exact / frames:.1f} AABB-intersecting pairs per world-frame")
    print(f"(a) key set unchanged: {same / total:.3f} of world-frames, {same_w / total_w:.3f} weighted by bodies")
    for (_, name), (h, c) in zip(SIZES, by_size):
        print(f"      {name}: {h / max(c, 1):.3f} ({c} world-frames)")
    for d in DELTAS:
        print(f"(b) delta {d:4.2f}: rebuild in {rebuilds[d] / frames:.3f} of world-frames, "
              f"candidates {cands[d] / max(exact, 1):.2f} x the exact pairs")


if __name__ == "__main__":
    main()

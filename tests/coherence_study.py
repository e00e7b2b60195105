"""Frame-to-frame coherence of the settled 4,096-world batch, measured with the oracle.

Two reuses would skip work without changing any result:

(a) the colouring is a pure function of a world's manifold key set (first-fit
    greedy in a fixed priority order), so a world whose key set equals the
    previous frame's could keep its colours;
(b) candidate pairs found from AABBs grown by a margin delta stay a superset of
    the AABB-intersecting pairs until some body's AABB leaves its grown box, so
    the binning could be skipped until then and only the exact filter run.

(c) fewer colours would mean fewer barrier-separated solve phases.  A world's
    contact colouring is an edge colouring of its dynamic bodies, so it needs
    at least the largest number of contacts on one dynamic body; the script
    compares the shipped hashed greedy order with that floor and with a
    degree-first greedy order.

This script measures all three: it settles the batch for 300
steps (the benchmark's settling), steps a seeded sample of worlds for a number
of frames, and prints (a) the fraction of world-frames whose key set is
unchanged (plain, weighted by body count, and by world size), and (b) per
delta, the fraction of world-frames that would rebuild and the candidate count
relative to the exact pair count, and (c) the mean contact colours per
world-frame under each rule.  CPU only.

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


M32 = 0xFFFFFFFF


def colour_mix(a, b):
    """r2d_colour_mix (resolve2d_gb300/csrc/r2d_colour.h) in Python integers."""
    h = (a * 0x9E3779B1 + b * 0x85EBCA77 + 0x165667B1) & M32
    h ^= h >> 16
    h = (h * 0x7FEB352D) & M32
    h ^= h >> 15
    h = (h * 0x846CA68B) & M32
    return h ^ (h >> 16)


def greedy_colours(edges, dyn, order):
    """Colours first-fit greedy uses over `edges` taken in `order`; only dynamic bodies conflict."""
    used, top = {}, 0
    for e in order:
        ends = [b for b in edges[e] if dyn[b]]
        taken = set().union(*(used.get(b, set()) for b in ends)) if ends else set()
        c = 0
        while c in taken:
            c += 1
        for b in ends:
            used.setdefault(b, set()).add(c)
        top = max(top, c + 1)
    return top


def colour_counts(keys, dyn):
    """(floor, hashed greedy, degree-first greedy) for one frame's manifold keys."""
    edges = [(int(min(a, b)), int(max(a, b))) for a, b in keys]
    deg = np.zeros(dyn.shape[0], int)
    for lo, hi in edges:
        deg[lo] += dyn[lo]
        deg[hi] += dyn[hi]
    hashed = sorted(range(len(edges)), key=lambda e: (colour_mix(*edges[e]), edges[e]))
    by_degree = sorted(range(len(edges)), key=lambda e: (-(deg[edges[e][0]] + deg[edges[e][1]]),
                                                          colour_mix(*edges[e]), edges[e]))
    return int(deg.max()), greedy_colours(edges, dyn, hashed), greedy_colours(edges, dyn, by_degree)


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
    colours = []
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
            if len(k):
                floor, hashed, by_degree = colour_counts(k, ~static)
                cc, _ = o.colours()
                assert hashed == int(cc.max()) + 1  # the restated rule is the oracle's
                colours.append((n, floor, hashed, by_degree))
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
    c = np.array(colours, float)
    big = c[:, 0] > 192
    for name, rows in (("all worlds", c), (">192 bodies", c[big])):
        print(f"(c) {name} ({len(rows)} world-frames): contact colours: floor {rows[:, 1].mean():.2f}, "
              f"hashed greedy {rows[:, 2].mean():.2f}, degree-first greedy {rows[:, 3].mean():.2f}")
    print(f"    hashed greedy above floor + 1 in {np.mean(c[:, 2] > c[:, 1] + 1):.3f} of world-frames")


if __name__ == "__main__":
    main()

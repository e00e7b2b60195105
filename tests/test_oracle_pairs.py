"""The oracle's candidate-pair tap on cases worked by hand from
Solver.updateManifolds (src/core/lib.zig:264-284): a pair reaches
performNarrowSAT when the two bodies share a spatial-hash bucket, are not both
static, are not excluded in either order, have no manifold yet, and their
AABBs intersect (aabb.zig:12-19, margin 0.01).  The GPU's taps are compared
with this one in the GPU parity tests."""

import numpy as np

from oracle import ORDER_COLOUR, Oracle
from resolve2d_gb300 import scenes


def _scene(builder, excl=None):
    ids, kind, opt = builder.arrays()
    ex = None if excl is None else (np.zeros(len(excl), np.uint32), np.array(excl, np.uint32))
    return scenes._concat("pairs", [(ids, kind, opt)], [0.0], 1 / 60, 1, 8, 1, excl=ex), ids


def _pairs(sc):
    o = Oracle.from_scene(sc)
    o.record_pairs()
    assert o.process(sc.dt, 1, 8, ORDER_COLOUR) == 0
    k, _ = o.manifolds()
    return {tuple(p) for p in o.pairs().tolist()}, {tuple(sorted(x)) for x in k.tolist()}


def test_aabb_overlap_without_contact_is_a_candidate():
    b = scenes._Builder()
    b.disc(0.0, 0.0, 0.5, 0.5)
    b.disc(0.8, 0.8, 0.5, 0.5)    # 1.13 apart: AABBs overlap, SAT rejects
    b.disc(0.0, -1.005, 0.5, 0.5)  # 0.005 inside the contact margin of body 0
    b.disc(9.0, 9.0, 0.5, 0.5)    # alone
    sc, _ = _scene(b)
    pairs, keys = _pairs(sc)
    assert pairs == {(0, 1), (0, 2)}
    assert keys == {(0, 2)}


def test_aabbs_just_apart_are_not_candidates():
    # |dx| = 1.02 > 0.5 + 0.5 + 0.01: the AABB test rejects them
    b = scenes._Builder()
    b.disc(0.0, 0.0, 0.5, 0.5)
    b.disc(1.02, 0.0, 0.5, 0.5)
    b.disc(1.0, 2.0, 0.5, 0.5)
    b.disc(1.0, 3.005, 0.5, 0.5)  # |dy| = 1.005 < 1.01: a candidate
    sc, _ = _scene(b)
    pairs, _ = _pairs(sc)
    assert pairs == {(2, 3)}


def test_static_pairs_and_exclusions_are_filtered():
    b = scenes._Builder()
    b.rect(0.0, 0.0, 4.0, 1.0, 0.5, static=True)
    b.rect(1.0, 0.0, 4.0, 1.0, 0.5, static=True)  # overlaps body 0: both static
    b.disc(0.0, 0.9, 0.5, 0.5)                     # on both boxes
    b.disc(0.0, 1.8, 0.5, 0.5)                     # on body 2, excluded from it
    ids = b.arrays()[0]
    sc, _ = _scene(b, excl=[[ids[3], ids[2]]])  # listed in the higher-lower order
    pairs, keys = _pairs(sc)
    assert (0, 1) not in pairs
    assert (2, 3) not in pairs
    assert {(0, 2), (1, 2)} <= pairs


def test_each_pair_once_across_shared_buckets():
    # a long static box spans many cells: bodies in several of its buckets
    # meet it in several queries, and the tap still lists each pair once
    b = scenes._Builder()
    b.rect(0.0, -0.5, 40.0, 1.0, 0.5, static=True)
    for k in range(8):
        b.disc(-14.0 + 4.0 * k, 0.49, 0.5, 0.5)
    sc, _ = _scene(b)
    o = Oracle.from_scene(sc)
    o.record_pairs()
    assert o.process(sc.dt, 1, 8, ORDER_COLOUR) == 0
    p = o.pairs()
    assert len({tuple(x) for x in p.tolist()}) == len(p) == 8
    assert (np.diff(p[:, 0].astype(np.int64) * 2**32 + p[:, 1]) > 0).all()

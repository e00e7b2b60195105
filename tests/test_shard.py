"""Dealing independent worlds out to ranks (resolve2d_gb300/shard.py) and
selecting them (Scene.select).  CPU only."""

import numpy as np
import pytest

from resolve2d_gb300 import scenes
from resolve2d_gb300.shard import balanced_shards


@pytest.fixture(scope="module")
def batch():
    return scenes.config3(nworlds=1024)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 8])
def test_shards_partition_the_worlds_and_balance_the_bodies(batch, n):
    counts = np.diff(batch.body_off).astype(np.int64)
    shards = balanced_shards(counts, n)
    assert len(shards) == n
    every = np.concatenate(shards)
    assert sorted(every.tolist()) == list(range(batch.nworlds))  # each world on exactly one rank
    for s in shards:
        assert np.all(np.diff(s) > 0)  # ascending within a rank
    totals = np.array([counts[s].sum() for s in shards])
    assert totals.max() - totals.mean() <= counts.max()  # the LPT bound: one world above the mean
    assert totals.max() / totals.mean() < 1.01  # and, on this distribution, within 1 %
    again = balanced_shards(counts, n)
    assert all(np.array_equal(a, b) for a, b in zip(shards, again))  # every rank deals the same


def test_more_ranks_than_worlds_and_bad_counts():
    shards = balanced_shards([5, 3], 4)
    assert [s.tolist() for s in shards] == [[0], [1], [], []]
    assert [s.tolist() for s in balanced_shards([], 2)] == [[], []]
    with pytest.raises(ValueError):
        balanced_shards([1, 2], 0)


def test_equal_counts_go_round_robin_by_index():
    assert [s.tolist() for s in balanced_shards([4, 4, 4, 4, 4], 2)] == [[0, 2, 4], [1, 3]]


def test_select_matches_the_contiguous_world_range(batch):
    a = batch.select(np.arange(10, 20))
    b = batch.worlds(10, 20)
    for f in ("ids", "kind", "opt", "body_off", "gravity"):
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f))
    assert (a.dt, a.sub_steps, a.iters) == (b.dt, b.sub_steps, b.iters)


def test_selected_shards_hold_every_body_once(batch):
    shards = balanced_shards(np.diff(batch.body_off), 3)
    parts = [batch.select(s) for s in shards]
    assert sum(p.nbodies for p in parts) == batch.nbodies
    assert sum(p.nworlds for p in parts) == batch.nworlds
    # a selected world is the same world: its bodies' options and its gravity
    w = int(shards[1][5])
    b0, b1 = batch.body_off[w], batch.body_off[w + 1]
    p = parts[1]
    np.testing.assert_array_equal(p.opt[:, p.body_off[5]: p.body_off[6]], batch.opt[:, b0:b1])
    assert p.gravity[5] == batch.gravity[w]

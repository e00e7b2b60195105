"""The benchmark scenes carry the decisions their configurations state.

Counts, sizes, solver parameters, joint layouts and seeds of configs 0-4, as
the generators in resolve2d_gb300/scenes.py fix them.  CPU only.
"""

import numpy as np

from resolve2d_gb300 import scenes as S


def dynamic(sc):
    return (sc.kind & S.KIND_STATIC) == 0


def rects(sc):
    return (sc.kind & S.KIND_RECT) != 0


def test_config0_grid_of_discs_and_rectangles():
    sc = S.config0()
    assert sc.nworlds == 1 and sc.nbodies == 201
    assert (sc.dt, sc.sub_steps, sc.iters, sc.steps) == (1 / 60, 1, 8, 600)
    dyn = dynamic(sc)
    assert dyn.sum() == 200
    assert (rects(sc) & dyn).sum() == 50 and (~rects(sc) & dyn).sum() == 150
    r = sc.opt[S.DIM0][dyn & ~rects(sc)]
    assert r.min() >= 0.2 and r.max() <= 0.5
    assert np.all(sc.opt[S.MU] == np.float32(0.4))
    assert np.all(sc.opt[S.VEL_X][dyn] == 0) and np.all(sc.opt[S.VEL_Y][dyn] == 0)


def test_config1_pyramid_rows_and_falling_discs():
    sc = S.config1()
    assert sc.nbodies == 12001
    assert (sc.dt, sc.iters, sc.steps) == (1 / 60, 10, 1000)
    dyn = dynamic(sc)
    boxes = dyn & rects(sc)
    discs = dyn & ~rects(sc)
    assert boxes.sum() == 10000 and discs.sum() == 2000
    assert np.all(sc.opt[S.DIM0][boxes] == 1.0) and np.all(sc.opt[S.DIM1][boxes] == 1.0)
    # rows of width 100, 100, 99, 99, ... stacked at unit spacing, the last partial
    y = np.round(sc.opt[S.POS_Y][boxes] - 0.5).astype(int)
    widths = np.bincount(y)
    expect, w = [], 100
    while sum(expect) < 10000:
        expect.append(min(w, 10000 - sum(expect)))
        if len(expect) % 2 == 0:
            w -= 1
    assert widths.tolist() == expect
    # disc heights U[60, 120] above the next row's centre line (half a unit above the top face)
    top = sc.opt[S.POS_Y][boxes].max() + 1.0
    r = sc.opt[S.DIM0][discs]
    assert r.min() >= 0.3 and r.max() <= 0.5
    h = sc.opt[S.POS_Y][discs] - top
    assert h.min() >= 60.0 - 1e-4 and h.max() <= 120.0 + 1e-4


def test_config2_box_chains_and_motors():
    sc = S.config2()
    assert sc.nbodies == 200004
    assert (sc.dt, sc.iters, sc.steps) == (1 / 120, 8, 300)
    st = ~dynamic(sc)
    assert st.sum() == 4  # the walls
    assert sc.ids.max() > 65535  # ids need 32 bits
    dyn = dynamic(sc)
    discs = dyn & ~rects(sc)
    frac = discs.sum() / dyn.sum()
    assert 0.68 < frac < 0.72
    assert sc.opt[S.DIM0][discs].min() >= 0.1 and sc.opt[S.DIM0][discs].max() <= 0.4
    dist = sc.jtype == S.JOINT_DISTANCE
    motor = sc.jtype == S.JOINT_MOTOR
    assert dist.sum() == 100000 and motor.sum() == 2000 and sc.jtype.size == 102000
    assert np.all(sc.jprm[dist, 3] == np.float32(0.5))  # rest length
    assert np.all(np.abs(sc.jprm[motor, 0]) == 50.0) and np.all(sc.jprm[motor, 2] == 10.0)
    assert len(set(sc.jid1[motor].tolist())) == 2000  # distinct bodies
    # neighbours in a chain do not collide with each other
    assert sc.xpairs.shape[0] == 100000


def test_config3_and_config4_batches():
    sc = S.config3()
    assert sc.nworlds == 4096 and sc.nbodies == 589055
    assert (sc.dt, sc.sub_steps, sc.iters) == (1 / 60, 1, 8)
    n = np.diff(sc.body_off) - 1  # each world also holds its static ground
    assert n.min() >= 16 and n.max() <= 512
    assert 100 < n.mean() < 160  # log-uniform on [16, 512]
    g = sc.gravity
    assert g.min() >= 5.0 and g.max() <= 15.0
    dyn = dynamic(sc)
    assert 0.58 < (dyn & ~rects(sc)).sum() / dyn.sum() < 0.62
    assert (~dynamic(sc)).sum() == 4096
    big = S.config4()
    assert big.nworlds == 16384 and big.steps == 3600

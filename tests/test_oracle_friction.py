"""Friction in the oracle's contact solve, against collision.zig:102-218.

preStep sets friction = sqrt(mu1 * mu2) (collision.zig:114).  calculateImpulses
clamps each point's accumulated tangential impulse to friction times its
accumulated normal impulse (collision.zig:186-190).  Consequences checked here,
on the CPU:
- a frictionless pair exchanges no tangential momentum at all;
- a sliding box slows at about mu * g;
- every point of a settled scene lies inside its Coulomb cone.
"""


import numpy as np

from oracle import ORDER_COLOUR, Oracle
from resolve2d_gb300 import scenes as S

DT = 1 / 60
P0, PF, APN, APT = 9, 12, 10, 11  # point 0's first float, floats a point, accumulated pn / pt


def world(bodies, g=9.81):
    b = S._Builder()
    for spec in bodies:
        getattr(b, spec[0])(*spec[1:])
    return Oracle.from_scene(S._concat("friction", [b.arrays()], [g], DT, 1, 8, 1))


def ground(mu):
    return ("rect", 0.0, -0.5, 200.0, 1.0, mu, 1.0, 0.0, 0.0, 0.0, 0.0, True)


def test_a_frictionless_pair_keeps_the_tangential_momentum_exactly():
    # mu = 0 on the ground: friction = sqrt(0 * 0.5) = 0, so max_pt = 0 and every
    # tangential increment is clamped away; gravity and the normal impulse are vertical
    o = world([ground(0.0), ("disc", 0.0, 0.49, 0.5, 0.5, 1.0, 3.0, 0.0)])
    px = o.state()[S.S_MOM_X, 1]
    for _ in range(60):
        assert o.process(DT, 1, 8, ORDER_COLOUR) == 0
        assert o.state()[S.S_MOM_X, 1] == px
    assert o.state()[S.S_POS_X, 1] > 2.9  # it slid about 3 units in the second


def test_a_sliding_box_slows_at_about_mu_g():
    mu, v0, frames = 0.5, 5.0, 30
    o = world([ground(mu), ("rect", 0.0, 0.495, 1.0, 1.0, mu, 1.0, v0, 0.0)])
    mass = float(o.props()[S.P_MASS, 1])
    for _ in range(frames):
        assert o.process(DT, 1, 8, ORDER_COLOUR) == 0
    v = float(o.state()[S.S_MOM_X, 1]) / mass
    want = v0 - mu * 9.81 * frames * DT  # friction = sqrt(mu * mu) = mu
    assert abs(v - want) < 0.1 * (v0 - want)
    assert abs(float(o.state()[S.S_ANGLE, 1])) < 0.05  # it slides flat rather than tipping


def test_every_settled_contact_lies_in_its_coulomb_cone():
    sc = S.random_scene(21, n=60, spin=True)
    o = Oracle.from_scene(sc)
    for _ in range(40):
        assert o.process(sc.dt, sc.sub_steps, sc.iters, ORDER_COLOUR) == 0
    keys, data = o.manifolds()
    mu = o.props()[S.P_MU]
    assert keys.shape[0] > 20
    checked = 0
    for (a, b), row in zip(keys, data):
        assert row[4] == np.sqrt(np.float32(mu[a] * mu[b]))  # the friction coefficient
        for p in range(2):
            if not row[5 + p]:
                continue
            pn, pt = row[P0 + PF * p + APN], row[P0 + PF * p + APT]
            assert pn >= 0.0
            assert abs(pt) <= row[4] * pn * (1 + 1e-6) + 1e-12
            checked += 1
    assert checked > 20

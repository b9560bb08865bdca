"""Rigid bodies on the CPU (rigid.comp; common.glsl:265-340; particles.comp:144-151,
222-248, 576): a yield-stress liquid's unyielded cells are labelled and joined into bodies
(each body's root its smallest cell), and the particles in them move with their body."""
import numpy as np

import tanks

DT = 1.0 / 240.0


def test_yield_stress_liquid_forms_bodies():
    ora, parts, _ = tanks.oracle_of(tanks.yield_stress(mat=5))
    assert ora.stats().caps & 4, "CAP_RIGID"
    for _ in range(24):
        ora.step(1, DT)
    rl = ora.field("rl", np.int32).reshape(-1, 2)
    rigid = rl[:, 0] >= 0
    assert rigid.any()
    roots = rl[rigid, 0]
    idx = np.nonzero(rigid)[0]
    assert np.all(roots <= idx), "every body's root is its smallest cell"
    assert np.all(rl[roots, 0] == roots), "roots point at themselves"
    p = ora.particles()
    assert np.isfinite(p["pos"]).all() and np.isfinite(p["vel"]).all()


def test_freezing_lava_becomes_one_body():
    ora, parts, _ = tanks.oracle_of(tanks.cooling_lava())
    assert ora.stats().caps & 6 == 6, "heat and rigid bodies"
    for _ in range(24):
        ora.step(1, DT)
    rl = ora.field("rl", np.int32).reshape(-1, 2)
    rigid = rl[:, 0] >= 0
    assert rigid.sum() > 100 and len(set(rl[rigid, 0].tolist())) >= 1

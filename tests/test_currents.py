"""Currents and drains on the CPU (params.rs:1113-1121, particles.comp:577-594, 809-835): a
drain removes liquid at its rate, a current drives the liquid in it along its direction and
never brakes it; set_currents keeps the first 16 and they survive a reset."""
import numpy as np

import tanks

DT = 1.0 / 240.0


def test_drain_and_current():
    t = tanks.currents()
    ora, parts, _ = tanks.oracle_of(t)
    n0 = len(parts)
    for _ in range(24):
        ora.step(1, DT)
    p = ora.particles()
    live = p[p["kind"] != 0]
    assert len(live) < n0, "the drain removed liquid"
    c = t.currents[0]
    inside = np.hypot(live["pos"][:, 0] - c["pos"][0], live["pos"][:, 1] - c["pos"][1]) < c["radius"]
    assert live["vel"][inside, 0].mean() > live["vel"][~inside, 0].mean() + 2.0, "the current drove its liquid"


def test_without_currents_nothing_drains():
    t = tanks.currents()
    t.currents = []
    ora, parts, _ = tanks.oracle_of(t)
    for _ in range(12):
        ora.step(1, DT)
    p = ora.particles()
    assert int((p["kind"] != 0).sum()) == len(parts)


def test_current_records_match_the_reference_layout():
    import sprout_gb300 as S
    assert S.CURRENT_DTYPE.itemsize == 24
    arr = S.current_array([{"pos": (1.0, 2.0), "radius": 3.0, "vel": (4.0, 5.0), "rate": -6.0}])
    assert arr.view(np.float32).tolist() == [1.0, 2.0, 3.0, 4.0, 5.0, -6.0]

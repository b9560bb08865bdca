"""Concentration families on the CPU: the library's rule for a custom liquid's diluent
(src/library.rs:318-330), and the oracle's miscible exchange (particles.comp:519-569 with
grid_prep.comp:67-68, 141-147): each family's concentrate is conserved, concentrations stay in
[0, 1], and diluent particles beside a concentrate join its family."""
import numpy as np

import tanks

DT = 1.0 / 240.0
HONEY, WATER = 1, 0


def rows_of(parts):
    live = parts[parts["kind"] != 0]
    return live, (live["kind"] & 255).astype(np.int64) - 1


def test_set_diluent_follows_the_library_rules():
    import sprout_gb300 as S
    p = S.SimParams()
    assert not p.set_diluent(HONEY, WATER), "a built-in row keeps its own diluent"
    assert not p.set_diluent(59, 59), "not itself"
    assert not p.set_diluent(59, HONEY), "a built-in concentrate is no diluent"
    assert not p.set_diluent(59, 96) and not p.set_diluent(96, 0), "rows past the table"
    assert p.set_diluent(59, WATER) and p.set_diluent(60, 59), "a plain built-in or a custom liquid"
    assert p.set_diluent(59, -1), "none"


def test_honey_and_water_exchange_and_conserve_the_concentrate():
    ora, parts, _ = tanks.oracle_of(tanks.honey_dam())
    honey0 = float((parts["kind"] & 255).astype(np.int64).__eq__(HONEY + 1).sum())
    for _ in range(24):
        ora.step(1, DT)
    live, row = rows_of(ora.particles())
    s = live["s"][row == HONEY]
    assert np.all((s >= 0.0) & (s <= 1.0))
    assert (row == HONEY).sum() > honey0, "water beside the honey joined the family"
    assert np.any((s > 0.0) & (s < 1.0)), "diluted honey"
    assert abs(float(s.astype(np.float64).sum()) - honey0) <= 1e-4 * honey0, "the concentrate is conserved"
    comp = ora.field("comp").reshape(-1, 4)
    assert np.any((comp[:, 2] > 0.0) & (comp[:, 2] < 1.0)), "cells hold family 0 at a mean concentration"


def test_no_exchange_without_a_mix_rate():
    ora, parts, _ = tanks.oracle_of(tanks.honey_dam(mix_rate=0.0))
    for _ in range(12):
        ora.step(1, DT)
    live, row = rows_of(ora.particles())
    assert np.all(live["s"][row == HONEY] == 1.0), "concentrations stay put"


def test_several_families_exchange_and_diluents_join():
    t = tanks.families_tank()
    ora, parts, _ = tanks.oracle_of(t)
    _, row0 = rows_of(parts)
    for _ in range(24):
        ora.step(1, DT)
    live, row = rows_of(ora.particles())
    s = live["s"]
    for fam_row, n0 in [(HONEY, (row0 == HONEY).sum()), (59, (row0 == 59).sum()), (61, (row0 == 61).sum())]:
        sf = s[row == fam_row].astype(np.float64)
        assert np.all((sf >= 0.0) & (sf <= 1.0))
        assert abs(sf.sum() - n0) <= 1e-4 * n0, f"family of row {fam_row} keeps its concentrate"
    assert (row == 61).sum() > (row0 == 61).sum(), "mat60 beside its concentrate joined family 2"
    assert (row == 60).sum() < (row0 == 60).sum()
    w, h = t.w, t.h
    mixb = ora.field("mixb").reshape(h, w, 2)
    assert np.any(mixb[..., 0] >= 0.0) and np.any(mixb[..., 1] >= 0.0), "families 1 and 2 on the grid"
    assert np.all((mixb == -1.0) | ((mixb >= 0.0) & (mixb <= 1.0)))

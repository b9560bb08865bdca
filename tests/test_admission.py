"""Admission of new liquid on the CPU: the brush's room per cell (src/brush.rs), and the
oracle's FluidSim::spawn / cell_counts (src/sim/mod.rs:2024-2046, 3350-3387) with count.comp
and claim.comp, checked against plain counts of its own particles."""
import numpy as np
import pytest

import tanks
from sprout_gb300 import admission as A

KIND_FRESH = 0x10000


def test_admission_fills_only_empty_cells_up_to_rest_density():
    # the reference's own known answers (src/brush.rs:251-264)
    adm = A.Admission([4, 7], [2, 1], [1, 0], 4, False)
    assert not adm.admit([4.5, 7.5]), "a cell with liquid is full"
    for p in [[5.25, 7.25], [5.75, 7.25], [5.25, 7.75], [5.75, 7.75]]:
        assert adm.admit(p)
    assert not adm.admit([5.5, 7.5]), "rest density reached"
    assert not adm.admit([9.5, 7.5]), "outside the window"
    stream = A.Admission([0, 0], [1, 1], [4], 4, True)
    assert stream.admit([0.5, 0.5]) and stream.admit([0.5, 0.5])
    assert not stream.admit([0.5, 0.5])


def test_window_covers_the_stroke_and_margin():
    lo, hi = A.window([10.0, 20.0], [4.5, 22.25], 3.0)
    assert lo == [1, 17] and hi == [14, 27]
    lo, hi = A.window([7.0, 7.0], [7.0, 7.0], 0.0)
    assert lo == [7, 7] and hi == [8, 8]


def small_tank(extra_rows: int = 1, capacity_extra: int = 2048):
    """A 96 x 64 dam break of custom liquid 59, with rows 60.. defined for spawning."""
    rows = [{"density": 1000.0, "viscosity": 1e-6, "tension": 0.0}] * (1 + extra_rows)
    t = tanks.layered_custom(96, 64, rows[:1], cell=0.002, ambient=20.0)
    for k in range(1, 1 + extra_rows):
        for name, val in rows[k].items():
            t.settings[f"mat{59 + k}.{name}"] = val
    t.fills = [([0.0, 0.0, 40.0, 38.0], 59, None)]
    t.settings["tension_mat59"] = 0.0
    t.capacity_extra = capacity_extra
    return t


def count_by_hand(parts, lo, hi):
    sw, sh = max(hi[0] - lo[0], 0), max(hi[1] - lo[1], 0)
    out = np.zeros((sh, sw), np.uint32)
    live = parts[(parts["kind"] & 255) != 0]
    c = np.floor(live["pos"]).astype(np.int64) - np.asarray(lo)
    m = (c[:, 0] >= 0) & (c[:, 1] >= 0) & (c[:, 0] < sw) & (c[:, 1] < sh)
    np.add.at(out, (c[m, 1], c[m, 0]), 1)
    return out


def test_oracle_cell_counts_match_a_plain_count():
    from oracle import oracle as O
    ora, parts, _ = tanks.oracle_of(small_tank())
    ora.step(3, 3 / 240.0)
    p = ora.particles()
    for lo, hi in [([0, 0], [96, 64]), ([10, 5], [31, 40]), ([40, 30], [40, 50]), ([95, 63], [96, 64])]:
        got = ora.cell_counts(lo, hi)
        assert got.shape == (max(hi[1] - lo[1], 0), max(hi[0] - lo[0], 0))
        assert np.array_equal(got, count_by_hand(p, lo, hi))
    assert ora.cell_counts([0, 0], [96, 64]).sum() == np.count_nonzero(p["kind"] & 255)
    with pytest.raises(ValueError):
        ora.cell_counts([-1, 0], [4, 4])
    with pytest.raises(ValueError):
        ora.cell_counts([0, 0], [97, 4])


def test_oracle_spawn_queues_then_places_with_fresh_ids():
    from oracle import oracle as O
    t = small_tank()
    ora, parts, (sdf, solid, region, temp) = tanks.oracle_of(t)
    ora.step(2, 2 / 240.0)
    n0 = len(ora.particles())
    new = O.fill_rect(96, 64, [60.0, 40.0, 70.0, 48.0], 59)
    new["vel"] = [0.0, -3.0]
    got = ora.spawn(new)
    assert got == len(new)
    # queued: counted by cell_counts, not yet in the slots
    assert len(ora.particles()) == n0
    lo, hi = [55, 35], [75, 52]
    assert ora.cell_counts(lo, hi).sum() == len(new)
    ora.step(1, 1 / 240.0)
    p = ora.particles()
    assert len(p) == n0 + len(new)
    ids = np.sort(p["id"][n0:])
    assert np.array_equal(ids, np.arange(len(parts), len(parts) + len(new)))
    # settled (rest concentration, enthalpy temperature) and no longer fresh after a substep
    assert np.all(p["s"][n0:] == 1.0) and np.all(p["kind"][n0:] & KIND_FRESH == 0)
    # a second spawn continues the ids
    more = O.fill_rect(96, 64, [60.0, 50.0, 62.0, 52.0], 59)
    assert ora.spawn(more) == len(more)
    ora.step(1, 1 / 240.0)
    p = ora.particles()
    assert p["id"].max() == len(parts) + len(new) + len(more) - 1


def test_oracle_spawn_of_a_new_material_widens_the_tank():
    from oracle import oracle as O
    t = small_tank(extra_rows=2)
    ora, parts, _ = tanks.oracle_of(t)
    ora.step(1, 1 / 240.0)
    before = ora.stats()
    new = O.fill_rect(96, 64, [60.0, 40.0, 66.0, 46.0], 60)
    assert ora.spawn(new) == len(new)
    ora.step(2, 2 / 240.0)
    after = ora.stats()
    assert after.n_slots == before.n_slots + len(new)
    p = ora.particles()
    assert np.count_nonzero((p["kind"] & 255) == 61) == len(new)


def test_oracle_spawn_without_a_material_is_skipped_and_the_queue_is_bounded():
    from oracle import oracle as O
    ora, parts, _ = tanks.oracle_of(small_tank())
    new = O.fill_rect(96, 64, [60.0, 40.0, 64.0, 44.0], 59)
    new["kind"][::2] = 0
    assert ora.spawn(new) == len(new) - (len(new) + 1) // 2
    big = np.repeat(O.fill_rect(96, 64, [60.0, 40.0, 61.0, 41.0], 59), 9000)
    assert ora.spawn(big) == 32768 - (len(new) - (len(new) + 1) // 2)
    assert ora.spawn(big[:10]) == 0


def test_oracle_claim_recycles_dead_slots_in_order():
    """With no fresh slot left, queued particles take dead slots (claim.comp); the ones
    beyond the dead slots are dropped."""
    from oracle import oracle as O
    t = small_tank(capacity_extra=16)
    ora, parts, _ = tanks.oracle_of(t)
    cap = len(parts) + 16
    # the eraser over part of the liquid
    tool = O.OTool()
    tool.pos[0], tool.pos[1], tool.radius, tool.mode = 20.0, 20.0, 4.0, 2
    ora.step(1, 1 / 240.0)
    ora.step(1, 1 / 240.0, tool)   # (the first substep after a reset has no grid to gather from)
    p = ora.particles()
    dead = int(np.count_nonzero(p["kind"] == 0))
    assert dead > 20
    new = O.fill_rect(96, 64, [60.0, 40.0, 72.0, 50.0], 59)
    assert len(new) > 16 + dead
    assert ora.spawn(new) == len(new)
    ora.step(0, 0.0)
    p = ora.particles()
    assert len(p) == cap
    live_new = np.sort(p["id"][(p["kind"] != 0) & (p["id"] >= len(parts))])
    # 16 fresh slots, then the dead ones in slot order: the first 16 + dead entries
    assert np.array_equal(live_new, np.arange(len(parts), len(parts) + 16 + dead))
    assert np.count_nonzero(p["kind"] == 0) == 0

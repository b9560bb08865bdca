"""Several phase groups in one tank on the CPU: the library's rule for a custom liquid's
group (src/library.rs:283-286), and the oracle's drift (particles.comp:374-502 with
grid_prep.comp:53, 172, 247-252): immiscible groups separate by density, and the materials of
one group sort themselves by density."""
import numpy as np

import tanks

DT = 1.0 / 240.0


def mean_heights(parts):
    live = parts[parts["kind"] != 0]
    row = (live["kind"] & 255).astype(np.int64) - 1
    return {int(r): float(live["pos"][row == r, 1].mean()) for r in np.unique(row)}, live


def test_set_group_follows_the_library_rules():
    import sprout_gb300 as S
    p = S.SimParams()
    assert not p.set_group(2, 0), "a built-in row keeps its group"
    assert not p.set_group(59, 4), "four groups"
    assert p.set_group(59, 1) and p.set_group(95, 3)


def test_oil_rises_through_water():
    ora, parts, _ = tanks.oracle_of(tanks.water_oil())
    before, _ = mean_heights(parts)
    for _ in range(40):
        ora.step(1, DT)
    after, live = mean_heights(ora.particles())
    assert np.isfinite(live["pos"]).all()
    assert after[2] > before[2] + 1.0, "the oil block rose"
    assert after[0] < before[0], "the water under it took its place"
    grho = ora.field("grho").reshape(-1, 4)
    assert np.any(grho[:, 1] > 0.0), "group 1's share x density on the grid"


def test_three_groups_separate():
    t = tanks.three_groups()
    ora, parts, _ = tanks.oracle_of(t)
    before, _ = mean_heights(parts)
    for _ in range(40):
        ora.step(1, DT)
    after, live = mean_heights(ora.particles())
    assert np.isfinite(live["pos"]).all()
    assert after[61] < before[61] - 5.0, "the dense group-2 liquid sank"
    assert after[59] > before[59] and after[60] > before[60], "the oil-like group rose"
    # group 1 sorts its two liquids: the cells carry its share x base density for that drift
    # (a sub-cell droplet's terminal velocity here is ~0.3 cells / s, too slow to see in 40
    # substeps; the GPU parity tests pin its arithmetic)
    gbase = ora.field("gbase").reshape(-1, 4)
    assert gbase[:, 0].max() > 0.0 and np.all(gbase[:, 2:] == 0.0)
    aux = ora.field("aux").reshape(-1, 4)
    assert aux[:, 2].max() > 0.5, "group 2's share in the cells it fills"


def test_builtin_rows_carry_the_reference_table():
    """Known answers of presets.rs for rows past the first three (every row comes from one
    table shared with the oracle)."""
    import sprout_gb300 as S
    p = S.SimParams()
    for key, want in [("density_mercury", 13534.0), ("viscosity_mercury", 1.13e-7), ("tension_mercury", 0.485),
                      ("density_ink", 1050.0), ("mix_rate_ink", 0.25), ("density_brine", 1200.0),
                      ("mix_rate_brine", 1.0), ("density_milk", 1030.0), ("mix_rate_milk", 0.8)]:
        assert abs(p.get(key) - want) <= 1e-6 * abs(want), key
    from oracle import oracle as O
    q = O.default_params()
    assert q.mat[8].group == 2 and q.mat[4].diluent == 0 and q.mat[11].diluent == 0 and q.mat[14].diluent == 0


def test_builtin_liquids_mix_and_separate():
    ora, parts, _ = tanks.oracle_of(tanks.builtin_mix())
    before, _ = mean_heights(parts)
    for _ in range(24):
        ora.step(1, DT)
    after, live = mean_heights(ora.particles())
    assert np.isfinite(live["pos"]).all()
    assert after[8] < before[8] - 2.0, "mercury sank"
    assert after[2] > before[2], "oil rose"
    row = (live["kind"] & 255).astype(np.int64) - 1
    assert np.any((row == 4) & (live["s"] < 1.0)) and np.any((row == 11) & (live["s"] < 1.0)), "ink and milk diluted"

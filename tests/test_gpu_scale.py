"""Parity of the engine with the oracle at the benchmark's own sizes, and with the persistent
solvers' blocks each taking several tiles.

At a grid's default launch shape the pressure and viscosity kernels run one block per 16 x 16
tile until the device is full (304 blocks here), so small grids give every block one tile and
never exercise the two-region staging pipeline that carries a block from one tile to the next.
The benchmark's 1024 x 576 pour gives each block 7 to 8 tiles per level-0 phase. These tests
force a few blocks on small tanks (every block then takes many tiles, unevenly) and run the
configurations themselves: the 384 x 216 dam break over its 200 substeps, the 512 x 288
stratified tank with the built-in honey, water and olive oil, and the 1024 x 576 full-physics
pour with its ten-level hierarchy. Everything is compared bit for bit, as in
test_gpu_parity.py: particles by id, every grid field, the accumulators, the viscosity
fields and the solvers' iteration counts.
"""
import numpy as np
import pytest

import tanks
from test_gpu_parity import compare_state, compare_viscosity, first_diff

pytestmark = pytest.mark.gpu

DT = 1.0 / 240.0


def oracle_threads():
    from oracle import oracle as O
    O.set_threads(O.threads_available())


def step_and_compare(sim, ora, substeps, check_every, viscosity=False):
    problems = []
    for k in range(substeps):
        sim.step(1, DT)
        ora.step(1, DT)
        if (k + 1) % check_every == 0 or k + 1 == substeps:
            problems += compare_state(sim, ora, f"substep {k + 1}")
            if viscosity:
                problems += [f"substep {k + 1}: {m}" for m in compare_viscosity(sim, ora)]
            a, b = sim.stats(), ora.stats()
            if (list(a.pressure_iters), a.pressure_iters_max, a.pressure2_iters) != (list(b.p_iters), b.p_it_max, b.p2_iters):
                problems.append(f"substep {k + 1}: pressure iterations {list(a.pressure_iters)}/{a.pressure_iters_max}/"
                                f"{a.pressure2_iters} vs {list(b.p_iters)}/{b.p_it_max}/{b.p2_iters}")
            if problems:
                break
    return problems


@pytest.mark.parametrize("blocks", [1, 7, 16])
def test_solver_blocks_taking_many_tiles_bit_exact(blocks):
    """The full-physics pour at 160 x 96 (60 level-0 tiles) with the pressure and viscosity
    kernels on `blocks` blocks: each block takes 4 to 60 tiles per phase through the staging
    pipeline, in uneven shares, and the results stay those of the oracle."""
    t = tanks.full_physics(160, 96, cell=0.0064)
    sim, _, _ = t.engine()
    sim.set_launch(pressure_blocks=blocks, pressure_blocks_mixed=blocks, viscosity_blocks=blocks)
    ora, _, _ = tanks.oracle_of(t)
    oracle_threads()
    problems = step_and_compare(sim, ora, 6, 3, viscosity=True)
    assert not problems, "\n".join(problems[:12])
    got = sim.launch()
    assert got["pressure_blocks"] == blocks and got["viscosity_blocks"] == blocks, got
    st = sim.stats()
    assert st.viscosity_mode == 2 and st.viscosity_iters_max > 0 and st.device_error == 0


def test_launch_shape_is_clamped_and_restored():
    t = tanks.dam_break(160, 96)
    sim, _, _ = t.engine()
    default = sim.launch()
    assert default["pressure_blocks"] == 60, default   # one per level-0 tile
    sim.set_launch(pressure_blocks=1 << 30)
    assert sim.launch()["pressure_blocks"] == 60       # at most one per tile
    sim.set_launch(pressure_blocks=3)
    sim.step(2, 2 * DT)
    assert sim.launch()["pressure_blocks"] == 3 and sim.stats().device_error == 0
    sim.set_launch()
    assert sim.launch() == default


def test_stratified_on_few_blocks_bit_exact():
    """The stratified tank at 192 x 108 (honey takes the implicit viscosity) on 5 pressure and
    3 viscosity blocks, against the oracle."""
    t = tanks.stratified(192, 108, builtins=True)
    sim, _, _ = t.engine()
    sim.set_launch(pressure_blocks=5, viscosity_blocks=3)
    ora, _, _ = tanks.oracle_of(t)
    oracle_threads()
    problems = step_and_compare(sim, ora, 8, 4, viscosity=True)
    assert not problems, "\n".join(problems[:12])


def test_dam_break_384_config_bit_exact():
    """The plain dam break at 384 x 216 (76,153 water particles, 9-level hierarchy) over the
    configuration's 200 substeps, compared every 25."""
    t = tanks.dam_break(384, 216)
    sim, parts, _ = t.engine()
    assert len(parts) == 76153
    ora, _, _ = tanks.oracle_of(t)
    oracle_threads()
    problems = step_and_compare(sim, ora, 200, 25)
    assert not problems, "\n".join(problems[:12])
    st = sim.stats()
    assert st.substeps == 200 and st.pressure_unconverged == 0 and st.device_error == 0


def test_stratified_512_config_bit_exact():
    """The stratified tank at 512 x 288 with the built-in honey, water and olive oil (344,080
    particles: family exchange, an immiscible oil layer, the implicit viscosity between two
    pressure solves) over 60 substeps, compared every 20."""
    t = tanks.stratified(512, 288, builtins=True)
    sim, parts, _ = t.engine()
    ora, _, _ = tanks.oracle_of(t)
    oracle_threads()
    problems = step_and_compare(sim, ora, 60, 20, viscosity=True)
    assert not problems, "\n".join(problems[:12])
    st = sim.stats()
    assert st.viscosity_mode == 2 and st.device_error == 0 and sim.launch()["pressure_blocks"] > 8


def test_full_physics_1024_config_bit_exact():
    """The full-physics pour at 1024 x 576 (2.29 M particles, eight liquids, heater strip,
    heat, surface tension, implicit viscosity between two pressure solves; a ten-level
    hierarchy with 2,304 level-0 tiles over the persistent kernels' blocks), 4 substeps."""
    t = tanks.full_physics(1024, 576)
    sim, parts, _ = t.engine()
    ora, _, _ = tanks.oracle_of(t)
    oracle_threads()
    problems = step_and_compare(sim, ora, 4, 2, viscosity=True)
    for name in ["therm", "dheat"]:
        n, k = first_diff(sim.field(name), ora.field(name))
        if n:
            problems.append(f"{name} differs in {n} values")
    if not np.array_equal(sim.field("ledger", np.uint64), ora.field("ledger", np.uint64)):
        problems.append("heat ledger differs")
    assert not problems, "\n".join(problems[:12])
    st = sim.stats()
    assert st.levels == 10 and st.thermal == 1 and st.viscosity_mode == 2 and st.device_error == 0


def test_tuned_launch_is_applied_and_bit_exact():
    """A grid size the autotuner has an entry for starts from the tuned block counts, and the
    results stay those of the oracle."""
    import json
    from pathlib import Path
    table = json.loads((Path(__file__).resolve().parents[1] / "sprout_gb300" / "tuned_launch.json").read_text())
    entry = next(s["best"] for s in table["sizes"] if s["grid"] == [256, 144])
    t = tanks.full_physics(256, 144, cell=0.004)
    sim, _, _ = t.engine()
    ora, _, _ = tanks.oracle_of(t)
    oracle_threads()
    problems = step_and_compare(sim, ora, 4, 2, viscosity=True)
    assert not problems, "\n".join(problems[:12])
    got = sim.launch()
    assert got["pressure_blocks"] == entry["pressure_blocks"] and got["viscosity_blocks"] == entry["viscosity_blocks"], (got, entry)

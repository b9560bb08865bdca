"""Admission on the GPU, bit for bit against the oracle: FluidSim::spawn (fresh slots, then
dead slots recycled as claim.comp does) and FluidSim::cell_counts (count.comp), alone and in a
batch. Particles are matched by their permanent id; the counts are integers."""
import numpy as np
import pytest

import tanks
from test_admission import small_tank
from test_gpu_parity import compare_state

pytestmark = pytest.mark.gpu

DT = 1.0 / 240.0
WINDOWS = [([0, 0], [96, 64]), ([10, 5], [31, 40]), ([55, 35], [75, 52]), ([40, 30], [40, 50])]


def pair(tank):
    from oracle import oracle as O
    O.set_threads(O.threads_available())
    sim, parts, _ = tank.engine()
    ora, _, _ = tanks.oracle_of(tank)
    return sim, ora, parts


def counts_agree(sim, ora):
    for lo, hi in WINDOWS:
        a, b = sim.cell_counts(lo, hi), ora.cell_counts(lo, hi)
        assert a.shape == b.shape and np.array_equal(a, b), f"cell_counts {lo}-{hi} differ"


def test_spawn_and_cell_counts_bit_exact():
    from oracle import oracle as O
    sim, ora, parts = pair(small_tank())
    for _ in range(3):
        sim.step(1, DT)
        ora.step(1, DT)
    counts_agree(sim, ora)
    new = O.fill_rect(96, 64, [60.0, 40.0, 70.0, 48.0], 59)
    new["vel"] = [0.0, -3.0]
    assert sim.spawn(new) == ora.spawn(new) == len(new)
    counts_agree(sim, ora)          # the queue is counted before it reaches the slots
    problems = []
    for k in range(8):
        sim.step(1, DT)
        ora.step(1, DT)
        problems += compare_state(sim, ora, f"substep {k + 1} after the spawn")
        if problems:
            break
    assert not problems, "\n".join(problems[:10])
    counts_agree(sim, ora)
    assert sim.stats().n_slots == ora.stats().n_slots == len(parts) + len(new)


def test_spawn_of_a_new_material_bit_exact():
    from oracle import oracle as O
    sim, ora, parts = pair(small_tank(extra_rows=2))
    sim.step(2, 2 * DT)
    ora.step(2, 2 * DT)
    new = O.fill_rect(96, 64, [60.0, 40.0, 66.0, 46.0], 60)
    assert sim.spawn(new) == ora.spawn(new) == len(new)
    problems = []
    for k in range(6):
        sim.step(1, DT)
        ora.step(1, DT)
        problems += compare_state(sim, ora, f"substep {k + 1} with the new liquid")
        if problems:
            break
    assert not problems, "\n".join(problems[:10])


def test_claim_of_dead_slots_bit_exact():
    """No fresh slots left: the queue recycles the slots the eraser emptied."""
    import sprout_gb300 as S
    from oracle import oracle as O
    sim, ora, parts = pair(small_tank(capacity_extra=16))
    sim.step(1, DT)
    ora.step(1, DT)
    tool = S.Tool()
    tool.pos[0], tool.pos[1], tool.radius, tool.mode = 20.0, 20.0, 4.0, 2
    otool = O.OTool()
    otool.pos[0], otool.pos[1], otool.radius, otool.mode = 20.0, 20.0, 4.0, 2
    sim.step(1, DT, tool)
    ora.step(1, DT, otool)
    assert not compare_state(sim, ora, "after the eraser")
    new = O.fill_rect(96, 64, [60.0, 40.0, 72.0, 50.0], 59)
    assert sim.spawn(new) == ora.spawn(new) == len(new)
    counts_agree(sim, ora)
    problems = []
    for k in range(6):
        sim.step(1, DT)
        ora.step(1, DT)
        problems += compare_state(sim, ora, f"substep {k + 1} after the claim")
        if problems:
            break
    assert not problems, "\n".join(problems[:10])
    counts_agree(sim, ora)


def test_spawn_in_a_batch_equals_alone():
    import sprout_gb300 as S
    from oracle import oracle as O
    new = O.fill_rect(96, 64, [60.0, 40.0, 70.0, 48.0], 59)
    alone, _, _ = small_tank().engine()
    a2, _, _ = small_tank().engine()
    b2, _, _ = tanks.dam_break(128, 72, width=0.3, height=0.5).engine()
    batch = S.Batch([a2, b2])
    for _ in range(2):
        alone.step(1, DT)
        batch.step(1)
    assert alone.spawn(new) == a2.spawn(new) == len(new)
    for _ in range(5):
        alone.step(1, DT)
        batch.step(1)
    batch.sync()
    pa, pb = alone.download_particles(), a2.download_particles()
    assert np.array_equal(pa.view(np.uint8), pb.view(np.uint8))
    for lo, hi in WINDOWS:
        assert np.array_equal(alone.cell_counts(lo, hi), a2.cell_counts(lo, hi))

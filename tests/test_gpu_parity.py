"""Parity of the CUDA engine with the CPU oracle on identical seeded inputs.

Both compute in FP32 with every operation rounded as written (the engine is compiled with
-fmad=false, the oracle with -ffp-contract=off) and both reduce the solver's dot products in
the reference's order, so the FP32 path is compared BIT FOR BIT: the fixed-point
accumulators, cell counts and cell-type flags (integer work) and every float field
(velocities, pressure, particle states). Particles are matched by their permanent id.
"""
import numpy as np
import pytest

import tanks

pytestmark = pytest.mark.gpu

GRID_FIELDS = ["vel", "cell", "comp", "coef", "sprop", "surf", "pjump", "pres", "prhs"]


def by_id(parts):
    live = parts[parts["kind"] != 0]
    return live[np.argsort(live["id"], kind="stable")]


def first_diff(a, b):
    a = np.asarray(a).view(np.uint32) if a.dtype == np.float32 else np.asarray(a)
    b = np.asarray(b).view(np.uint32) if b.dtype == np.float32 else np.asarray(b)
    bad = np.nonzero(a != b)[0]
    return (len(bad), int(bad[0])) if len(bad) else (0, -1)


def compare_state(sim, ora, tag):
    msgs = []
    g = by_id(sim.download_particles())
    o = by_id(ora.particles())
    if len(g) != len(o) or not np.array_equal(g["id"], o["id"]):
        msgs.append(f"{tag}: live particle sets differ ({len(g)} vs {len(o)})")
    else:
        for f in ["pos", "vel", "c", "s", "kind", "t"]:
            n, k = first_diff(g[f].ravel(), o[f].ravel())
            if n:
                msgs.append(f"{tag}: particle {f} differs in {n} values (first flat index {k})")
    for name in GRID_FIELDS:
        a, b = sim.field(name), ora.field(name)
        n, k = first_diff(a, b)
        if n:
            msgs.append(f"{tag}: field {name} differs in {n} values (first {k}: {a[k]} vs {b[k]})")
    a, b = sim.field("acc", np.int32), ora.field("acc", np.int32)
    n, k = first_diff(a, b)
    if n:
        msgs.append(f"{tag}: accumulators differ in {n} ints (first {k})")
    return msgs


def run_pair(tank: "tanks.Tank", substeps: int, check_every: int = 1):
    sim, _, _ = tank.engine()
    ora, _, _ = tanks.oracle_of(tank)
    from oracle import oracle as O
    O.set_threads(O.threads_available())
    dt = 1.0 / 240.0
    problems = []
    for k in range(substeps):
        sim.step(1, dt)
        ora.step(1, dt)
        if (k + 1) % check_every == 0 or k + 1 == substeps:
            problems += compare_state(sim, ora, f"substep {k + 1}")
            if problems:
                break
    return sim, ora, problems


def test_first_substep_is_bit_exact():
    t = tanks.dam_break(96, 64)
    sim, ora, problems = run_pair(t, 1)
    assert not problems, "\n".join(problems)
    # the sorted order: the engine keeps particles in a stable counting-sort order by cell
    ora.sort()
    g, o = sim.download_particles(), ora.particles()
    assert np.array_equal(g.view(np.uint8), o.view(np.uint8)), "sort permutation differs"


def test_dam_break_stays_bit_exact():
    t = tanks.dam_break(128, 72)
    sim, ora, problems = run_pair(t, 24, check_every=4)
    assert not problems, "\n".join(problems)
    a, b = sim.stats(), ora.stats()
    assert list(a.pressure_iters) == list(b.p_iters)
    assert a.pressure_iters_max == b.p_it_max and a.pressure_unconverged == b.p_unconv == 0
    assert a.umax_grid == b.umax_grid and a.umax_part == b.umax_part


def test_counts_and_flags_bit_exact_midrun():
    t = tanks.dam_break(160, 96, width=0.5, height=0.5)
    sim, ora, problems = run_pair(t, 10, check_every=10)
    assert not problems, "\n".join(problems)
    # cell-type flags: face states and liquid level, and the tiles with unknowns
    assert np.array_equal(sim.field("ptile", np.uint32)[: ora.field("ptile", np.uint32).size],
                          ora.field("ptile", np.uint32))
    cnt = sim.field("count", np.uint32)
    pos = by_id(ora.particles())["pos"]
    cells = np.clip(pos[:, 1].astype(np.int64), 0, 95) * 160 + np.clip(pos[:, 0].astype(np.int64), 0, 159)
    assert np.array_equal(cnt, np.bincount(cells, minlength=160 * 96).astype(np.uint32))


def test_surface_tension_and_heat_bit_exact():
    rows = [
        {"density": 1000.0, "viscosity": 1e-6, "tension": 0.072, "heat_capacity": 4182.0, "conductivity": 0.6},
        {"density": 1400.0, "viscosity": 2e-6, "tension": 0.05, "heat_capacity": 2500.0, "conductivity": 0.3},
        {"density": 900.0, "viscosity": 1.5e-6, "tension": 0.03, "heat_capacity": 2000.0, "conductivity": 0.2},
    ]
    t = tanks.layered_custom(128, 72, rows, cell=0.002, heater_rows=4, columns=False)
    # leave the top quarter empty: a free surface for the tension to act on
    t.fills = [(r[:3] + [min(r[3], 0.75 * t.h)], m, temp) for r, m, temp in t.fills]
    t.settings["fixed_hz"] = 2000.0
    sim, ora, problems = run_pair(t, 12, check_every=4)
    assert not problems, "\n".join(problems)
    assert sim.stats().thermal == 1
    for name in ["therm", "dheat"]:
        n, k = first_diff(sim.field(name), ora.field(name))
        assert n == 0, f"{name} differs"
    assert np.array_equal(sim.field("ledger", np.uint64), ora.field("ledger", np.uint64))


VISC_FIELDS = ["vw", "vs", "vd", "p2keep", "vma", "vmb", "vmd"]


def compare_viscosity(sim, ora):
    msgs = []
    for name in VISC_FIELDS:
        n, k = first_diff(sim.field(name), ora.field(name))
        if n:
            msgs.append(f"viscosity field {name} differs in {n} values (first {k})")
    for name in ["tiles", "vtile"]:
        if not np.array_equal(sim.field(name, np.uint32), ora.field(name, np.uint32)):
            msgs.append(f"tile flags {name} differ")
    a, b = sim.stats(), ora.stats()
    if (a.viscosity_iters, a.viscosity_iters_max, a.viscosity_unconverged) != (b.v_iters, b.v_it_max, b.v_unconv):
        msgs.append(f"viscosity iterations differ: {a.viscosity_iters}/{a.viscosity_iters_max} vs {b.v_iters}/{b.v_it_max}")
    if a.viscosity_residual_max != b.v_res_max:
        msgs.append(f"viscosity residual differs: {a.viscosity_residual_max} vs {b.v_res_max}")
    if (a.pressure2_iters_max, a.pressure2_unconverged) != (b.p2_it_max, b.p2_unconv):
        msgs.append("second pressure solve differs")
    return msgs


def test_implicit_viscosity_bit_exact():
    """Honey, water and oil: the honey layer takes the implicit MG-PCG viscosity solve between
    two pressure solves (visc*.comp, vmg*.comp, rhs_visc.comp, project_visc.comp)."""
    t = tanks.stratified(128, 72)
    sim, ora, problems = run_pair(t, 8, check_every=4)
    assert not problems, "\n".join(problems)
    st = sim.stats()
    assert st.viscosity_mode == 2 and st.viscosity_iters_max > 0 and st.pressure2_iters_max > 0
    problems = compare_viscosity(sim, ora)
    assert not problems, "\n".join(problems)


def test_implicit_viscosity_variants_bit_exact():
    """One pressure solve after the viscosity, one sweep per level, two coarse levels, no
    warm starts: the other recordings of record_viscosity_solve."""
    t = tanks.stratified(160, 96, extra={"viscous_projection": 0, "viscosity_mg_sweeps": 1,
                                         "viscosity_mg_levels": 2, "viscosity_warm": 0})
    sim, ora, problems = run_pair(t, 6, check_every=3)
    assert not problems, "\n".join(problems)
    st = sim.stats()
    assert st.viscosity_mode == 2 and st.viscosity_iters_max > 0 and st.pressure2_iters_max == 0
    problems = compare_viscosity(sim, ora)
    assert not problems, "\n".join(problems)


def test_jacobi_preconditioned_viscosity_bit_exact():
    """viscosity_precond 0: the reference's Jacobi-preconditioned iteration (visc_iter.comp,
    visc_update.comp) in place of the multigrid one, warm starts on."""
    t = tanks.stratified(160, 96, extra={"viscosity_precond": 0})
    sim, ora, problems = run_pair(t, 6, check_every=3)
    assert not problems, "\n".join(problems)
    st = sim.stats()
    assert st.viscosity_mode == 2 and st.viscosity_iters_max > 0
    problems = compare_viscosity(sim, ora)
    assert not problems, "\n".join(problems)


def test_full_physics_pour_bit_exact():
    """The full-physics pour at 160 x 96 (same physical tank, 6.4 mm cells): eight liquids,
    heater strip, surface tension, heat and the implicit viscosity together."""
    t = tanks.full_physics(160, 96, cell=0.0064)
    sim, ora, problems = run_pair(t, 8, check_every=4)
    assert not problems, "\n".join(problems)
    st = sim.stats()
    assert st.thermal == 1 and st.viscosity_mode == 2
    problems = compare_viscosity(sim, ora)
    for name in ["therm", "dheat"]:
        n, k = first_diff(sim.field(name), ora.field(name))
        if n:
            problems.append(f"{name} differs in {n} values")
    if not np.array_equal(sim.field("ledger", np.uint64), ora.field("ledger", np.uint64)):
        problems.append("heat ledger differs")
    a, b = sim.stats(), ora.stats()
    if (list(a.pressure_iters), a.pressure2_iters) != (list(b.p_iters), b.p2_iters):
        problems.append(f"pressure iterations differ: {list(a.pressure_iters)}/{a.pressure2_iters} vs "
                        f"{list(b.p_iters)}/{b.p2_iters}")
    assert not problems, "\n".join(problems)


def test_currents_and_drains_bit_exact():
    """A current driving the liquid and a drain removing it (particles.comp:577-594, 809-835)."""
    sim, ora, problems = run_pair(tanks.currents(), 16)
    assert not problems, "\n".join(problems[:10])
    assert sim.stats().n_live < len(tanks.currents().engine()[1])


def test_frame_blocking_reports_the_time_covered():
    sim, _, _ = tanks.dam_break(96, 64).engine()
    adv = sim.frame_blocking(4, 4 / 240.0)
    assert abs(adv - 4 / 240.0) < 1e-6
    assert abs(sim.dt_estimate() - 1 / 240.0) < 1e-9


@pytest.mark.parametrize("name", ["dam_break", "stratified", "elastic", "claims"])
def test_slot_order_is_the_oracles(name):
    """The engine and the oracle both sort the particles by cell after every substep (a
    stable counting sort in slot order), so they hold every particle in the same slot: the
    particle arrays are equal slot for slot, not only by id (what the render side's passes
    that rank by slot, look.comp's specks, rely on). "claims": particles erased, then new ones
    queued into the freed slots."""
    DT = 1.0 / 240.0
    if name == "claims":
        import sprout_gb300 as S
        from oracle import oracle as O
        from test_gpu_admission import pair, small_tank
        sim, ora, _ = pair(small_tank(capacity_extra=16))
        sim.step(1, DT)
        ora.step(1, DT)
        tool = S.Tool()
        tool.pos[0], tool.pos[1], tool.radius, tool.mode = 20.0, 20.0, 4.0, 2
        otool = O.OTool()
        otool.pos[0], otool.pos[1], otool.radius, otool.mode = 20.0, 20.0, 4.0, 2
        sim.step(1, DT, tool)
        ora.step(1, DT, otool)
        new = O.fill_rect(96, 64, [60.0, 40.0, 72.0, 50.0], 59)
        assert sim.spawn(new) == ora.spawn(new) == len(new)
        for _ in range(4):
            sim.step(1, DT)
            ora.step(1, DT)
    else:
        make = {"dam_break": lambda: tanks.dam_break(96, 64), "stratified": lambda: tanks.stratified(96, 64),
                "elastic": lambda: tanks.elastic_drop()}[name]
        sim, ora, problems = run_pair(make(), 6)
        assert not problems, "\n".join(problems[:10])
    g, o = sim.download_particles(), ora.particles()
    assert len(g) == len(o)
    bad = np.nonzero(g.view(np.uint8).reshape(len(g), -1).any(axis=1) != o.view(np.uint8).reshape(len(o), -1).any(axis=1))[0]
    assert np.array_equal(g.view(np.uint8), o.view(np.uint8)), f"particles differ slot for slot ({len(bad)} live/dead mismatches)"

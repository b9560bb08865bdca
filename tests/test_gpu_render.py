"""The render side's cell passes on the device (sprout_sim_render: cell_optics.comp, light.comp,
optics_blur.comp, sss.comp, flow_map.comp, glow.comp) against the oracle's restatement (osim_render) on the same grid, bit for bit
in their RGBA16F texels: the state after a few substeps is itself bit-exact between engine and
oracle (run_pair), and both passes take the engine's optics table, which test_optics.py pins to
its own restatement. Tanks that reach the branches: eight custom liquids over a heater (glow,
group temperatures), honey in water (a concentrate: the diluent's fading tint), water under
olive oil (the other groups' layers, iridescence), cooling lava (frozen shares, the quenched
skin against air and wall), a magnetisable liquid near a magnet (its share)."""
import numpy as np
import pytest

import sprout_gb300 as S
import tanks
from test_gpu_parity import run_pair

pytestmark = pytest.mark.gpu


def render_pair(tank, substeps, inv_speed=1.0 / 80.0):
    sim, ora, problems = run_pair(tank, substeps)
    assert not problems, "\n".join(problems[:10])
    sim.render(inv_speed)
    e = (sim.download_render("raw"), sim.download_render("smoothed"), sim.download_render("glow"))
    table = S.SimParams(tank.settings)
    for row, dil in tank.diluents.items():
        table.set_diluent(row, dil)
    for row, grp in tank.groups.items():
        table.set_group(row, grp)
    o = ora.render(table.optics_table(), inv_speed, int(table.get("sss_iters")))
    render_pair.ora, render_pair.table = ora, table
    return sim, e, o


def diff(a, b, what):
    ua, ub = a.view(np.uint16), b.view(np.uint16)
    bad = np.argwhere(ua != ub)
    if len(bad) == 0:
        return None
    l, y, x, c = bad[0]
    return f"{what}: {len(bad)} half words differ, first layer {l} cell ({x}, {y}) channel {c}: {a[l, y, x, c]} vs {b[l, y, x, c]}"


@pytest.mark.parametrize("name", ["full_physics", "honey_dam", "water_oil", "cooling_lava", "magnetic"])
def test_cell_passes_bit_exact(name):
    tank = {"full_physics": lambda: tanks.full_physics(96, 64, cell=0.0106),
            "honey_dam": lambda: tanks.honey_dam(), "water_oil": lambda: tanks.water_oil(),
            "cooling_lava": lambda: tanks.cooling_lava(), "magnetic": lambda: tanks.magnetic()}[name]()
    sim, (er, es, eg), (orw, osm, og, _, _) = render_pair(tank, 6)
    for a, b, what in ((er, orw, "raw"), (es, osm, "smoothed")):
        m = diff(a, b, what)
        assert m is None, m
    assert np.array_equal(eg.view(np.uint16), og.view(np.uint16)), "glow"
    # a second frame: sss.comp starts from the last call's light under the surface
    from oracle import oracle as O
    for _ in range(2):
        sim.step(1, 1 / 240.0)
        render_pair.ora.step(1, 1 / 240.0)
    sim.render(1 / 80.0)
    o2 = render_pair.ora.render(render_pair.table.optics_table(), 1 / 80.0, int(render_pair.table.get("sss_iters")))
    m = diff(sim.download_render("smoothed"), o2[1], "smoothed, second frame")
    assert m is None, m
    assert float(es[20, ..., :3].astype(np.float32).max()) > 0.0
    # the layers hold something: occupancy (4.w), a look key (12), the light from above (raw 10 yzw)
    assert float(er[4, ..., 3].astype(np.float32).max()) > 0.5
    assert float(er[12, ..., :3].astype(np.float32).max()) > 0.0
    assert 0.0 < float(er[10, ..., 1].astype(np.float32).min()) <= 1.0
    if name == "magnetic":   # the spikes' spacing and phase in every cell, their height where the field is strong
        assert float(er[13, ..., 3].astype(np.float32).min()) > 0.0
        assert float(np.abs(er[14, ..., :2].astype(np.float32)).max()) > 0.5
    if name == "cooling_lava":   # lava near 760 C glows (a heater at 327 C is below the Draper point)
        assert float(er[3, ..., :3].astype(np.float32).max()) > 0.0
        assert float(eg[..., :3].astype(np.float32).max()) > 0.0


def test_render_is_what_the_reference_draws():
    """Plain facts of the passes: the light falls off downwards through liquid and is 1 above
    it; the smoothing keeps a uniform field's level; nothing is drawn in empty cells."""
    tank = tanks.dam_break(96, 64)
    sim, _, _ = tank.engine()
    sim.step(2, 2 / 240.0)
    sim.render(1 / 80.0)
    raw = sim.download_render("raw").astype(np.float32)
    occ = raw[4, ..., 3]
    light = raw[10, ..., 1]
    assert np.all(light[-1] == 1.0) or np.all(light[-1] >= light[0])
    col = light[:, 10]
    assert np.all(np.diff(col[::-1]) <= 0.0)   # from the top down, never brighter
    assert np.all(raw[0][occ == 0.0] == 0.0)


def test_flow_map_bit_exact():
    """flow_map.comp over frames of a dam break against the oracle, with record_cell_optics'
    clock and key: the first call on a new tank carries nothing; a call after substeps advances
    the map by the simulated time since the last call and swaps its copies; a call with no
    substep since the last records nothing (the map, its copy and sss.comp's warm start stay as
    they were); crossing t = 2 s restarts the short period's second pair (zw: floor(t / 4 +
    0.5) changes); a reset clears the map."""
    tank = tanks.dam_break(96, 64)
    sim, _, _ = render_pair(tank, 6)
    ora, table = render_pair.ora, render_pair.table
    inv = 1.0 / 80.0

    def frame(substeps):
        for _ in range(substeps):
            sim.step(1, 1 / 240.0)
            ora.step(1, 1 / 240.0)
        sim.render(inv)
        o = ora.render(table.optics_table(), inv, int(table.get("sss_iters")))
        e_flow, e_par = sim.download_render("flow"), sim.flow_parity()
        assert e_par == o[4], f"flow parity {e_par} vs {o[4]}"
        m = diff(e_flow, o[3], "flow map")
        assert m is None, m
        m = diff(sim.download_render("smoothed"), o[1], "smoothed")
        assert m is None, m
        return e_flow, e_par

    f0 = sim.download_render("flow")
    assert not np.any(f0.view(np.uint16)), "the first call on a new tank carries nothing"
    p0 = sim.flow_parity()
    f1, p1 = frame(4)
    assert p1 == 1 - p0
    moved = f1[2 * p1].astype(np.float32)
    assert np.abs(moved).max() > 0.0, "the liquid moved the map"
    sm1 = sim.download_render("smoothed")
    f2, p2 = frame(0)   # nothing new: nothing recorded
    assert p2 == p1 and np.array_equal(f2.view(np.uint16), f1.view(np.uint16))
    assert np.array_equal(sim.download_render("smoothed").view(np.uint16), sm1.view(np.uint16))
    for n in (4, 3, 5):
        frame(n)
    # up to just before t = 2 s, then across it
    done = 6 + 4 + 3 + 4 + 5
    frame(476 - done)
    f3, p3 = frame(8)
    short_zw = f3[2 * p3, ..., 2:].astype(np.float32)
    short_xy = f3[2 * p3, ..., :2].astype(np.float32)
    assert not np.any(short_zw), "the short period's second pair restarted at t = 2 s"
    assert np.abs(short_xy).max() > 0.0
    # a reset of the same sim: the next call clears the map and keeps the copy that holds it
    _, parts, _ = tank.engine()
    sim.reset(parts)
    sim.step(2, 2 / 240.0)
    sim.render(inv)
    assert not np.any(sim.download_render("flow").view(np.uint16))
    assert sim.flow_parity() == p3


def test_look_bit_exact():
    """look.comp on a dam break of water carrying mica platelets (cloud 0.05, platelets 1/20
    as thick as wide, 15 um): over frames with substeps between, every particle's platelet
    orientation (the packed second moment, matched by particle id: the engine's sort moves the
    state every substep, the oracle's only periodically) and the set of particles listed for the
    look splat equal the oracle's; the flow turns the platelets away from isotropy."""
    mica = {"mat0.cloud": 0.05, "mat0.cloud_shape": 0.05, "mat0.cloud_size": 1.5e-5}
    tank = tanks.dam_break(96, 64, extra=mica)
    sim, _, _ = render_pair(tank, 4)
    ora, table = render_pair.ora, render_pair.table
    inv = 1.0 / 80.0

    for n in (0, 3, 2, 4, 1):
        for _ in range(n):
            sim.step(1, 1 / 240.0)
            ora.step(1, 1 / 240.0)
        sim.render(inv)
        ora.render(table.optics_table(), inv, int(table.get("sss_iters")))
        e_st, e_list = sim.download_look()
        o_st, o_list = ora.look()
        ep, op = sim.download_particles(), ora.particles()
        assert len(e_st) == len(ep) and len(o_st) == len(op)
        # every live particle's state, by id (the slot's stored id is the particle's)
        e_live, o_live = ep["kind"] != 0, op["kind"] != 0
        assert np.array_equal(e_st[e_live, 0], ep["id"][e_live]) and np.array_equal(o_st[o_live, 0], op["id"][o_live])
        eb = dict(zip(ep["id"][e_live].tolist(), e_st[e_live, 2].tolist()))
        ob = dict(zip(op["id"][o_live].tolist(), o_st[o_live, 2].tolist()))
        assert eb == ob, f"{sum(eb[k] != ob.get(k) for k in eb)} particles' platelet states differ"
        assert sorted(ep["id"][e_list].tolist()) == sorted(op["id"][o_list].tolist())
        assert len(e_list) == int(e_live.sum())
    a = e_st[e_live, 2]
    axx = (a & 1023) / 1023.0
    assert np.abs(axx - 1.0 / 3.0).max() > 0.05, "the flow turned the platelets"


def test_spray_bit_exact():
    """spray.comp on a dam break of water that fizzes and foams: over frames with substeps
    between, the pool (every entry bit for bit: the engine hands entries out in the same
    deterministic order as the oracle, emissions ranked by cell), its free stack, the list
    of live entries, the foam counted per cell and the counters equal the oracle's; bubbles
    are made, rise, turn to foam and burst."""
    fizzy = {"mat0.fizz": 1.0, "mat0.foam": 0.6, "mat0.froth": 0.5}
    tank = tanks.dam_break(96, 64, extra=fizzy)
    sim, _, _ = render_pair(tank, 4)
    ora, table = render_pair.ora, render_pair.table
    inv, amount = 1.0 / 80.0, float(table.get("bubbles"))
    seen = set()
    for n in (0, 3, 4, 2, 6, 1, 5):
        for _ in range(n):
            sim.step(1, 1 / 240.0)
            ora.step(1, 1 / 240.0)
        sim.render(inv)
        ora.render(table.optics_table(), inv, int(table.get("sss_iters")), amount)
        ep, es, es1, el, ef, ec = sim.download_spray()
        op, os_, os1, ol, of, oc = ora.spray()
        assert ec == oc, f"counters {ec} vs {oc}"
        assert np.array_equal(es, os_) and np.array_equal(es1, os1) and np.array_equal(el, ol), "free stacks or list"
        assert np.array_equal(ef, of), "foam per cell"
        bad = np.nonzero(ep.view(np.uint32).reshape(-1, 8) != op.view(np.uint32).reshape(-1, 8))[0]
        assert len(bad) == 0, f"{len(np.unique(bad))} pool entries differ, first {bad[0]}: {ep[bad[0]]} vs {op[bad[0]]}"
        seen |= set((ep["info"][el] & 3).tolist())
    assert ec[0] > 0 and ec[2] > 0, "bubbles were made and live"
    assert {1, 2} <= seen, f"bubbles and foam seen ({seen})"


def test_specks_bit_exact():
    """look.comp's specks and spray.comp's move_dust on a dam break of water carrying sand
    (dust 0.02): new particles bring their share of the specks into the pool's second part
    (ranked by particle slot, the engine's slot order being the oracle's), the specks settle,
    rest on the floor and are stirred up again, and lay their share of the colour into the dust
    field that cell_optics.comp reads on the next frame. Over frames: the whole pool, both free
    stacks, the list, the foam and resting-speck counts, the counters and the raw cell layers
    (layer 18 the dust field) equal the oracle's bit for bit."""
    sandy = {"mat0.dust": 0.02}
    tank = tanks.dam_break(96, 64, extra=sandy)
    sim, ora, problems = run_pair(tank, 4)
    assert not problems, "\n".join(problems[:10])
    table = S.SimParams(tank.settings)
    inv = 1.0 / 80.0
    states = set()
    for n in (0, 3, 4, 2, 6, 5):
        for _ in range(n):
            sim.step(1, 1 / 240.0)
            ora.step(1, 1 / 240.0)
        sim.render(inv)
        o = ora.render(table.optics_table(), inv, int(table.get("sss_iters")), float(table.get("bubbles")), has_dust=True)
        m = diff(sim.download_render("raw"), o[0], "raw")
        assert m is None, m
        ep, es, es1, el, ef, ec = sim.download_spray()
        op, os_, os1, ol, of, oc = ora.spray()
        assert ec == oc, f"counters {ec} vs {oc}"
        assert np.array_equal(es1, os1) and np.array_equal(el, ol), "specks' free stack or list"
        assert np.array_equal(ef, of), "counts per cell"
        bad = np.nonzero(ep.view(np.uint32).reshape(-1, 8) != op.view(np.uint32).reshape(-1, 8))[0]
        assert len(bad) == 0, f"{len(np.unique(bad))} pool entries differ, first {bad[0]}: {ep[bad[0]]} vs {op[bad[0]]}"
        specks = ep[el][(ep["info"][el] & 8) != 0]
        states |= set((specks["info"] & 3).tolist())
    assert ec[4] > 0, "specks came in"
    assert {1, 2} <= states, f"specks suspended and resting ({states})"
    raw = sim.download_render("raw").astype(np.float32)
    assert float(raw[18, ..., 3].max()) > 0.0, "the dust field coloured the liquid"

"""The render side's cell passes on the device (sprout_sim_render: cell_optics.comp, light.comp,
optics_blur.comp) against the oracle's restatement (osim_render) on the same grid, bit for bit
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
    sim, (er, es, eg), (orw, osm, og) = render_pair(tank, 6)
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

"""Tank descriptions: the synthetic workloads of the engine's tests and benchmark.

A tank is a grid, named parameter settings (as `--set k=v`, src/sim/params.rs:986), scene
shapes (src/scene.rs) and rectangles filled with rest-density particles (maps::fill_rect,
src/maps.rs:466). Rows of custom liquids are `mat<row>`. The description is plain data, so
other implementations (the tests' CPU oracle) can be built from the same one.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

@dataclass
class Tank:
    w: int
    h: int
    settings: dict = field(default_factory=dict)
    shapes: list = field(default_factory=list)      # dicts: kind box/circle, c, half/r, angle, temp
    fills: list = field(default_factory=list)       # (rect, material row, temperature or None)
    capacity_extra: int = 64
    diluents: dict = field(default_factory=dict)    # custom row -> its diluent's row (a family)
    groups: dict = field(default_factory=dict)      # custom row -> its phase group (0-3)
    currents: list = field(default_factory=list)    # dicts: pos, radius, vel, rate (negative: a drain)
    magnets: list = field(default_factory=list)     # dicts: pos, radius, strength (T), dir
    # applied to the filled particles before the reset (both implementations): a function of
    # the particle array returning the array to start from (a velocity field, a selection)
    prepare: object = None

    # ---- the engine -----------------------------------------------------------------------
    def engine(self):
        import sprout_gb300 as S
        p = S.SimParams(self.settings)
        for row, dil in self.diluents.items():
            if not p.set_diluent(row, dil):
                raise ValueError(f"row {row} cannot take diluent {dil}")
        for row, grp in self.groups.items():
            if not p.set_group(row, grp):
                raise ValueError(f"row {row} cannot take phase group {grp}")
        sc = S.Scene(self.w, self.h)
        for s in self.shapes:
            if s["kind"] == "box":
                sc.add_box(s["c"], s["half"], s.get("angle", 0.0), s.get("temp"))
            else:
                sc.add_circle(s["c"], s["r"], s.get("temp"))
        sdf, solid, region, temp = sc.rasterize()
        parts = None
        for rect, mat, t in self.fills:
            before = 0 if parts is None else len(parts)
            parts = sc.fill_rect(rect, mat, parts)
            if t is not None:
                parts["t"][before:] = t
                parts["kind"][before:] |= 0x20000   # KIND_REAL_T: a temperature to settle
        if self.prepare is not None:
            parts = self.prepare(parts)
        sim = S.FluidSim(self.w, self.h, len(parts) + self.capacity_extra, p)
        if self.currents:
            sim.set_currents(self.currents)
        if self.magnets:
            sim.set_magnets(self.magnets)
        sim.set_solids(sdf, solid, region, temp)
        sim.reset(parts)
        return sim, parts, (sdf, solid, region, temp)



# ---- the configurations the benchmark names, at their sizes or scaled down ------------------

def dam_break(w: int = 384, h: int = 216, cell: float = 0.002, width: float = 0.4, height: float = 0.6,
              tol: float = 1e-5, extra: dict | None = None, mat: int = 0) -> Tank:
    """A plain dam break: liquid row `mat` (0 water, 1 honey, 2 oil) over the left `width` and
    bottom `height` of a closed box, fixed 1/240 s substeps, no surface tension (the 384 x 216
    water form is the first configuration). Honey takes the implicit viscosity solve."""
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": tol, "tension_water": 0.0}
    if mat == 1:
        s["tension_honey"] = 0.0
    elif mat == 2:
        s["tension_oil"] = 0.0
    s.update(extra or {})
    return Tank(w, h, s, [], [([0.0, 0.0, width * w, height * h], mat, None)])


def layered_custom(w: int, h: int, rows: list[dict], cell: float = 0.001, heater_rows: int = 0,
                   heater_temp: float = 326.85, ambient: float = 19.85, tol: float = 1e-5,
                   columns: bool = True, seed: int = 0, extra: dict | None = None) -> Tank:
    """Several custom liquids (rows 59.. of the material table) filling the tank in vertical
    columns (or horizontal layers), optionally over a heater strip held at `heater_temp`."""
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": tol, "ambient_temp": ambient}
    for k, props in enumerate(rows):
        r = 59 + k
        for name, val in props.items():
            s[f"mat{r}.{name}"] = val
    s.update(extra or {})
    shapes = []
    if heater_rows > 0:
        # a box over the bottom rows, held at the heater temperature (solid floor strip)
        shapes.append({"kind": "box", "c": [w / 2.0, 3.0 + heater_rows / 2.0], "half": [w / 2.0, heater_rows / 2.0],
                       "angle": 0.0, "temp": heater_temp})
    rng = np.random.default_rng(seed)
    fills = []
    n = len(rows)
    if columns:
        edges = np.sort(rng.uniform(0.0, 1.0, n - 1)) if n > 1 else np.array([])
        edges = np.concatenate([[0.0], edges, [1.0]])
        for k in range(n):
            fills.append(([edges[k] * w, 0.0, edges[k + 1] * w, float(h)], 59 + k, ambient))
    else:
        for k in range(n):
            fills.append(([0.0, k * h / n, float(w), (k + 1) * h / n], 59 + k, ambient))
    return Tank(w, h, s, shapes, fills)


# The three layers of the stratified tank: honey, water, olive oil (rho in kg/m^3, kinematic
# viscosity mu / rho in m^2/s), each a fifth of the height.
STRATIFIED_LAYERS = [
    {"density": 1420.0, "viscosity": 10.0 / 1420.0, "tension": 0.0},
    {"density": 1000.0, "viscosity": 1e-3 / 1000.0, "tension": 0.0},
    {"density": 910.0, "viscosity": 0.08 / 910.0, "tension": 0.0},
]


def stratified(w: int = 512, h: int = 288, cell: float = 0.002, tol: float = 1e-5,
               extra: dict | None = None, builtins: bool = False) -> Tank:
    """Honey, water and olive oil stacked bottom to top, each 20% of the height (the second
    configuration at 512 x 288); the honey layer takes the implicit viscosity solve.

    Three custom liquids (one phase group, no exchange) with the layers' properties by
    default. With `builtins` the layers are the built-in honey, water and olive oil rows with
    those properties: honey is a water concentrate (presets.rs:61-90), so the two exchange
    concentration at its mix rate (1.5 / s) and water that gains some becomes honey; olive oil
    is phase group 1, immiscible, drifting against the water with no interfacial tension
    (tension_oil_water 0: at 2 mm cells a tension would want substeps below the fixed 1/240 s)."""
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": tol, "viscosity_tol": tol}
    rows = [59, 60, 61]
    for k, props in enumerate(STRATIFIED_LAYERS):
        for name, val in props.items():
            s[f"mat{59 + k}.{name}"] = val
    if builtins:
        rows = [1, 0, 2]
        for k, mat in enumerate(["honey", "water", "oil"]):
            for name, val in STRATIFIED_LAYERS[k].items():
                s[f"{name}_{mat}"] = val
        s["tension_oil_water"] = 0.0
    s.update(extra or {})
    fills = [([0.0, k * 0.2 * h, float(w), (k + 1) * 0.2 * h], rows[k], None) for k in range(3)]
    return Tank(w, h, s, [], fills)


def full_physics(w: int = 1024, h: int = 576, cell: float = 0.001, n_liquids: int = 8, seed: int = 0,
                 heater_rows: int = 8, tol: float = 1e-5, extra: dict | None = None) -> Tank:
    """The full-physics pour (the 1024 x 576 configuration): `n_liquids` custom liquids in
    seeded random vertical columns over the whole tank, rho uniform in 800-13500 kg/m^3,
    dynamic viscosity log-uniform in 1e-3-50 Pa s, surface tension uniform in 0.02-0.5 N/m;
    293 K everywhere over a 600 K heater strip along the bottom `heater_rows` rows; heat
    diffusion, surface tension and implicit viscosity all on."""
    rng = np.random.default_rng(seed)
    rows = []
    for _ in range(n_liquids):
        rho = float(rng.uniform(800.0, 13500.0))
        mu = float(np.exp(rng.uniform(np.log(1e-3), np.log(50.0))))
        rows.append({"density": rho, "viscosity": min(mu / rho, 0.5), "tension": float(rng.uniform(0.02, 0.5))})
    ex = {"viscosity_tol": tol}
    ex.update(extra or {})
    return layered_custom(w, h, rows, cell=cell, heater_rows=heater_rows, heater_temp=326.85,
                          ambient=19.85, tol=tol, columns=True, seed=seed + 1, extra=ex)


# ---- many tanks: the batched and serving configurations ---------------------------------------

# the grid sizes both draw from, and the serving mix's weights of them
UNEVEN_SIZES = [(128, 72), (256, 144), (384, 216), (512, 288), (768, 432), (1024, 576)]
SERVING_WEIGHTS = [0.30, 0.25, 0.20, 0.12, 0.08, 0.05]


def config3_liquid(rng) -> dict:
    """One liquid from the full-physics pour's ranges: rho uniform in 800-13500 kg/m^3, dynamic
    viscosity log-uniform in 1e-3-50 Pa s, surface tension uniform in 0.02-0.5 N/m."""
    rho = float(rng.uniform(800.0, 13500.0))
    mu = float(np.exp(rng.uniform(np.log(1e-3), np.log(50.0))))
    return {"density": rho, "viscosity": min(mu / rho, 0.5), "tension": float(rng.uniform(0.02, 0.5))}


def uneven_dam_breaks(n: int = 64, seed: int = 0, weights: list | None = None, tol: float = 1e-5,
                      extra: dict | None = None) -> list:
    """Seeded dam breaks of uneven sizes (the batched configuration: 64 tanks, sizes uniform
    over UNEVEN_SIZES; the serving mix: sizes by SERVING_WEIGHTS). Each tank is the same
    physical box, 1.024 m wide (cell size 1.024 m / width), fixed 1/240 s substeps; its liquid
    block covers a seeded 0.2-0.6 of the width and 0.3-0.8 of the height and holds one or two
    liquids (side by side) drawn from the full-physics pour's ranges; pressure and viscosity
    to `tol`."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        k = int(rng.choice(len(UNEVEN_SIZES), p=weights)) if weights is not None else int(rng.integers(len(UNEVEN_SIZES)))
        w, h = UNEVEN_SIZES[k]
        fw, fh = float(rng.uniform(0.2, 0.6)), float(rng.uniform(0.3, 0.8))
        nliq = int(rng.integers(1, 3))
        s = {"cell_size": 1.024 / w, "fixed_hz": 240.0, "pressure_tol": tol, "viscosity_tol": tol}
        for j in range(nliq):
            for name, val in config3_liquid(rng).items():
                s[f"mat{59 + j}.{name}"] = val
        s.update(extra or {})
        x1, y1 = fw * w, fh * h
        if nliq == 1:
            fills = [([0.0, 0.0, x1, y1], 59, None)]
        else:
            xm = float(int(x1 * rng.uniform(0.3, 0.7)))
            fills = [([0.0, 0.0, xm, y1], 59, None), ([xm, 0.0, x1, y1], 60, None)]
        out.append(Tank(w, h, s, [], fills))
    return out

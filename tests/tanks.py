"""The workloads of the tests: sprout_gb300.workloads' tank descriptions, built for the engine
(Tank.engine) and for the CPU oracle (oracle_of)."""
from sprout_gb300.workloads import *  # noqa: F401,F403
from sprout_gb300.workloads import Tank


def oracle_of(tank: Tank):
    from oracle import oracle as O
    return O.build_tank(tank)


def honey_dam(w: int = 96, h: int = 64, cell: float = 0.002, mix_rate: float | None = None) -> Tank:
    """A water column falling onto a layer of the built-in honey (a water concentrate): the
    two meet, exchange concentration, and water that gains some becomes honey."""
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": 1e-5, "viscosity_tol": 1e-5,
         "tension_water": 0.0, "tension_honey": 0.0, "viscosity_honey": 2e-4}
    if mix_rate is not None:
        s["mix_rate_honey"] = mix_rate
    fills = [([0.0, 0.0, float(w), 0.3 * h], 1, None), ([0.0, 0.3 * h, 0.4 * w, 0.8 * h], 0, None)]
    return Tank(w, h, s, [], fills)


def families_tank(w: int = 96, h: int = 64, cell: float = 0.002) -> Tank:
    """Three concentration families in one tank: honey in water (the primary family, 0), a
    custom water concentrate (mat59, family 1) and a concentrate (mat61, family 2) of another
    custom liquid (mat60), each block beside its diluent."""
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": 1e-5, "viscosity_tol": 1e-5,
         "tension_water": 0.0, "tension_honey": 0.0, "viscosity_honey": 2e-4}
    for row, props in {59: {"density": 1200.0, "viscosity": 1e-4, "mix_rate": 2.0},
                       60: {"density": 900.0, "viscosity": 1e-5},
                       61: {"density": 1100.0, "viscosity": 5e-4, "mix_rate": 3.0}}.items():
        for name, val in dict(props, tension=0.0).items():
            s[f"mat{row}.{name}"] = val
    sx, sy = w / 96.0, h / 64.0
    box = lambda x0, y0, x1, y1: [x0 * sx, y0 * sy, x1 * sx, y1 * sy]
    fills = [(box(48, 0, 96, 16), 1, None), (box(0, 0, 48, 16), 59, None), (box(0, 16, 30, 50), 0, None),
             (box(60, 30, 90, 50), 60, None), (box(60, 16, 90, 30), 61, None)]
    return Tank(w, h, s, [], fills, diluents={59: 0, 61: 60})



def around(rect, holes):
    """Rectangles covering `rect` less the `holes` (x0, y0, x1, y1 in whole cells), so that
    liquid filled around blocks of other liquids does not land on them (fill_rect does not
    look at what is already there)."""
    x0, y0, x1, y1 = rect
    ys = sorted({y0, y1, *[v for hh in holes for v in (hh[1], hh[3]) if y0 < v < y1]})
    out = []
    for ya, yb in zip(ys, ys[1:]):
        cuts = sorted((max(hh[0], x0), min(hh[2], x1)) for hh in holes if hh[1] <= ya and hh[3] >= yb and hh[0] < x1 and hh[2] > x0)
        x = x0
        for ca, cb in cuts:
            if ca > x:
                out.append([float(x), float(ya), float(ca), float(yb)])
            x = max(x, cb)
        if x < x1:
            out.append([float(x), float(ya), float(x1), float(yb)])
    return out


def water_oil(w: int = 96, h: int = 64, cell: float = 0.002) -> Tank:
    """A block of the built-in olive oil (phase group 1) under water: immiscible, it drifts
    up through the water and meets it with the groups' pair tension."""
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": 1e-5, "tension_water": 0.0, "tension_oil": 0.0}
    oil = [int(0.3 * w), int(0.1 * h), int(0.6 * w), int(0.35 * h)]
    fills = [([float(v) for v in oil], 2, None)]
    fills += [(r, 0, None) for r in around([0, 0, w, int(0.6 * h)], [oil])]
    return Tank(w, h, s, [], fills)


def three_groups(w: int = 96, h: int = 64, cell: float = 0.002) -> Tank:
    """Water with two oil-like custom liquids stacked in one block, the lighter below (group 1
    sorts them by density), and a dense metal-like custom liquid (group 2) above: three
    phase groups."""
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": 1e-5, "viscosity_tol": 1e-5, "tension_water": 0.0}
    for row, props in {59: {"density": 850.0, "viscosity": 5e-5}, 60: {"density": 960.0, "viscosity": 2e-5},
                       61: {"density": 3000.0, "viscosity": 1e-6}}.items():
        for name, val in dict(props, tension=0.0).items():
            s[f"mat{row}.{name}"] = val
    sx, sy = w / 96.0, h / 64.0
    box = lambda x0, y0, x1, y1: [int(x0 * sx), int(y0 * sy), int(x1 * sx), int(y1 * sy)]
    a, b, c = box(10, 4, 40, 14), box(10, 14, 40, 24), box(60, 26, 80, 36)
    fills = [([float(v) for v in a], 59, None), ([float(v) for v in b], 60, None), ([float(v) for v in c], 61, None)]
    fills += [(r, 0, None) for r in around([0, 0, w, int(36 * sy)], [a, b, c])]
    return Tank(w, h, s, [], fills, groups={59: 1, 60: 1, 61: 2})


def builtin_mix(w: int = 96, h: int = 64, cell: float = 0.002) -> Tank:
    """Built-in liquids side by side: water, ink and milk (water concentrates: two families),
    olive oil (phase group 1) and mercury (phase group 2), no surface tension."""
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": 1e-5, "viscosity_tol": 1e-5}
    for k in ["water", "ink", "milk", "oil", "mercury"]:
        s[f"tension_{k}"] = 0.0
    for k in ["tension_oil_water", "tension_metal_water", "tension_metal_oil"]:
        s[k] = 0.0
    sx, sy = w / 96.0, h / 64.0
    box = lambda x0, y0, x1, y1: [int(x0 * sx), int(y0 * sy), int(x1 * sx), int(y1 * sy)]
    ink, milk, oil, hg = box(8, 4, 28, 16), box(40, 4, 60, 16), box(66, 4, 86, 14), box(40, 30, 52, 40)
    fills = [([float(v) for v in ink], 4, None), ([float(v) for v in milk], 11, None),
             ([float(v) for v in oil], 2, None), ([float(v) for v in hg], 8, None)]
    fills += [(r, 0, None) for r in around([0, 0, w, int(36 * sy)], [ink, milk, oil, hg])]
    return Tank(w, h, s, [], fills)


def shear_thinning(w: int = 96, h: int = 64, cell: float = 0.002, mat: int = 7) -> Tank:
    """A dam break of a Carreau (shear-thinning) built-in, blood by default (soap: 19), beside
    water: rheo.comp sets each cell's viscosity from its shear rate."""
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": 1e-5, "viscosity_tol": 1e-5, "tension_water": 0.0,
         "tension_" + {7: "blood", 19: "soap"}[mat]: 0.0}
    sx, sy = w / 96.0, h / 64.0
    box = lambda x0, y0, x1, y1: [float(int(x0 * sx)), float(int(y0 * sy)), float(int(x1 * sx)), float(int(y1 * sy))]
    fills = [(box(4, 4, 40, 44), mat, None), (box(60, 4, 92, 20), 0, None)]
    return Tank(w, h, s, [], fills)


def settling(w: int = 96, h: int = 64, cell: float = 0.002, mat: int = 51) -> Tank:
    """A suspension over clear water: silt (51, grains of 0.1 mm, a water concentrate) by
    default, or mud (3: also shear-thinning). Its grains settle through the water below."""
    key = {51: "silt", 3: "mud"}[mat]
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": 1e-5, "viscosity_tol": 1e-5,
         "tension_water": 0.0, f"tension_{key}": 0.0}
    fills = [([0.0, 0.0, float(w), float(int(0.3 * h))], 0, None),
             ([0.0, float(int(0.3 * h)), float(w), float(int(0.55 * h))], mat, None)]
    return Tank(w, h, s, [], fills)


def currents(w: int = 96, h: int = 64, cell: float = 0.002) -> Tank:
    """A resting pool with a current driving its left half to the right and a drain near the
    right wall's floor."""
    t = dam_break(w, h, width=1.0, height=0.5)
    t.currents = [{"pos": (0.25 * w, 0.2 * h), "radius": 0.15 * h, "vel": (60.0, 5.0), "rate": 20.0},
                  {"pos": (0.85 * w, 0.08 * h), "radius": 0.1 * h, "vel": (0.0, 0.0), "rate": -30.0}]
    return t


def magnetic(w: int = 96, h: int = 64, cell: float = 0.002, mat: int = 37, demag: float = 0.0) -> Tank:
    """A pool of a magnetic built-in ("magnetic", 37, or ferrofluid, 13) over water with a
    magnet above it, north pole up: the field's energy pulls the liquid towards the magnet."""
    key = {37: "magnetic", 13: "ferrofluid"}[mat]
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": 1e-5, "viscosity_tol": 1e-5,
         "tension_water": 0.0, f"tension_{key}": 0.0, "magnet_demag": demag}
    fills = [([0.0, 0.0, float(w), float(int(0.2 * h))], 0, None),
             ([float(int(0.3 * w)), float(int(0.2 * h)), float(int(0.7 * w)), float(int(0.35 * h))], mat, None)]
    t = Tank(w, h, s, [], fills)
    t.magnets = [{"pos": (0.5 * w, 0.45 * h), "radius": 4.0, "strength": 1.0, "dir": (0.0, 1.0)}]
    return t


def elastic_drop(w: int = 96, h: int = 64, cell: float = 0.002, mat: int = 12) -> Tank:
    """A block of a viscoelastic built-in (slime, 12, or putty, 33) falling into water: its
    particles carry an upper-convected Maxwell stress that elastic.comp turns into force."""
    key = {12: "slime", 33: "putty"}[mat]
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": 1e-5, "viscosity_tol": 1e-5,
         "tension_water": 0.0, f"tension_{key}": 0.0}
    fills = [([0.0, 0.0, float(w), float(int(0.25 * h))], 0, None),
             ([float(int(0.35 * w)), float(int(0.45 * h)), float(int(0.65 * w)), float(int(0.7 * h))], mat, None)]
    return Tank(w, h, s, [], fills)


def yield_stress(w: int = 96, h: int = 64, cell: float = 0.002, mat: int = 5) -> Tank:
    """A dam break of a yield-stress built-in (molten chocolate, 5, or clay slip, 6): where
    its stress stays below the yield stress it moves as rigid bodies (rigid.comp)."""
    key = {5: "chocolate", 6: "clay"}[mat]
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": 1e-5, "viscosity_tol": 1e-5, f"tension_{key}": 0.0}
    fills = [([0.0, 0.0, float(int(0.4 * w)), float(int(0.6 * h))], mat, None)]
    return Tank(w, h, s, [], fills)


def cooling_lava(w: int = 96, h: int = 64, cell: float = 0.002) -> Tank:
    """A blob of lava (9) at 760 C, near its solidus, falling through 20 C air onto the floor: it loses heat to
    the air and the walls and its crust freezes into rigid bodies."""
    s = {"cell_size": cell, "fixed_hz": 240.0, "pressure_tol": 1e-5, "viscosity_tol": 1e-5, "tension_lava": 0.0}
    fills = [([float(int(0.3 * w)), float(int(0.2 * h)), float(int(0.6 * w)), float(int(0.5 * h))], 9, 760.0)]
    return Tank(w, h, s, [], fills)

"""The reference's physics known-answer checks (src/validate.rs), restated as scenarios that
run on either implementation: the CPU oracle (tests/test_validate.py checks it against the
reference's own thresholds) and the engine (tests/test_gpu_validate.py checks the same
thresholds and that the engine matches the oracle bit for bit).

Each scenario is built as the reference builds it: a 512 x 288 grid (validate.rs:16) with the
default parameters (1 cm cells, the adaptive substep, water's default surface tension), a
scene of box walls (scene.rs WALL = 3 cells), particles from maps::fill_rect, and advanced by
FluidSim::advance_blocking for the scenario's seconds of simulated time. Measurements and
thresholds follow validate.rs line by line (cited per scenario).
"""
from __future__ import annotations

import math

import numpy as np

from sprout_gb300.workloads import Tank

GRID = (512, 288)    # validate.rs:16
WALL = 3.0           # scene.rs:8
PPC = 4              # params.rs:11
G_CELLS = 9.81 / 0.01   # SimParams::g_cells at the default gravity and cell size (params.rs:900-902)


class Runner:
    """One tank on one implementation: advance(seconds) as FluidSim::advance_blocking,
    particles() as download_particles (live ones), stats() as the solver statistics."""

    def __init__(self, tank: Tank, impl: str):
        self.impl = impl
        if impl == "engine":
            self.sim, self.parts0, _ = tank.engine()
        else:
            from oracle import oracle as O
            self.sim, self.parts0, _ = O.build_tank(tank)
            O.set_threads(O.threads_available())

    def advance(self, seconds: float):
        if seconds > 0.0:
            self.sim.advance_blocking(seconds)

    def particles(self) -> np.ndarray:
        ps = self.sim.download_particles() if self.impl == "engine" else self.sim.particles()
        return ps[ps["kind"] != 0]

    def stats(self):
        """(pressure unconverged, substeps, most iterations, viscosity unconverged)"""
        s = self.sim.stats()
        if self.impl == "engine":
            return s.pressure_unconverged, s.substeps, s.pressure_iters_max, s.viscosity_unconverged
        return s.p_unconv, s.substeps, s.p_it_max, s.v_unconv


# ---- measurements (validate.rs:73-123) -----------------------------------------------------

def percentile(v, q: float) -> float:
    """validate.rs:114-121: the k-th smallest with k = floor((n - 1) q) taken in f32."""
    v = np.asarray(v, np.float32)
    if len(v) == 0:
        return 0.0
    k = int(np.float32(len(v) - 1) * np.float32(q))
    return float(np.partition(v, k)[k])


def rms_speed(ps) -> float:
    v = ps["vel"].astype(np.float64)
    return math.sqrt(float((v[:, 0] ** 2 + v[:, 1] ** 2).sum()) / max(len(ps), 1))


def mode_amplitude(ps, pick, shape, component: int) -> float:
    """validate.rs:1109-1118: least-squares amplitude of a velocity component along shape(pos)."""
    sel = ps[pick(ps["pos"])]
    f = shape(sel["pos"]).astype(np.float64)
    return float((f * sel["vel"][:, component].astype(np.float64)).sum() / max((f * f).sum(), 1e-12))


def particles_where(bbox, inside, vel, grad):
    """validate.rs:1087-1106: the filled particles inside `inside`, with velocity field `vel`
    and its gradient (du/dx, du/dy, dv/dx, dv/dy) as the APIC matrix."""
    def prepare(ps):
        ps = ps[inside(ps["pos"])].copy()
        ps["vel"] = vel(ps["pos"])
        ps["c"] = grad(ps["pos"])
        return ps
    return prepare


def wall_box(x0, y0, x1, y1):
    return {"kind": "box", "c": [(x0 + x1) * 0.5, (y0 + y1) * 0.5], "half": [(x1 - x0) * 0.5, (y1 - y0) * 0.5],
            "angle": 0.0}


# ---- scenarios: (tank, run) where run(runner) returns [(what, measured, ok)] -------------------

def hydrostatic(seconds: float = 10.0):
    """validate.rs:124-138: a pool of water 100 cells deep must stay at rest (rms speed under
    1 % of sqrt(g h)) and keep its level (within 2 %) and its particles."""
    tank = Tank(*GRID, {}, [], [([0.0, 0.0, 512.0, 100.0 + WALL], 0, None)])

    def run(r: Runner):
        n0 = len(r.particles())
        r.advance(seconds)
        ps = r.particles()
        top = percentile(ps["pos"][:, 1], 0.995) - WALL
        v_ref = math.sqrt(G_CELLS * 100.0)
        rms = rms_speed(ps) / v_ref
        return [("particles conserved", (n0, len(ps)), n0 == len(ps)),
                ("surface level (cells)", top, abs(top / 100.0 - 1.0) < 0.02),
                ("residual motion rms / sqrt(g h)", rms, rms < 0.01)]
    return tank, run


def sealed(which: str):
    """validate.rs:140-175: liquid with no free surface. "box": a closed box of walls full of
    water for 3 s; "tank": the whole tank filled to the lid for 2 s. Nothing may leave, the
    liquid stays at rest (rms under 1 % of sqrt(g 80)), every pressure solve converges."""
    if which == "box":
        shapes = [wall_box(194.0, 0.0, 200.0, 86.0), wall_box(300.0, 0.0, 306.0, 86.0), wall_box(194.0, 80.0, 306.0, 86.0)]
        fill, seconds, lid = [200.0, 0.0, 300.0, 80.0], 3.0, 80.0
    else:
        shapes, fill, seconds, lid = [], [0.0, 0.0, 512.0, 288.0], 2.0, 80.0
    tank = Tank(*GRID, {}, shapes, [(fill, 0, None)])

    def run(r: Runner):
        n0 = len(r.parts0)
        r.advance(seconds)
        ps = r.particles()
        x, y = ps["pos"][:, 0], ps["pos"][:, 1]
        escaped = int(((y > lid + 1.0) | (x < 199.0) | (x > 301.0)).sum()) if which == "box" else 0
        rms = rms_speed(ps) / math.sqrt(G_CELLS * 80.0)
        unconv = r.stats()[0]
        return [(f"{which}: liquid stays where it is", (n0, len(ps), escaped), len(ps) == n0 and escaped == 0),
                (f"{which}: at rest rms / sqrt(g h)", rms, rms < 0.01),
                (f"{which}: pressure solves converged", unconv, unconv == 0)]
    return tank, run


# Martin & Moyce (1952), a column twice as tall as wide: front Z = x / a at T = t sqrt(2 g / a)
MARTIN_MOYCE = [(1.19, 1.44), (1.63, 1.89), (1.98, 2.33), (2.32, 2.78), (2.65, 3.22), (2.98, 3.67), (3.33, 4.11)]


def dam_break():
    """validate.rs:177-211: a water column 60 x 120 cells collapses; its surge front stays
    within 20 % of the experiment and its speed dZ/dT between 1.2 and 1.6."""
    a = 60.0
    tank = Tank(*GRID, {}, [], [([0.0, 0.0, WALL + a, WALL + 2.0 * a], 0, None)])

    def run(r: Runner):
        t, worst, fronts = 0.0, 0.0, []
        for tt, z_ref in MARTIN_MOYCE:
            target = float(np.float32(tt) / np.sqrt(np.float32(2.0 * G_CELLS / a), dtype=np.float32))
            r.advance(target - t)
            t = target
            ps = r.particles()
            front = (percentile(ps["pos"][:, 0], 0.999) - WALL) / a
            if abs(front / z_ref - 1.0) > abs(worst):
                worst = front / z_ref - 1.0
            fronts.append((tt, front))
        speed = (fronts[6][1] - fronts[2][1]) / (fronts[6][0] - fronts[2][0])
        return [("front vs experiment, worst deviation", worst, abs(worst) < 0.20),
                ("front speed dZ/dT", speed, 1.2 < speed < 1.6)]
    return tank, run


def ritter():
    """validate.rs:213-238: a reservoir 300 x 30 cells released at once: at the dam site the
    depth holds at 4/9 of the reservoir's and the flow at 2/3 sqrt(g h0) (Ritter 1892), each
    within 10 %, sampled at 0.6-0.9 s."""
    length, h0 = 300.0, 30.0
    tank = Tank(*GRID, {}, [], [([0.0, 0.0, WALL + length, WALL + h0], 0, None)])

    def run(r: Runner):
        c0 = math.sqrt(G_CELLS * h0)
        depth = speed = 0.0
        t = 0.0
        for target in (0.6, 0.7, 0.8, 0.9):
            r.advance(target - t)
            t = target
            ps = r.particles()
            band = ps[np.abs(ps["pos"][:, 0] - (WALL + length)) < 3.0]
            depth += len(band) / (6.0 * PPC)
            speed += float(band["vel"][:, 0].sum()) / max(len(band), 1)
        depth, speed = depth / 4 / h0, speed / 4 / c0
        return [("depth at the dam site / h0", depth, abs(depth / (4.0 / 9.0) - 1.0) < 0.10),
                ("flow speed at the dam site / sqrt(g h0)", speed, abs(speed / (2.0 / 3.0) - 1.0) < 0.10)]
    return tank, run


VISC_SETTINGS = {"gravity": 0.0, "viscosity_water": 0.01, "viscosity_honey": 0.01, "viscosity_oil": 0.01,
                 "tension_water": 0.0, "tension_honey": 0.0, "tension_oil": 0.0, "tension_oil_water": 0.0}
NU_CELLS = 0.01 / (0.01 * 0.01)   # SimParams::nu_cells: 100 cells^2 / s


def viscosity(which: str):
    """validate.rs:1120-1230: viscosity alone in zero gravity (nu = 0.01 m^2/s = 100 cells^2/s).
    "free": a free slab 40 cells thick with u = A cos(pi y / H) decays at nu (pi/H)^2 (5 %);
    "floor": the slab on the no-slip floor with u = A sin(pi y / 2H) decays at nu (pi/2H)^2
    (10 %); "disc": a disc in rigid rotation keeps over 95 % of its angular momentum for 1 s,
    and every viscosity solve converges."""
    h, a = 40.0, 20.0
    pi = math.pi
    if which == "free":
        y0, k, t = 100.0, pi / h, 1.0
        prep = particles_where([80.0, y0, 432.0, y0 + h], lambda p: np.ones(len(p), bool),
                               lambda p: np.stack([a * np.cos(k * (p[:, 1] - y0)), np.zeros(len(p))], 1),
                               lambda p: np.stack([np.zeros(len(p)), -a * k * np.sin(k * (p[:, 1] - y0)),
                                                   np.zeros(len(p)), np.zeros(len(p))], 1))
        shape = lambda p: np.cos(np.float32(k) * (p[:, 1] - np.float32(y0)))
        bbox, tol = [80.0, y0, 432.0, y0 + h], 0.05
    elif which == "floor":
        y0, k, t = WALL, pi / (2.0 * h), 2.0
        prep = particles_where([80.0, y0, 432.0, y0 + h], lambda p: np.ones(len(p), bool),
                               lambda p: np.stack([a * np.sin(k * (p[:, 1] - y0)), np.zeros(len(p))], 1),
                               lambda p: np.stack([np.zeros(len(p)), a * k * np.cos(k * (p[:, 1] - y0)),
                                                   np.zeros(len(p)), np.zeros(len(p))], 1))
        shape = lambda p: np.sin(np.float32(k) * (p[:, 1] - np.float32(y0)))
        bbox, tol = [80.0, y0, 432.0, y0 + h], 0.10
    else:
        c, rad, omega = (256.0, 144.0), 50.0, 2.0
        prep = particles_where([c[0] - rad, c[1] - rad, c[0] + rad, c[1] + rad],
                               lambda p: np.hypot(p[:, 0] - c[0], p[:, 1] - c[1]) < rad,
                               lambda p: np.stack([-omega * (p[:, 1] - c[1]), omega * (p[:, 0] - c[0])], 1),
                               lambda p: np.tile(np.array([0.0, -omega, omega, 0.0]), (len(p), 1)))
        bbox = [c[0] - rad, c[1] - rad, c[0] + rad, c[1] + rad]
    tank = Tank(*GRID, dict(VISC_SETTINGS), [], [(bbox, 0, None)], prepare=prep)

    def run(r: Runner):
        if which == "disc":
            def angular(ps):
                x, y = ps["pos"][:, 0].astype(np.float64), ps["pos"][:, 1].astype(np.float64)
                vx, vy = ps["vel"][:, 0].astype(np.float64), ps["vel"][:, 1].astype(np.float64)
                return float(((x - x.mean()) * vy - (y - y.mean()) * vx).sum())
            l0 = angular(r.particles())
            r.advance(1.0)
            l1 = angular(r.particles())
            unconv = r.stats()[3]
            return [("rigid rotation keeps its angular momentum", l1 / l0, l1 / l0 > 0.95),
                    ("viscosity solves converged", unconv, unconv == 0)]
        mid = lambda p: (p[:, 0] > 180.0) & (p[:, 0] < 332.0)
        a0 = mode_amplitude(r.particles(), mid, shape, 0)
        r.advance(t)
        a1 = mode_amplitude(r.particles(), mid, shape, 0)
        rate = math.log(a0 / a1) / t
        theory = NU_CELLS * k * k
        return [(f"{which} slab: decay rate / theory", rate / theory, abs(rate / theory - 1.0) < tol)]
    return tank, run


SCENARIOS = {
    "hydrostatic": hydrostatic,
    "sealed_box": lambda: sealed("box"),
    "sealed_tank": lambda: sealed("tank"),
    "dam_break": dam_break,
    "ritter": ritter,
    "viscosity_free": lambda: viscosity("free"),
    "viscosity_floor": lambda: viscosity("floor"),
    "viscosity_disc": lambda: viscosity("disc"),
}

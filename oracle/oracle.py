"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: the checker the parity tests compare the CUDA engine with. Only
tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may import this module.
The oracle restates the reference's substep (shaders/*.comp and src/sim/mod.rs); see
oracle/sprout_oracle.c for the file:line of each part.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

PARTICLE_DTYPE = np.dtype(
    [("pos", "<f4", 2), ("vel", "<f4", 2), ("c", "<f4", 4), ("s", "<f4"), ("kind", "<u4"),
     ("id", "<u4"), ("t", "<f4")]
)
assert PARTICLE_DTYPE.itemsize == 48


class OMat(C.Structure):
    _fields_ = [
        ("group", C.c_uint32), ("diluent", C.c_int32),
        ("density", C.c_float), ("density_solid", C.c_float), ("viscosity", C.c_float),
        ("rheology", C.c_uint32), ("temp_model", C.c_uint32),
        ("temp_b", C.c_float), ("temp_c", C.c_float), ("temp_ref", C.c_float),
        ("tension", C.c_float), ("contact_angle", C.c_float), ("mix_rate", C.c_float),
        ("grain", C.c_float), ("load", C.c_float),
        ("heat_capacity", C.c_float), ("conductivity", C.c_float), ("expansion", C.c_float),
        ("melt_lo", C.c_float), ("melt_hi", C.c_float), ("latent", C.c_float),
        ("emissivity", C.c_float), ("boil", C.c_float), ("latent_vap", C.c_float),
        ("freeze_shift", C.c_float), ("spawn_temp", C.c_float),
        ("shear_modulus", C.c_float), ("susceptibility", C.c_float), ("skin", C.c_float),
        ("friction", C.c_float), ("self_heat", C.c_float), ("volatility", C.c_float),
        ("react_with", C.c_int32), ("react_rate", C.c_float), ("fume", C.c_float),
        ("yield_stress", C.c_float), ("flow_index", C.c_float), ("shear_time", C.c_float), ("visc_ratio", C.c_float),
        ("saturation", C.c_float),
        ("relax_time", C.c_float),
    ]


class OSimParams(C.Structure):
    _fields_ = [
        ("cell_size", C.c_float), ("gravity", C.c_float),
        ("pair_tension", (C.c_float * 4) * 4),
        ("ambient_temp", C.c_float), ("heat_rate", C.c_float), ("air_cooling", C.c_float),
        ("contact_heat", C.c_float), ("eddy_heat", C.c_float), ("evaporation", C.c_uint32),
        ("rigid_viscosity", C.c_float), ("heat_power", C.c_float), ("steam", C.c_uint32),
        ("droplet_cells", C.c_float), ("cfl", C.c_float), ("advection_order", C.c_uint32),
        ("dt_max", C.c_float), ("fixed_hz", C.c_float), ("pressure_tol", C.c_float),
        ("pressure_max_iters", C.c_uint32), ("correction_tol", C.c_float),
        ("viscosity_tol", C.c_float), ("viscosity_max_iters", C.c_uint32),
        ("implicit_viscosity_min", C.c_float),
        ("viscous_projection", C.c_uint32), ("viscous_warm", C.c_uint32),
        ("viscosity_warm", C.c_uint32), ("viscosity_precond", C.c_uint32),
        ("viscosity_mg_levels", C.c_uint32), ("viscosity_mg_sweeps", C.c_uint32),
        ("spray_cfl", C.c_float), ("speed_cap", C.c_float), ("correction_time", C.c_float),
        ("correction_max", C.c_float), ("correction_deadband", C.c_float),
        ("correction_step_max", C.c_float), ("crowd_jitter", C.c_float),
        ("tool_crowd_max", C.c_float), ("apic_clamp", C.c_float), ("curvature_max", C.c_float),
        ("slip_cap", C.c_uint32), ("sealed_vent", C.c_uint32),
        ("mat", OMat * 96),
        ("magnet_demag", C.c_float),
        ("elastic_stress_max", C.c_float), ("elastic_step_max", C.c_float),
        ("rigid_contact", C.c_uint32), ("rigid_friction", C.c_float),
        ("iters_margin", C.c_float),
    ]


class OTool(C.Structure):
    _fields_ = [("pos", C.c_float * 2), ("vel", C.c_float * 2), ("radius", C.c_float),
                ("mode", C.c_int32), ("strength", C.c_float)]


class OShape(C.Structure):
    _fields_ = [("kind", C.c_int32), ("c", C.c_float * 2), ("half", C.c_float * 2),
                ("r", C.c_float), ("angle", C.c_float), ("temp", C.c_float)]


class OStats(C.Structure):
    _fields_ = [
        ("substeps", C.c_uint64), ("sim_time", C.c_float), ("dt", C.c_float), ("dt_prev", C.c_float),
        ("p_iters", C.c_uint32 * 2), ("p_done", C.c_uint32 * 2), ("p2_iters", C.c_uint32),
        ("v_iters", C.c_uint32), ("v_done", C.c_uint32),
        ("p_it_max", C.c_uint32), ("p_unconv", C.c_uint32), ("v_it_max", C.c_uint32),
        ("v_unconv", C.c_uint32), ("p2_it_max", C.c_uint32), ("p2_unconv", C.c_uint32),
        ("solves", C.c_uint32), ("p_res_max", C.c_float), ("v_res_max", C.c_float),
        ("p_rr", C.c_float * 2), ("p_bb", C.c_float * 2), ("v_rr", C.c_float), ("v_r0", C.c_float),
        ("umax_grid", C.c_float), ("umax_part", C.c_float),
        ("n_slots", C.c_uint32), ("caps", C.c_uint32), ("acc_stride", C.c_uint32),
        ("thermal", C.c_uint32), ("viscosity_mode", C.c_uint32), ("levels", C.c_uint32),
        ("tail", C.c_uint32),
    ]


def build(force: bool = False) -> Path:
    """Compiles the oracle (gcc, no fused multiply-add) into oracle/_build/liboracle.so."""
    src = HERE / "sprout_oracle.c"
    if LIB.exists() and not force and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off", "-fopenmp", "-fPIC",
           "-shared", "-o", str(LIB), str(src), "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P = C.POINTER
        L.oparams_default.argtypes = [P(OSimParams)]
        L.oscene_rasterize.argtypes = [C.c_int, C.c_int, C.c_int, P(OShape), P(C.c_float),
                                       P(C.c_float), P(C.c_uint32), P(C.c_float)]
        L.oscene_rasterize.restype = C.c_int
        L.oscene_sdf.argtypes = [C.c_int, C.c_int, C.c_int, P(OShape), C.c_float, C.c_float]
        L.oscene_sdf.restype = C.c_float
        L.ofill_rect.argtypes = [C.c_int, C.c_int, C.c_int, P(OShape), P(C.c_float), C.c_uint32,
                                 C.c_void_p, C.c_uint32, C.c_uint32]
        L.ofill_rect.restype = C.c_uint32
        L.osim_create.argtypes = [C.c_int, C.c_int, C.c_uint32, P(OSimParams)]
        L.osim_create.restype = C.c_void_p
        L.osim_destroy.argtypes = [C.c_void_p]
        L.osim_set_params.argtypes = [C.c_void_p, P(OSimParams)]
        L.osim_set_solids.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.osim_reset.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32]
        L.osim_set_currents.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32]
        L.osim_set_magnets.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32]
        L.osim_set_magnets.restype = C.c_int
        L.osim_set_currents.restype = C.c_int
        L.osim_reset.restype = C.c_int
        L.osim_spawn.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32]
        L.osim_spawn.restype = C.c_int
        L.osim_cell_counts.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int), C.c_void_p, C.c_size_t]
        L.osim_cell_counts.restype = C.c_long
        L.osim_step.argtypes = [C.c_void_p, C.c_uint32, C.c_float, P(OTool)]
        L.osim_step.restype = C.c_int
        L.osim_sort.argtypes = [C.c_void_p]
        L.osim_particles.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32]
        L.osim_particles.restype = C.c_uint32
        L.osim_field.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p, C.c_size_t]
        L.osim_field.restype = C.c_long
        L.osim_stats.argtypes = [C.c_void_p, P(OStats)]
        L.osim_visc_operator.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.osim_visc_operator.restype = C.c_long
        L.osim_vmg_apply.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.osim_vmg_apply.restype = C.c_long
        L.osim_set_threads.argtypes = [C.c_int]
        L.osim_render.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p]
        L.osim_render.restype = C.c_long
        L.osim_flow_map.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_uint32]
        L.osim_flow_map.restype = C.c_long
        L.osim_recorded_iters.argtypes = [C.c_void_p, C.c_void_p]
        L.osim_recorded_iters.restype = None
        L.osim_look.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_uint32]
        L.osim_look.restype = C.c_long
        L.osim_look_state.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
        L.osim_look_state.restype = C.c_long
        L.osim_spray.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float]
        L.osim_spray.restype = C.c_long
        L.osim_spray_state.argtypes = [C.c_void_p] + [C.c_void_p] * 6
        L.osim_set_dust.argtypes = [C.c_void_p, C.c_int]
        L.osim_set_dust.restype = None
        L.osim_spray_state.restype = C.c_long
        L.o_expf.argtypes = [C.c_float]
        L.o_expf.restype = C.c_float
        for fn in ("o_sinf", "o_cosf"):
            getattr(L, fn).argtypes = [C.c_float]
            getattr(L, fn).restype = C.c_float
        L.o_atan2.argtypes = [C.c_float, C.c_float]
        L.o_atan2.restype = C.c_float
        _lib = L
    return _lib


def default_params() -> OSimParams:
    p = OSimParams()
    lib().oparams_default(C.byref(p))
    return p


def shapes_array(shapes) -> tuple:
    arr = (OShape * max(len(shapes), 1))()
    for k, s in enumerate(shapes):
        arr[k].kind = 0 if s["kind"] == "circle" else 1
        arr[k].c[0], arr[k].c[1] = s["c"]
        if s["kind"] == "circle":
            arr[k].r = s["r"]
        else:
            arr[k].half[0], arr[k].half[1] = s["half"]
            arr[k].angle = s.get("angle", 0.0)
        t = s.get("temp")
        arr[k].temp = -2e9 if t is None else t
    return arr, len(shapes)


def rasterize(w: int, h: int, shapes=()):
    arr, n = shapes_array(shapes)
    sdf = np.zeros((h + 1) * (w + 1), np.float32)
    solid = np.zeros((h * w, 4), np.float32)
    region = np.zeros(h * w, np.uint32)
    temp = np.zeros(h * w, np.float32)
    f = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    heated = lib().oscene_rasterize(w, h, n, arr, f(sdf), f(solid), region.ctypes.data_as(C.POINTER(C.c_uint32)), f(temp))
    return sdf, solid, region, (temp if heated else None)


def fill_rect(w: int, h: int, rect, material: int, shapes=(), existing: np.ndarray | None = None):
    arr, n = shapes_array(shapes)
    n0 = 0 if existing is None else len(existing)
    r = (C.c_float * 4)(*rect)
    count = lib().ofill_rect(w, h, n, arr, r, material, None, n0, n0)
    out = np.zeros(count, PARTICLE_DTYPE)
    if existing is not None:
        out[:n0] = existing
    lib().ofill_rect(w, h, n, arr, r, material, out.ctypes.data, n0, count)
    return out


class OracleSim:
    """The oracle behind the same calls as FluidSim (src/sim/mod.rs:862-)."""

    def __init__(self, w: int, h: int, capacity: int, params: OSimParams):
        self.w, self.h = w, h
        self.params = params
        self.h_ = lib().osim_create(w, h, capacity, C.byref(params))
        if not self.h_:
            raise ValueError("oracle: bad grid")

    def close(self):
        if self.h_:
            lib().osim_destroy(self.h_)
            self.h_ = None

    __del__ = close

    def set_solids(self, sdf, solid, region, temp=None):
        self._keep = (np.ascontiguousarray(sdf, np.float32), np.ascontiguousarray(solid, np.float32),
                      np.ascontiguousarray(region, np.uint32),
                      None if temp is None else np.ascontiguousarray(temp, np.float32))
        a, b, c, d = self._keep
        lib().osim_set_solids(self.h_, a.ctypes.data, b.ctypes.data, c.ctypes.data, None if d is None else d.ctypes.data)

    def reset(self, particles: np.ndarray) -> int:
        p = np.ascontiguousarray(particles, PARTICLE_DTYPE)
        self.sim_time, self.dt_est = 0.0, float(np.float32(1.0) / np.float32(240.0))
        self._resets = getattr(self, "_resets", 0) + 1
        self._stain_valid = False
        return lib().osim_reset(self.h_, p.ctypes.data, len(p))

    # The host loop of FluidSim::advance_blocking (src/sim/mod.rs:3284-3312) over the oracle,
    # with the engine's host arithmetic: the substep count and target of each step call, the
    # simulated time and the CFL estimate read back after it (poll_readbacks).
    fixed_hz = 0.0
    sliver = float(np.float32(0.02))   # min_substep_share as a float

    def dt_estimate(self) -> float:
        if self.fixed_hz > 0.0:
            return float(np.float32(1.0) / np.float32(self.fixed_hz))
        return self.dt_est

    def _poll(self):
        st = self.field("step")
        advanced, dt_cfl, comp = float(st[1]), float(st[8]), float(st[11:12].view(np.float32)[0])
        t = advanced - comp
        if t > self.sim_time:
            self.sim_time = t
        if dt_cfl > 0.0:
            self.dt_est = dt_cfl

    def advance_blocking(self, seconds: float):
        goal = self.sim_time + seconds
        for _ in range(1000000):
            left = goal - self.sim_time
            dt = self.dt_estimate()
            if left <= self.sliver * dt:
                break
            nn = max(round(left / dt), 1.0) if self.fixed_hz > 0.0 else float(np.ceil(left / dt))
            n = int(min(max(nn, 1.0), 16.0))
            target = n * dt if self.fixed_hz > 0.0 else left
            self.step(n, float(np.float32(target)))
            self._poll()
            if self.fixed_hz > 0.0 and (goal - self.sim_time) < 0.5 * dt:
                break

    def set_magnets(self, magnets):
        from sprout_gb300 import magnet_array
        arr = magnet_array(magnets)
        return lib().osim_set_magnets(self.h_, arr.ctypes.data if len(arr) else None, len(arr))

    def set_currents(self, currents):
        from sprout_gb300 import current_array
        arr = current_array(currents)
        return lib().osim_set_currents(self.h_, arr.ctypes.data if len(arr) else None, len(arr))

    def spawn(self, particles: np.ndarray) -> int:
        """FluidSim::spawn: how many were queued (0 when their materials do not fit)."""
        p = np.ascontiguousarray(particles, PARTICLE_DTYPE)
        return lib().osim_spawn(self.h_, p.ctypes.data, len(p))

    def cell_counts(self, lo, hi) -> np.ndarray:
        """FluidSim::cell_counts: live particles per cell of [lo, hi), shape (rows, columns)."""
        a, b = (C.c_int * 2)(*lo), (C.c_int * 2)(*hi)
        n = lib().osim_cell_counts(self.h_, a, b, None, 0)
        if n < 0:
            raise ValueError("oracle: window outside the grid")
        out = np.zeros(n, np.uint32)
        lib().osim_cell_counts(self.h_, a, b, out.ctypes.data, n)
        return out.reshape(max(hi[1] - lo[1], 0), max(hi[0] - lo[0], 0))

    def n_slots_(self) -> int:
        return int(lib().osim_particles(self.h_, None, 0))

    def spray(self):
        """spray.comp's pool: (entries, bubbles' stack, specks' stack, listed entries, counts
        (4, h, w), state (8)) as FluidSim.download_spray gives them."""
        from sprout_gb300 import DIFFUSE_DTYPE, POOL_MAX
        st = (C.c_uint32 * 8)()
        pool = np.zeros(POOL_MAX, DIFFUSE_DTYPE)
        stack, stack1, lst = (np.zeros(POOL_MAX, np.uint32) for _ in range(3))
        counts = np.zeros(4 * self.w * self.h, np.uint32)
        lib().osim_spray_state(self.h_, pool.ctypes.data, stack.ctypes.data, stack1.ctypes.data, lst.ctypes.data,
                               counts.ctypes.data, st)
        s = [int(x) for x in st]
        return pool, stack[: s[1]], stack1[: s[5]], lst[: s[2]], counts.reshape(4, self.h, self.w), s

    def look(self):
        """look.comp's state per slot (n, 4) uint32 and the slots the last render listed."""
        n = lib().osim_look_state(self.h_, None, 0)
        st = np.zeros((max(n, 0), 4), np.uint32)
        if n > 0:
            lib().osim_look_state(self.h_, st.ctypes.data, st.size)
        return st, getattr(self, "_look_list", np.zeros(0, np.uint32))

    def recorded_iters(self) -> list:
        """FluidSim::recorded_iters: [first pressure solve, second, viscosity]."""
        v = (C.c_uint32 * 3)()
        lib().osim_recorded_iters(self.h_, v)
        return [int(x) for x in v]

    def step(self, substeps: int, target: float = 0.0, tool: OTool | None = None):
        if substeps > 0:
            self._substeps = getattr(self, "_substeps", 0) + substeps
        return lib().osim_step(self.h_, substeps, target, None if tool is None else C.byref(tool))

    def sort(self):
        lib().osim_sort(self.h_)

    def particles(self) -> np.ndarray:
        n = lib().osim_particles(self.h_, None, 0)
        out = np.zeros(n, PARTICLE_DTYPE)
        lib().osim_particles(self.h_, out.ctypes.data, n)
        return out

    def render(self, optics: np.ndarray, inv_speed: float = 1.0 / 60.0, sss_iters: int = 4, bubbles: float = 1.0,
               has_dust: bool = False):
        """FluidSim::record_cell_optics (mod.rs:1626-1712) on the current grid, from the optics
        table `optics` (96 rows of 240 bytes): cell_optics.comp, light.comp, optics_blur.comp,
        sss.comp, flow_map.comp and glow.comp. Returns (raw (20, h, w, 4), smooth (24, h, w, 4),
        glow (ceil(h / 2), ceil(w / 2), 4), flow (4, h, w, 4), flow parity) as float16 arrays.
        Every buffer persists between calls (sss.comp's warm start, the flow map), and a call
        records nothing when no substep, reset, other table or other inv_speed came since the
        last one (the reference's optics_key; parameter changes between two calls with no
        substep are not tracked here). The clock (stain_at): the simulated time after the last
        substep, the compensated sum step.comp keeps, minus the last call's, clamped to
        0 .. 0.25 s and zero on the first call on a new tank, which also clears the flow map."""
        tab = np.ascontiguousarray(optics)
        assert tab.nbytes == 96 * 240
        nc = self.w * self.h
        hw, hh = (self.w + 1) // 2, (self.h + 1) // 2
        if getattr(self, "_smooth", None) is None:
            self._smooth = np.zeros(24 * nc * 4, np.uint16)
            self._raw = np.zeros(20 * nc * 4, np.uint16)
            self._flow = np.zeros(4 * nc * 4, np.uint16)
            self._ga, self._gb = np.zeros(hw * hh * 4, np.uint16), np.zeros(hw * hh * 4, np.uint16)
            self._parity, self._stain, self._key = 0, 0.0, None
        valid = getattr(self, "_stain_valid", False)
        if not valid:
            self._flow[:] = 0
        st = self.field("step")
        now = float(st[1]) - float(st[11:12].view(np.float32)[0])
        dt = np.float32(min(max(now - self._stain, 0.0), 0.25)) if valid else np.float32(0.0)
        self._stain, self._stain_valid = now, True
        key = (getattr(self, "_substeps", 0), getattr(self, "_resets", 0), tab.tobytes(),
               int(np.float32(inv_speed).view(np.uint32)))
        if key != self._key:
            self._key = key
            lib().osim_set_dust(self.h_, 1 if has_dust else 0)   # a liquid with specks in the tank
            lib().osim_render(self.h_, tab.ctypes.data, inv_speed, sss_iters, self._raw.ctypes.data,
                              self._smooth.ctypes.data, self._ga.ctypes.data, self._gb.ctypes.data)
            if dt > 0.0:
                lib().osim_flow_map(self.h_, self._smooth.ctypes.data, self._flow.ctypes.data, float(dt),
                                    float(np.float32(now)), self._parity)
                self._parity = 1 - self._parity
            # record_look: particles of a liquid without a look are left as they are, so the
            # pass runs whether or not the tank holds such a liquid
            lst = np.zeros(max(self.n_slots_(), 1), np.uint32)
            n = lib().osim_look(self.h_, tab.ctypes.data, float(dt), lst.ctypes.data, len(lst))
            self._look_list = lst[: min(max(n, 0), len(lst))].copy()
            lib().osim_spray(self.h_, self._smooth.ctypes.data, tab.ctypes.data, float(dt), float(bubbles))
        return (self._raw.copy().view(np.float16).reshape(20, self.h, self.w, 4),
                self._smooth.copy().view(np.float16).reshape(24, self.h, self.w, 4),
                self._gb.copy().view(np.float16).reshape(hh, hw, 4),
                self._flow.copy().view(np.float16).reshape(4, self.h, self.w, 4), self._parity)

    def field(self, name: str, dtype=np.float32) -> np.ndarray:
        n = lib().osim_field(self.h_, name.encode(), None, 0)
        if n < 0:
            raise KeyError(name)
        buf = np.zeros(n // np.dtype(dtype).itemsize, dtype)
        lib().osim_field(self.h_, name.encode(), buf.ctypes.data, n)
        return buf

    def visc_operator(self, x: np.ndarray):
        """The implicit viscosity's level-0 matrix and its matrix-free form applied to x
        (float32, 2 per cell): (unknown count, A_assembled x, A_matrix_free x)."""
        x = np.ascontiguousarray(x, np.float32)
        y0 = np.zeros_like(x)
        y1 = np.zeros_like(x)
        n = lib().osim_visc_operator(self.h_, x.ctypes.data, y0.ctypes.data, y1.ctypes.data)
        return n, y0, y1

    def vmg_apply(self, level: int, x: np.ndarray) -> np.ndarray:
        """The assembled viscosity matrix of multigrid `level` applied to x (2 per cell)."""
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros_like(x)
        if lib().osim_vmg_apply(self.h_, level, x.ctypes.data, y.ctypes.data) < 0:
            raise ValueError(level)
        return y

    def stats(self) -> OStats:
        s = OStats()
        lib().osim_stats(self.h_, C.byref(s))
        return s


def set_threads(n: int):
    lib().osim_set_threads(n)


def threads_available() -> int:
    return len(os.sched_getaffinity(0))


# ---- building the oracle's tank from a workload description -----------------------------

def _builtin_rows() -> dict:
    """Built-in row keys (presets.rs BUILTINS order), from the table's header."""
    import re
    inc = Path(__file__).resolve().parents[1] / "sprout_gb300" / "csrc" / "builtin_rows.inc"
    return {k: int(r) for r, k in re.findall(r"(\d+):([a-z_]+)", inc.read_text().split("*/", 2)[1])}


BUILTIN_ROWS = _builtin_rows()
MAT_FIELDS = {f for f, _ in OMat._fields_} - {"group", "diluent", "rheology", "react_with"}


def _row(name: str) -> int:
    if name in BUILTIN_ROWS:
        return BUILTIN_ROWS[name]
    if name.startswith("mat"):
        return int(name[3:])
    raise KeyError(name)


# material fields only the render side reads (the optics table the tests take from the engine)
RENDER_ONLY = {"cloud", "cloud_size", "cloud_ior", "cloud_shape", "dust", "dust_size", "dust_density",
               "dust_shape", "dust_reflect", "foam", "froth", "fizz"}

PAIR_TENSIONS = {"tension_oil_water": (0, 1), "tension_metal_water": (0, 2), "tension_metal_oil": (1, 2),
                 "tension_melt_water": (0, 3), "tension_melt_oil": (1, 3), "tension_melt_metal": (2, 3)}


def apply_setting(p: OSimParams, key: str, v: float):
    """The oracle-side counterpart of SimParams::set for the names the workloads use."""
    if key in PAIR_TENSIONS:
        a, b = PAIR_TENSIONS[key]
        p.pair_tension[a][b] = p.pair_tension[b][a] = float(v)
        return
    prop = row = None
    if "." in key:
        mat, prop = key.split(".", 1)
        row = _row(mat)
    else:
        for f in sorted(MAT_FIELDS, key=len, reverse=True):
            if key.startswith(f + "_"):
                try:
                    row, prop = _row(key[len(f) + 1:]), f
                    break
                except (KeyError, ValueError):
                    pass
    if prop is not None:
        m = p.mat[row]
        if prop in RENDER_ONLY and prop not in dict(m._fields_):
            return   # read by the optics table (the engine's SimParams), not by a substep
        typ = dict(m._fields_)[prop]
        setattr(m, prop, int(v) if typ in (C.c_uint32, C.c_int32) else float(v))
        return
    names = dict(p._fields_)
    if key not in names:
        raise KeyError(key)
    setattr(p, key, int(round(v)) if names[key] is C.c_uint32 else float(v))


def build_tank(tank, threads: int | None = None):
    """(OracleSim, particles, solids) for a workload description (sprout_gb300.workloads.Tank)."""
    p = default_params()
    for k, v in tank.settings.items():
        apply_setting(p, k, v)
    for row, dil in getattr(tank, "diluents", {}).items():
        p.mat[row].diluent = dil
    for row, grp in getattr(tank, "groups", {}).items():
        p.mat[row].group = grp
    sdf, solid, region, temp = rasterize(tank.w, tank.h, tank.shapes)
    parts = None
    for rect, mat, t in tank.fills:
        before = 0 if parts is None else len(parts)
        parts = fill_rect(tank.w, tank.h, rect, mat, tank.shapes, parts)
        if t is not None:
            parts["t"][before:] = t
            parts["kind"][before:] |= 0x20000
    if getattr(tank, "prepare", None) is not None:
        parts = tank.prepare(parts)
    sim = OracleSim(tank.w, tank.h, len(parts) + tank.capacity_extra, p)
    sim.fixed_hz = float(p.fixed_hz)
    sim.sliver = float(max(np.float32(tank.settings.get("min_substep_share", 0.02)), np.float32(1e-6)))
    if getattr(tank, "currents", None):
        sim.set_currents(tank.currents)
    if getattr(tank, "magnets", None):
        sim.set_magnets(tank.magnets)
    sim.set_solids(sdf, solid, region, temp)
    rc = sim.reset(parts)
    if rc != 0:
        raise RuntimeError(f"the oracle does not carry this tank ({rc})")
    if threads is not None:
        set_threads(threads)
    return sim, parts, (sdf, solid, region, temp)

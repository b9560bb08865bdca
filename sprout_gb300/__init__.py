"""sprout_gb300: a GB300 (sm_103a) engine for Sprout's per-substep 2D APIC/PIC fluid solver.

The engine is the C-ABI library libsprout_gpu.so (include/sprout_gpu.h); this module is a
thin ctypes layer over it with the reference's names: SimParams (with `set` by name, as
`--set k=v` / SimParams::set), Scene (Scene::rasterize, maps::fill_rect) and FluidSim
(reset, step, step_blocking, advance_blocking, download_particles, download_pressure,
stats). The library must have been built (sprout_gb300/build.py); nothing here falls back
to a CPU path.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libsprout_gpu.so"

PARTICLE_DTYPE = np.dtype(
    [("pos", "<f4", 2), ("vel", "<f4", 2), ("c", "<f4", 4), ("s", "<f4"), ("kind", "<u4"),
     ("id", "<u4"), ("t", "<f4")]
)
assert PARTICLE_DTYPE.itemsize == 48

SPROUT_OK = 0
ERRORS = {
    -1: "SPROUT_E_ARG", -2: "SPROUT_E_NOMEM", -3: "SPROUT_E_CAPACITY", -4: "SPROUT_E_DIVERGED",
    -5: "SPROUT_E_TIMEOUT", -6: "SPROUT_E_CUDA", -7: "SPROUT_E_UNSUPPORTED",
}

# Every entry point include/sprout_gpu.h declares.
EXPORTS = [
    "sprout_last_error", "sprout_version", "sprout_params_new", "sprout_params_free", "sprout_params_copy",
    "sprout_params_set", "sprout_params_get", "sprout_params_set_diluent", "sprout_params_set_group", "sprout_scene_new", "sprout_scene_free", "sprout_scene_add_box",
    "sprout_scene_add_circle", "sprout_scene_sdf", "sprout_scene_rasterize", "sprout_fill_rect",
    "sprout_sim_create", "sprout_sim_destroy", "sprout_sim_set_params", "sprout_sim_set_solids",
    "sprout_sim_reset", "sprout_sim_set_currents", "sprout_sim_set_magnets", "sprout_sim_frame_blocking", "sprout_sim_dt_estimate", "sprout_sim_step", "sprout_sim_step_blocking", "sprout_sim_advance_blocking",
    "sprout_sim_sync", "sprout_sim_download_particles", "sprout_sim_download_pressure",
    "sprout_sim_download_field", "sprout_sim_stats", "sprout_sim_device_bytes", "sprout_sim_profile",
    "sprout_sim_profile_passes", "sprout_pressure_solve_static", "sprout_sim_set_precision",
    "sprout_batch_create", "sprout_batch_destroy", "sprout_batch_add", "sprout_batch_remove", "sprout_batch_size",
    "sprout_batch_set_precision", "sprout_batch_step", "sprout_batch_sync", "sprout_batch_profile",
    "sprout_batch_step_subset", "sprout_batch_tickets", "sprout_device_memory", "sprout_sim_trace_enable",
    "sprout_sim_trace_read", "sprout_sim_spawn", "sprout_sim_cell_counts", "sprout_sim_set_launch",
    "sprout_sim_get_launch", "sprout_sim_debug_stall", "sprout_batch_set_launch", "sprout_sim_request_stats",
    "sprout_sim_poll_stats", "sprout_pacer_new", "sprout_pacer_free", "sprout_pacer_reset", "sprout_pacer_speed",
    "sprout_pacer_plan", "sprout_device_count", "sprout_set_device", "sprout_get_device",
    "sprout_scene_rasterize_device", "sprout_sim_set_scene", "sprout_spout", "sprout_sim_emit_stream",
    "sprout_sim_emit_paint", "sprout_sim_emit_rain", "sprout_sim_emitter_seed", "sprout_sim_emitted",
    "sprout_params_optics", "sprout_params_set_color", "sprout_sim_render", "sprout_sim_download_render",
    "sprout_params_get_color", "sprout_params_get_row", "sprout_sim_flow_parity", "sprout_sim_recorded_iters",
    "sprout_sim_download_look", "sprout_sim_download_spray", "sprout_sim_draw", "sprout_sim_download_draw",
]

# One row of the optics table (material.rs GpuOptics): 15 four-word fields, 240 bytes.
OPTICS_FIELDS = ["absorb", "solid", "opt", "sty", "idx", "fx", "fx2", "lum", "hot", "thermo", "scat", "opt2", "dust",
                 "dust2", "dcol"]
OPTICS_DTYPE = np.dtype([(f, "<i4" if f == "idx" else "<f4", 4) for f in OPTICS_FIELDS])
assert OPTICS_DTYPE.itemsize == 240
RENDER_LAYERS = 20
# spray.comp's pool entry (the reference's Diffuse) and the pool's size (mod.rs DIFFUSE_MAX)
DIFFUSE_DTYPE = np.dtype([("pos", np.float32, 2), ("vel", np.float32, 2), ("life", np.float32), ("r", np.float32),
                          ("info", np.uint32), ("z", np.float32)])
DIFFUSE_MAX = 1 << 16
POOL_MAX = DIFFUSE_MAX + (1 << 17)   # then the specks' part (mod.rs DUST_MAX)

STAGES = ["advance", "sort", "p2g", "grid", "pressure", "project", "viscosity", "project2"]


class SproutError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Tool(C.Structure):
    """ToolState (src/sim/params.rs:1141-1150)."""
    _fields_ = [("pos", C.c_float * 2), ("vel", C.c_float * 2), ("radius", C.c_float), ("mode", C.c_int32),
                ("strength", C.c_float)]

    @staticmethod
    def whirl(pos, radius: float, speed: float, clockwise: bool = False) -> "Tool":
        """ToolState::whirl (params.rs:1175-1181) with the rim speed in cells/s."""
        t = Tool()
        t.pos[0], t.pos[1] = pos
        t.vel[0] = -speed if clockwise else speed
        t.radius, t.mode, t.strength = radius, 7, 30.0
        return t


class SolverStats(C.Structure):
    _fields_ = [
        ("substeps", C.c_uint64), ("sim_time", C.c_double), ("dt", C.c_float), ("dt_prev", C.c_float),
        ("pressure_iters", C.c_uint32 * 2), ("pressure_iters_max", C.c_uint32),
        ("pressure_unconverged", C.c_uint32), ("pressure2_iters_max", C.c_uint32),
        ("pressure2_unconverged", C.c_uint32), ("viscosity_iters_max", C.c_uint32),
        ("viscosity_unconverged", C.c_uint32), ("solves", C.c_uint32),
        ("pressure_residual", C.c_float), ("pressure_residual_max", C.c_float),
        ("viscosity_residual_max", C.c_float), ("umax_grid", C.c_float), ("umax_part", C.c_float),
        ("n_slots", C.c_uint32), ("n_live", C.c_uint32), ("caps", C.c_uint32), ("acc_stride", C.c_uint32),
        ("thermal", C.c_uint32), ("viscosity_mode", C.c_uint32), ("levels", C.c_uint32), ("tail", C.c_uint32),
        ("device_error", C.c_uint32), ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
        ("viscosity_iters", C.c_uint32), ("viscosity_residual", C.c_float), ("pressure2_iters", C.c_uint32),
        ("pressure_true_residual", C.c_float), ("pressure_true_residual_max", C.c_float),
        ("pressure_replacements", C.c_uint32),
    ]


class Spout(C.Structure):
    """SproutSpout: brush::Spout (direction, speed cells/s, width cells)."""
    _fields_ = [("direction", C.c_float * 2), ("speed", C.c_float), ("width", C.c_float)]

    @staticmethod
    def make(kind: str, rate: float, radius: float, degrees: float = 0.0) -> "Spout":
        """Spout::pour / jet / faucet."""
        s = Spout()
        _check(lib().sprout_spout({"pour": 0, "jet": 1, "faucet": 2}[kind], degrees, rate, radius, C.byref(s)))
        return s


class StreamState:
    """brush::Stream: simulated seconds the stream has run (0 for a new stroke)."""

    def __init__(self, time: float = 0.0):
        self.time = time


class Launch(C.Structure):
    """SproutLaunch: block counts of the persistent solvers (0: the default)."""
    _fields_ = [("pressure_blocks", C.c_uint32), ("pressure_blocks_mixed", C.c_uint32),
                ("viscosity_blocks", C.c_uint32), ("batch_viscosity", C.c_uint32), ("reserved", C.c_uint32 * 4)]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k in ("pressure_blocks", "pressure_blocks_mixed", "viscosity_blocks",
                                                   "batch_viscosity")}


class Census(C.Structure):
    """SproutStats (Stats, src/sim/mod.rs:130-136): live particles, per material row its
    particles and the sum of their concentrations."""
    _fields_ = [("live", C.c_uint32), ("count", C.c_uint32 * 96), ("conc", C.c_float * 96)]


class Plan(C.Structure):
    """SproutPlan (pacing.rs Plan): substeps, target and expected simulated seconds."""
    _fields_ = [("substeps", C.c_uint32), ("target", C.c_float), ("expected", C.c_float)]


_lib = None


def lib() -> C.CDLL:
    """The engine library. Raises if it has not been built: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m sprout_gb300.build` (CUDA toolkit required)")
    L = C.CDLL(str(LIB_PATH))
    P, V = C.POINTER, C.c_void_p
    sig = {
        "sprout_last_error": ([], C.c_char_p), "sprout_version": ([], C.c_char_p),
        "sprout_params_new": ([P(V)], C.c_int), "sprout_params_free": ([V], C.c_int),
        "sprout_params_copy": ([V, P(V)], C.c_int),
        "sprout_params_set": ([V, C.c_char_p, C.c_float, P(C.c_int)], C.c_int),
        "sprout_params_get": ([V, C.c_char_p, P(C.c_float), P(C.c_int)], C.c_int),
        "sprout_params_set_diluent": ([V, C.c_uint32, C.c_int32, P(C.c_int)], C.c_int),
        "sprout_params_set_group": ([V, C.c_uint32, C.c_uint32, P(C.c_int)], C.c_int),
        "sprout_scene_new": ([C.c_uint32, C.c_uint32, P(V)], C.c_int), "sprout_scene_free": ([V], C.c_int),
        "sprout_scene_add_box": ([V] + [C.c_float] * 6, C.c_int),
        "sprout_scene_add_circle": ([V] + [C.c_float] * 4, C.c_int),
        "sprout_scene_sdf": ([V, C.c_float, C.c_float, P(C.c_float)], C.c_int),
        "sprout_scene_rasterize": ([V, V, V, V, V, P(C.c_int)], C.c_int),
        "sprout_scene_rasterize_device": ([V, V, V, V, V, P(C.c_int)], C.c_int),
        "sprout_sim_set_scene": ([V, V], C.c_int),
        "sprout_fill_rect": ([V, P(C.c_float), C.c_uint32, C.c_uint32, V, C.c_uint32, P(C.c_uint32)], C.c_int),
        "sprout_sim_create": ([C.c_uint32, C.c_uint32, C.c_uint32, V, P(V)], C.c_int),
        "sprout_sim_destroy": ([V], C.c_int), "sprout_sim_set_params": ([V, V], C.c_int),
        "sprout_sim_set_solids": ([V, V, V, V, V], C.c_int),
        "sprout_sim_reset": ([V, V, C.c_uint32], C.c_int),
        "sprout_sim_set_currents": ([V, V, C.c_uint32], C.c_int),
        "sprout_sim_set_magnets": ([V, V, C.c_uint32], C.c_int),
        "sprout_sim_frame_blocking": ([V, C.c_uint32, C.c_float, V, P(C.c_double)], C.c_int),
        "sprout_sim_dt_estimate": ([V, P(C.c_float)], C.c_int),
        "sprout_sim_step": ([V, C.c_uint32, C.c_float, P(Tool)], C.c_int),
        "sprout_sim_step_blocking": ([V, C.c_uint32, P(Tool)], C.c_int),
        "sprout_sim_advance_blocking": ([V, C.c_double, P(Tool)], C.c_int),
        "sprout_sim_sync": ([V], C.c_int),
        "sprout_sim_spawn": ([V, V, C.c_uint32, P(C.c_uint32)], C.c_int),
        "sprout_sim_cell_counts": ([V, P(C.c_int32), P(C.c_int32), V, C.c_size_t, P(C.c_size_t)], C.c_int),
        "sprout_spout": ([C.c_int, C.c_float, C.c_float, C.c_float, V], C.c_int),
        "sprout_sim_emit_stream": ([V, V, P(C.c_double), P(C.c_float), P(C.c_float), C.c_float, C.c_uint32], C.c_int),
        "sprout_sim_emit_paint": ([V, P(C.c_float), P(C.c_float), C.c_float, C.c_uint32, C.c_int, C.c_uint32], C.c_int),
        "sprout_sim_emit_rain": ([V, P(C.c_float), C.c_float, C.c_uint32, C.c_uint32], C.c_int),
        "sprout_sim_emitter_seed": ([V, C.c_uint32], C.c_int),
        "sprout_sim_emitted": ([V, P(C.c_uint64), P(C.c_uint32)], C.c_int),
        "sprout_params_optics": ([V, V, C.c_uint32], C.c_int),
        "sprout_params_set_color": ([V, C.c_uint32, C.c_char_p, P(C.c_float), P(C.c_int)], C.c_int),
        "sprout_sim_render": ([V, C.c_float], C.c_int),
        "sprout_sim_draw": ([V, C.c_float, C.c_float, C.c_float, C.c_uint32, C.c_uint32], C.c_int),
        "sprout_sim_download_draw": ([V, C.c_int, V, C.c_size_t, P(C.c_uint32)], C.c_int),
        "sprout_sim_flow_parity": ([V, P(C.c_uint32)], C.c_int),
        "sprout_sim_recorded_iters": ([V, P(C.c_uint32)], C.c_int),
        "sprout_sim_download_look": ([V, V, C.c_size_t, V, C.c_size_t, P(C.c_uint32), P(C.c_uint32)], C.c_int),
        "sprout_sim_download_spray": ([V, V, C.c_size_t, V, V, V, C.c_size_t, V, C.c_size_t, P(C.c_uint32)], C.c_int),
        "sprout_params_get_color": ([V, C.c_uint32, C.c_char_p, P(C.c_float), P(C.c_int)], C.c_int),
        "sprout_params_get_row": ([V, C.c_uint32, P(C.c_int32), P(C.c_int32)], C.c_int),
        "sprout_sim_download_render": ([V, C.c_int, V, C.c_size_t, P(C.c_size_t)], C.c_int),
        "sprout_sim_download_particles": ([V, V, C.c_uint32, P(C.c_uint32)], C.c_int),
        "sprout_sim_download_pressure": ([V, V], C.c_int),
        "sprout_sim_download_field": ([V, C.c_char_p, V, C.c_size_t, P(C.c_size_t)], C.c_int),
        "sprout_sim_stats": ([V, P(SolverStats)], C.c_int),
        "sprout_sim_device_bytes": ([V, P(C.c_size_t)], C.c_int),
        "sprout_sim_profile": ([V, C.c_uint32, P(C.c_float)], C.c_int),
        "sprout_sim_profile_passes": ([V, P(C.c_float), C.c_uint32], C.c_int),
        "sprout_sim_set_precision": ([V, C.c_int], C.c_int),
        "sprout_batch_create": ([P(V)], C.c_int),
        "sprout_batch_destroy": ([V], C.c_int),
        "sprout_batch_add": ([V, V], C.c_int),
        "sprout_batch_remove": ([V, V], C.c_int),
        "sprout_batch_size": ([V, P(C.c_uint32)], C.c_int),
        "sprout_batch_set_precision": ([V, C.c_int], C.c_int),
        "sprout_batch_step": ([V, C.c_uint32], C.c_int),
        "sprout_batch_sync": ([V], C.c_int),
        "sprout_batch_profile": ([V, C.c_uint32, P(C.c_float)], C.c_int),
        "sprout_batch_step_subset": ([V, P(C.c_uint32), C.c_uint32], C.c_int),
        "sprout_batch_tickets": ([V, P(C.c_uint64), P(C.c_uint64)], C.c_int),
        "sprout_device_memory": ([P(C.c_size_t), P(C.c_size_t)], C.c_int),
        "sprout_sim_trace_enable": ([V, C.c_uint32], C.c_int),
        "sprout_sim_trace_read": ([V, V, C.c_size_t, P(C.c_size_t), P(C.c_uint32)], C.c_int),
        "sprout_device_count": ([P(C.c_int)], C.c_int), "sprout_set_device": ([C.c_int], C.c_int),
        "sprout_get_device": ([P(C.c_int)], C.c_int),
        "sprout_pacer_new": ([P(V)], C.c_int), "sprout_pacer_free": ([V], C.c_int),
        "sprout_pacer_reset": ([V], C.c_int), "sprout_pacer_speed": ([V, P(C.c_float)], C.c_int),
        "sprout_pacer_plan": ([V, C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_float, P(Plan)], C.c_int),
        "sprout_sim_request_stats": ([V], C.c_int),
        "sprout_sim_poll_stats": ([V, P(Census), P(C.c_int)], C.c_int),
        "sprout_sim_set_launch": ([V, P(Launch)], C.c_int),
        "sprout_sim_get_launch": ([V, P(Launch)], C.c_int),
        "sprout_sim_debug_stall": ([V, C.c_uint32, C.c_uint32, C.c_uint32], C.c_int),
        "sprout_batch_set_launch": ([V, P(Launch)], C.c_int),
        "sprout_pressure_solve_static": ([C.c_uint32, C.c_uint32, V, V, V, V, C.c_float, C.c_float, C.c_uint32, V,
                                          P(C.c_uint32), P(C.c_float)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(rc: int):
    if rc != SPROUT_OK:
        raise SproutError(rc, lib().sprout_last_error().decode())


CURRENT_DTYPE = np.dtype([("pos", "<f4", 2), ("radius", "<f4"), ("vel", "<f4", 2), ("rate", "<f4")])


def current_array(currents) -> np.ndarray:
    """Current records (src/sim/params.rs:1113-1121) from dicts with pos, radius, vel, rate."""
    arr = np.zeros(len(currents), CURRENT_DTYPE)
    for k, c in enumerate(currents):
        arr[k]["pos"] = c["pos"]
        arr[k]["radius"] = c["radius"]
        arr[k]["vel"] = c.get("vel", (0.0, 0.0))
        arr[k]["rate"] = c["rate"]
    return arr


MAGNET_DTYPE = np.dtype([("pos", "<f4", 2), ("radius", "<f4"), ("strength", "<f4"), ("dir", "<f4", 2)])


def magnet_array(magnets) -> np.ndarray:
    """Magnet records (src/sim/params.rs:1082-1087) from dicts with pos, radius, strength, dir."""
    arr = np.zeros(len(magnets), MAGNET_DTYPE)
    for k, m in enumerate(magnets):
        arr[k]["pos"] = m["pos"]
        arr[k]["radius"] = m["radius"]
        arr[k]["strength"] = m["strength"]
        arr[k]["dir"] = m.get("dir", (0.0, 1.0))
    return arr


class SimParams:
    """SimParams (src/sim/params.rs:149-451) behind the engine's table of names."""

    def __init__(self, settings: dict | None = None):
        self._h = C.c_void_p()
        _check(lib().sprout_params_new(C.byref(self._h)))
        for k, v in (settings or {}).items():
            if not self.set(k, v):
                raise KeyError(f"unknown parameter {k!r}")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().sprout_params_free(self._h)
            self._h = None

    def set(self, key: str, value: float) -> bool:
        """SimParams::set: False for an unknown name or NaN; clamps to the range."""
        ok = C.c_int()
        _check(lib().sprout_params_set(self._h, key.encode(), float(value), C.byref(ok)))
        return bool(ok.value)

    def set_diluent(self, row: int, diluent: int) -> bool:
        """A custom liquid's diluent as the library's loader resolves it (library.rs:318-330):
        False for a built-in row or a diluent the loader would drop."""
        ok = C.c_int()
        _check(lib().sprout_params_set_diluent(self._h, int(row), int(diluent), C.byref(ok)))
        return bool(ok.value)

    def set_color(self, row: int, field: str, rgb) -> bool:
        """A colour of a material row (color, color_solid, color_hot, cloud_color, dust_color,
        glow_color; sRGB 0..1), as a custom liquid's library entry gives it."""
        ok = C.c_int()
        _check(lib().sprout_params_set_color(self._h, int(row), field.encode(), (C.c_float * 3)(*rgb), C.byref(ok)))
        return bool(ok.value)

    def get_color(self, row: int, field: str) -> tuple:
        rgb, ok = (C.c_float * 3)(), C.c_int()
        _check(lib().sprout_params_get_color(self._h, int(row), field.encode(), rgb, C.byref(ok)))
        if not ok.value:
            raise KeyError(field)
        return tuple(rgb)

    def row_kind(self, row: int) -> tuple[int, int]:
        """(phase group, diluent row or -1) of a material row."""
        g, dil = C.c_int32(), C.c_int32()
        _check(lib().sprout_params_get_row(self._h, int(row), C.byref(g), C.byref(dil)))
        return g.value, dil.value

    def optics_table(self, rows: int = 96) -> np.ndarray:
        """material.rs optics_table: one OPTICS_DTYPE row per material row."""
        out = np.zeros(rows, OPTICS_DTYPE)
        _check(lib().sprout_params_optics(self._h, out.ctypes.data, rows))
        return out

    def set_group(self, row: int, group: int) -> bool:
        """A custom liquid's phase group as the library's loader reads it (library.rs:283-286):
        0 aqueous, 1 oil-like, 2 metal, 3 silicate; False for a built-in row."""
        ok = C.c_int()
        _check(lib().sprout_params_set_group(self._h, int(row), int(group), C.byref(ok)))
        return bool(ok.value)

    def get(self, key: str) -> float:
        v, ok = C.c_float(), C.c_int()
        _check(lib().sprout_params_get(self._h, key.encode(), C.byref(v), C.byref(ok)))
        if not ok.value:
            raise KeyError(key)
        return v.value


class Scene:
    """Scene (src/scene.rs): box walls plus boxes and circles, optionally held at a temperature."""

    def __init__(self, w: int, h: int):
        self.w, self.h = w, h
        self._h = C.c_void_p()
        _check(lib().sprout_scene_new(w, h, C.byref(self._h)))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().sprout_scene_free(self._h)
            self._h = None

    def add_box(self, c, half, angle: float = 0.0, temp: float | None = None):
        _check(lib().sprout_scene_add_box(self._h, c[0], c[1], half[0], half[1], angle, math.nan if temp is None else temp))

    def add_circle(self, c, r: float, temp: float | None = None):
        _check(lib().sprout_scene_add_circle(self._h, c[0], c[1], r, math.nan if temp is None else temp))

    def sdf(self, x: float, y: float) -> float:
        d = C.c_float()
        _check(lib().sprout_scene_sdf(self._h, x, y, C.byref(d)))
        return d.value

    def rasterize(self, device: bool = False):
        """(sdf, solid[n,4], region, temp or None), as Scene::rasterize fills SolidField;
        with `device` computed on the current CUDA device (the same fields, bit for bit)."""
        w, h = self.w, self.h
        sdf = np.zeros((h + 1) * (w + 1), np.float32)
        solid = np.zeros((h * w, 4), np.float32)
        region = np.zeros(h * w, np.uint32)
        temp = np.zeros(h * w, np.float32)
        heated = C.c_int()
        fn = lib().sprout_scene_rasterize_device if device else lib().sprout_scene_rasterize
        _check(fn(self._h, sdf.ctypes.data, solid.ctypes.data, region.ctypes.data, temp.ctypes.data, C.byref(heated)))
        return sdf, solid, region, (temp if heated.value else None)

    def fill_rect(self, rect, material: int, existing: np.ndarray | None = None) -> np.ndarray:
        """maps::fill_rect: appends rest-density particles of `material` in rect to `existing`."""
        n0 = 0 if existing is None else len(existing)
        r = (C.c_float * 4)(*rect)
        n = C.c_uint32()
        _check(lib().sprout_fill_rect(self._h, r, material, n0, None, 0, C.byref(n)))
        out = np.zeros(n0 + n.value, PARTICLE_DTYPE)
        if existing is not None:
            out[:n0] = existing
        _check(lib().sprout_fill_rect(self._h, r, material, n0, out[n0:].ctypes.data, n.value, C.byref(n)))
        return out


class FluidSim:
    """FluidSim (src/sim/mod.rs:862-) on the current CUDA device."""

    def __init__(self, w: int, h: int, capacity: int, params: SimParams):
        self.w, self.h = w, h
        self._h = C.c_void_p()
        _check(lib().sprout_sim_create(w, h, capacity, params._h, C.byref(self._h)))

    def close(self):
        if getattr(self, "_h", None):
            lib().sprout_sim_destroy(self._h)
            self._h = None

    __del__ = close

    def set_params(self, params: SimParams):
        _check(lib().sprout_sim_set_params(self._h, params._h))

    def set_solids(self, sdf, solid, region, temp=None):
        a = np.ascontiguousarray(sdf, np.float32)
        b = np.ascontiguousarray(solid, np.float32)
        c = np.ascontiguousarray(region, np.uint32)
        d = None if temp is None else np.ascontiguousarray(temp, np.float32)
        _check(lib().sprout_sim_set_solids(self._h, a.ctypes.data, b.ctypes.data, c.ctypes.data,
                                           None if d is None else d.ctypes.data))

    def set_scene(self, scene: "Scene"):
        """set_solids with the scene rasterised on the device, straight into the sim's buffers."""
        _check(lib().sprout_sim_set_scene(self._h, scene._h))

    def reset(self, particles: np.ndarray):
        p = np.ascontiguousarray(particles, PARTICLE_DTYPE)
        _check(lib().sprout_sim_reset(self._h, p.ctypes.data, len(p)))

    def frame_blocking(self, substeps: int, target: float, tool: "Tool | None" = None) -> float:
        """FluidSim::frame_blocking: steps and waits; the simulated seconds covered."""
        adv = C.c_double()
        _check(lib().sprout_sim_frame_blocking(self._h, substeps, float(target), None if tool is None else C.byref(tool), C.byref(adv)))
        return adv.value

    def dt_estimate(self) -> float:
        """FluidSim::dt_estimate: the substep length the next step will most likely take, s."""
        dt = C.c_float()
        _check(lib().sprout_sim_dt_estimate(self._h, C.byref(dt)))
        return dt.value

    def set_magnets(self, magnets):
        """FluidSim::set_magnets: dipoles {pos, radius, strength, dir} (cells, T); the first 8
        are kept, across resets."""
        arr = magnet_array(magnets)
        _check(lib().sprout_sim_set_magnets(self._h, arr.ctypes.data if len(arr) else None, len(arr)))

    def set_currents(self, currents):
        """FluidSim::set_currents: zones {pos, radius, vel, rate} (cells, cells / s, 1 / s; a
        negative rate drains); the first 16 are kept, across resets."""
        arr = current_array(currents)
        _check(lib().sprout_sim_set_currents(self._h, arr.ctypes.data if len(arr) else None, len(arr)))

    def spawn(self, particles: np.ndarray) -> int:
        """FluidSim::spawn: queues particles for the next step; returns how many were taken
        (0 when their materials do not fit the tank)."""
        p = np.ascontiguousarray(particles, PARTICLE_DTYPE)
        n = C.c_uint32()
        _check(lib().sprout_sim_spawn(self._h, p.ctypes.data if len(p) else None, len(p), C.byref(n)))
        return n.value

    def cell_counts(self, lo, hi) -> np.ndarray:
        """FluidSim::cell_counts: live particles per cell of the window [lo, hi), queued ones
        included, as an array of (rows, columns)."""
        a, b = (C.c_int32 * 2)(*lo), (C.c_int32 * 2)(*hi)
        n = C.c_size_t()
        _check(lib().sprout_sim_cell_counts(self._h, a, b, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.uint32)
        if n.value:
            _check(lib().sprout_sim_cell_counts(self._h, a, b, out.ctypes.data, n.value, C.byref(n)))
        return out.reshape(max(hi[1] - lo[1], 0), max(hi[0] - lo[0], 0))

    # ---- the render side's cell passes (record_cell_optics without a window) --------------
    def render(self, inv_speed: float = 1.0 / 60.0):
        """record_cell_optics on the device (no wait): cell_optics.comp, light.comp,
        optics_blur.comp, sss.comp, flow_map.comp and glow.comp; nothing when nothing changed
        since the last call."""
        _check(lib().sprout_sim_render(self._h, inv_speed))

    def recorded_iters(self) -> list:
        """FluidSim::recorded_iters: [first pressure solve, second, viscosity] (blocking)."""
        v = (C.c_uint32 * 3)()
        _check(lib().sprout_sim_recorded_iters(self._h, v))
        return [int(x) for x in v]

    def download_spray(self):
        """spray.comp's pool: (entries (196608, DIFFUSE_DTYPE), bubbles' free stack, specks'
        free stack, listed entries, counts (4, h, w): foam x 2, resting specks x 2, state (8))."""
        st = (C.c_uint32 * 8)()
        pool = np.zeros(POOL_MAX, DIFFUSE_DTYPE)
        stack, stack1, lst = (np.zeros(POOL_MAX, np.uint32) for _ in range(3))
        counts = np.zeros(4 * self.w * self.h, np.uint32)
        _check(lib().sprout_sim_download_spray(self._h, pool.ctypes.data, POOL_MAX, stack.ctypes.data, stack1.ctypes.data,
                                               lst.ctypes.data, POOL_MAX, counts.ctypes.data, counts.size, st))
        s = [int(x) for x in st]
        return pool, stack[: s[1]], stack1[: s[5]], lst[: s[2]], counts.reshape(4, self.h, self.w), s

    def download_look(self):
        """look.comp's state: (per slot (id, 0, packed A, 0) as uint32 (n, 4), the listed slots)."""
        n, m = C.c_uint32(), C.c_uint32()
        _check(lib().sprout_sim_download_look(self._h, None, 0, None, 0, C.byref(n), C.byref(m)))
        st = np.zeros((n.value, 4), np.uint32)
        ls = np.zeros(max(m.value, 1), np.uint32)
        _check(lib().sprout_sim_download_look(self._h, st.ctypes.data, st.size, ls.ctypes.data, ls.size,
                                              C.byref(n), C.byref(m)))
        return st, ls[: m.value]

    def flow_parity(self) -> int:
        """The copy of the flow map that holds it now (blocking)."""
        v = C.c_uint32()
        _check(lib().sprout_sim_flow_parity(self._h, C.byref(v)))
        return int(v.value)

    def download_render(self, which: str = "smoothed") -> np.ndarray:
        """The layers as float16: "raw" (20, h, w, 4), "smoothed" (24, h, w, 4), "glow"
        (ceil(h / 2), ceil(w / 2), 4) or "flow" (4, h, w, 4)."""
        k = {"raw": 0, "smoothed": 1, "glow": 2, "flow": 3}[which]
        n = C.c_size_t()
        _check(lib().sprout_sim_download_render(self._h, k, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.uint16)
        _check(lib().sprout_sim_download_render(self._h, k, out.ctypes.data, n.value, C.byref(n)))
        shape = {0: (RENDER_LAYERS, self.h, self.w, 4), 1: (24, self.h, self.w, 4),
                 2: ((self.h + 1) // 2, (self.w + 1) // 2, 4), 3: (4, self.h, self.w, 4)}[k]
        return out.view(np.float16).reshape(shape)

    def draw(self, center, zoom: float, size):
        """Renderer::render's particle fields for a view of size = (width, height) pixels centred
        on `center` (cells) at `zoom` pixels per cell, and the wet map (no wait)."""
        _check(lib().sprout_sim_draw(self._h, float(center[0]), float(center[1]), float(zoom), int(size[0]), int(size[1])))

    def download_draw(self, which: str = "sharp") -> np.ndarray:
        """An image of the last draw: "sharp", "tint", "share", "wide" or "look" as (h, w, 4)
        float16, "wet" as (H, W, 4) float32; None when it was never drawn."""
        k = {"sharp": 0, "tint": 1, "share": 2, "wide": 3, "wet": 4, "look": 5}[which]
        dims = (C.c_uint32 * 2)()
        _check(lib().sprout_sim_download_draw(self._h, k, None, 0, dims))
        w, h = int(dims[0]), int(dims[1])
        if w == 0:
            return None
        out = np.zeros((h, w, 4), np.float32 if k == 4 else np.float16)
        _check(lib().sprout_sim_download_draw(self._h, k, out.ctypes.data, out.nbytes, dims))
        return out

    # ---- the brush's emitters on the device (World::emit without a read-back) -------------
    def emit_stream(self, spout: "Spout", stream: "StreamState", frm, to, seconds: float, material: int):
        """World::stream: the frame's particles of the spout's stream, admitted on the device."""
        t = C.c_double(stream.time)
        _check(lib().sprout_sim_emit_stream(self._h, C.byref(spout), C.byref(t), (C.c_float * 2)(*frm),
                                            (C.c_float * 2)(*to), seconds, material))
        stream.time = t.value

    def emit_paint(self, frm, to, radius: float, count: int, spray: bool, material: int):
        """World::paint (stamp: frm == to, count 32768; spray: the sparse launched lattice)."""
        _check(lib().sprout_sim_emit_paint(self._h, (C.c_float * 2)(*frm), (C.c_float * 2)(*to), radius, count,
                                           1 if spray else 0, material))

    def emit_rain(self, at, radius: float, count: int, material: int):
        """World::rain: `count` drops from the cloud around `at`."""
        _check(lib().sprout_sim_emit_rain(self._h, (C.c_float * 2)(*at), radius, count, material))

    def emitter_seed(self, rng: int):
        _check(lib().sprout_sim_emitter_seed(self._h, rng & 0xFFFFFFFF))

    def emitted(self) -> tuple[int, int]:
        """(particles the emitters have queued in all, in the last emission); blocking."""
        t, last = C.c_uint64(), C.c_uint32()
        _check(lib().sprout_sim_emitted(self._h, C.byref(t), C.byref(last)))
        return t.value, last.value

    def step(self, substeps: int, target: float = 0.0, tool: Tool | None = None):
        _check(lib().sprout_sim_step(self._h, substeps, target, None if tool is None else C.byref(tool)))

    def step_blocking(self, substeps: int, tool: Tool | None = None):
        _check(lib().sprout_sim_step_blocking(self._h, substeps, None if tool is None else C.byref(tool)))

    def advance_blocking(self, seconds: float, tool: Tool | None = None):
        _check(lib().sprout_sim_advance_blocking(self._h, seconds, None if tool is None else C.byref(tool)))

    def sync(self):
        _check(lib().sprout_sim_sync(self._h))

    def download_particles(self) -> np.ndarray:
        n = C.c_uint32()
        _check(lib().sprout_sim_download_particles(self._h, None, 0, C.byref(n)))
        out = np.zeros(n.value, PARTICLE_DTYPE)
        _check(lib().sprout_sim_download_particles(self._h, out.ctypes.data, n.value, C.byref(n)))
        return out

    def download_pressure(self) -> np.ndarray:
        out = np.zeros((self.h * self.w, 2), np.float32)
        _check(lib().sprout_sim_download_pressure(self._h, out.ctypes.data))
        return out

    def field(self, name: str, dtype=np.float32) -> np.ndarray:
        b = C.c_size_t()
        _check(lib().sprout_sim_download_field(self._h, name.encode(), None, 0, C.byref(b)))
        out = np.zeros(b.value // np.dtype(dtype).itemsize, dtype)
        _check(lib().sprout_sim_download_field(self._h, name.encode(), out.ctypes.data, b.value, C.byref(b)))
        return out

    def stats(self) -> SolverStats:
        s = SolverStats()
        _check(lib().sprout_sim_stats(self._h, C.byref(s)))
        return s

    def profile(self, substeps: int) -> float:
        """Device ms of `substeps` more substeps (CUDA events on the sim's stream)."""
        ms = C.c_float()
        _check(lib().sprout_sim_profile(self._h, substeps, C.byref(ms)))
        return ms.value

    def set_precision(self, mode: str | int):
        """The pressure solve's precision: "plain" (0, FP32 as the reference) or "mixed" (1:
        BF16 matrices, FP32 dot products with FP64 totals, step lengths and convergence test, the
        true residual at the end as float pairs)."""
        m = {"plain": 0, "mixed": 1}.get(mode, mode)
        _check(lib().sprout_sim_set_precision(self._h, int(m)))

    def trace_on(self, rows: int = 4096):
        """Turns the solvers' phase trace on (rows: barrier generations kept; 0: off)."""
        _check(lib().sprout_sim_trace_enable(self._h, rows))

    def trace(self) -> np.ndarray:
        """The phase trace so far: (rows, blocks + 1) device ns, 0 where never written."""
        w, c = C.c_size_t(), C.c_uint32()
        _check(lib().sprout_sim_trace_read(self._h, None, 0, C.byref(w), C.byref(c)))
        out = np.zeros(w.value, np.uint64)
        if w.value:
            _check(lib().sprout_sim_trace_read(self._h, out.ctypes.data, w.value, C.byref(w), C.byref(c)))
        return out.reshape(-1, max(c.value, 1))

    def profile_passes(self) -> dict:
        """One substep stage by stage: device ms per stage (STAGES)."""
        ms = (C.c_float * len(STAGES))()
        _check(lib().sprout_sim_profile_passes(self._h, ms, len(STAGES)))
        return dict(zip(STAGES, list(ms)))

    def device_bytes(self) -> int:
        b = C.c_size_t()
        _check(lib().sprout_sim_device_bytes(self._h, C.byref(b)))
        return b.value

    def request_stats(self):
        """FluidSim::request_stats: records the census of the particles (asynchronous)."""
        _check(lib().sprout_sim_request_stats(self._h))

    def poll_stats(self) -> "Census | None":
        """FluidSim::poll_stats: the census once the device has finished it, else None."""
        out, ready = Census(), C.c_int()
        _check(lib().sprout_sim_poll_stats(self._h, C.byref(out), C.byref(ready)))
        return out if ready.value else None

    def set_launch(self, pressure_blocks: int = 0, pressure_blocks_mixed: int = 0, viscosity_blocks: int = 0):
        """Block counts of the persistent pressure and viscosity solves (0: the default, one
        block per tile up to what the device holds). Results do not depend on them."""
        lc = Launch(pressure_blocks, pressure_blocks_mixed, viscosity_blocks, 0)
        _check(lib().sprout_sim_set_launch(self._h, C.byref(lc)))

    def launch(self) -> dict:
        """The block counts in effect."""
        lc = Launch()
        _check(lib().sprout_sim_get_launch(self._h, C.byref(lc)))
        return lc.as_dict()

    def debug_stall(self, block: int, stall_ns: int, spin_limit: int):
        """Failure injection for tests: block `block` of later persistent solves arrives
        stall_ns late at each grid barrier and waits give up after spin_limit polls."""
        _check(lib().sprout_sim_debug_stall(self._h, block, stall_ns, spin_limit))


class Pacer:
    """Pacer (src/pacing.rs): plans each frame's substeps from the frame length, the step
    length and the measured device cost of a substep."""

    def __init__(self):
        self._h = C.c_void_p()
        _check(lib().sprout_pacer_new(C.byref(self._h)))

    def close(self):
        if getattr(self, "_h", None):
            lib().sprout_pacer_free(self._h)
            self._h = None

    __del__ = close

    def plan(self, frame_dt: float, dt: float, fixed: bool, time_scale: float, cost: float, budget: float) -> Plan:
        out = Plan()
        _check(lib().sprout_pacer_plan(self._h, frame_dt, dt, int(fixed), time_scale, cost, budget, C.byref(out)))
        return out

    def reset(self):
        _check(lib().sprout_pacer_reset(self._h))

    def speed(self) -> float:
        v = C.c_float()
        _check(lib().sprout_pacer_speed(self._h, C.byref(v)))
        return v.value


def pressure_solve_static(w: int, h: int, mga_ptr: int, mgd_ptr: int, rhs_ptr: int, x_ptr: int, tol_p: float,
                          tol_psi: float, max_iters: int = 60, stream: int | None = None):
    """The pressure solve on a system held on the device, using no allocation (device pointers
    in; see sprout_pressure_solve_static in include/sprout_gpu.h). Returns (iterations, |r|/|b|)."""
    iters = (C.c_uint32 * 2)()
    res = C.c_float()
    _check(lib().sprout_pressure_solve_static(w, h, mga_ptr, mgd_ptr, rhs_ptr, x_ptr, tol_p, tol_psi, max_iters, stream,
                                              iters, C.byref(res)))
    return list(iters), res.value


class Batch:
    """Many FluidSims advanced together: one CUDA graph per substep, their pressure solves
    in one persistent kernel (sprout_batch_*). Each tank's results equal stepping it alone."""

    def __init__(self, sims=(), precision: str | int = "plain"):
        self._h = C.c_void_p()
        _check(lib().sprout_batch_create(C.byref(self._h)))
        self.sims = []
        self.set_precision(precision)
        for s in sims:
            self.add(s)

    def close(self):
        if getattr(self, "_h", None):
            lib().sprout_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def add(self, sim: FluidSim):
        _check(lib().sprout_batch_add(self._h, sim._h))
        self.sims.append(sim)

    def remove(self, sim: FluidSim):
        _check(lib().sprout_batch_remove(self._h, sim._h))
        self.sims.remove(sim)

    def set_precision(self, mode: str | int):
        m = {"plain": 0, "mixed": 1}.get(mode, mode)
        _check(lib().sprout_batch_set_precision(self._h, int(m)))

    def step(self, substeps: int = 1):
        _check(lib().sprout_batch_step(self._h, substeps))

    def step_subset(self, members):
        """One substep of the members at these indices only (continuous batching)."""
        idx = (C.c_uint32 * len(members))(*members)
        _check(lib().sprout_batch_step_subset(self._h, idx, len(members)))

    def tickets(self):
        """(issued, completed): step calls so far and how many have finished on the device."""
        a, b = C.c_uint64(), C.c_uint64()
        _check(lib().sprout_batch_tickets(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def sync(self):
        _check(lib().sprout_batch_sync(self._h))

    def profile(self, substeps: int) -> float:
        ms = C.c_float()
        _check(lib().sprout_batch_profile(self._h, substeps, C.byref(ms)))
        return ms.value

    def set_launch(self, pressure_blocks: int = 0, pressure_blocks_mixed: int = 0, viscosity_blocks: int = 0,
                   batch_viscosity: int = 0):
        """Block counts of the batch's persistent solves (0: defaults); batch_viscosity 0 the
        default, 1 always one batched viscosity solve, 2 one solve per tank."""
        lc = Launch(pressure_blocks, pressure_blocks_mixed, viscosity_blocks, batch_viscosity)
        _check(lib().sprout_batch_set_launch(self._h, C.byref(lc)))


def set_device(device: int):
    """Sims and batches created on this thread from now on live on `device`."""
    _check(lib().sprout_set_device(device))


def device_count() -> int:
    n = C.c_int()
    _check(lib().sprout_device_count(C.byref(n)))
    return n.value


def device_memory():
    """(free, total) bytes of the current device."""
    a, b = C.c_size_t(), C.c_size_t()
    _check(lib().sprout_device_memory(C.byref(a), C.byref(b)))
    return a.value, b.value

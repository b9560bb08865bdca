"""CPU restatement of the optics table (src/sim/material.rs:600-980: optics_table and the
helpers it calls), in the reference's single-precision arithmetic.

Test infrastructure: the checker of the engine's table (optics.cpp, read through
sprout_params_optics). It takes a material row's inputs from the engine's parameter set
(SimParams::get, the colours and the row's group and diluent) and recomputes the row:
numpy float32 for the arithmetic, the platform's libm (powf, logf, log10f, expf, sinf, cosf,
cbrtf) where material.rs calls f32 methods, so both round the same way.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import math

import numpy as np

f32 = np.float32
_m = ctypes.CDLL(ctypes.util.find_library("m"))
for _n, _k in (("powf", 2), ("logf", 1), ("log10f", 1), ("expf", 1), ("sinf", 1), ("cosf", 1), ("cbrtf", 1)):
    getattr(_m, _n).restype = ctypes.c_float
    getattr(_m, _n).argtypes = [ctypes.c_float] * _k


def powf(x, y): return f32(_m.powf(float(x), float(y)))
def logf(x): return f32(_m.logf(float(x)))
def log10f(x): return f32(_m.log10f(float(x)))
def expf(x): return f32(_m.expf(float(x)))
def sinf(x): return f32(_m.sinf(float(x)))
def cosf(x): return f32(_m.cosf(float(x)))
def cbrtf(x): return f32(_m.cbrtf(float(x)))
def sqrtf(x): return f32(np.sqrt(f32(x)))
def clamp(v, lo, hi): return min(max(f32(v), f32(lo)), f32(hi))


PI = f32(math.pi)
WAVELENGTHS = (f32(610.0e-9), f32(550.0e-9), f32(465.0e-9))
LV_BODY, DUST_DRAW_MAX, DUST_PACKING, FOAM_DRAIN_WATER = f32(16.0), f32(4.0), f32(0.6), f32(0.02)
KT = f32(f32(1.380649e-23) * f32(293.15))
MAX_COEFFICIENT = f32(2000.0)
FILM_UNIT, EVAP_WATER, COAT_SPEED = f32(1.0e-4), f32(1.0e-7), f32(0.05)
TWO_THIRDS = f32(f32(2.0) / f32(3.0))
RADS_PER_DEG = f32(PI / f32(180.0))
T_REF = f32(20.0)

FIELDS = ["density", "viscosity", "tension", "contact_angle", "melt_lo", "melt_hi", "emissivity", "boil", "opacity",
          "metal", "gloss", "foam", "volatility", "froth", "fizz", "luminous", "glow_shear", "thermo_lo", "thermo_hi",
          "solids", "cloud", "cloud_size", "cloud_ior", "cloud_shape", "dust", "dust_size", "dust_density",
          "dust_shape", "dust_reflect", "ior"]
COLOURS = ["color", "color_solid", "color_hot", "cloud_color", "dust_color", "glow_color"]


class Mat:
    """The inputs of one material row."""

    def __init__(self, params, row: int):
        for f in FIELDS:
            setattr(self, f, f32(params.get(f"mat{row}.{f}")))
        for c in COLOURS:
            setattr(self, c, tuple(f32(v) for v in params.get_color(row, c)))
        self.group, self.diluent = params.row_kind(row)

    def freezes(self) -> bool:
        return self.melt_hi > f32(-273.0)


def linear(c):
    return tuple(f32(v / f32(12.92)) if v <= f32(0.04045) else powf(f32(f32(v + f32(0.055)) / f32(1.055)), f32(2.4))
                 for v in c)


def tint_depth(m):
    clear = f32(f32(1.0) - clamp(m.opacity, 0.0, 1.0))
    return f32(f32(0.5) + f32(f32(f32(30.0) * clear) * clear))


def particle_shape(d, r):
    d = max(f32(d), f32(1e-9))
    if r >= TWO_THIRDS:
        return f32(f32(1.5) / d), d, d
    t = f32(d * max(f32(r), f32(0.005)))
    half = f32(f32(0.5) * d)
    return (f32(f32(half + t) / f32(d * t)), f32(f32(f32(f32(1.5) * d) * t) / f32(half + t)),
            f32(d * cbrtf(f32(f32(1.5) * max(f32(r), f32(0.005))))))


def scattering_efficiency(x_vol, x_path, m):
    m = max(f32(m), f32(1e-3))
    mm = f32(m * m)
    k = f32(f32(mm - f32(1.0)) / f32(mm + f32(2.0)))
    x2 = f32(x_vol * x_vol)
    qr = f32(f32(f32(f32(f32(8.0) / f32(3.0)) * f32(x2 * x2)) * k) * k)
    rho = f32(f32(f32(2.0) * x_path) * f32(abs(f32(m - f32(1.0)))))
    if rho < f32(1e-2):
        qa = f32(f32(f32(0.5) * rho) * rho)
    else:
        qa = f32(f32(f32(2.0) - f32(f32(f32(4.0) / rho) * sinf(rho))) +
                 f32(f32(f32(4.0) / f32(rho * rho)) * f32(f32(1.0) - cosf(rho))))
    if qr <= 0.0 or qa <= 0.0:
        return f32(0.0)
    return f32(f32(1.0) / f32(f32(f32(1.0) / qr) + f32(f32(1.0) / qa)))


def asymmetry(x, m):
    large = clamp(f32(f32(1.0) - f32(f32(0.6) * f32(abs(f32(m - f32(1.0)))))), 0.3, 0.98)
    return f32(f32(f32(large * x) * x) / f32(f32(x * x) + f32(2.5)))


def albedo_of(color):
    out = []
    for r in linear(color):
        r = clamp(r, 1e-3, 0.995)
        q = f32(f32(f32(1.0) - r) / f32(f32(1.0) + r))
        out.append(max(f32(f32(1.0) - f32(q * q)), f32(1e-4)))
    return out


def cloud_scattering(m, cell):
    if m.cloud <= 0.0:
        return [f32(0.0)] * 3, f32(0.0)
    a_v, chord, d_eq = particle_shape(m.cloud_size, m.cloud_shape)
    n_med = max(m.ior, f32(1.0))
    rel = f32(m.cloud_ior / n_med)
    s, g_sum = [], f32(0.0)
    for c in range(3):
        k = f32(f32(PI * n_med) / WAVELENGTHS[c])
        q = scattering_efficiency(f32(k * d_eq), f32(k * chord), rel)
        g = asymmetry(f32(k * d_eq), rel)
        g_sum = f32(g_sum + g)
        s.append(f32(f32(f32(f32(clamp(m.cloud, 0.0, 0.74) * a_v) * q) * f32(f32(1.0) - g)) * f32(cell)))
    return s, f32(g_sum / f32(3.0))


def coefficients(m, color, cell):
    depth = tint_depth(m)
    lin = [clamp(v, 1e-3, 0.995) for v in linear(color)]
    s, _ = cloud_scattering(m, cell)
    w = albedo_of(m.cloud_color)
    a = [f32(f32(f32(-logf(lin[c])) / depth) + f32(f32(s[c] * f32(f32(1.0) - w[c])) / w[c])) for c in range(3)]
    sc = list(s)
    if m.metal > 0.0:
        wm = albedo_of(color)
        k = clamp(m.metal, 0.0, 1.0)
        for c in range(3):
            sm = f32(6.0)
            a[c] = f32(a[c] + f32(k * f32(f32(f32(sm * f32(f32(1.0) - wm[c])) / wm[c]) - a[c])))
            sc[c] = f32(sc[c] + f32(k * f32(sm - sc[c])))
    return [min(v, MAX_COEFFICIENT) for v in a], [min(v, MAX_COEFFICIENT) for v in sc]


def packed(a, s):
    return [a[0], a[1], a[2], f32(f32(f32(s[0] + s[1]) + s[2]) / f32(3.0))]


def fullness(m):
    def ss(x, lo, hi):
        t = clamp(f32(f32(x - f32(lo)) / f32(f32(hi) - f32(lo))), 0.0, 1.0)
        return f32(f32(t * t) * f32(f32(3.0) - f32(f32(2.0) * t)))
    return max(ss(log10f(max(m.viscosity, f32(1e-9))), -5.3, -2.7), ss(m.contact_angle, 100.0, 145.0))


def volatile_share(m):
    if m.boil >= f32(1.0e8) and m.volatility <= 0.0:
        return f32(0.0)
    return clamp(f32(f32(f32(f32(1.0) - m.solids) - m.cloud) - m.dust), 0.0, 1.0)


def vapour_pressure(boil, t):
    if boil >= f32(1.0e8):
        return f32(0.0)
    tb = f32(boil + f32(273.15))
    tk = max(f32(f32(t) + f32(273.15)), f32(1.0))
    return expf(clamp(f32(f32(10.6) * f32(f32(1.0) - f32(tb / tk))), -60.0, 5.0))


def evaporation(m, t, speed):
    rel = f32(vapour_pressure(m.boil, t) / max(vapour_pressure(f32(100.0), T_REF), f32(1e-12)))
    vol = f32(m.volatility * f32(50.0)) if (m.boil >= f32(1.0e8) and m.volatility > 0.0) else rel
    return f32(f32(f32(EVAP_WATER * vol) * f32(speed)) / FILM_UNIT)


def freezes_on_contact(m):
    return m.freezes() and m.melt_lo > f32(300.0)


def wetting(m):
    if freezes_on_contact(m):
        return f32(0.0)
    w = f32(f32(0.5) * f32(f32(1.0) + cosf(f32(m.contact_angle * RADS_PER_DEG))))
    return clamp(f32(f32(w - f32(0.15)) / f32(0.85)), 0.0, 1.0)


def coat_thickness(m, gravity):
    if freezes_on_contact(m):
        return f32(0.0)
    sigma = max(m.tension, f32(1e-3))
    rho = max(m.density, f32(1.0))
    lc = sqrtf(f32(sigma / f32(rho * max(f32(gravity), f32(0.1)))))
    ca = min(f32(f32(f32(m.viscosity * rho) * COAT_SPEED) / sigma), f32(1.0))
    wet = f32(f32(0.5) * f32(f32(1.0) + cosf(f32(m.contact_angle * RADS_PER_DEG))))
    return f32(f32(f32(f32(f32(0.94) * lc) * powf(ca, TWO_THIRDS)) * wet) / FILM_UNIT)


def dry_scatter(m):
    rigid = m.cloud_ior >= f32(1.5)
    n = max(m.ior, f32(1.0))

    def gain(np_):
        g = f32(f32(np_ - f32(1.0)) / max(f32(abs(f32(np_ - n))), f32(0.02)))
        return clamp(f32(g * g), 1.0, 6.0)
    wr = f32(m.dust + (m.cloud if rigid else f32(0.0)))
    ws = f32(0.0) if rigid else m.cloud
    if f32(wr + ws) <= 0.0:
        return f32(1.0)
    npv = f32(1.55) if (m.dust > 0.0 and not rigid) else max(m.cloud_ior, f32(1.55))
    return f32(f32(f32(wr * gain(npv)) + f32(ws * f32(0.33))) / f32(wr + ws))


def iridescence(m, pair, cell):
    if m.group in (0, 2):
        return f32(0.0)
    spread = f32(f32(f32(0.072) - m.tension) - f32(pair))
    a, s = coefficients(m, m.color, cell)
    murk = f32(f32(f32(f32(a[0] + a[1]) + a[2]) / f32(3.0)) + f32(f32(f32(s[0] + s[1]) + s[2]) / f32(3.0)))
    return f32(f32(clamp(f32(spread / f32(0.01)), 0.0, 1.0) * clamp(f32(f32(abs(f32(m.ior - f32(1.33)))) / f32(0.1)), 0.0, 1.0))
               * f32(f32(1.0) - clamp(f32(murk / f32(1.5)), 0.0, 1.0)))


def crust(m):
    if not m.freezes():
        return f32(0.0)
    return clamp(f32(f32(m.melt_lo - f32(400.0)) / f32(400.0)), 0.0, 1.0)


def mean_area_factor(r):
    if r >= TWO_THIRDS:
        return f32(f32(0.25) * PI)
    return f32(f32(0.25) * f32(f32(f32(0.5) * PI) + f32(PI * max(f32(r), f32(0.005)))))


def dust_specks(m, cell):
    zero = [f32(0.0)] * 4
    if m.dust <= 0.0:
        return f32(0.0), zero
    a_v, _, _ = particle_shape(m.dust_size, m.dust_shape)
    phi = clamp(m.dust, 0.0, 0.6)
    cell = f32(cell)
    sigma = f32(f32(f32(phi * a_v) * f32(2.0)) * cell)
    s_red = f32(f32(0.5) * sigma)
    area = f32(f32(f32(m.dust_size * m.dust_size) * mean_area_factor(m.dust_shape)) / f32(cell * cell))
    tau = f32(sigma * LV_BODY)
    n_vis = f32(f32(f32(1.0) - expf(f32(-tau))) / max(area, f32(1e-9)))
    n = min(n_vis, DUST_DRAW_MAX)
    if n <= f32(1e-6):
        return f32(0.0), zero
    undrawn = max(f32(f32(1.0) - f32(n / n_vis)), f32(0.0))
    w = albedo_of(m.dust_color)
    r0 = clamp(m.dust_reflect, 0.0, 1.0)
    per = f32(undrawn / n)
    out = []
    for c in range(3):
        wc = f32(r0 + f32(f32(f32(1.0) - r0) * w[c]))
        out.append(f32(f32(f32(s_red * f32(f32(1.0) - wc)) / max(wc, f32(1e-4))) * per))
    out.append(f32(s_red * per))
    return n, out


def optics_row(params, row: int, cell, ambient, drying, gravity, pair0):
    """material.rs:921-978: one row as (field, four values) pairs in GpuOptics order."""
    m = Mat(params, row)
    sl = linear(m.color_solid)
    a, s = coefficients(m, m.color, cell)
    ah, sh = coefficients(m, m.color_hot, cell)
    mean = f32(f32(f32(s[0] + s[1]) + s[2]) / f32(3.0))
    _, g = cloud_scattering(m, cell)
    ratio = [f32(v / mean) for v in s] if mean > f32(1e-9) else [f32(1.0)] * 3
    plate_k = max(f32(f32(1.0) - min(f32(m.cloud_shape / TWO_THIRDS), f32(1.0))), f32(0.0))
    am = f32(f32(f32(a[0] + a[1]) + a[2]) / f32(3.0))
    plate = f32(0.0)
    if m.cloud > 0.0:
        plate = f32(f32(f32(plate_k * f32(f32(1.0) - expf(f32(f32(-4.0) * mean)))) * mean) / f32(f32(mean + am) + f32(1e-6)))
    eta = max(f32(m.viscosity * m.density), f32(1e-6))
    dsz = max(m.cloud_size, f32(1e-9))
    dr = f32(f32(f32(3.0) * KT) / f32(f32(f32(f32(f32(4.0) * eta) * dsz) * dsz) * dsz)) if plate_k > 0.0 else f32(0.0)
    ar = clamp(m.cloud_shape, 0.005, 1.0)
    bret = f32(f32(f32(ar * ar) - f32(1.0)) / f32(f32(ar * ar) + f32(1.0)))
    n_draw, per = dust_specks(m, cell)
    dl = linear(m.dust_color)
    pack = f32(f32(n_draw * DUST_PACKING) / max(m.dust, f32(1e-6))) if m.dust > 0.0 else f32(0.0)
    drain = f32(f32(FOAM_DRAIN_WATER * eta) / f32(1.0e-3))
    vshare = volatile_share(m)
    evap = evaporation(m, ambient, drying)
    coat = coat_thickness(m, gravity)
    if vshare > 0.0 and evap > 0.0:
        dry_time = clamp(f32(f32(max(coat, f32(0.2)) * vshare) / evap), 0.2, 600.0)
    else:
        dry_time = f32(600.0)
    gl = linear(m.glow_color)
    return {
        "absorb": packed(a, s),
        "solid": [sl[0], sl[1], sl[2], tint_depth(m)],
        "opt": [m.opacity, plate, m.metal, m.gloss],
        "sty": [fullness(m), m.foam, dry_time, m.emissivity],
        # f32::round: half away from zero (the value is positive)
        "idx": [m.diluent, m.group, int(math.floor(float(f32(dry_scatter(m) * f32(1000.0))) + 0.5)), 0],
        "fx": [vshare, coat, iridescence(m, pair0[min(m.group, 3)], cell), crust(m)],
        "fx2": [m.froth, m.fizz, n_draw, drain],
        "lum": [f32(gl[0] * m.luminous), f32(gl[1] * m.luminous), f32(gl[2] * m.luminous), m.glow_shear],
        "hot": packed(ah, sh),
        "thermo": [m.thermo_lo, m.thermo_hi, wetting(m), f32(1.0) if (m.group == 0 and m.tension < f32(0.04)) else f32(0.0)],
        "scat": [ratio[0], ratio[1], ratio[2], g],
        "opt2": [m.ior, dr, bret, evap],
        "dust": per,
        "dust2": [f32(f32(0.5) * m.dust_size), m.dust_density, m.dust_shape, m.dust_reflect],
        "dcol": [dl[0], dl[1], dl[2], pack],
    }

"""CPU restatement of the brush's emitters: src/brush.rs (Spout, Stream::advance, stroke,
spray_velocity, Admission) and World::emit's sources (src/world.rs:609-743: paint, rain,
stream, admission, rand, solid_distance), in the reference's f32 / f64 arithmetic.

Test infrastructure: the checker of the engine's device emitters (emit.cu). It produces the
particles World::emit hands to FluidSim::spawn, from the counts FluidSim::cell_counts reads
back and the solid distances of the tank's node field, so that a test can queue them through
the engine's host spawn path and compare with what the device emitters queued. Pinned to the
reference's own brush.rs tests (tests/test_brush.py).

Two functions are the engine's own where the reference calls libm: hypot (the double sum of
squares rounded once, which is what glibc's hypotf returns) and the spray's sin / cos of its
small jitter angle (a Taylor series in FP64 rounded once; glibc's sinf / cosf agree to an ulp).
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32
PPC = 4                                   # sim::PPC
POUR_SPEED = (f32(60.0), f32(400.0))      # brush.rs:5
JET_SPEED = f32(320.0)                    # brush.rs:7
STREAM_FILL = f32(1.5)                    # brush.rs:11
GOLDEN = 0.6180339887498949               # brush.rs:58
SPRAY_SPEED = f32(260.0)                  # brush.rs:121
SPRAY_SHARE = f32(0.15)
SPRAY_SPACING = f32(1.5)
RAIN_SPEED = f32(200.0)                   # brush.rs:129
RAIN_SHARE = f32(0.3)
RAIN_SPAN = f32(3.0)
SPRAY_SPREAD = f32(0.25)                  # brush.rs:198
SPRAY_SPEED_SPREAD = f32(0.25)
SPAWN_MAX = 32768                         # mod.rs:63
RADS_PER_DEG = f32(f32(math.pi) / f32(180.0))


def hypot32(a, b) -> np.float32:
    return f32(math.sqrt(float(a) * float(a) + float(b) * float(b)))


def sincos_spread(x) -> tuple[np.float32, np.float32]:
    """sin and cos of a small angle (|x| <= 0.25): Taylor series in FP64, rounded once."""
    x = float(f32(x))
    x2 = x * x
    sn = 1.0 / 1307674368000.0
    for c in (6227020800.0, 39916800.0, 362880.0, 5040.0, 120.0, 6.0):
        sn = 1.0 / c - x2 * sn
    sn = x - x * x2 * sn
    cs = 1.0 / 20922789888000.0
    for c in (87178291200.0, 479001600.0, 3628800.0, 40320.0, 720.0, 24.0):
        cs = 1.0 / c - x2 * cs
    cs = 0.5 - x2 * cs
    cs = 1.0 - x2 * cs
    return f32(sn), f32(cs)


# ---- brush.rs ------------------------------------------------------------------------------

_libm = None


def _sincosf(r):
    """sinf / cosf of the platform's libm (what f32::sin_cos calls in the reference)."""
    global _libm
    if _libm is None:
        import ctypes
        import ctypes.util
        _libm = ctypes.CDLL(ctypes.util.find_library("m"))
        _libm.sinf.restype = _libm.cosf.restype = ctypes.c_float
        _libm.sinf.argtypes = _libm.cosf.argtypes = [ctypes.c_float]
    return f32(_libm.sinf(float(r))), f32(_libm.cosf(float(r)))


def jet_direction(degrees) -> tuple:
    s, c = _sincosf(f32(f32(degrees) * RADS_PER_DEG))
    return (s, f32(-c))


class Spout:
    """brush::Spout (brush.rs:18-58)."""

    def __init__(self, direction, speed, width):
        self.direction = (f32(direction[0]), f32(direction[1]))
        self.speed = f32(speed)
        self.width = f32(width)

    @staticmethod
    def _new(direction, speed, rate, radius):
        speed = f32(speed)
        return Spout(direction, speed, min(f32(f32(rate) / f32(f32(PPC) * speed)), f32(f32(2.0) * f32(radius))))

    @staticmethod
    def pour(rate, radius):
        speed = f32(f32(rate) / f32(f32(f32(PPC) * f32(2.0)) * f32(radius)))
        speed = min(max(speed, POUR_SPEED[0]), POUR_SPEED[1])
        return Spout._new((f32(0.0), f32(-1.0)), speed, rate, radius)

    @staticmethod
    def jet(degrees, rate, radius):
        return Spout._new(jet_direction(degrees), JET_SPEED, rate, radius)

    @staticmethod
    def faucet(degrees, rate, radius):
        p = Spout.pour(rate, radius)
        return Spout(jet_direction(degrees), p.speed, p.width)

    def rate(self) -> np.float32:
        return f32(f32(f32(PPC) * self.speed) * self.width)

    def velocity(self):
        return (f32(self.direction[0] * self.speed), f32(self.direction[1] * self.speed))


class Stream:
    """brush::Stream (brush.rs:78-116)."""

    def __init__(self):
        self.time = 0.0

    def advance(self, spout: Spout, frm, to, seconds, limit: int) -> list:
        rate = float(spout.rate())
        start, end = self.time, self.time + float(f32(seconds))
        self.time = end
        half = f32(f32(0.5) * spout.width)
        side = (f32(-spout.direction[1]), spout.direction[0])
        frm = (f32(frm[0]), f32(frm[1]))
        to = (f32(to[0]), f32(to[1]))

        def index(t):
            return int(max(math.floor(rate * t - 0.5) + 1.0, 0.0))

        out = []
        for k in range(index(start - float(f32(half / spout.speed))), index(end)):
            kg = k * GOLDEN
            across = f32(f32(f32(kg - math.floor(kg)) - f32(0.5)) * spout.width)
            arc = f32(np.sqrt(max(f32(half * half - across * across), f32(0.0))))
            appears = (k + 0.5) / rate + float(f32((half - arc) / spout.speed))
            if appears < start or appears >= end:
                continue
            t = f32((appears - start) / (end - start))
            along = f32(f32(f32(end - appears) * spout.speed) - arc)
            x = f32(f32(f32(frm[0] + f32(f32(to[0] - frm[0]) * t)) + f32(side[0] * across)) + f32(spout.direction[0] * along))
            y = f32(f32(f32(frm[1] + f32(f32(to[1] - frm[1]) * t)) + f32(side[1] * across)) + f32(spout.direction[1] * along))
            out.append((x, y))
        if len(out) > limit:
            out = out[len(out) - limit:]
        return out


def offset_from_stroke(p, frm, to, length2):
    dx, dy = f32(to[0] - frm[0]), f32(to[1] - frm[1])
    t = f32(0.0)
    if length2 > 0.0:
        t = f32(f32(f32(f32(p[0] - frm[0]) * dx) + f32(f32(p[1] - frm[1]) * dy)) / length2)
        t = min(max(t, f32(0.0)), f32(1.0))
    return (f32(f32(p[0] - frm[0]) - f32(t * dx)), f32(f32(p[1] - frm[1]) - f32(t * dy)))


def stroke(frm, to, radius, grid, spacing) -> list:
    """brush::stroke (brush.rs:134-153)."""
    frm = (f32(frm[0]), f32(frm[1]))
    to = (f32(to[0]), f32(to[1]))
    radius, spacing = f32(radius), f32(spacing)
    dx, dy = f32(to[0] - frm[0]), f32(to[1] - frm[1])
    length2 = f32(f32(dx * dx) + f32(dy * dy))

    def index(v, limit, rnd):
        return int(rnd(float(f32(min(max(f32(v), f32(0.0)), f32(limit)) / spacing))))

    lo = [index(min(frm[0], to[0]) - radius, grid[0], math.floor), index(min(frm[1], to[1]) - radius, grid[1], math.floor)]
    hi = [index(max(frm[0], to[0]) + radius, grid[0], math.ceil), index(max(frm[1], to[1]) + radius, grid[1], math.ceil)]
    out = []
    for y in range(lo[1], hi[1]):
        for x in range(lo[0], hi[0]):
            p = (f32(f32(f32(x) + f32(0.5)) * spacing), f32(f32(f32(y) + f32(0.5)) * spacing))
            d = offset_from_stroke(p, frm, to, length2)
            if f32(f32(d[0] * d[0]) + f32(d[1] * d[1])) <= f32(radius * radius):
                out.append(p)
    return out


def spray_velocity(p, frm, to, radius, jitter):
    """brush::spray_velocity (brush.rs:177-193); None for the dense centre."""
    frm = (f32(frm[0]), f32(frm[1]))
    to = (f32(to[0]), f32(to[1]))
    radius = f32(radius)
    dx, dy = f32(to[0] - frm[0]), f32(to[1] - frm[1])
    length2 = f32(f32(dx * dx) + f32(dy * dy))
    off = offset_from_stroke(p, frm, to, length2)
    dist = hypot32(off[0], off[1])
    if dist < f32(radius * f32(0.7)) or dist < f32(1e-4):
        return None
    s, c = sincos_spread(f32(f32(f32(f32(jitter[0]) * f32(2.0)) - f32(1.0)) * SPRAY_SPREAD))
    speed = f32(SPRAY_SPEED * f32(f32(1.0) + f32(f32(f32(f32(jitter[1]) * f32(2.0)) - f32(1.0)) * SPRAY_SPEED_SPREAD)))
    nx, ny = f32(off[0] / dist), f32(off[1] / dist)
    return (f32(f32(f32(nx * c) - f32(ny * s)) * speed), f32(f32(f32(nx * s) + f32(ny * c)) * speed))


def window(frm, to, margin):
    """Admission::window (brush.rs:219-224)."""
    m = f32(margin)
    lo = [int(math.floor(f32(min(f32(frm[c]), f32(to[c])) - m))) for c in range(2)]
    hi = [int(math.ceil(f32(max(f32(frm[c]), f32(to[c])) + m))) + 1 for c in range(2)]
    return lo, hi


class Admission:
    """brush::Admission (brush.rs:203-238)."""

    def __init__(self, lo, size, counts, ppc: int, stream: bool):
        self.lo, self.size = list(lo), list(size)
        full = int(f32(f32(ppc) * STREAM_FILL))
        counts = np.asarray(counts, np.int64).ravel()
        self.room = (np.maximum(full - counts, 0) if stream else np.where(counts == 0, ppc, 0)).astype(np.int64)

    def admit(self, pos) -> bool:
        cx = int(math.floor(f32(pos[0]))) - self.lo[0]
        cy = int(math.floor(f32(pos[1]))) - self.lo[1]
        if cx < 0 or cy < 0 or cx >= self.size[0] or cy >= self.size[1]:
            return False
        k = cy * self.size[0] + cx
        if self.room[k] == 0:
            return False
        self.room[k] -= 1
        return True


# ---- World::emit's sources (world.rs) ------------------------------------------------------

class World:
    """The parts of World that emit: its generator, the node distances of its solids, and a
    `counts(lo, hi)` callable that reads the tank's live particles per cell (FluidSim::
    cell_counts, the queued ones included). Each source returns the particles it hands to
    FluidSim::spawn as (pos, vel) pairs."""

    def __init__(self, w: int, h: int, sdf: np.ndarray, counts, rng: int = 0x12345678):
        self.w, self.h = w, h
        self.sdf = np.asarray(sdf, np.float32).reshape(h + 1, w + 1)
        self.counts = counts
        self.rng = rng

    def rand(self) -> np.float32:
        r = self.rng
        r ^= (r << 13) & 0xFFFFFFFF
        r ^= r >> 17
        r ^= (r << 5) & 0xFFFFFFFF
        self.rng = r
        return f32(f32(r >> 8) / f32(16777216.0))

    def solid_distance(self, p) -> np.float32:
        x = min(max(f32(p[0]), f32(0.0)), f32(f32(self.w) - f32(1e-3)))
        y = min(max(f32(p[1]), f32(0.0)), f32(f32(self.h) - f32(1e-3)))
        i, j = int(x), int(y)
        fx, fy = f32(x - f32(i)), f32(y - f32(j))
        d = self.sdf
        bottom = f32(f32(d[j, i] * f32(f32(1.0) - fx)) + f32(d[j, i + 1] * fx))
        top = f32(f32(d[j + 1, i] * f32(f32(1.0) - fx)) + f32(d[j + 1, i + 1] * fx))
        return f32(f32(bottom * f32(f32(1.0) - fy)) + f32(top * fy))

    def admission(self, frm, to, margin, stream: bool) -> Admission:
        lo, hi = window(frm, to, margin)
        lo = [min(max(lo[0], 0), self.w), min(max(lo[1], 0), self.h)]
        hi = [min(max(hi[0], lo[0]), self.w), min(max(hi[1], lo[1]), self.h)]
        return Admission(lo, [hi[0] - lo[0], hi[1] - lo[1]], self.counts(lo, hi), PPC, stream)

    def paint(self, frm, to, radius, count: int, spray: bool) -> list:
        count = min(count, SPAWN_MAX)
        if count == 0:
            return []
        spacing = SPRAY_SPACING if spray else f32(f32(1.0) / f32(np.sqrt(f32(PPC))))
        cand = stroke(frm, to, radius, (self.w, self.h), spacing)
        for i in range(len(cand) - 1, 0, -1):
            j = min(int(f32(self.rand() * f32(i + 1))), i)
            cand[i], cand[j] = cand[j], cand[i]
        adm = self.admission(frm, to, f32(f32(radius) + f32(1.0)), False)
        out = []
        for pos in cand:
            if spray:
                jx = self.rand()
                jy = self.rand()
                pos = (f32(pos[0] + f32(f32(f32(jx - f32(0.5)) * f32(0.6)) * spacing)),
                       f32(pos[1] + f32(f32(f32(jy - f32(0.5)) * f32(0.6)) * spacing)))
            if self.solid_distance(pos) <= f32(0.4):
                continue
            vel = (f32(0.0), f32(0.0))
            if spray:
                jitter = (self.rand(), self.rand())
                vel = spray_velocity(pos, frm, to, radius, jitter)
                if vel is None:
                    continue
            if not adm.admit(pos):
                continue
            out.append((pos, vel))
            if len(out) == count:
                break
        return out

    def rain(self, at, radius, count: int) -> list:
        half = f32(f32(radius) * RAIN_SPAN)
        count = min(count, SPAWN_MAX)
        if count == 0:
            return []
        at = (f32(at[0]), f32(at[1]))
        frm, to = (f32(at[0] - half), at[1]), (f32(at[0] + half), at[1])
        adm = self.admission(frm, to, f32(3.0), False)
        out = []
        for _ in range(count):
            rx = self.rand()
            ry = self.rand()
            pos = (f32(at[0] + f32(f32(f32(rx * f32(2.0)) - f32(1.0)) * half)),
                   f32(at[1] + f32(f32(f32(ry * f32(2.0)) - f32(1.0)) * f32(2.0))))
            if self.solid_distance(pos) <= f32(0.4) or not adm.admit(pos):
                continue
            speed = f32(RAIN_SPEED * f32(f32(0.8) + f32(f32(0.4) * self.rand())))
            vx = f32(f32(self.rand() - f32(0.5)) * f32(12.0))
            out.append((pos, (vx, f32(-speed))))
        return out

    def stream(self, stream: Stream, spout: Spout, frm, to, seconds) -> list:
        positions = stream.advance(spout, frm, to, seconds, SPAWN_MAX)
        reach = f32(f32(f32(spout.speed * f32(seconds)) + spout.width) + f32(1.0))
        adm = self.admission(frm, to, reach, True)
        v = spout.velocity()
        return [(p, v) for p in positions if self.solid_distance(p) > f32(0.4) and adm.admit(p)]

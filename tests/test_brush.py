"""The CPU restatement of the brush's emitters (oracle/brush.py), pinned to the reference's own
brush.rs tests (src/brush.rs:244-384, restated with their thresholds), and the engine's host
helper for spouts (sprout_spout) against it. The device emitters are checked against this
restatement in test_gpu_emit.py."""
import math

import numpy as np
import pytest

from oracle import brush as B

f32 = np.float32


def run_stream(spout, frames, dt, sweep):
    st, allp, v = B.Stream(), [], spout.velocity()
    for f in range(frames):
        allp = [(f32(p[0] + f32(v[0] * f32(dt))), f32(p[1] + f32(v[1] * f32(dt)))) for p in allp]
        frm = (f32(100.0 + sweep * dt * f), 100.0)
        to = (f32(100.0 + sweep * dt * (f + 1)), 100.0)
        allp.extend(st.advance(spout, frm, to, dt, 1 << 62))
    return allp


def test_a_stroke_is_the_same_however_it_is_cut_into_frames():
    whole = B.stroke((10.0, 10.0), (80.0, 10.0), 2.0, (100, 30), 0.5)
    parts = B.stroke((10.0, 10.0), (45.0, 10.0), 2.0, (100, 30), 0.5)
    parts += B.stroke((45.0, 10.0), (80.0, 10.0), 2.0, (100, 30), 0.5)
    assert set(whole) <= set(parts) and set(parts) <= set(whole)
    dot = B.stroke((20.0, 20.0), (20.0, 20.0), 3.0, (100, 100), 0.5)
    area = math.pi * 9.0 * 4.0
    assert abs(len(dot) - area) < 0.1 * area


def test_admission_fills_only_empty_cells_up_to_rest_density():
    a = B.Admission([4, 7], [2, 1], [1, 0], 4, False)
    assert not a.admit((4.5, 7.5))
    for p in [(5.25, 7.25), (5.75, 7.25), (5.25, 7.75), (5.75, 7.75)]:
        assert a.admit(p)
    assert not a.admit((5.5, 7.5)) and not a.admit((9.5, 7.5))
    s = B.Admission([0, 0], [1, 1], [4], 4, True)
    assert s.admit((0.5, 0.5)) and s.admit((0.5, 0.5)) and not s.admit((0.5, 0.5))


def test_the_pour_fills_the_brush_at_the_speed_the_flow_needs():
    sp = B.Spout.pour(12000.0, 9.0)
    assert abs(sp.width - 18.0) < 1e-4 and abs(sp.speed - 12000.0 / 72.0) < 1e-3
    assert abs(sp.rate() - 12000.0) < 1.0
    tr = B.Spout.pour(1000.0, 9.0)
    assert tr.speed == B.POUR_SPEED[0] and tr.width < 5.0 and abs(tr.rate() - 1000.0) < 1.0
    fl = B.Spout.pour(1e6, 9.0)
    assert fl.speed == B.POUR_SPEED[1] and fl.width == 18.0 and fl.rate() < 30000.0
    jet = B.Spout.jet(90.0, 12000.0, 9.0)
    assert abs(jet.velocity()[0] - B.JET_SPEED) < 1e-3 and abs(jet.rate() - 12000.0) < 1.0


def test_a_stream_is_the_same_however_time_is_cut_into_frames():
    sp = B.Spout.pour(12000.0, 9.0)
    for sweep in (0.0, 300.0):
        whole, cut = run_stream(sp, 1, 0.1, sweep), run_stream(sp, 25, 0.004, sweep)
        corners = int(f32(B.PPC * (162.0 - 0.5 * math.pi * 81.0)))
        assert abs(len(whole) - (1200 - corners)) <= 2, len(whole)
        assert len(whole) == len(cut)
        c = np.array(cut, np.float64)
        worst = max(np.min(np.hypot(c[:, 0] - a[0], c[:, 1] - a[1])) for a in whole)
        assert worst < 0.02, (sweep, worst)


def test_a_stream_is_evenly_packed_at_rest_density():
    for sp, dt in [(B.Spout.pour(12000.0, 9.0), 1 / 60), (B.Spout.pour(1500.0, 9.0), 1 / 144),
                   (B.Spout.jet(40.0, 30000.0, 20.0), 1 / 30)]:
        pts = np.array(run_stream(sp, 12, dt, 0.0), np.float64)
        half = 0.5 * float(sp.width)
        area = float(sp.width) * float(sp.speed) * 12.0 * dt - (2.0 - 0.5 * math.pi) * half * half
        assert abs(len(pts) / area - B.PPC) < 0.02 * B.PPC, (len(pts), area)
        near = min(np.min(np.hypot(pts[:i, 0] - pts[i, 0], pts[:i, 1] - pts[i, 1])) for i in range(1, len(pts)))
        assert near > 0.9 / math.sqrt(B.PPC), near


def test_a_stream_has_a_round_top_that_fills_the_brush():
    pts = np.array(run_stream(B.Spout.pour(12000.0, 9.0), 1, 0.02, 0.0), np.float64)
    up = pts[pts[:, 1] > 100.0]
    assert np.count_nonzero(np.hypot(up[:, 0] - 100.0, up[:, 1] - 100.0) > 9.0 + 1e-3) == 0

    def top(lo, hi):
        sel = pts[(pts[:, 0] - 100.0 >= lo) & (pts[:, 0] - 100.0 < hi)]
        return sel[:, 1].max() if len(sel) else -np.inf   # the reference folds from f32::MIN
    assert abs(top(-1.0, 1.0) - 109.0) < 0.3
    assert top(8.0, 9.0) < 104.5 and top(-9.0, -8.0) < 104.5


def test_a_stream_drops_a_backlog_instead_of_releasing_it():
    sp, st = B.Spout.pour(12000.0, 9.0), B.Stream()
    assert len(st.advance(sp, (0.0, 0.0), (0.0, 0.0), 1.0, 500)) == 500
    assert abs(len(st.advance(sp, (0.0, 0.0), (0.0, 0.0), 0.01, 500)) - 120) <= 10


def test_jet_aim_covers_a_full_turn():
    for ang, exp in [(0.0, (0.0, -1.0)), (90.0, (1.0, 0.0)), (180.0, (0.0, 1.0)), (270.0, (-1.0, 0.0))]:
        d = B.jet_direction(ang)
        assert abs(d[0] - exp[0]) < 1e-5 and abs(d[1] - exp[1]) < 1e-5


def test_spray_has_no_dense_centre_and_keeps_its_launch_speed():
    c, mid = (20.0, 20.0), (0.5, 0.5)
    assert B.spray_velocity(c, c, c, 9.0, mid) is None
    assert B.spray_velocity((23.0, 20.0), c, c, 9.0, mid) is None
    for off in [(8.0, 0.0), (-8.0, 0.0), (0.0, 8.0), (5.0, -5.0)]:
        p = (f32(c[0] + off[0]), f32(c[1] + off[1]))
        v = B.spray_velocity(p, c, c, 9.0, mid)
        assert abs(math.hypot(v[0], v[1]) - float(B.SPRAY_SPEED)) < 0.001
        assert v[0] * off[0] + v[1] * off[1] > 0.0
        for j in [(0.0, 0.0), (1.0, 1.0), (0.2, 0.9)]:
            v = B.spray_velocity(p, c, c, 9.0, j)
            sp = math.hypot(v[0], v[1])
            assert sp >= 260.0 * 0.75 - 1e-3 and sp <= 260.0 * 1.25 + 1e-3
            cos = (v[0] * off[0] + v[1] * off[1]) / (sp * math.hypot(*off))
            assert cos >= math.cos(0.25) - 1e-4
    v = B.spray_velocity((30.0, 28.0), (20.0, 20.0), (40.0, 20.0), 9.0, mid)
    assert abs(v[0]) < 1e-3 and v[1] > 0.0


def test_own_sin_and_cos_stay_within_an_ulp_of_libm():
    """The spray's jitter angle takes the engine's own sin / cos (FP64 Taylor series, rounded
    once); against the platform's sinf / cosf (what the reference's f32::sin_cos calls) they
    agree to an ulp over the whole jitter range."""
    import ctypes
    import ctypes.util
    libm = ctypes.CDLL(ctypes.util.find_library("m"))
    libm.sinf.restype = libm.cosf.restype = ctypes.c_float
    libm.sinf.argtypes = libm.cosf.argtypes = [ctypes.c_float]
    worst = 0
    for x in np.linspace(-0.25, 0.25, 20001, dtype=np.float32):
        s, c = B.sincos_spread(x)
        for mine, ref in ((s, libm.sinf(float(x))), (c, libm.cosf(float(x)))):
            d = abs(int(np.array(mine, np.float32).view(np.int32)) - int(np.array(ref, np.float32).view(np.int32)))
            worst = max(worst, d)
    assert worst <= 1


def test_engine_spout_matches_the_restatement():
    """sprout_spout (the C ABI's Spout::pour / jet / faucet, host arithmetic) against the
    restatement, bit for bit (needs the built library, not a GPU)."""
    S = pytest.importorskip("sprout_gb300")
    for kind, deg, rate, rad in [("pour", 0.0, 12000.0, 9.0), ("pour", 0.0, 1000.0, 9.0), ("pour", 0.0, 1e6, 9.0),
                                 ("jet", 90.0, 12000.0, 9.0), ("jet", 40.0, 30000.0, 20.0),
                                 ("faucet", 135.0, 5000.0, 6.0)]:
        e = S.Spout.make(kind, rate, rad, deg)
        o = {"pour": lambda: B.Spout.pour(rate, rad), "jet": lambda: B.Spout.jet(deg, rate, rad),
             "faucet": lambda: B.Spout.faucet(deg, rate, rad)}[kind]()
        got = np.array([e.direction[0], e.direction[1], e.speed, e.width], np.float32)
        want = np.array([o.direction[0], o.direction[1], o.speed, o.width], np.float32)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (kind, got, want)

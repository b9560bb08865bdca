"""Scene::rasterize on the device (sprout_scene_rasterize_device, sprout_sim_set_scene)
against the host restatement (sprout_scene_rasterize, scene.cpp), bit for bit: node
distances with the chamfer union depth inside overlapping solids, open volumes, the sealing of
enclosed pockets, face fractions, smoothed occupancy, regions (ids capped at 31) with their
vents, and held temperatures. The host restatement is itself pinned to the reference's scene
tests (test_oracle_golden.py) and equal to the oracle's (test_host.py)."""
import time

import numpy as np
import pytest

import sprout_gb300 as S
import tanks

pytestmark = pytest.mark.gpu


def same(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def compare(scene):
    h_sdf, h_solid, h_region, h_temp = scene.rasterize()
    d_sdf, d_solid, d_region, d_temp = scene.rasterize(device=True)
    problems = []
    for name, a, b in [("sdf", h_sdf, d_sdf), ("solid", h_solid, d_solid), ("region", h_region, d_region)]:
        if not same(a, b):
            bad = np.flatnonzero(np.asarray(a).view(np.uint32).ravel() != np.asarray(b).view(np.uint32).ravel())
            problems.append(f"{name}: {len(bad)} values differ (first {bad[0]})")
    if (h_temp is None) != (d_temp is None) or (h_temp is not None and not same(h_temp, d_temp)):
        problems.append("temp differs")
    return problems, (h_sdf, h_solid, h_region, h_temp)


def ring(sc, x0, y0, x1, y1, t=1.0):
    """Four thin boxes enclosing [x0, x1] x [y0, y1] (cells)."""
    cx, cy = (x0 + x1) / 2, (y0 + y1) / 2
    hx, hy = (x1 - x0) / 2, (y1 - y0) / 2
    sc.add_box([cx, y0 - t], [hx + 2 * t, t])
    sc.add_box([cx, y1 + t], [hx + 2 * t, t])
    sc.add_box([x0 - t, cy], [t, hy + 2 * t])
    sc.add_box([x1 + t, cy], [t, hy + 2 * t])


def test_walls_only_and_timing_at_1024():
    sc = S.Scene(1024, 576)
    problems, _ = compare(sc)
    assert not problems, problems
    t0 = time.perf_counter()
    sc.rasterize()
    host = time.perf_counter() - t0
    sc.rasterize(device=True)   # warm
    t0 = time.perf_counter()
    sc.rasterize(device=True)
    dev = time.perf_counter() - t0
    print(f"rasterize 1024x576: host {host * 1e3:.1f} ms, device {dev * 1e3:.1f} ms (with copies)")


def test_overlapping_rotated_shapes_union_depth():
    sc = S.Scene(384, 216)
    sc.add_box([120.0, 60.0], [40.0, 8.0], 0.35)
    sc.add_box([150.0, 70.0], [30.0, 10.0], -0.6)
    sc.add_circle([140.0, 65.0], 18.0)
    sc.add_circle([300.0, 150.0], 25.5)
    sc.add_box([300.0, 120.0], [50.0, 6.0], 0.05)
    sc.add_box([40.0, 200.0], [60.0, 20.0], 0.0)   # overlapping the top wall
    problems, (sdf, solid, region, _) = compare(sc)
    assert not problems, problems
    assert (sdf < -3.0).sum() > 100   # the union depth reached inside the overlaps


def test_pockets_are_sealed_and_regions_numbered():
    sc = S.Scene(256, 144)
    ring(sc, 20.0, 20.0, 23.0, 23.0)        # a 3 x 3 pocket: sealed
    ring(sc, 60.0, 20.0, 63.0, 25.0)        # a 3 x 5 pocket: sealed
    for k in range(40):                     # 40 enclosures of 5 x 5 open cells: regions 1.. (ids cap at 31)
        x, y = 12.0 + (k % 10) * 22.0, 50.0 + (k // 10) * 22.0
        ring(sc, x, y, x + 5.0, y + 5.0)
    problems, (sdf, solid, region, _) = compare(sc)
    assert not problems, problems
    ids = region & 255
    assert ids.max() == 31 and np.count_nonzero(region & 256) >= 32


def test_held_temperatures():
    sc = S.Scene(192, 108)
    sc.add_box([96.0, 10.0], [90.0, 4.0], 0.0, 300.0)
    sc.add_circle([50.0, 60.0], 10.0, -20.0)
    sc.add_circle([55.0, 62.0], 6.0, 80.0)   # overlaps the first: the later one wins
    sc.add_box([150.0, 60.0], [10.0, 10.0], 0.3)   # insulating
    problems, (_, _, _, temp) = compare(sc)
    assert not problems, problems
    assert temp is not None and np.any(temp == 300.0) and np.any(temp == 80.0)


def test_set_scene_steps_as_set_solids():
    """A tank whose solids are rasterised on the device into the sim's own buffers steps bit
    for bit as the same tank given the host's arrays."""
    t = tanks.dam_break(160, 96)
    t.shapes = [{"kind": "box", "c": [110.0, 20.0], "half": [20.0, 4.0], "angle": 0.4},
                {"kind": "circle", "c": [60.0, 70.0], "r": 9.0}]
    a, parts, _ = t.engine()
    b = S.FluidSim(t.w, t.h, len(parts) + t.capacity_extra, S.SimParams(t.settings))
    sc = S.Scene(t.w, t.h)
    sc.add_box([110.0, 20.0], [20.0, 4.0], 0.4)
    sc.add_circle([60.0, 70.0], 9.0)
    b.set_scene(sc)
    b.reset(parts)
    for _ in range(6):
        a.step(1, 1 / 240.0)
        b.step(1, 1 / 240.0)
    pa, pb = a.download_particles(), b.download_particles()
    assert np.array_equal(pa.view(np.uint8), pb.view(np.uint8))

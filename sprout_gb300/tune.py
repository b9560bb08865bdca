"""The launch autotuner: picks, per grid size, the block counts of the persistent pressure and
viscosity solves (plain and mixed precision) and the viscosity smoother's sweeps per level,
from candidates timed on the device with CUDA events.

What it may choose, and why only that:
- Block counts. Each persistent solve runs its phases over the active tiles of a level; a
  block takes tiles blockIdx, blockIdx + blocks, ... and every block sums the same per-tile
  partials in the same order, so the results are bit-identical at any count (the tests check
  1 to 16 blocks on a 60-tile grid against the oracle). Fewer blocks mean fewer arrivals at
  each grid barrier but more tiles per block; the best count depends on the grid and on how
  many of its tiles are active.
- Viscosity sweeps (viscosity_mg_sweeps, 1 or 2 red-black sweeps per level visit). This is a
  parameter of the reference's solver (params.rs:437-442): both counts solve to the same
  tolerance, one with more, cheaper iterations. The tuner reports the faster one; a caller
  opts in by setting the parameter (the library never changes a parameter by itself).
- Not the tile shape: the 16 x 16 tile is the reference's work group (mg_down.comp:18), and
  its partial sums are reduced in that work group's tree order (reduce.glsl); another shape
  would change the bits of every dot product and so the iteration counts.

The table is written as JSON (sprout_gb300/tuned_launch.json) and as a C table compiled
into the library (csrc/tuned_launch.inc): a sim whose grid size is in the table starts from
its counts unless the caller sets its own (sprout_sim_set_launch).

    python -m sprout_gb300.tune [--sizes 128x72,256x144,...] [--substeps 6]
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
JSON_OUT = HERE / "tuned_launch.json"
INC_OUT = HERE / "csrc" / "tuned_launch.inc"

DEFAULT_SIZES = [(128, 72), (256, 144), (384, 216), (512, 288), (768, 432), (1024, 576)]


def representative(w: int, h: int, seed: int = 0):
    """A tank of this grid size that runs both solves: the full-physics pour's liquids (eight
    columns, heater, tension) at the same physical size as the 1024 x 576 pour."""
    from .workloads import full_physics
    return full_physics(w, h, cell=0.001 * 1024 / w, seed=seed)


def candidates(nwg: int, sms: int = 152) -> list[int]:
    """Block counts to try: the default (one per tile, at most what fits: 0), whole multiples
    of the SM count and fractions of the tile count."""
    c = {0}
    for m in (0.5, 1, 1.5, 2, 3, 4):
        b = int(sms * m)
        if 1 <= b < nwg:
            c.add(b)
    for f in (0.25, 0.5, 0.75):
        b = int(nwg * f)
        if b >= 8:
            c.add(b)
    return sorted(c)


def time_stages(tank, launch: dict, precision: str, substeps: int, warmup: int = 3) -> tuple[float, float, dict]:
    """(pressure ms, viscosity ms) per substep and the stage times, from CUDA events, with
    `launch` applied to a fresh copy of the tank after `warmup` substeps."""
    sim, _, _ = tank.engine()
    sim.set_precision(precision)
    sim.set_launch(**launch)
    dt = 1.0 / 240.0
    for _ in range(warmup):
        sim.step(1, dt)
    p = v = 0.0
    st = {}
    for _ in range(substeps):
        st = sim.profile_passes()
        p += st["pressure"] + st["project2"]   # both pressure solves (project2 holds the second)
        v += st["viscosity"]
    eff = sim.launch()
    sim.close()
    return p / substeps, v / substeps, eff


def tune_size(w: int, h: int, substeps: int, sweeps: bool = True) -> dict:
    tank = representative(w, h)
    nwg = ((w + 15) // 16) * ((h + 15) // 16)
    out = {"grid": [w, h], "tiles": nwg, "trials": []}
    best = {}
    for prec, key in (("plain", "pressure_blocks"), ("mixed", "pressure_blocks_mixed")):
        res = []
        for b in candidates(nwg):
            pm, vm, eff = time_stages(tank, {key: b, "viscosity_blocks": b}, prec, substeps)
            res.append((pm, b, vm, eff))
            out["trials"].append({"precision": prec, "blocks": b, "effective": eff, "pressure_ms": pm, "viscosity_ms": vm})
        pm, b, _, eff = min(res)
        best[key] = eff[key]
        if prec == "plain":
            vm, vb, veff = min((r[2], r[1], r[3]) for r in res)
            best["viscosity_blocks"] = veff["viscosity_blocks"]
            best["_ms"] = {"pressure": pm, "viscosity": vm}
    if sweeps:
        timing = {}
        for nu in (1, 2):
            t = representative(w, h)
            t.settings["viscosity_mg_sweeps"] = float(nu)
            _, vm, _ = time_stages(t, {"viscosity_blocks": best["viscosity_blocks"]}, "plain", substeps)
            timing[nu] = vm
        best["viscosity_mg_sweeps"] = min(timing, key=timing.get)
        out["sweeps_ms"] = timing
    out["best"] = best
    return out


def write_tables(results: list[dict], device: str, out_dir: Path | None = None):
    json_out = JSON_OUT if out_dir is None else out_dir / JSON_OUT.name
    inc_out = INC_OUT if out_dir is None else out_dir / INC_OUT.name
    json_out.write_text(json.dumps({"device": device, "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
                                    "sizes": results}, indent=1) + "\n")
    lines = ["// Generated by sprout_gb300/tune.py from timed candidates on " + device + ": the persistent",
             "// solvers' block counts per grid size (w, h, plain pressure, mixed pressure, viscosity).",
             "// Results do not depend on them; a count a device cannot hold is lowered to what fits."]
    for r in results:
        b = r["best"]
        lines.append(f"{{{r['grid'][0]}, {r['grid'][1]}, {b['pressure_blocks']}, {b['pressure_blocks_mixed']}, "
                     f"{b['viscosity_blocks']}}},")
    inc_out.write_text("\n".join(lines) + "\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default=",".join(f"{w}x{h}" for w, h in DEFAULT_SIZES))
    ap.add_argument("--substeps", type=int, default=6)
    ap.add_argument("--no-sweeps", action="store_true")
    ap.add_argument("--write", action="store_true", help="write tuned_launch.json and csrc/tuned_launch.inc")
    ap.add_argument("--out-dir", default=None, help="write the two tables there instead of into the package")
    a = ap.parse_args()
    from . import build
    build.build()
    import torch
    dev = torch.cuda.get_device_name(0)
    results = []
    for s in a.sizes.split(","):
        w, h = (int(v) for v in s.split("x"))
        r = tune_size(w, h, a.substeps, sweeps=not a.no_sweeps)
        print(json.dumps({"grid": r["grid"], "best": r["best"], "sweeps_ms": r.get("sweeps_ms")}), flush=True)
        results.append(r)
    if a.write:
        write_tables(results, dev, Path(a.out_dir) if a.out_dir else None)
    print(json.dumps({"device": dev, "sizes": [r["best"] | {"grid": r["grid"]} for r in results]}))


if __name__ == "__main__":
    main()

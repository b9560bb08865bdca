"""Benchmark of the engine's substep: particle-steps/s on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference] [--workload NAME]

A step is one substep of the whole tank (sort, P2G, grid passes, pressure solve, projection,
the implicit viscosity and the second projection where the tank needs them, G2P/advection) on
a seeded synthetic tank (sprout_gb300.workloads); by default the full-physics pour at
1024 x 576 (8 liquids, heater, surface tension, implicit viscosity). `value` is
live particles x substeps / device seconds with the tank resident on the device
(CUDA events on the engine's stream; a tank whose substep touches more than the 129 MB L2,
as the default one does, runs back to back, a smaller one behind a 512 MB write before every
timed substep, which `config.l2` states); `e2e` is the same metric through the public API with a host
round trip every step (the step call's host -> device copies and the stats read-back).
Under torchrun (N > 1) every rank advances its own tank (replicas: one tank does not
shard), the timed region is bracketed by barriers and the slowest rank's time counts.

`--impl reference` times the reference's algorithm on the host cores instead: the CPU
oracle (a C restatement of the reference's shaders, all host threads), on the same tank.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s at 1024x576, mixed vs plain, equal residual; p50/p99 step latency"
UNIT = "particle-steps/s"


def workload(name: str, rank: int):
    from sprout_gb300 import workloads as WL
    if name == "full_physics_1024":
        # The full-physics pour: 1024 x 576, 1 mm cells, 8 seeded liquids in random vertical
        # columns over the whole tank (rho 800-13500, mu 1e-3-50 Pa s log-uniform, tension
        # 0.02-0.5 N/m), 293 K over a 600 K heater strip on the bottom 8 rows, heat diffusion,
        # surface tension and implicit viscosity on, pressure and viscosity to 1e-5.
        t = WL.full_physics(1024, 576, cell=0.001, n_liquids=8, seed=0, heater_rows=8, tol=1e-5)
        desc = {"workload": "full_physics_pour_1024x576", "grid": [1024, 576], "cell_size_m": 0.001,
                "fill": "8 liquids, seeded vertical columns, whole tank", "ppc": 4, "substep_s": 1 / 240,
                "pressure_tol": 1e-5, "viscosity_tol": 1e-5, "solver": "plain fp32 MGPCG + implicit viscosity MG-PCG",
                "heater": "600 K, bottom 8 rows", "surface_tension": "0.02-0.5 N/m", "seed": 0}
    elif name == "stratified_512":
        # built-in honey (a water concentrate, mix rate 1.5 / s) and water exchange concentration;
        # the built-in olive oil is immiscible (phase group 1) and drifts against the water
        t = WL.stratified(512, 288, cell=0.002, tol=1e-5, builtins=True)
        desc = {"workload": "stratified_honey_water_oil_512x288", "grid": [512, 288], "cell_size_m": 0.002,
                "fill": "honey / water / olive oil layers, 20% of the height each", "ppc": 4, "substep_s": 1 / 240,
                "family": "honey in water, mix rate 1.5/s", "groups": "aqueous + olive oil, no pair tension",
                "pressure_tol": 1e-5, "viscosity_tol": 1e-5, "solver": "plain fp32 MGPCG + implicit viscosity MG-PCG"}
    elif name == "dam_break_1024":
        # 1024 x 576 MAC grid, 1 mm cells, water over the left 40 % and bottom 60 %, 4 particles
        # per cell, closed box, fixed 1/240 s substeps, pressure to relative residual 1e-5.
        t = WL.dam_break(1024, 576, cell=0.001, width=0.4, height=0.6, tol=1e-5)
        desc = {"workload": "dam_break_1024x576", "grid": [1024, 576], "cell_size_m": 0.001,
                "fill": "water, left 40% x bottom 60%", "ppc": 4, "substep_s": 1 / 240, "pressure_tol": 1e-5,
                "solver": "plain fp32 MGPCG", "surface_tension": 0, "viscosity": "explicit (water)"}
    elif name == "dam_break_384":
        t = WL.dam_break(384, 216, cell=0.002, width=0.4, height=0.6, tol=1e-5)
        desc = {"workload": "dam_break_384x216", "grid": [384, 216], "cell_size_m": 0.002,
                "fill": "water, left 40% x bottom 60%", "ppc": 4, "substep_s": 1 / 240, "pressure_tol": 1e-5,
                "solver": "plain fp32 MGPCG"}
    else:
        raise SystemExit(f"unknown workload {name}")
    desc["l2"] = l2_note(t)[1]
    return t, desc


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, n in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_setup(n_gpus: int):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allreduce_max(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


L2_BYTES = 129 * 1000 * 1000   # GB300 L2


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_oracle_rate(tank, seconds_budget: float = 15.0):
    """The oracle (the reference's algorithm restated in C) on all host threads, a bounded sample."""
    from oracle import oracle as O
    threads = O.threads_available()
    sim, parts, _ = O.build_tank(tank, threads=threads)
    dt = 1.0 / 240.0
    sim.step(1, dt)   # first substep: scatter only
    t0 = time.perf_counter()
    sim.step(1, dt)
    one = time.perf_counter() - t0
    n = int(max(1, min(20, seconds_budget / max(one, 1e-3))))
    t0 = time.perf_counter()
    sim.step(n, n * dt)
    el = time.perf_counter() - t0
    live = int(np.count_nonzero(sim.particles()["kind"]))
    return {"value": live * n / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} substeps of the same tank after 2 warm-up substeps, {el:.1f} s"}, live, el / n


def run_reference(args, rank, world, pg, budget_s: float = 90.0):
    """The reference's algorithm on the host cores (the oracle, all threads): up to `steps`
    substeps of the same tank after `warmup` (at most 3) warm-up substeps, stopping early once
    `budget_s` seconds of timed work have run, so the whole run ends within a few minutes."""
    tank, desc = workload(args.workload, rank)
    if rank != 0:
        return
    from oracle import oracle as O
    threads = O.threads_available()
    sim, parts, _ = O.build_tank(tank, threads=threads)
    dt = 1.0 / 240.0
    warm = min(args.warmup, 3)
    for _ in range(warm):
        sim.step(1, dt)
    done = 0
    t0 = time.perf_counter()
    while done < args.steps:
        sim.step(1, dt)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    live = int(np.count_nonzero(sim.particles()["kind"]))
    value = live * done / el
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / done * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded tank, no dataset)", "config": desc,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{done} of {args.steps} substeps timed after {warm} warm-up substeps, {el:.1f} s"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def kernels_per_substep(stats, settings: dict) -> int:
    n = 2 + 7 + 1 + 1             # step + advance; scan x3 + place + cell sort + crowd sort + gather; p2g;
                                  # the frame's end (the recorded iteration counts, each profiled substep)
    n += 4 + 1                    # grid_prep, coef/smooth, curvature, jumps; rhs
    caps = int(stats.caps)
    n += 1 if caps & 8 else 0     # rheo.comp
    n += 1 if caps & 64 else 0    # settle.comp
    n += 2 if caps & 16 else 0    # magnet.comp, both modes
    n += 1 if stats.thermal else 0
    n += 2 if stats.viscosity_mode == 1 else 0
    n += 1 + 1                    # pressure (persistent), project
    if stats.viscosity_mode == 2:
        levels = min(max(int(settings.get("viscosity_mg_levels", 1)), 1), stats.tail)
        n += 3 + levels + 1       # visc_setup, split, diag, coarse builds, the solve (persistent)
        if int(settings.get("viscous_projection", 1)) != 0:
            n += 3                # rhs_visc, second pressure solve, project_visc
    return n


def active_viscosity_cells(sim, w: int, h: int) -> int:
    """Cells of the tiles that take the implicit viscosity solve."""
    tiles = sim.field("tiles", np.uint32)
    tw = (w + 15) // 16
    n = 0
    for t in np.nonzero(tiles)[0]:
        x0, y0 = (t % tw) * 16, (t // tw) * 16
        n += (min(x0 + 16, w) - x0) * (min(y0 + 16, h) - y0)
    return int(n)


def l2_note(tank) -> tuple[bool, str]:
    """Whether a tank's substep fits in L2 (then each timed substep runs behind a 512 MB write),
    from the bytes it touches at least: every particle slot read and written (48 B each, 4 per
    cell at most) and ~400 B of per-cell grid records. The same in both arms' config."""
    touched = (96 * 4 + 400) * tank.w * tank.h
    flush = touched <= L2_BYTES
    return flush, (f"~{touched / 1e6:.0f} MB touched per substep <= L2 (129 MB): a 512 MB write before each "
                   "timed substep, substeps alone timed" if flush else
                   f"~{touched / 1e6:.0f} MB touched per substep > L2 (129 MB): no flush")


def device_resident(sim, tank, args, pg, local):
    """ms of `steps` substeps after `warmup`, CUDA events on the sim's stream (max over ranks)."""
    dt = 1.0 / 240.0
    for _ in range(args.warmup):
        sim.step(1, dt)
    sim.sync()
    flush, _ = l2_note(tank)
    barrier(pg)
    sim.sync()
    if flush:
        import torch
        scratch = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
        ms = 0.0
        for _ in range(args.steps):
            scratch.fill_(1)
            torch.cuda.synchronize()
            ms += sim.profile(1)
        del scratch
    else:
        ms = sim.profile(args.steps)
    sim.sync()
    barrier(pg)
    return allreduce_max(pg, ms)


def end_to_end(tank, args, pg):
    """The same metric through the public API on a fresh copy of the tank, over the same
    substep indices as the device-resident timing (warmup, then steps): each step call
    uploads its inputs (the step's batch words, parameters when they change) and reads the
    step's result back (the solver statistics), all inside the timed region."""
    sim, _, _ = tank.engine()
    dt = 1.0 / 240.0
    for _ in range(args.warmup):
        sim.step(1, dt)
    sim.sync()
    live = sim.stats().n_live
    h0 = sim.stats()
    lat = []
    barrier(pg)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        a = time.perf_counter()
        sim.step(1, dt)
        sim.stats()               # the step's result read back to the host (blocking)
        lat.append(time.perf_counter() - a)
    el = time.perf_counter() - t0
    el = allreduce_max(pg, el)
    h1 = sim.stats()
    value = allreduce_sum(pg, float(live)) * args.steps / el
    return {"value": value, "unit": UNIT,
            "h2d_bytes_per_step": (h1.h2d_bytes - h0.h2d_bytes) / args.steps,
            # h1's own read is counted in h1 - h0 with the loop's reads, all the same size
            "d2h_bytes_per_step": (h1.d2h_bytes - h0.d2h_bytes) / (args.steps + 1),
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "substeps": f"{args.warmup + 1}..{args.warmup + args.steps} of a fresh copy of the tank (as value)"}


def run_batched(args, pg, rank: int = 0, world: int = 1) -> dict:
    """The batched configuration: 64 seeded dam breaks of uneven sizes (128 x 72 .. 1024 x
    576), one or two liquids each from the full-physics ranges, mixed precision, stepped as
    one batch (one captured graph per substep, the solves as persistent kernels over the
    flattened tile lists); then the same tanks in plain FP32. Under torchrun each rank steps
    its share of the tanks (sprout_gb300.placement), with no exchange on the data path."""
    import sprout_gb300 as S
    from sprout_gb300 import placement
    from sprout_gb300 import workloads as WL
    t0 = time.perf_counter()
    tanks = WL.uneven_dam_breaks(args.batch_tanks, seed=0)
    mine = placement.my_tanks(tanks, rank, world)
    sims = [tanks[i].engine()[0] for i in mine]
    b = S.Batch(sims, "mixed")
    setup = time.perf_counter() - t0
    out = {"workload": f"{len(tanks)} uneven dam breaks (128x72..1024x576, 1-2 config-3 liquids), seed 0",
           "setup_s": setup, "placement": f"{len(mine)} of {len(tanks)} tanks on this rank (greedy by cells + particles/4)"}
    from sprout_gb300 import bytes_model as BM
    unknowns = None
    for prec in ("mixed", "plain"):
        b.set_precision(prec)
        b.step(args.warmup)
        b.sync()
        live = sum(s.stats().n_live for s in sims)
        barrier(pg)
        ms = allreduce_max(pg, b.profile(args.steps))
        sts = [s.stats() for s in sims]
        if unknowns is None:   # level-0 unknowns of each tank's pressure system
            unknowns = [int(np.count_nonzero(s_.field("mgd")[: s_.w * s_.h] > 0.0)) for s_ in sims]
        # the algorithmic bytes of the last substep's batched pressure launches (both solves),
        # from each tank's iterations: the numerator of the batched solver's roofline
        pbytes = sum(BM.pressure_bytes(u, max(x.pressure_iters)) for u, x in zip(unknowns, sts))
        pbytes2 = sum(u * (44 + (x.pressure2_iters + 1) * BM.PRESSURE_ITER) for u, x in zip(unknowns, sts)
                      if x.pressure2_iters > 0)
        out[prec] = {"value": allreduce_sum(pg, float(live)) * args.steps / (ms / 1e3), "unit": UNIT,
                     "ms_per_step": ms / args.steps, "particles": int(live),
                     "pressure_unconverged": int(sum(x.pressure_unconverged for x in sts)),
                     "device_errors": int(sum(1 for x in sts if x.device_error)),
                     "pressure_algorithmic_bytes_last_substep": {"first_solve": pbytes, "second_solve": pbytes2}}
        if prec == "mixed":
            out[prec]["pressure_true_residual_max_fp64"] = float(max(x.pressure_true_residual_max for x in sts))
    out["launch"] = {"batch_blocks": "one per tile of the tanks, at most what fits (2 per SM)"}
    b.close()
    # the same tanks on the single-scene path, one after another, plain FP32: each tank's own
    # captured substep, `steps` substeps each after 2 more warm-up substeps
    seq_ms = 0.0
    for s_ in sims:
        s_.set_precision("plain")
        s_.step(2, 2 / 240.0)
        seq_ms += s_.profile(args.steps)
    live = sum(s_.stats().n_live for s_ in sims)
    seq_ms = allreduce_max(pg, seq_ms)
    out["plain_single_scene"] = {"value": allreduce_sum(pg, float(live)) * args.steps / (seq_ms / 1e3), "unit": UNIT,
                                 "ms_per_step": seq_ms / args.steps,
                                 "how": "the same tanks stepped one at a time through their own captured substeps, plain FP32"}
    out["ratio_mixed_batched_vs_plain_single_scene"] = out["mixed"]["value"] / out["plain_single_scene"]["value"]
    for s_ in sims:
        s_.close()
    return out


def run_serving(args) -> dict:
    """The serving mix: a seeded Poisson stream of scene-step requests (1-8 substeps each) at
    `serve_rate` per second over resident tanks whose sizes follow the mix's weights, mixed
    precision, continuous batching (sprout_gb300.serving)."""
    from sprout_gb300 import serving
    r = serving.run(scenes=args.serve_tanks, rate=args.serve_rate, seconds=args.serve_seconds, precision="mixed")
    r["target_p99_ms"] = 16.0
    return r


def stage_runs(sim, substeps: int = 5) -> list:
    """(per-stage device ms, stats after it) of `substeps` consecutive ungraphed substeps, each
    stage bracketed by CUDA events: one substep's figures move with host launch jitter, so the
    line reports medians."""
    return [(sim.profile_passes(), sim.stats()) for _ in range(substeps)]


def median_stages(runs) -> dict:
    return {k: float(np.median([r[0][k] for r in runs])) for k in runs[0][0]}


def draw_timing(sim, tank) -> dict:
    """The renderer's particle fields (sprout_sim_draw: the splat and tint fields, the wide
    field, the wet map) for a 1920 x 1080 view of the whole tank after the timed substeps: host
    ms per call including a sync, median of 10 after 3."""
    import time
    zoom = min(1920.0 / tank.w, 1080.0 / tank.h)
    center = (tank.w * 0.5, tank.h * 0.5)
    for _ in range(3):
        sim.draw(center, zoom, (1920, 1080))
    sim.sync()
    ts = []
    for _ in range(10):
        t0 = time.perf_counter()
        sim.draw(center, zoom, (1920, 1080))
        sim.sync()
        ts.append((time.perf_counter() - t0) * 1e3)
    sharp, tint = sim.download_draw("sharp"), sim.download_draw("tint")
    return {"view": "1920x1080", "zoom_px_per_cell": zoom, "ms_median": float(np.median(ts)), "ms_min": float(min(ts)),
            "sharp_texels": list(sharp.shape[1::-1]), "tint_texels": None if tint is None else list(tint.shape[1::-1]),
            "kernels": "k_splat x2, k_fields_out x2, k_down, k_blur x2, k_wet_clock, k_wet"}


def run_engine(args, rank, world, local, pg):
    import sprout_gb300 as S
    from sprout_gb300 import bytes_model as BM
    try:
        import torch
        torch.cuda.set_device(local)
    except Exception:
        pass
    tank, desc = workload(args.workload, rank)
    sim, parts, _ = tank.engine()
    live = None
    with Clocks(local) as clk:
        ms = device_resident(sim, tank, args, pg, local)
    st1 = sim.stats()
    live = st1.n_live
    live_all = allreduce_sum(pg, float(live))
    value = live_all * args.steps / (ms / 1e3)
    run = {"particles": int(live), "pressure_iters_last": list(st1.pressure_iters),
           "pressure_residual": st1.pressure_residual, "pressure_unconverged": st1.pressure_unconverged,
           "viscosity_iters_last": st1.viscosity_iters, "viscosity_residual": st1.viscosity_residual,
           "viscosity_unconverged": st1.viscosity_unconverged, "pressure2_iters_last": st1.pressure2_iters,
           "launch": sim.launch()}
    # ---- per-stage times (CUDA events) and the roofline of the dominant stage ---------------
    runs = stage_runs(sim)
    stages = median_stages(runs)
    hbm, src = peaks()
    unknowns = int(np.count_nonzero(sim.field("mgd")[: tank.w * tank.h] > 0))
    top = max(stages, key=stages.get)
    st2 = runs[-1][1]
    active = active_viscosity_cells(sim, tank.w, tank.h) if st2.viscosity_mode == 2 else 0
    run["viscosity_active_cells"] = active
    per = []   # (achieved GB/s, algorithmic bytes, stage ms) of each profiled substep
    for ms_k, stk in runs:
        algo_k = BM.stage_bytes(top, stk.n_live, tank.w * tank.h, unknowns,
                                max(stk.pressure_iters[0], stk.pressure_iters[1]), stk.acc_stride,
                                bool(stk.thermal), stk.viscosity_mode, active_cells=active,
                                visc_iterations=stk.viscosity_iters, iterations2=stk.pressure2_iters)
        per.append((algo_k / (ms_k[top] * 1e-3) / 1e9, algo_k, ms_k[top]))
    achieved, algo, top_ms = sorted(per)[len(per) // 2]
    roof = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "peak_source": src, "traffic": None,
            "algorithmic_bytes": algo, "stage_ms": top_ms,
            "sample": f"median over {len(per)} profiled substeps of the stage's algorithmic bytes / its time"}
    traffic_file = ROOT / "profiles" / "traffic.json"
    if traffic_file.exists():
        tr = json.loads(traffic_file.read_text())
        v = tr.get(args.workload, {}).get(top)
        if v:
            roof["traffic"] = v
            roof["traffic_source"] = (f"profiles/traffic.json: dram__bytes_read.sum + dram__bytes_write.sum of one "
                                      f"launch of this stage's kernel on this workload ({tr.get('command', 'ncu')}), "
                                      "not measured in this run")
    # ---- the mixed-precision solve on the same tank (BF16 matrices, FP64 scalars) -----------
    mixed = None
    if args.precision in ("both", "mixed"):
        msim, _, _ = tank.engine()
        msim.set_precision("mixed")
        mms = device_resident(msim, tank, args, pg, local)
        mst = msim.stats()
        mlive = mst.n_live
        mstages = median_stages(stage_runs(msim))
        mixed = {"value": allreduce_sum(pg, float(mlive)) * args.steps / (mms / 1e3), "unit": UNIT,
                 "ms_per_step": mms / args.steps, "stages_ms": mstages,
                 "pressure_iters_last": list(mst.pressure_iters), "pressure2_iters_last": mst.pressure2_iters,
                 "pressure_residual_max": mst.pressure_residual_max, "pressure_unconverged": mst.pressure_unconverged,
                 "pressure_true_residual_max_fp64": mst.pressure_true_residual_max,
                 "refinement": {"residual_replacements": mst.pressure_replacements,
                                "rule": "true residual b - A x (float-pair products and sums of the FP32 values) checked each time the "
                                        "carried |r| falls 100x; adopted where it exceeds twice the carried one and "
                                        "ten times the FP32 rounding floor eps |A| |x|"},
                 "storage": "BF16 couplings + FP32 row-sum-keeping diagonal on every level; FP32 vectors",
                 "dots": "FP32 sums (the plain solve's trees), FP64 totals, step lengths and convergence test",
                 "speedup_vs_plain": (ms / args.steps) / (mms / args.steps)}
    # ---- end to end through the public API, on a fresh copy over the same substeps ----------
    e2e = end_to_end(tank, args, pg)
    draw = draw_timing(sim, tank)
    batched = run_batched(args, pg, rank, world) if args.batch_tanks > 0 else None
    serving_r = run_serving(args) if (args.serve_seconds > 0 and world == 1) else None
    if rank != 0:
        return
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded tank, no dataset)", "config": desc,
            "parallelism": f"replicas x{world}", "run": run,
            "clocks": clk.summary(), "e2e": e2e, "gpu_launches": kernels_per_substep(st2, tank.settings) * args.steps,
            "roofline": roof, "stages_ms": stages, "latency_ms": {"p50": e2e["p50_ms"], "p99": e2e["p99_ms"]}}
    line["draw"] = draw
    if mixed is not None:
        line["mixed"] = mixed
    if batched is not None:
        batched["ratio_mixed_batched_vs_plain_single"] = batched["mixed"]["value"] / value
        batched["ratio_plain_batched_vs_plain_single"] = batched["plain"]["value"] / value
        batched["target_ratio"] = 3.0
        line["batched"] = batched
    if serving_r is not None:
        line["serving"] = serving_r
    if not args.no_cpu_baseline:
        # the checkers, on the host: the oracle's rate, and the FP64 reference solution of each
        # arm's last pressure system
        cb, _, _ = cpu_oracle_rate(tank)
        line["cpu_baseline"] = cb
        from oracle.fp64_mgpcg import FP64MGPCG, accuracy
        acc = {}
        for name, s_ in [("plain", sim)] + ([("mixed", msim)] if mixed is not None else []):
            a = accuracy(s_.field("mga"), s_.field("mgd"), s_.field("prhs"), s_.field("pres"), tank.w, tank.h, columns=(0,))
            f = FP64MGPCG(s_.field("mga"), s_.field("mgd"), tank.w, tank.h)
            b = np.asarray(s_.field("prhs"), np.float64).reshape(tank.h, tank.w, 4)[..., :2]
            x64, _ = f.solve(b)
            floor = float(f.residual(x64.astype(np.float32).astype(np.float64), b)[0])
            acc[name] = {"pressure_error_vs_fp64": a[0]["error_vs_fp64"], "pressure_residual_fp64": a[0]["residual_fp64"],
                         "fp32_floor": floor}
        acc["system"] = "the last pressure solve of each arm's tank, solved again by an FP64 MGPCG to 1e-12"
        acc["fp32_floor"] = ("|b - A fl32(x*)| / |b|: the true residual that rounding the FP64 solution x* to FP32 "
                             "leaves, the scale below which no FP32 iterate's true residual goes")
        line["accuracy"] = acc
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="full_physics_1024",
                    choices=["full_physics_1024", "stratified_512", "dam_break_1024", "dam_break_384"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", default="both", choices=["plain", "mixed", "both"],
                    help="plain: the reference's FP32 arithmetic (the headline value); mixed: also time "
                         "the mixed-precision pressure solve on the same tank (reported under 'mixed')")
    ap.add_argument("--batch-tanks", type=int, default=64,
                    help="tanks of the batched configuration's leg (0: skip it)")
    ap.add_argument("--serve-seconds", type=float, default=10.0,
                    help="seconds of the serving mix's arrival stream (the configuration runs 60; 0: skip it)")
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--serve-tanks", type=int, default=512)
    ap.add_argument("--batch-only", action="store_true",
                    help="run only the batched configuration's leg and print it (a profiler's capture of the "
                         "batched solves)")
    ap.add_argument("--draw-only", action="store_true",
                    help="step the workload five substeps, time only the renderer's particle fields for a "
                         "1920 x 1080 view of it and print them (a profiler's capture of the draw)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local, pg = dist_setup(args.gpus)
    try:
        if args.impl == "reference":
            run_reference(args, rank, world, pg)
        else:
            from sprout_gb300 import build
            build.build()
            if args.batch_only:
                print(json.dumps({"batched": run_batched(args, pg, rank, world)}), flush=True)
            elif args.draw_only:
                tank, _ = workload(args.workload, rank)
                sim, _, _ = tank.engine()
                sim.step(5, 5 / 240.0)
                sim.sync()
                print(json.dumps({"draw": draw_timing(sim, tank)}), flush=True)
            else:
                run_engine(args, rank, world, local, pg)
    finally:
        if pg is not None:
            pg.destroy_process_group()


if __name__ == "__main__":
    main()

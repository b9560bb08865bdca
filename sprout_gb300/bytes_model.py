"""Algorithmic bytes of each stage of a substep: the unique bytes a stage must move (every
field it needs read once, every field it produces written once), in the FP32 engine's own
layouts. These are the numerators of the roofline figures the benchmark reports; traffic
measured by ncu above them means re-reads.

Per live particle (48-byte records): advance reads and writes the particle (96) and writes
its new cell and rank (8); the sort moves it once more (96) with its permutation entry
(4 written, 4 read, 4 read by the placement); P2G reads it once (48).
Per cell: see the per-stage tables below (float4 records = 16 bytes).
"""
from __future__ import annotations

PARTICLE = {"advance": 48 + 48 + 8, "sort": 8 + 4 + 4 + 4 + 48 + 48, "p2g": 48}


def cell_bytes(stage: str, stride: int, thermal: bool, visc_mode: int) -> int:
    """Bytes per grid cell of one launch of `stage`."""
    if stage == "advance":
        return 16 + 16 + 4 + (32 if thermal else 0)          # vel, comp, sdf (+ dheat, hcell)
    if stage == "sort":
        return 4 + 4 + 4 + 4 + 4 + 4                          # count clear + read, start write + read + add
    if stage == "p2g":
        return 4 + 4 * stride                                  # start (row ranges), accumulators written once
    if stage == "grid":
        prep = 4 * stride + 16 + 16 + 8 + 16 + 16 + 16 + (32 if thermal else 0) + 8
        coef_smooth = 16 + 16 + 16 + 8 + 16
        curv = 8 + 16 + 4 + 8 + 16
        apply = 16 + 16 + 16 + 16 + 8
        heat = (16 * 5 + 8 + 4) if thermal else 0
        visc = (16 + 16 + 16 + 16 + 16 + 16 + 8) if visc_mode == 1 else 0
        if visc_mode == 2:   # visc_setup, split, diag with the level-0 matrix, coarse builds
            visc = (16 + 16 + 16 + 16 + 16) + (16 + 16 + 16 + 8) + (16 + 16 + 8 + 8 + 16 + 16 + 8 + 16) + 20
        rhs = 16 + 16 + 16 + 16 + 8 + 16 + 4 + 8 + 16 + 4 + 16
        return prep + coef_smooth + curv + apply + heat + visc + rhs
    if stage == "project":
        return 16 + 16 + 8 + 16 + 8 + 4 + 4 + 16
    raise KeyError(stage)


# The pressure solve, per level-0 unknown: the set-up (warm-start scaling 16, the residual
# r = b - A x with its matrix row 20 + x 8 + b 8 + r 8, the coarse-matrix build 0.33 of a
# row 20 + 20), then per iteration: apply (z 8, p_old 8, matrix 20, p 8, q 8 = 52), update
# fused with the way down (x 8 + 8, p 8, r 8 + 8, q 8, z_pre 8, coarse rhs 2 = 58), the way up
# (rhs 8, z_pre 8, coarse z 2, matrix 20, z 8 = 46): 156 on level 0, and a third more on the
# coarser levels (the hierarchy holds 1/3 of the cells again).
PRESSURE_SETUP = 16 + 44 + 14
PRESSURE_ITER_L0 = 52 + 58 + 46
PRESSURE_ITER = PRESSURE_ITER_L0 + (38 + 46) / 3.0


def pressure_bytes(unknowns: int, iterations: int) -> float:
    return unknowns * (PRESSURE_SETUP + (iterations + 1) * PRESSURE_ITER)


# The implicit viscosity solve, per cell of an active tile (both faces, float2 vectors of 8
# bytes, the level-0 matrix 16 + 16 + 8 = 40): set-up (strain: vw 16, vel 16, vs 16; start:
# vs 16, coef 16, vw 16, r 8, z 8; warm start: vd 8, vw 16, coef 16, vel 16 + 8, r 8 + 8; the
# first way down and up as one iteration's) and per iteration: the update fused with the way
# down (z 8, p 8 + 8, A z 8, q 8 + 8, r 8 + 8, vel 16 + 8, vd 8 + 8, matrix 40, vmx 8, coarse
# rhs 2 = 162), the way up with A z (r 8, matrix 40, vmx 8, coarse z 2, q 8, z 8, A z 8 = 82)
# and the coarse levels a quarter of the cells each way (down 58 + up 66) / 4.
VISC_SETUP = 48 + 64 + 104
VISC_ITER = 162 + 82 + (58 + 66) / 4.0


def viscosity_bytes(active_cells: int, iterations: int) -> float:
    return active_cells * (VISC_SETUP + (iterations + 1) * VISC_ITER)


# The second projection: rhs_visc per cell (mgd 4 + 4 x 4, mga 16, prhs 16 + 16 + neighbours'
# P1 16, solid 16 x 3, vel 16 x 3 = 180 read, prhs 16 + pres 8 + p2keep 4 written), the
# second pressure solve on the same hierarchy (no build, no scaling), project_visc per cell
# (mgd 4 x 3, pres 8 x 3, prhs 16 x 3, coef 16, vel 16 + 8, p2keep 4 = 128).
PROJECT2_CELL = 180 + 28 + 128


def stage_bytes(stage: str, particles: int, cells: int, unknowns: int, iterations: int, stride: int,
                thermal: bool, visc_mode: int, active_cells: int = 0, visc_iterations: int = 0,
                iterations2: int = 0) -> float:
    if stage == "pressure":
        return pressure_bytes(unknowns, iterations)
    if stage == "viscosity":
        return viscosity_bytes(active_cells, visc_iterations)
    if stage == "project2":
        return cells * PROJECT2_CELL + unknowns * (44 + (iterations2 + 1) * PRESSURE_ITER)
    return particles * PARTICLE.get(stage, 0) + cells * cell_bytes(stage, stride, thermal, visc_mode)

"""Admission of new liquid under a brush: which cells of a window may take more particles.

The caller of FluidSim::cell_counts (src/world.rs:729-736): the window around a stroke
(Admission::window, src/brush.rs:219-224), clamped to the grid, the live particles per cell of
that window read back from the engine (count.comp, one integer per cell, no particle read
back), and the room that leaves each cell (Admission::new / admit, src/brush.rs:209-238):
painted liquid only fills empty cells, up to rest density; a stream fills cells up to
STREAM_FILL times rest density.
"""
from __future__ import annotations

import math

import numpy as np

PPC = 4               # particles per cell at rest density (src/sim/params.rs:11)
STREAM_FILL = 1.5     # src/brush.rs:11


def window(frm, to, margin: float) -> tuple[list[int], list[int]]:
    """The cells [lo, hi) covering everything within `margin` of the segment frm-to, in the
    reference's f32 arithmetic (brush.rs:219-224)."""
    f = [np.float32(v) for v in frm]
    t = [np.float32(v) for v in to]
    m = np.float32(margin)
    lo = [int(math.floor(min(f[k], t[k]) - m)) for k in range(2)]
    hi = [int(math.ceil(max(f[k], t[k]) + m)) + 1 for k in range(2)]
    return lo, hi


class Admission:
    """Room per cell of a window at `lo`, `size` cells across (brush.rs:203-238)."""

    def __init__(self, lo, size, counts, ppc: int = PPC, stream: bool = False):
        self.lo = [int(lo[0]), int(lo[1])]
        self.size = [int(size[0]), int(size[1])]
        counts = np.asarray(counts, np.int64).ravel()
        if stream:
            full = int(np.float32(ppc) * np.float32(STREAM_FILL))
            self.room = np.maximum(full - counts, 0)
        else:
            self.room = np.where(counts == 0, ppc, 0)

    def admit(self, pos) -> bool:
        """Takes one particle's worth of room at `pos`, if its cell has any left."""
        cx = int(math.floor(np.float32(pos[0]))) - self.lo[0]
        cy = int(math.floor(np.float32(pos[1]))) - self.lo[1]
        if cx < 0 or cy < 0 or cx >= self.size[0] or cy >= self.size[1]:
            return False
        k = cy * self.size[0] + cx
        if self.room[k] == 0:
            return False
        self.room[k] -= 1
        return True


def for_stroke(sim, frm, to, margin: float, stream: bool) -> Admission:
    """World::admission (src/world.rs:729-736): the stroke's window clamped to the grid (a
    stroke wholly past the edge gets an empty window), filled from sim.cell_counts."""
    lo, hi = window(frm, to, margin)
    gw, gh = sim.w, sim.h
    lo = [min(max(lo[0], 0), gw), min(max(lo[1], 0), gh)]
    hi = [min(max(hi[0], lo[0]), gw), min(max(hi[1], lo[1]), gh)]
    counts = sim.cell_counts(lo, hi)
    return Admission(lo, [hi[0] - lo[0], hi[1] - lo[1]], counts, PPC, stream)

"""FP64 reference solve of the pressure system: multigrid-preconditioned CG in double precision.

Test and measurement infrastructure (the tests' checker and the benchmark's accuracy figure),
never part of the engine. It takes the level-0 system the engine (or the oracle) assembled —
the 5-point matrix of rhs.comp as couplings `mga` (left, right, down, up) and diagonal `mgd`,
unknowns where mgd > 0, right-hand sides prhs.xy (pressure * dt and the density-correction
potential) — and solves A x = b for both columns to a relative residual of 1e-12 in FP64,
so that the FP32 and mixed-precision solutions can be stated as an error against it.

The preconditioner is the same kind as the reference's (mg.glsl): 2 x 2 aggregation with
Galerkin coarse matrices (mg_build.comp), symmetric red-black Gauss-Seidel (red then black on
the way down, black then red on the way up), down to a few cells, all in FP64 numpy arrays.
"""
from __future__ import annotations

import numpy as np

# neighbour q: 0 left (x - 1), 1 right (x + 1), 2 below (y - 1), 3 above (y + 1)
OMEGA = 1.8   # coarse-correction weight, as mg_up.comp
NB = [(-1, 0), (1, 0), (0, -1), (0, 1)]


def _nb(a: np.ndarray, dx: int, dy: int) -> np.ndarray:
    """out[y, x] = a[y + dy, x + dx], zero outside."""
    out = np.zeros_like(a)
    h, w = a.shape[:2]
    ys, yd = slice(max(0, dy), h + min(0, dy)), slice(max(0, -dy), h - max(0, dy))
    xs, xd = slice(max(0, dx), w + min(0, dx)), slice(max(0, -dx), w - max(0, dx))
    out[yd, xd] = a[ys, xs]
    return out


class Level:
    def __init__(self, D: np.ndarray, W: np.ndarray):
        self.D = D                          # (h, w)
        self.unk = D > 0.0
        # couplings only between unknowns
        self.W = np.stack([W[q] * self.unk * _nb(self.unk, *NB[q]) for q in range(4)])
        self.red = (np.add.outer(np.arange(D.shape[0]), np.arange(D.shape[1])) & 1) == 0
        self.inv = np.where(self.unk, 1.0 / np.where(self.unk, D, 1.0), 0.0)

    def apply(self, x: np.ndarray) -> np.ndarray:
        y = self.D[..., None] * x
        for q in range(4):
            y -= self.W[q][..., None] * _nb(x, *NB[q])
        return y * self.unk[..., None]

    def sweep(self, x: np.ndarray, b: np.ndarray, red: bool) -> np.ndarray:
        s = b.copy()
        for q in range(4):
            s += self.W[q][..., None] * _nb(x, *NB[q])
        m = (self.red if red else ~self.red) & self.unk
        return np.where(m[..., None], s * self.inv[..., None], x)

    def coarse(self) -> "Level":
        h, w = self.D.shape
        hc, wc = (h + 1) // 2, (w + 1) // 2
        pad = lambda a: np.pad(a, ((0, 2 * hc - h), (0, 2 * wc - w)))
        D = pad(self.D * self.unk)
        Wq = [pad(self.W[q]) for q in range(4)]
        ys, xs = np.meshgrid(np.arange(2 * hc), np.arange(2 * wc), indexing="ij")
        Dc = D.reshape(hc, 2, wc, 2).sum(axis=(1, 3))
        Ac = np.zeros((4, hc, wc))
        for q, (dx, dy) in enumerate(NB):
            inside = ((xs + dx) >> 1 == xs >> 1) & ((ys + dy) >> 1 == ys >> 1)
            Dc -= (Wq[q] * inside).reshape(hc, 2, wc, 2).sum(axis=(1, 3))
            Ac[q] = (Wq[q] * ~inside).reshape(hc, 2, wc, 2).sum(axis=(1, 3))
        keep = Dc > 1e-12
        return Level(np.where(keep, Dc, 0.0), Ac * keep)


def _prolong(xc: np.ndarray, shape) -> np.ndarray:
    return np.repeat(np.repeat(xc, 2, axis=0), 2, axis=1)[: shape[0], : shape[1]]


def _restrict(r: np.ndarray, shape_c) -> np.ndarray:
    hc, wc = shape_c
    h, w = r.shape[:2]
    rp = np.pad(r, ((0, 2 * hc - h), (0, 2 * wc - w), (0, 0)))
    return rp.reshape(hc, 2, wc, 2, r.shape[2]).sum(axis=(1, 3))


class FP64MGPCG:
    def __init__(self, mga: np.ndarray, mgd: np.ndarray, w: int, h: int):
        D = np.asarray(mgd[: w * h], np.float64).reshape(h, w)
        A = np.asarray(mga[: 4 * w * h], np.float64).reshape(h, w, 4)
        self.levels = [Level(D, np.moveaxis(A, 2, 0))]
        while self.levels[-1].D.size > 16:
            self.levels.append(self.levels[-1].coarse())

    def vcycle(self, b: np.ndarray, l: int = 0) -> np.ndarray:
        L = self.levels[l]
        x = np.zeros_like(b)
        if l == len(self.levels) - 1:
            for k in range(40):
                x = L.sweep(x, b, k % 2 == 0)
            for k in range(40):
                x = L.sweep(x, b, k % 2 == 1)
            return x
        x = L.sweep(x, b, True)
        x = L.sweep(x, b, False)
        r = (b - L.apply(x)) * L.unk[..., None]
        xc = self.vcycle(_restrict(r, self.levels[l + 1].D.shape), l + 1)
        x = x + OMEGA * _prolong(xc, L.D.shape) * L.unk[..., None]
        x = L.sweep(x, b, False)
        x = L.sweep(x, b, True)
        return x

    def solve(self, b: np.ndarray, tol: float = 1e-12, max_iters: int = 400):
        """Both columns of b (h, w, 2) at once, each with its own step lengths. Returns x and
        the relative residual reached per column."""
        L0 = self.levels[0]
        b = np.asarray(b, np.float64) * L0.unk[..., None]
        x = np.zeros_like(b)
        r = b.copy()
        bb = np.einsum("ijk,ijk->k", b, b)
        z = self.vcycle(r)
        p = z.copy()
        rz = np.einsum("ijk,ijk->k", r, z)
        for _ in range(max_iters):
            rr = np.einsum("ijk,ijk->k", r, r)
            if np.all(rr <= tol * tol * np.maximum(bb, 1e-300)):
                break
            q = L0.apply(p)
            pq = np.einsum("ijk,ijk->k", p, q)
            alpha = np.where(pq > 0, rz / np.where(pq > 0, pq, 1.0), 0.0)
            x += alpha * p
            r -= alpha * q
            z = self.vcycle(r)
            rz_new = np.einsum("ijk,ijk->k", r, z)
            beta = np.where(rz > 0, rz_new / np.where(rz > 0, rz, 1.0), 0.0)
            p = z + beta * p
            rz = rz_new
        res = b - L0.apply(x)
        rel = np.sqrt(np.einsum("ijk,ijk->k", res, res) / np.maximum(bb, 1e-300))
        return x, rel

    def residual(self, x: np.ndarray, b: np.ndarray) -> np.ndarray:
        """Relative residual |b - A x| / |b| per column, in FP64, of a given solution."""
        L0 = self.levels[0]
        b = np.asarray(b, np.float64) * L0.unk[..., None]
        r = b - L0.apply(np.asarray(x, np.float64) * L0.unk[..., None])
        bb = np.einsum("ijk,ijk->k", b, b)
        return np.sqrt(np.einsum("ijk,ijk->k", r, r) / np.maximum(bb, 1e-300))


def accuracy(mga, mgd, prhs, pres, w: int, h: int, columns=(0, 1)) -> dict:
    """The FP64 reference solution of the last pressure system and the error of `pres` (the
    engine's solution, (w*h, 2)) against it, per column: relative L2 error over the unknowns
    and the relative residual of `pres` in FP64."""
    s = FP64MGPCG(mga, mgd, w, h)
    b = np.asarray(prhs, np.float64).reshape(h, w, 4)[..., :2]
    x64, rel64 = s.solve(b)
    xe = np.asarray(pres, np.float64).reshape(h, w, 2) * s.levels[0].unk[..., None]
    res_e = s.residual(xe, b)
    out = {}
    for c in columns:
        nrm = np.linalg.norm(x64[..., c])
        out[c] = {"error_vs_fp64": float(np.linalg.norm(xe[..., c] - x64[..., c]) / nrm) if nrm > 0 else 0.0,
                  "residual_fp64": float(res_e[c]), "fp64_residual": float(rel64[c])}
    return out

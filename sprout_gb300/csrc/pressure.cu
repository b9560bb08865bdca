// The pressure solve as ONE persistent cooperative kernel per solve on sm_103a.
//
// Multigrid-preconditioned conjugate gradients on the two potentials (pressure * dt and
// the density-correction potential) side by side, each with its own step lengths and
// convergence flag (reduce_tail.glsl:61-116), preconditioned by an aggregation V-cycle:
// Galerkin 2 x 2 coarse matrices (mg_build.comp:147-197, mg_tail.comp:44-70), red-black
// Gauss-Seidel from zero on the way down with restriction of the residual (mg_down.comp),
// coarse correction with omega = 1.8 and the mirrored sweep on the way up (mg_up.comp),
// and the small levels (<= 1500 cells) in one thread block (mg_tail.comp:159-225).
//
// What the reference spreads over ~15 dispatches and barriers per iteration, with a
// host-recorded iteration count, runs here inside one kernel with a device-decided exit:
// the phases are separated by a grid-wide barrier (bounded spin; on timeout every block
// sets the error word and leaves), every block computes the solve's scalars itself from the
// per-tile partial sums (the same work-group trees and strided totals as
// reduce.glsl / reduce_tail.glsl, so every block gets identical values), and the residual
// update of conjugate gradients is fused into the first restriction of the next V-cycle by
// double-buffering the level-0 residual.
#include <cuda_runtime.h>

#include "dev_common.cuh"
#include "kernels.h"
#include "solve_common.cuh"

namespace sprout {

namespace {

using namespace solve;

__constant__ int NBX[4] = {-1, 1, 0, 0};
__constant__ int NBY[4] = {0, 0, -1, 1};

struct Solve {
    float rz[2], alpha[2], beta[2], bb[2], rr[2];
    uint32_t done[2], iters[2];
};

struct Ctx {
    DevScene d;
    Lv L0;
};

// ---- setup phases ---------------------------------------------------------------------

// cg_scale.comp: warm start from last substep's potential rescaled to this substep.
DEV void phase_cg_scale(const DevScene& d, int mode) {
    Lv F = lev(d.lv, 0);
    const float ratio = d.S->dt / d.S->dt_prev;
    const int T = tiles_x(F) * tiles_y(F);
    for (int t = blockIdx.x; t < T; t += gridDim.x) {
        if (d.ptile[F.toff + t] == 0u) continue;
        int cx = (t % tiles_x(F)) * 16 + (threadIdx.x & 15), cy = (t / tiles_x(F)) * 16 + (threadIdx.x >> 4);
        if (!l_inside(F, cx, cy)) continue;
        int i = l_at(F, cx, cy);
        if (d.mgd[i] > 0.0f) {
            float p = d.pres[i].x;
            if (mode == 1) p -= d.p2keep[i];
            else d.p2keep[i] = 0.0f;
            d.pres[i].x = p * ratio;
        } else {
            d.pres[i] = make_float2(0.0f, 0.0f);
        }
    }
}

DEV bool unknown(const DevScene& d, const Lv& L, int x, int y) { return l_inside(L, x, y) && d.mgd[l_at(L, x, y)] > 0.0f; }

// mg_build.comp: coarse level l + 1 from level l over the tiles of the coarse level.
DEV void phase_mg_build(const DevScene& d, int l) {
    Lv F = lev(d.lv, l), C = lev(d.lv, l + 1);
    const int tfx = tiles_x(F), tfy = tiles_y(F), tcx = tiles_x(C);
    const int T = tcx * tiles_y(C);
    __shared__ uint32_t s_state;
    for (int t = blockIdx.x; t < T; t += gridDim.x) {
        const int tx = t % tcx, ty = t / tcx;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t on = 0u;
            for (int k = 0; k < 4; k++) {
                int fx = 2 * tx + (k & 1), fy = 2 * ty + (k >> 1);
                if (fx < tfx && fy < tfy) on |= d.ptile[F.toff + fy * tfx + fx];
            }
            uint32_t slot = (uint32_t)C.toff + (uint32_t)t;
            uint32_t was = d.ptile[slot];
            d.ptile[slot] = on != 0u ? 1u : 0u;
            s_state = (on != 0u ? 1u : 0u) | (was != 0u ? 2u : 0u);
        }
        __syncthreads();
        const uint32_t state = s_state;
        if (state == 0u) continue;
        const int Cx = tx * 16 + (threadIdx.x & 15), Cy = ty * 16 + (threadIdx.x >> 4);
        if (Cx >= C.w || Cy >= C.h) continue;
        const int o = l_at(C, Cx, Cy);
        if ((state & 1u) == 0u) {
            d.mgd[o] = 0.0f;
            d.mga[o] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            continue;
        }
        float D = 0.0f;
        float4 A = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (int k = 0; k < 4; k++) {
            int cx = 2 * Cx + (k & 1), cy = 2 * Cy + (k >> 1);
            if (!unknown(d, F, cx, cy)) continue;
            int i = l_at(F, cx, cy);
            D += d.mgd[i];
            float4 w = d.mga[i];
            for (int q = 0; q < 4; q++) {
                int nx = cx + NBX[q], ny = cy + NBY[q];
                if (!unknown(d, F, nx, ny)) continue;
                float wd = wcomp(w, q);
                if ((nx >> 1) == Cx && (ny >> 1) == Cy) D -= wd;
                else if (q == 0) A.x += wd;
                else if (q == 1) A.y += wd;
                else if (q == 2) A.z += wd;
                else A.w += wd;
            }
        }
        d.mgd[o] = D > 1e-7f ? D : 0.0f;
        d.mga[o] = D > 1e-7f ? A : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// cg_init.comp: r = b - A x, partial sums of b.b into part[n + tile].
DEV void phase_cg_init(const DevScene& d, float2* r0, float4* buf) {
    Lv F = lev(d.lv, 0);
    const int T = tiles_x(F) * tiles_y(F);
    const int n = d.nwg;
    for (int t = blockIdx.x; t < T; t += gridDim.x) {
        if (d.ptile[F.toff + t] == 0u) {
            if (threadIdx.x == 0) d.partials[n + t] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            continue;
        }
        const int cx = (t % tiles_x(F)) * 16 + (threadIdx.x & 15), cy = (t / tiles_x(F)) * 16 + (threadIdx.x >> 4);
        float4 a4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (l_inside(F, cx, cy)) {
            const int i = l_at(F, cx, cy);
            const float D = d.mgd[i];
            if (D > 0.0f) {
                float2 x = d.pres[i];
                float4 w = d.mga[i];
                float axx = D * x.x, axy = D * x.y;
                for (int q = 0; q < 4; q++) {
                    int nx = cx + NBX[q], ny = cy + NBY[q];
                    if (unknown(d, F, nx, ny)) {
                        float wd = wcomp(w, q);
                        float2 pn = d.pres[l_at(F, nx, ny)];
                        axx -= wd * pn.x;
                        axy -= wd * pn.y;
                    }
                }
                float4 b = d.prhs[i];
                r0[i] = make_float2(b.x - axx, b.y - axy);
                a4 = make_float4(b.x * b.x, b.y * b.y, 0.0f, 0.0f);
            } else {
                r0[i] = make_float2(0.0f, 0.0f);
            }
        }
        buf[threadIdx.x] = a4;
        block_tree(buf);
        if (threadIdx.x == 0) d.partials[n + t] = buf[0];
        __syncthreads();
    }
}

// ---- the V-cycle --------------------------------------------------------------------------

// The residual of level-0 cell j as the next iterate sees it: fused with the update
// r -= alpha q of cg_update.comp, or as stored.
struct Rsrc {
    const float2* r;      // level-0 residual before the update (or the level's rhs)
    const float2* q;      // A p, for the fused update (null: no update)
    float ax, ay;
    DEV float2 at(int i) const {
        float2 v = r[i];
        if (q) {
            float2 qq = q[i];
            v.x = v.x - ax * qq.x;
            v.y = v.y - ay * qq.y;
        }
        return v;
    }
};

// mg_down black(): value of black cell n after the half-sweep from zero.
DEV float2 down_black(const DevScene& d, const Lv& L, const Rsrc& R, int nx, int ny) {
    int i = l_at(L, nx, ny);
    float4 w = d.mga[i];
    float2 sum = R.at(i);
    for (int q = 0; q < 4; q++) {
        int mx = nx + NBX[q], my = ny + NBY[q];
        if (!unknown(d, L, mx, my)) continue;
        int j = l_at(L, mx, my);
        float wd = wcomp(w, q);
        float2 rj = R.at(j);
        float dj = d.mgd[j];
        sum.x += wd * rj.x / dj;
        sum.y += wd * rj.y / dj;
    }
    float di = d.mgd[i];
    return make_float2(sum.x / di, sum.y / di);
}

// mg_down.comp on level l. On level 0 with `upd` it also applies cg_update.comp:
// x += alpha p and the residual update into r_out.
DEV void phase_down(const DevScene& d, int l, const Rsrc& R, float2* r_out, const float2* p, float2* sz) {
    Lv F = lev(d.lv, l), C = lev(d.lv, l + 1);
    const int tx_n = tiles_x(F);
    const int T = tx_n * tiles_y(F);
    const int lx = threadIdx.x & 15, ly = threadIdx.x >> 4;
    float2* mgr_c = d.mgr;   // coarse right-hand sides live at the coarse level's offset
    for (int t = blockIdx.x; t < T; t += gridDim.x) {
        if (d.ptile[F.toff + t] == 0u) continue;
        const int cx = (t % tx_n) * 16 + lx, cy = (t / tx_n) * 16 + ly;
        const bool red = ((cx + cy) & 1) == 0;
        float2 z = make_float2(0.0f, 0.0f);
        if (l_inside(F, cx, cy)) {
            const int i = l_at(F, cx, cy);
            const float D = d.mgd[i];
            if (D > 0.0f) {
                if (red) {
                    float2 r = R.at(i);
                    z = make_float2(r.x / D, r.y / D);
                } else {
                    z = down_black(d, F, R, cx, cy);
                }
                if (r_out) {
                    // cg_update.comp: x += alpha p, r -= alpha q (unknowns of active tiles)
                    float2 pp = p[i];
                    float2 x = d.pres[i];
                    x.x += R.ax * pp.x;
                    x.y += R.ay * pp.y;
                    d.pres[i] = x;
                    r_out[i] = R.at(i);
                }
            }
            d.mgx[i] = z;
        }
        sz[threadIdx.x] = z;
        __syncthreads();
        if (((lx | ly) & 1) == 0) {
            const int Cx = cx >> 1, Cy = cy >> 1;
            if (Cx < C.w && Cy < C.h) {
                float sx = 0.0f, sy = 0.0f;
                for (int k = 0; k < 2; k++) {
                    int qx = cx + k, qy = cy + k;
                    if (!unknown(d, F, qx, qy)) continue;
                    float4 w = d.mga[l_at(F, qx, qy)];
                    int lqx = lx + k, lqy = ly + k;
                    for (int q = 0; q < 4; q++) {
                        int nx = qx + NBX[q], ny = qy + NBY[q];
                        if (!unknown(d, F, nx, ny)) continue;
                        int lnx = lqx + NBX[q], lny = lqy + NBY[q];
                        bool here = lnx >= 0 && lny >= 0 && lnx < 16 && lny < 16;
                        float2 zb = here ? sz[lny * 16 + lnx] : down_black(d, F, R, nx, ny);
                        float wd = wcomp(w, q);
                        sx += wd * zb.x;
                        sy += wd * zb.y;
                    }
                }
                mgr_c[l_at(C, Cx, Cy)] = make_float2(sx, sy);
            }
        }
        __syncthreads();
    }
}

// The tail levels' state in each block's shared memory (dynamic): per tail cell the matrix
// row (couplings, diagonal), the iterate and the right-hand side, at its offset from the
// first tail level (the slots of mg_tail.comp).
struct Tail {
    float4* a;
    float* dg;
    float2* x;
    float2* r;
    int base, T, nf;
};

DEV bool t_unknown(const Tail& tl, const Lv& L, int x, int y) { return l_inside(L, x, y) && tl.dg[L.off - tl.base + y * L.w + x] > 0.0f; }

// mg_tail.comp mode 1 in every block's shared memory, once per solve: the first tail
// level's matrix from global memory, then the Galerkin matrices of the coarser tail levels
// (the arithmetic of mg_build.comp). Block 0 also stores them for inspection.
DEV void tail_setup(const DevScene& d, const Tail& tl) {
    for (int s = threadIdx.x; s < tl.nf; s += NT) {
        tl.a[s] = d.mga[tl.base + s];
        tl.dg[s] = d.mgd[tl.base + s];
    }
    __syncthreads();
    for (int l = d.lv.tail; l < d.lv.n - 1; l++) {
        Lv F = lev(d.lv, l), C = lev(d.lv, l + 1);
        const int o = F.off - tl.base, oc = C.off - tl.base;
        for (int t = threadIdx.x; t < C.w * C.h; t += NT) {
            int ccx = t % C.w, ccy = t / C.w;
            float D = 0.0f;
            float4 A = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            for (int k = 0; k < 4; k++) {
                int cx = 2 * ccx + (k & 1), cy = 2 * ccy + (k >> 1);
                if (!t_unknown(tl, F, cx, cy)) continue;
                int i = o + cy * F.w + cx;
                D += tl.dg[i];
                float4 w = tl.a[i];
                for (int q = 0; q < 4; q++) {
                    int nx = cx + NBX[q], ny = cy + NBY[q];
                    if (!t_unknown(tl, F, nx, ny)) continue;
                    float wd = wcomp(w, q);
                    if ((nx >> 1) == ccx && (ny >> 1) == ccy) D -= wd;
                    else if (q == 0) A.x += wd;
                    else if (q == 1) A.y += wd;
                    else if (q == 2) A.z += wd;
                    else A.w += wd;
                }
            }
            tl.dg[oc + t] = D > 1e-7f ? D : 0.0f;
            tl.a[oc + t] = D > 1e-7f ? A : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (blockIdx.x == 0) {
                d.mgd[C.off + t] = tl.dg[oc + t];
                d.mga[C.off + t] = tl.a[oc + t];
            }
        }
        __syncthreads();
    }
}

// mg_up black(): new value of black cell n after the coarse correction. The coarse level's
// finished values come from zc (row width zw): global memory, or this block's shared copy
// of the first tail level.
DEV float2 up_black(const DevScene& d, const Lv& L, const float2* zc, int zw, const float2* rhs, int nx, int ny) {
    int i = l_at(L, nx, ny);
    float4 w = d.mga[i];
    float2 sum = rhs[i];
    for (int q = 0; q < 4; q++) {
        int mx = nx + NBX[q], my = ny + NBY[q];
        if (!unknown(d, L, mx, my)) continue;
        float2 xm = d.mgx[l_at(L, mx, my)];
        float2 zcv = zc[(my >> 1) * zw + (mx >> 1)];
        float wd = wcomp(w, q);
        sum.x += wd * (xm.x + MG_OMEGA * zcv.x);
        sum.y += wd * (xm.y + MG_OMEGA * zcv.y);
    }
    float di = d.mgd[i];
    return make_float2(sum.x / di, sum.y / di);
}

// mg_up.comp on level l; on level 0 (flag) the partial sums r.z, r.r into part[tile].
DEV void phase_up(const DevScene& d, int l, bool flag, const float2* rhs, const float2* zc, float2* sz, float4* buf) {
    Lv F = lev(d.lv, l), C = lev(d.lv, l + 1);
    const int tx_n = tiles_x(F);
    const int T = tx_n * tiles_y(F);
    const int lx = threadIdx.x & 15, ly = threadIdx.x >> 4;
    for (int t = blockIdx.x; t < T; t += gridDim.x) {
        if (d.ptile[F.toff + t] == 0u) {
            if (flag && threadIdx.x == 0) d.partials[t] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            continue;
        }
        const int cx = (t % tx_n) * 16 + lx, cy = (t / tx_n) * 16 + ly;
        const bool red = ((cx + cy) & 1) == 0;
        const bool unk = unknown(d, F, cx, cy);
        float2 z = make_float2(0.0f, 0.0f);
        if (unk && !red) z = up_black(d, F, zc, C.w, rhs, cx, cy);
        sz[threadIdx.x] = z;
        __syncthreads();
        float4 a4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (l_inside(F, cx, cy)) {
            const int i = l_at(F, cx, cy);
            if (unk) {
                float2 r = rhs[i];
                if (red) {
                    float4 w = d.mga[i];
                    float sx = r.x, sy = r.y;
                    for (int q = 0; q < 4; q++) {
                        int nx = cx + NBX[q], ny = cy + NBY[q];
                        if (!unknown(d, F, nx, ny)) continue;
                        int lnx = lx + NBX[q], lny = ly + NBY[q];
                        bool here = lnx >= 0 && lny >= 0 && lnx < 16 && lny < 16;
                        float2 zb = here ? sz[lny * 16 + lnx] : up_black(d, F, zc, C.w, rhs, nx, ny);
                        float wd = wcomp(w, q);
                        sx += wd * zb.x;
                        sy += wd * zb.y;
                    }
                    float di = d.mgd[i];
                    z = make_float2(sx / di, sy / di);
                }
                a4 = make_float4(r.x * z.x, r.y * z.y, r.x * r.x, r.y * r.y);
            }
            d.mgz[i] = z;
        }
        if (flag) {
            buf[threadIdx.x] = a4;
            block_tree(buf);
            if (threadIdx.x == 0) d.partials[t] = buf[0];
        }
        __syncthreads();
    }
}

// mg_tail.comp mode 0, computed by EVERY block in its own shared memory: the V-cycle on the
// tail levels, right-hand side the first tail level's mgr, result left in tl.x (the first
// tail level's slots). Every block gets the same values; the way up of the level above
// reads them from its own copy, so no grid barrier follows the tail.
DEV void phase_tail(const DevScene& d, const Tail& tl) {
    const int first = d.lv.tail, last = d.lv.n - 1;
    for (int s = threadIdx.x; s < tl.nf; s += NT) tl.r[s] = d.mgr[tl.base + s];
    __syncthreads();
    auto sweep = [&](const Lv& L, int colour, bool zero) {
        const int o = L.off - tl.base;
        for (int t = threadIdx.x; t < L.w * L.h; t += NT) {
            int x = t % L.w, y = t / L.w;
            int s = o + t;
            float D = tl.dg[s];
            if (D <= 0.0f || ((x + y) & 1) != colour) {
                if (zero) tl.x[s] = make_float2(0.0f, 0.0f);
                continue;
            }
            float2 sum = tl.r[s];
            if (!zero) {
                float4 w = tl.a[s];
                for (int q = 0; q < 4; q++) {
                    int nx = x + NBX[q], ny = y + NBY[q];
                    if (t_unknown(tl, L, nx, ny)) {
                        float wd = wcomp(w, q);
                        float2 xn = tl.x[o + ny * L.w + nx];
                        sum.x += wd * xn.x;
                        sum.y += wd * xn.y;
                    }
                }
            }
            tl.x[s] = make_float2(sum.x / D, sum.y / D);
        }
        __syncthreads();
    };
    for (int l = first; l < last; l++) {
        Lv L = lev(d.lv, l), C = lev(d.lv, l + 1);
        const int o = L.off - tl.base, oc = C.off - tl.base;
        sweep(L, 0, true);
        sweep(L, 1, false);
        for (int t = threadIdx.x; t < C.w * C.h; t += NT) {
            int ccx = t % C.w, ccy = t / C.w;
            float sumx = 0.0f, sumy = 0.0f;
            for (int k = 0; k < 4; k++) {
                int cx = 2 * ccx + (k & 1), cy = 2 * ccy + (k >> 1);
                if (!t_unknown(tl, L, cx, cy)) continue;
                int s = o + cy * L.w + cx;
                float4 w = tl.a[s];
                float Ds = tl.dg[s];
                float2 xs = tl.x[s];
                float azx = Ds * xs.x, azy = Ds * xs.y;
                for (int q = 0; q < 4; q++) {
                    int nx = cx + NBX[q], ny = cy + NBY[q];
                    if (t_unknown(tl, L, nx, ny)) {
                        float wd = wcomp(w, q);
                        float2 xn = tl.x[o + ny * L.w + nx];
                        azx -= wd * xn.x;
                        azy -= wd * xn.y;
                    }
                }
                float2 rh = tl.r[s];
                sumx += rh.x - azx;
                sumy += rh.y - azy;
            }
            tl.r[oc + t] = make_float2(sumx, sumy);
        }
        __syncthreads();
    }
    {
        Lv L = lev(d.lv, last);
        sweep(L, 0, true);
        for (int s = 1; s < 9; s++) sweep(L, s & 1, false);
    }
    for (int l = last - 1; l >= first; l--) {
        Lv F = lev(d.lv, l), C = lev(d.lv, l + 1);
        const int o = F.off - tl.base, oc = C.off - tl.base;
        for (int t = threadIdx.x; t < F.w * F.h; t += NT) {
            int x = t % F.w, y = t / F.w;
            if (((x + y) & 1) == 0) continue;
            int s = o + t;
            float D = tl.dg[s];
            if (D <= 0.0f) continue;
            float4 w = tl.a[s];
            float2 sum = tl.r[s];
            for (int q = 0; q < 4; q++) {
                int nx = x + NBX[q], ny = y + NBY[q];
                if (!t_unknown(tl, F, nx, ny)) continue;
                float wd = wcomp(w, q);
                float2 xn = tl.x[o + ny * F.w + nx];
                float2 xc = tl.x[oc + (ny >> 1) * C.w + (nx >> 1)];
                sum.x += wd * (xn.x + MG_OMEGA * xc.x);
                sum.y += wd * (xn.y + MG_OMEGA * xc.y);
            }
            tl.x[s] = make_float2(sum.x / D, sum.y / D);
        }
        __syncthreads();
        sweep(F, 0, false);
    }
    if (blockIdx.x == 0)   // the first tail level's result, for inspection
        for (int s = threadIdx.x; s < tl.nf; s += NT) d.mgz[tl.base + s] = tl.x[s];
}

// One V-cycle: level 0's right-hand side through R (fused with the CG update when R.q is
// set), result in mgz of level 0, partials of r.z and r.r. Returns false on a barrier timeout.
DEV bool vcycle(const DevScene& d, const Tail& tl, const Rsrc& R, float2* r_out, const float2* p, const float2* r_new, float2* sz, float4* buf) {
    const int tail = d.lv.tail;
    for (int l = 0; l < tail; l++) {
        Rsrc Rl = R;
        if (l > 0) Rl = Rsrc{d.mgr, nullptr, 0.0f, 0.0f};
        phase_down(d, l, Rl, l == 0 ? r_out : nullptr, p, sz);
        if (!grid_sync(d.K)) return false;
    }
    phase_tail(d, tl);
    for (int l = tail - 1; l >= 0; l--) {
        const float2* zc = (l == tail - 1) ? tl.x : d.mgz + lev(d.lv, l + 1).off;
        phase_up(d, l, l == 0, l == 0 ? r_new : d.mgr, zc, sz, buf);
        if (!grid_sync(d.K)) return false;
    }
    return true;
}

// cg_apply.comp: p = z + beta p_old, q = A p, partial sums of p.q into part[n + tile].
DEV void phase_apply(const DevScene& d, const Solve& K, const float2* p_old, float2* p_new, float4* buf) {
    Lv F = lev(d.lv, 0);
    const int tx_n = tiles_x(F);
    const int T = tx_n * tiles_y(F);
    const int n = d.nwg;
    const bool nob = K.beta[0] == 0.0f && K.beta[1] == 0.0f;
    auto direction = [&](int i) {
        float2 z = d.mgz[i];
        if (nob) return z;
        float2 po = p_old[i];
        return make_float2(K.beta[0] != 0.0f ? z.x + K.beta[0] * po.x : z.x, K.beta[1] != 0.0f ? z.y + K.beta[1] * po.y : z.y);
    };
    for (int t = blockIdx.x; t < T; t += gridDim.x) {
        if (d.ptile[F.toff + t] == 0u) {
            if (threadIdx.x == 0) d.partials[n + t] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            continue;
        }
        const int cx = (t % tx_n) * 16 + (threadIdx.x & 15), cy = (t / tx_n) * 16 + (threadIdx.x >> 4);
        float4 a4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (l_inside(F, cx, cy)) {
            const int i = l_at(F, cx, cy);
            const float D = d.mgd[i];
            if (D > 0.0f) {
                float2 pp = direction(i);
                float4 w = d.mga[i];
                float qx = D * pp.x, qy = D * pp.y;
                for (int q = 0; q < 4; q++) {
                    int nx = cx + NBX[q], ny = cy + NBY[q];
                    if (unknown(d, F, nx, ny)) {
                        float2 pn = direction(l_at(F, nx, ny));
                        float wd = wcomp(w, q);
                        qx -= wd * pn.x;
                        qy -= wd * pn.y;
                    }
                }
                p_new[i] = pp;
                d.cgq[i] = make_float2(qx, qy);
                a4 = make_float4(0.0f, 0.0f, pp.x * qx, pp.y * qy);
            } else {
                p_new[i] = make_float2(0.0f, 0.0f);
            }
        }
        buf[threadIdx.x] = a4;
        block_tree(buf);
        if (threadIdx.x == 0) d.partials[n + t] = buf[0];
        __syncthreads();
    }
}

}  // namespace

// The whole pressure solve. `second`: the solve after the implicit viscosity (cg_reduce
// mode 8/9: same matrix and hierarchy, density correction counted as solved).
__global__ void __launch_bounds__(NT) k_mgpcg(DevScene d, int second, int scale_mode) {
    __shared__ float2 sz[NT];
    __shared__ float4 buf[NT];
    __shared__ Solve K;
    extern __shared__ __align__(16) unsigned char tail_smem[];
    const DevParams* P = d.P;
    const int n = d.nwg;
    Tail tl;
    {
        const Lv F = lev(d.lv, d.lv.tail), E = lev(d.lv, d.lv.n - 1);
        tl.base = F.off;
        tl.T = E.off + E.w * E.h - F.off;
        tl.nf = F.w * F.h;
        tl.a = reinterpret_cast<float4*>(tail_smem);
        tl.x = reinterpret_cast<float2*>(tl.a + tl.T);
        tl.r = tl.x + tl.T;
        tl.dg = reinterpret_cast<float*>(tl.r + tl.T);
    }
    if (!second) {
        phase_cg_scale(d, scale_mode);
        for (int l = 1; l <= d.lv.tail; l++) {
            if (!grid_sync(d.K)) return;
            phase_mg_build(d, l - 1);
        }
        if (!grid_sync(d.K)) return;
    }
    tail_setup(d, tl);
    float2* r_cur = d.mgr;    // level 0 of mgr: the residual, double-buffered with mgr2
    float2* r_nxt = d.mgr2;
    phase_cg_init(d, r_cur, buf);
    if (!grid_sync(d.K)) return;
    if (!vcycle(d, tl, Rsrc{r_cur, nullptr, 0.0f, 0.0f}, nullptr, nullptr, r_cur, sz, buf)) return;
    {
        float4 a = total(d.partials, n, buf), b = total(d.partials + n, n, buf);
        if (threadIdx.x == 0) {
            K.bb[0] = b.x;
            K.bb[1] = b.y;
            K.rz[0] = a.x;
            K.rz[1] = a.y;
            K.rr[0] = a.z;
            K.rr[1] = a.w;
            K.beta[0] = K.beta[1] = 0.0f;
            K.alpha[0] = K.alpha[1] = 0.0f;
            K.iters[0] = K.iters[1] = 0u;
            float tx = P->tol[0], ty = P->tol[1];
            K.done[0] = a.z <= tx * tx * b.x ? 1u : 0u;
            K.done[1] = a.w <= ty * ty * b.y ? 1u : 0u;
            if (second) K.done[1] = 1u;
        }
        __syncthreads();
    }
    float2* p_old = d.cgp;
    float2* p_new = d.cgp2;
    for (uint32_t it = 0; it < P->pressure_max_iters; it++) {
        if (K.done[0] && K.done[1]) break;
        phase_apply(d, K, p_old, p_new, buf);
        if (!grid_sync(d.K)) return;
        {
            float4 b = total(d.partials + n, n, buf);
            if (threadIdx.x == 0) {
                float ax = 0.0f, ay = 0.0f;
                if (K.done[0] == 0u && b.z > 0.0f) ax = K.rz[0] / b.z;
                if (K.done[1] == 0u && b.w > 0.0f) ay = K.rz[1] / b.w;
                K.alpha[0] = ax;
                K.alpha[1] = ay;
            }
            __syncthreads();
        }
        Rsrc R{r_cur, d.cgq, K.alpha[0], K.alpha[1]};
        if (!vcycle(d, tl, R, r_nxt, p_new, r_nxt, sz, buf)) return;
        {
            float4 a = total(d.partials, n, buf);
            if (threadIdx.x == 0) {
                uint32_t was0 = K.done[0], was1 = K.done[1];
                K.iters[0] += 1u - was0;
                K.iters[1] += 1u - was1;
                float tx = P->tol[0], ty = P->tol[1];
                uint32_t now0 = a.z <= tx * tx * K.bb[0] ? 1u : 0u, now1 = a.w <= ty * ty * K.bb[1] ? 1u : 0u;
                uint32_t d0 = was0 > now0 ? was0 : now0, d1 = was1 > now1 ? was1 : now1;
                float bx = 0.0f, by = 0.0f;
                if (d0 == 0u && K.rz[0] > 0.0f) bx = a.x / K.rz[0];
                if (d1 == 0u && K.rz[1] > 0.0f) by = a.y / K.rz[1];
                K.beta[0] = bx;
                K.beta[1] = by;
                K.rz[0] = a.x;
                K.rz[1] = a.y;
                K.rr[0] = mixf(a.z, K.rr[0], (float)was0);
                K.rr[1] = mixf(a.w, K.rr[1], (float)was1);
                K.done[0] = d0;
                K.done[1] = d1;
            }
            __syncthreads();
        }
        float2* t = p_old;
        p_old = p_new;
        p_new = t;
        t = r_cur;
        r_cur = r_nxt;
        r_nxt = t;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        SolveState* G = d.K;
        for (int c = 0; c < 2; c++) {
            G->p_rz[c] = K.rz[c];
            G->p_alpha[c] = K.alpha[c];
            G->p_beta[c] = K.beta[c];
            G->p_bb[c] = K.bb[c];
            G->p_rr[c] = K.rr[c];
            G->p_done[c] = K.done[c];
            if (!second) G->p_iters[c] = K.iters[c];
        }
        if (second) G->p2_iters = K.iters[0];
        G->solves += 1u;
        if (!second) {
            uint32_t m = K.iters[0] > K.iters[1] ? K.iters[0] : K.iters[1];
            if (m > G->p_it_max) G->p_it_max = m;
            if (K.done[0] == 0u) G->p_unconv += 1u;
        } else {
            if (K.iters[0] > G->p2_it_max) G->p2_it_max = K.iters[0];
            if (K.done[0] == 0u) G->p2_unconv += 1u;
        }
        float rel = K.bb[0] > 0.0f ? sqrtf(K.rr[0] / K.bb[0]) : 0.0f;
        G->p_res_max = maxf(G->p_res_max, rel);
    }
}

size_t pressure_smem(const Levels& lv) {
    int T = lv.off[lv.n - 1] + lv.w[lv.n - 1] * lv.h[lv.n - 1] - lv.off[lv.tail];
    return (size_t)T * (sizeof(float4) + 2 * sizeof(float2) + sizeof(float));
}

int pressure_blocks_max(int device, size_t smem) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    // Opt in to the dynamic shared memory the largest tank so far needs (static + dynamic
    // above 48 KB needs it; the attribute belongs to the kernel, shared by every sim).
    static size_t opted = 0;
    if (smem > opted) {
        cudaFuncSetAttribute(k_mgpcg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        opted = smem;
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mgpcg, NT, smem);
    return sms * per;
}

cudaError_t launch_pressure(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st, int second) {
    // barrier counter back to zero (a solve left by a timeout may have stopped mid-barrier)
    cudaMemsetAsync(&d.K->bar_count, 0, sizeof(uint32_t), st);
    // cg_scale mode 1: with the viscosity between two solves, the first starts from last
    // substep's P1 alone (viscous_warm, mod.rs:2979-2983)
    int scale_mode = (!second && cfg.visc_mode == 2 && cfg.twice && cfg.viscous_warm) ? 1 : 0;
    void* args[] = {(void*)&d, &second, &scale_mode};
    return cudaLaunchCooperativeKernel((const void*)k_mgpcg, dim3(cfg.mg_blocks), dim3(NT), args, pressure_smem(d.lv), st);
}

}  // namespace sprout

namespace sprout {

// ---- the pressure solve on caller buffers, with no allocation ----------------------------
//
// For callers that cannot allocate device memory themselves or through this library: code
// running where cudaMalloc is unavailable or forbidden (a host whose allocator owns the whole
// device, a capture-time or real-time path that must not allocate, an FFI host with a fixed
// memory budget). The multigrid hierarchy, the Krylov vectors and the solve's scalars live
// in one file-scope device array of fixed size, which every GPU that loads this library
// holds until the process exits.

constexpr int kStaticMaxCells = 512 * 288;   // the largest grid the array holds (147,456 cells)
constexpr int kStaticMaxLevels = kMaxLevels;

// Byte layout of the array for kStaticMaxCells (every level of the hierarchy adds at most a
// third again: 4/3 n + one cell per level).
constexpr size_t kStaticTotal = (size_t)kStaticMaxCells * 4 / 3 + 64;
constexpr size_t kStaticTiles = (size_t)kStaticMaxCells / 256 * 2 + 256;
constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kStaticBytes =
    align256(sizeof(DevParams)) + align256(sizeof(StepState)) + align256(sizeof(SolveState)) +
    align256((size_t)kStaticMaxCells * sizeof(float4)) +          // rhs as the engine lays it out
    align256((size_t)kStaticMaxCells * sizeof(float)) +           // viscous part of the warm start
    align256(kStaticTiles * sizeof(uint32_t)) +                   // tile flags of every level
    align256(2 * ((size_t)kStaticMaxCells / 256 + 64) * sizeof(float4)) +   // per-tile partial sums
    align256(kStaticTotal * sizeof(float4)) + align256(kStaticTotal * sizeof(float)) +
    3 * align256(kStaticTotal * sizeof(float2)) + 4 * align256((size_t)kStaticMaxCells * sizeof(float2));

static __device__ __align__(256) unsigned char g_solve_scratch[kStaticBytes];

namespace {

Levels static_levels(int w, int h) {
    Levels L;
    L.w[0] = w;
    L.h[0] = h;
    L.n = 1;
    while (L.w[L.n - 1] * L.h[L.n - 1] > 4 && L.n < kStaticMaxLevels) {
        L.w[L.n] = (L.w[L.n - 1] + 1) / 2;
        L.h[L.n] = (L.h[L.n - 1] + 1) / 2;
        L.n++;
    }
    int total = 0;
    for (int l = 0; l < L.n; l++) {
        L.off[l] = total;
        total += L.w[l] * L.h[l];
    }
    L.total = total;
    int tail = L.n - 1;
    for (int l = 1; l < L.n; l++)
        if (L.w[l] * L.h[l] <= 1500) { tail = l; break; }
    L.tail = tail < 1 ? 1 : (tail > L.n - 1 ? L.n - 1 : tail);
    int tiles = 0;
    for (int l = 0; l <= L.tail; l++) {
        L.toff[l] = tiles;
        tiles += ((L.w[l] + 15) / 16) * ((L.h[l] + 15) / 16);
    }
    L.tiles = tiles;
    return L;
}

// Prepares a solve in the array: the level-0 matrix and right-hand side copied in, every
// coarse matrix and tile flag cleared (a call starts as the first solve of a fresh tank),
// the level-0 tile flags from the diagonal, the scalars reset.
__global__ void k_static_prep(DevScene d, const float4* mga, const float* mgd, const float2* rhs, float tol_p,
                              float tol_psi, uint32_t max_iters) {
    const int n0 = d.W * d.H;
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    for (int i = t0; i < d.lv.total; i += stride) {
        if (i < n0) {
            d.mga[i] = mga[i];
            d.mgd[i] = mgd[i];
            float2 b = rhs[i];
            d.prhs[i] = make_float4(b.x, b.y, 0.0f, 0.0f);
            d.p2keep[i] = 0.0f;
        } else {
            d.mga[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            d.mgd[i] = 0.0f;
        }
    }
    const int tw = (d.W + 15) / 16, th = (d.H + 15) / 16;
    for (int t = t0; t < d.lv.tiles; t += stride) {
        uint32_t on = 0u;
        if (t < tw * th) {
            const int x0 = (t % tw) * 16, y0 = (t / tw) * 16;
            for (int y = y0; y < y0 + 16 && y < d.H && !on; y++)
                for (int x = x0; x < x0 + 16 && x < d.W; x++)
                    if (mgd[y * d.W + x] > 0.0f) { on = 1u; break; }
        }
        d.ptile[t] = on;
    }
    if (t0 == 0) {
        DevParams* P = const_cast<DevParams*>(d.P);
        P->tol[0] = tol_p;
        P->tol[1] = tol_psi;
        P->pressure_max_iters = max_iters;
        d.S->dt = 1.0f;
        d.S->dt_prev = 1.0f;
        SolveState* K = d.K;
        unsigned char* k = reinterpret_cast<unsigned char*>(K);
        for (size_t b = 0; b < sizeof(SolveState); b++) k[b] = 0;
    }
}

struct StaticSlot {
    int ready;
    unsigned char* base;
};
StaticSlot g_slots[64];

}  // namespace

void sprout_internal_set_error(const char* msg);

}  // namespace sprout

extern "C" int sprout_pressure_solve_static(uint32_t w, uint32_t h, const float* mga, const float* mgd, const float* rhs,
                                            float* x, float tol_p, float tol_psi, uint32_t max_iters, void* stream,
                                            uint32_t* iters_out, float* residual_out) {
    using namespace sprout;
    if (!mga || !mgd || !rhs || !x) {
        sprout_internal_set_error("null argument");
        return -1;
    }
    if (w < 16 || h < 16 || (size_t)w * h > (size_t)kStaticMaxCells) {
        sprout_internal_set_error("grid outside 16 x 16 .. 147,456 cells, the most the fixed solve array holds");
        return -3;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        sprout_internal_set_error("no current CUDA device");
        return -6;
    }
    StaticSlot& slot = g_slots[dev];
    if (!slot.ready) {
        // With this device current: the array's device address (its host-side name is only
        // a stand-in). Done on the first call on each device.
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_solve_scratch);
        if (e != cudaSuccess || ptr == nullptr) {
            sprout_internal_set_error(cudaGetErrorString(e));
            return -6;
        }
        slot.base = static_cast<unsigned char*>(ptr);
        slot.ready = 1;
    }
    const Levels L = static_levels((int)w, (int)h);
    DevScene d{};
    d.W = (int)w;
    d.H = (int)h;
    d.ncell = (int)(w * h);
    d.lv = L;
    d.nwg = (int)(((w + 15) / 16) * ((h + 15) / 16));
    unsigned char* p = slot.base;
    auto take = [&](size_t bytes) { unsigned char* q = p; p += align256(bytes); return q; };
    DevParams* P = reinterpret_cast<DevParams*>(take(sizeof(DevParams)));
    d.P = P;
    d.S = reinterpret_cast<StepState*>(take(sizeof(StepState)));
    d.K = reinterpret_cast<SolveState*>(take(sizeof(SolveState)));
    d.prhs = reinterpret_cast<float4*>(take((size_t)kStaticMaxCells * sizeof(float4)));
    d.p2keep = reinterpret_cast<float*>(take((size_t)kStaticMaxCells * sizeof(float)));
    d.ptile = reinterpret_cast<uint32_t*>(take(kStaticTiles * sizeof(uint32_t)));
    d.partials = reinterpret_cast<float4*>(take(2 * ((size_t)kStaticMaxCells / 256 + 64) * sizeof(float4)));
    d.mga = reinterpret_cast<float4*>(take(kStaticTotal * sizeof(float4)));
    d.mgd = reinterpret_cast<float*>(take(kStaticTotal * sizeof(float)));
    d.mgx = reinterpret_cast<float2*>(take(kStaticTotal * sizeof(float2)));
    d.mgz = reinterpret_cast<float2*>(take(kStaticTotal * sizeof(float2)));
    d.mgr = reinterpret_cast<float2*>(take(kStaticTotal * sizeof(float2)));
    d.mgr2 = reinterpret_cast<float2*>(take((size_t)kStaticMaxCells * sizeof(float2)));
    d.cgp = reinterpret_cast<float2*>(take((size_t)kStaticMaxCells * sizeof(float2)));
    d.cgp2 = reinterpret_cast<float2*>(take((size_t)kStaticMaxCells * sizeof(float2)));
    d.cgq = reinterpret_cast<float2*>(take((size_t)kStaticMaxCells * sizeof(float2)));
    d.pres = reinterpret_cast<float2*>(x);
    if ((size_t)(p - slot.base) > kStaticBytes || (size_t)L.total > kStaticTotal || (size_t)L.tiles > kStaticTiles) {
        sprout_internal_set_error("fixed solve array layout overflow");
        return -3;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_static_prep<<<128, 256, 0, st>>>(d, reinterpret_cast<const float4*>(mga), mgd, reinterpret_cast<const float2*>(rhs),
                                       tol_p, tol_psi, max_iters);
    const size_t smem = pressure_smem(L);
    int blocks = pressure_blocks_max(dev, smem);
    if (blocks > d.nwg) blocks = d.nwg;
    if (blocks < 1) blocks = 1;
    int second = 0, scale_mode = 0;
    void* args[] = {(void*)&d, &second, &scale_mode};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_mgpcg, dim3(blocks), dim3(NT), args, smem, st);
    if (e != cudaSuccess) {
        sprout_internal_set_error(cudaGetErrorString(e));
        return -6;
    }
    if (iters_out || residual_out) {
        SolveState K;
        e = cudaMemcpyAsync(&K, d.K, sizeof K, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            sprout_internal_set_error(cudaGetErrorString(e));
            return -6;
        }
        if (K.error) {
            sprout_internal_set_error("a bounded device-side wait ran out (grid barrier of the pressure solve)");
            return -5;
        }
        if (iters_out) {
            iters_out[0] = K.p_iters[0];
            iters_out[1] = K.p_iters[1];
        }
        if (residual_out) *residual_out = K.p_bb[0] > 0.0f ? sqrtf(K.p_rr[0] / K.p_bb[0]) : 0.0f;
    }
    return 0;
}

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
//
// Two precisions, one kernel template:
//   Plain  the reference's arithmetic: every value FP32, the dot products summed in FP32 in
//          the reference's order (bit-exact with the oracle).
//   Mixed  the V-cycle's matrices (every level's couplings) stored in BF16 and computed in
//          FP32; the CG operator (level 0's matrix), every vector, iterate, residual and
//          direction stay FP32; the dot products summed in FP32 as the plain solve sums
//          them, their totals widened to FP64 for the step lengths and the convergence
//          test; the refinement's checks and the closing true residual b - A x evaluated
//          as float pairs (products exact, sums compensated). The BF16 couplings come with
//          an FP32 diagonal that keeps each row's exact excess over them (see Mixed::setA).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "dev_common.cuh"
#include "kernels.h"
#include "solve_common.cuh"

namespace sprout {

namespace {

using namespace solve;

__constant__ int NBX[4] = {-1, 1, 0, 0};
__constant__ int NBY[4] = {0, 0, -1, 1};


// ---- the two precisions ---------------------------------------------------------------

struct Plain {
    static constexpr bool kMixed = false;
    using acc = float;
    using acc4 = float4;
    DEV static float4 A(const DevScene& d, int i) { return d.mga[i]; }
    DEV static float Dg(const DevScene& d, int i) { return d.mgd[i]; }
    DEV static void setA(const DevScene& d, int i, float4 a, float dg) { d.mga[i] = a; d.mgd[i] = dg; }
    DEV static void setX(const DevScene& d, int i, float2 v) { d.mgx[i] = v; }
    DEV static float2 Z(const DevScene& d, int i) { return d.mgz[i]; }
    DEV static void setZ(const DevScene& d, int i, float2 v) { d.mgz[i] = v; }
    DEV static float2 R(const DevScene& d, int i) { return d.mgr[i]; }   // a coarse level's rhs
    DEV static void setR(const DevScene& d, int i, float2 v) { d.mgr[i] = v; }
    DEV static acc4* part(const DevScene& d) { return d.partials; }
    DEV static acc4 zero4() { return make_float4(0.0f, 0.0f, 0.0f, 0.0f); }
    // the four products a_k b_k of a cell's partial sums, and a total as the scalars use it
    DEV static acc4 prod4(float a0, float b0, float a1, float b1, float a2, float b2, float a3, float b3) {
        return make_float4(a0 * b0, a1 * b1, a2 * b2, a3 * b3);
    }
    DEV static float4 fin(acc4 a) { return a; }
    // the stored matrix as a tile region stages it: bytes per row of couplings, their address,
    // the diagonal's array, and the row read from its staged slot in FP32
    static constexpr int kABytes = 16;
    DEV static const void* Araw(const DevScene& d, int i) { return d.mga + i; }
    DEV static const float* Dptr(const DevScene& d) { return d.mgd; }
    DEV static float4 Aslot(const float4& slot) { return slot; }
    // a / D with D's staged slot (the diagonal): the shader's IEEE division; quotp is zero
    // unless the slot is positive
    DEV static float quot(float a, float slot) { return divz(a, slot); }
    DEV static float2 quot(float2 a, float slot) { return divz(a, slot); }
    DEV static float quotp(float a, float slot) { return divp(a, slot); }
};

// a pair of BF16 values in 32 bits (x in the low half), rounded to nearest even
DEV uint32_t pack(float2 v) {
    __nv_bfloat162 h = __floats2bfloat162_rn(v.x, v.y);
    return *reinterpret_cast<const uint32_t*>(&h);
}
DEV float2 unpack(uint32_t u) { return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u)); }

struct Mixed {
    static constexpr bool kMixed = true;
    using acc = double;
    // the dot products' partial sums and totals in FP32 as the plain solve takes them (the
    // reference's trees), widened to FP64 for the step lengths and the convergence test
    using acc4 = float4;
    // the hierarchy in BF16: a row's four couplings as two bfloat162 in a uint2
    DEV static float4 A(const DevScene& d, int i) {
        const uint2 u = d.hga[i];
        const float2 a = unpack(u.x), b = unpack(u.y);
        return make_float4(a.x, a.y, b.x, b.y);
    }
    DEV static float Dg(const DevScene& d, int i) { return d.hgd[i]; }
    // A row whose couplings m (a mask of the unknown neighbours) link it to other unknowns:
    // the couplings rounded to BF16, the diagonal rebuilt as its excess over the FP32
    // couplings plus the rounded ones, so that every row sum (the air, solid and vent terms
    // that keep a sealed region's matrix definite) is kept exactly and the stored matrix
    // stays a weighted graph Laplacian plus the same non-negative diagonal.
    DEV static void setA(const DevScene& d, int i, float4 a, float dg, int m = 15) {
        const uint2 u = make_uint2(pack(make_float2(a.x, a.y)), pack(make_float2(a.z, a.w)));
        d.hga[i] = u;
        if (dg <= 0.0f) {
            d.hgd[i] = 0.0f;
            d.hgi[i] = 0.0f;
            return;
        }
        const float2 lo = unpack(u.x), hi = unpack(u.y);
        const float c32 = ((m & 1) ? a.x : 0.0f) + ((m & 2) ? a.y : 0.0f) + ((m & 4) ? a.z : 0.0f) + ((m & 8) ? a.w : 0.0f);
        const float c16 = ((m & 1) ? lo.x : 0.0f) + ((m & 2) ? lo.y : 0.0f) + ((m & 4) ? hi.x : 0.0f) + ((m & 8) ? hi.y : 0.0f);
        const float D = (dg - c32) + c16;
        d.hgd[i] = D;
        d.hgi[i] = D > 0.0f ? 1.0f / D : 0.0f;
    }
    // the vectors stay FP32 on every level: rounding them would make the V-cycle a
    // nonlinear operator, which conjugate gradients does not tolerate (it stagnates near the
    // rounding level); the matrices are fixed during a solve, so the V-cycle built on their
    // BF16 copies stays a linear, symmetric positive definite preconditioner
    DEV static void setX(const DevScene& d, int i, float2 v) { d.mgx[i] = v; }
    DEV static float2 Z(const DevScene& d, int i) { return d.mgz[i]; }
    DEV static void setZ(const DevScene& d, int i, float2 v) { d.mgz[i] = v; }
    DEV static float2 R(const DevScene& d, int i) { return d.mgr[i]; }
    DEV static void setR(const DevScene& d, int i, float2 v) { d.mgr[i] = v; }
    DEV static acc4* part(const DevScene& d) { return d.partials; }
    DEV static acc4 zero4() { return make_float4(0.0f, 0.0f, 0.0f, 0.0f); }
    DEV static acc4 prod4(float a0, float b0, float a1, float b1, float a2, float b2, float a3, float b3) {
        return make_float4(a0 * b0, a1 * b1, a2 * b2, a3 * b3);
    }
    DEV static Dbl4 fin(acc4 a) { return Dbl4{(double)a.x, (double)a.y, (double)a.z, (double)a.w}; }
    static constexpr int kABytes = 8;
    DEV static const void* Araw(const DevScene& d, int i) { return d.hga + i; }
    // the level passes stage the inverse diagonal in the diagonal's slot (positive exactly
    // where the diagonal is) and multiply by it instead of dividing: a V-cycle is a
    // preconditioner here, not the reference's arithmetic, and ten IEEE divisions per black
    // cell were most of a way down's instructions
    DEV static const float* Dptr(const DevScene& d) { return d.hgi; }
    DEV static float quot(float a, float slot) { return a * slot; }
    DEV static float2 quot(float2 a, float slot) { return make_float2(a.x * slot, a.y * slot); }
    DEV static float quotp(float a, float slot) { return slot > 0.0f ? a * slot : 0.0f; }
    // the BF16 row copied into the first 8 bytes of the slot, widened on reading
    DEV static float4 Aslot(const float4& slot) {
        const uint2 u = *reinterpret_cast<const uint2*>(&slot);
        const float2 a = unpack(u.x), b = unpack(u.y);
        return make_float4(a.x, a.y, b.x, b.y);
    }
};

template <class T>
struct Solve {
    T rz[2], alpha[2], beta[2], bb[2], rr[2];
    T rmark;   // mixed precision: the pressure column's r.r at the last residual check
    uint32_t done[2], iters[2];
    uint32_t bad;   // a total was not finite: the solve stopped (SolveState ERR_DIVERGED)
    uint32_t replaced;   // residual replacements in this solve
    uint32_t floor_hit;  // a check found the carried residual near the FP32 rounding floor
    uint32_t adopt;      // a batch: this iteration's check adopts the true residual
};

template <class A4>
DEV bool finite4(const A4& a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z) && isfinite(a.w); }

// ---- setup phases ---------------------------------------------------------------------

// Unknowns of the V-cycle's level (M's copy of the diagonal) and of the CG operator.
template <class M>
DEV bool unknown(const DevScene& d, const Lv& L, int x, int y) { return l_inside(L, x, y) && M::Dg(d, l_at(L, x, y)) > 0.0f; }
DEV bool unknown_op(const DevScene& d, const Lv& L, int x, int y) { return l_inside(L, x, y) && d.mgd[l_at(L, x, y)] > 0.0f; }


// cg_scale.comp on level-0 tile t: warm start from last substep's potential rescaled to
// this substep. Mixed: also level 0's matrix in BF16 for the V-cycle (every cell: rhs.comp
// rewrote them all).
template <class M>
DEV void cg_scale_tile(const DevScene& d, int t, int mode) {
    const Lv F = lev(d.lv, 0);
    const float ratio = d.S->dt / d.S->dt_prev;
    const int cx = (t % tiles_x(F)) * 16 + (threadIdx.x & 15), cy = (t / tiles_x(F)) * 16 + (threadIdx.x >> 4);
    if (!l_inside(F, cx, cy)) return;
    const int i = l_at(F, cx, cy);
    if (M::kMixed) {
        int m = 0;
        for (int q = 0; q < 4; q++) m |= unknown_op(d, F, cx + NBX[q], cy + NBY[q]) ? (1 << q) : 0;
        Mixed::setA(d, i, d.mga[i], d.mgd[i], m);
    }
    if (d.ptile[F.toff + t] == 0u) return;
    if (d.mgd[i] > 0.0f) {
        float p = d.pres[i].x;
        if (mode == 1) p -= d.p2keep[i];
        else d.p2keep[i] = 0.0f;
        d.pres[i].x = p * ratio;
    } else {
        d.pres[i] = make_float2(0.0f, 0.0f);
    }
}

// mg_build.comp on tile t of coarse level l + 1, from level l.
template <class M>
DEV void mg_build_tile(const DevScene& d, int l, int t) {
    const Lv F = lev(d.lv, l), C = lev(d.lv, l + 1);
    const int tfx = tiles_x(F), tfy = tiles_y(F), tcx = tiles_x(C);
    __shared__ uint32_t s_state;
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
    if (state == 0u) return;
    const int Cx = tx * 16 + (threadIdx.x & 15), Cy = ty * 16 + (threadIdx.x >> 4);
    if (Cx >= C.w || Cy >= C.h) return;
    const int o = l_at(C, Cx, Cy);
    if ((state & 1u) == 0u) {
        M::setA(d, o, make_float4(0.0f, 0.0f, 0.0f, 0.0f), 0.0f);
        return;
    }
    float D = 0.0f;
    float4 A = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int k = 0; k < 4; k++) {
        int cx = 2 * Cx + (k & 1), cy = 2 * Cy + (k >> 1);
        if (!unknown<M>(d, F, cx, cy)) continue;
        int i = l_at(F, cx, cy);
        D += M::Dg(d, i);
        float4 w = M::A(d, i);
        for (int q = 0; q < 4; q++) {
            int nx = cx + NBX[q], ny = cy + NBY[q];
            if (!unknown<M>(d, F, nx, ny)) continue;
            float wd = wcomp(w, q);
            if ((nx >> 1) == Cx && (ny >> 1) == Cy) D -= wd;
            else if (q == 0) A.x += wd;
            else if (q == 1) A.y += wd;
            else if (q == 2) A.z += wd;
            else A.w += wd;
        }
    }
    M::setA(d, o, D > 1e-7f ? A : make_float4(0.0f, 0.0f, 0.0f, 0.0f), D > 1e-7f ? D : 0.0f);
}

// cg_init.comp on level-0 tile t: r = b - A x (the FP32 operator), the tile's sum of b.b
// into part[n + t] (or, with `rr`, of r.r into part[t]).
template <class M>
DEV void residual_tile(const DevScene& d, int t, float2* r0, typename M::acc4* buf, bool rr) {
    using acc = typename M::acc;
    const Lv F = lev(d.lv, 0);
    const int n = d.nwg;
    typename M::acc4* part = M::part(d) + (rr ? 0 : n);
    if (d.ptile[F.toff + t] == 0u) {
        if (threadIdx.x == 0) part[t] = M::zero4();
        return;
    }
    const int cx = (t % tiles_x(F)) * 16 + (threadIdx.x & 15), cy = (t / tiles_x(F)) * 16 + (threadIdx.x >> 4);
    typename M::acc4 a4 = M::zero4();
    if (l_inside(F, cx, cy)) {
        const int i = l_at(F, cx, cy);
        const float D = d.mgd[i];
        if (D > 0.0f) {
            float2 x = d.pres[i];
            float4 w = d.mga[i];
            float axx = D * x.x, axy = D * x.y;
            for (int q = 0; q < 4; q++) {
                int nx = cx + NBX[q], ny = cy + NBY[q];
                if (unknown_op(d, F, nx, ny)) {
                    float wd = wcomp(w, q);
                    float2 pn = d.pres[l_at(F, nx, ny)];
                    axx -= wd * pn.x;
                    axy -= wd * pn.y;
                }
            }
            float4 b = d.prhs[i];
            const float2 r = make_float2(b.x - axx, b.y - axy);
            r0[i] = r;
            if (rr) a4 = M::prod4(0.0f, 0.0f, 0.0f, 0.0f, r.x, r.x, r.y, r.y);
            else a4 = M::prod4(b.x, b.x, b.y, b.y, 0.0f, 0.0f, 0.0f, 0.0f);
        } else {
            r0[i] = make_float2(0.0f, 0.0f);
        }
    }
    buf[threadIdx.x] = a4;
    block_tree(buf);
    if (threadIdx.x == 0) part[t] = buf[0];
    __syncthreads();
}

// Tiles of level l of one scene.
DEV int level_tiles(const DevScene& d, int l) {
    const Lv L = lev(d.lv, l);
    return tiles_x(L) * tiles_y(L);
}

// ---- the V-cycle --------------------------------------------------------------------------

// The right-hand side a way down reads: level 0's residual (FP32), fused with the update
// r -= alpha q of cg_update.comp when q is set; or a coarse level's, through M.
template <class M>
struct Rsrc {
    const float2* r;      // level-0 residual before the update (null: a coarse level)
    const float2* q;      // A p, for the fused update (null: no update)
    float ax, ay;
    DEV float2 at(const DevScene& d, int i) const {
        if (!r) return M::R(d, i);
        float2 v = r[i];
        if (q) {
            float2 qq = q[i];
            v.x = v.x - ax * qq.x;
            v.y = v.y - ay * qq.y;
        }
        return v;
    }
};

// The tail levels' state in each block's shared memory (dynamic, FP32 in both precisions):
// per tail cell the matrix row (couplings, diagonal), the iterate and the right-hand side,
// at its offset from the first tail level (the slots of mg_tail.comp).
struct Tail {
    float4* a;    // couplings of tail cells aoff .. T - 1 (at a[s - aoff])
    float* dg;
    float2* x;
    float2* r;
    uint8_t* m;   // per cell: bit q set when neighbour q is an unknown, bit 4 when the cell is
    int base, T, nf;
    int aoff;     // 0: every level's couplings in shared memory; nf: the first tail level's read
                  // from the level's stored matrix (a batch, whose blocks then fit four per SM)
};

// The couplings of tail cell s, from shared memory or (the first level of a batch's tail)
// from the level's stored matrix: the same values tail_setup would have copied.
template <class M>
DEV float4 tail_a(const DevScene& d, const Tail& tl, int s) {
    return s < tl.aoff ? M::A(d, tl.base + s) : tl.a[s - tl.aoff];
}

DEV bool t_unknown(const Tail& tl, const Lv& L, int x, int y) { return l_inside(L, x, y) && tl.dg[L.off - tl.base + y * L.w + x] > 0.0f; }

// The tail of scene d laid out in the dynamic shared memory at smem; its right-hand sides at
// r_store if given (they are live only inside the tail phase, so a caller may keep them in
// bytes that other phases use), else after the iterates.
DEV Tail make_tail(const DevScene& d, unsigned char* smem, float2* r_store = nullptr, bool first_global = false) {
    Tail tl;
    const Lv F = lev(d.lv, d.lv.tail), E = lev(d.lv, d.lv.n - 1);
    tl.base = F.off;
    tl.T = E.off + E.w * E.h - F.off;
    tl.nf = F.w * F.h;
    tl.aoff = first_global ? tl.nf : 0;
    tl.a = reinterpret_cast<float4*>(smem);
    tl.x = reinterpret_cast<float2*>(tl.a + (tl.T - tl.aoff));
    if (r_store) {
        tl.r = r_store;
        tl.dg = reinterpret_cast<float*>(tl.x + tl.T);
    } else {
        tl.r = tl.x + tl.T;
        tl.dg = reinterpret_cast<float*>(tl.r + tl.T);
    }
    tl.m = reinterpret_cast<uint8_t*>(tl.dg + tl.T);
    return tl;
}

// Cells of the tail levels, and the tail's bytes with and without its right-hand sides.
__host__ __device__ inline int tail_cells(const Levels& lv) { return lv.off[lv.n - 1] + lv.w[lv.n - 1] * lv.h[lv.n - 1] - lv.off[lv.tail]; }
__host__ __device__ inline size_t tail_bytes(int T, bool with_r, int aoff = 0) {
    const size_t per = sizeof(float2) + (with_r ? sizeof(float2) : 0) + sizeof(float) + 1;
    return ((size_t)T * per + (size_t)(T - aoff) * sizeof(float4) + 15) / 16 * 16;
}
// The first tail level's cells (a batch keeps their couplings out of shared memory).
__host__ __device__ inline int tail_first_cells(const Levels& lv) { return lv.w[lv.tail] * lv.h[lv.tail]; }

// mg_tail.comp mode 1 in every block's shared memory, once per solve: the first tail
// level's matrix from global memory, then the Galerkin matrices of the coarser tail levels
// (the arithmetic of mg_build.comp). Block 0 also stores them for inspection.
template <class M>
DEV void tail_setup(const DevScene& d, const Tail& tl, bool writer) {
    for (int s = threadIdx.x; s < tl.nf; s += NT) {
        if (s >= tl.aoff) tl.a[s - tl.aoff] = M::A(d, tl.base + s);
        tl.dg[s] = M::Dg(d, tl.base + s);
    }
    __syncthreads();
    for (int l = d.lv.tail; l < d.lv.n - 1; l++) {
        Lv F = lev(d.lv, l), C = lev(d.lv, l + 1);
        const int o = F.off - tl.base, oc = C.off - tl.base;
        for (int t = threadIdx.x; t < C.w * C.h; t += NT) {
            const int ccy = qdiv(t, C.wm), ccx = t - ccy * C.w;
            float D = 0.0f;
            float4 A = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            for (int k = 0; k < 4; k++) {
                int cx = 2 * ccx + (k & 1), cy = 2 * ccy + (k >> 1);
                if (!t_unknown(tl, F, cx, cy)) continue;
                int i = o + cy * F.w + cx;
                D += tl.dg[i];
                float4 w = tail_a<M>(d, tl, i);
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
            tl.a[oc + t - tl.aoff] = D > 1e-7f ? A : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (writer) M::setA(d, C.off + t, tl.a[oc + t - tl.aoff], tl.dg[oc + t]);
        }
        __syncthreads();
    }
    // the unknowns around every tail cell, for the sweeps
    for (int l = d.lv.tail; l < d.lv.n; l++) {
        const Lv L = lev(d.lv, l);
        const int o = L.off - tl.base;
        for (int t = threadIdx.x; t < L.w * L.h; t += NT) {
            const int y = qdiv(t, L.wm), x = t - y * L.w;
            uint32_t m = tl.dg[o + t] > 0.0f ? 16u : 0u;
            for (int q = 0; q < 4; q++) m |= t_unknown(tl, L, x + NBX[q], y + NBY[q]) ? (1u << q) : 0u;
            tl.m[o + t] = (uint8_t)m;
        }
    }
    __syncthreads();
}

// Where a way up reads the coarse level's finished values: this block's shared copy of the
// first tail level (s), or the level in global memory through M (at offset off).
struct Zc {
    const float2* s;
    int off, w;
};

// A level's tile and RH cells around it staged in shared memory, RW x RW slots: the
// diagonal (zero outside the level), the couplings, up to three vector fields, and for the
// tile's own cells (one per thread) two more vectors and the operator's diagonal. A tile body
// comes in two halves: stage_* issues every load of the tile as an asynchronous copy into a
// Region (zero-filled outside the level), and finish_* runs once they have landed and reads
// only the slots, each as the shader reads its field (a diagonal that is not positive as
// zero, BF16 couplings widened, the fused residual update applied). Its values are the same,
// value for value, as reading the fields from global memory one after another. Every block
// holds two Regions: while one tile computes, the copies of its next tile are in flight
// (pipe_active).
constexpr int RH = 2;
constexpr int RW = 16 + 2 * RH;
constexpr int RN = RW * RW;
struct Region {
    float dg[RN];
    float4 a[RN];
    float2 u[RN], v[RN];
    union {
        float2 w[RN];   // a way up: each slot's coarse-grid value
        struct {        // a way down fused with the CG update: the tile's own p, x and diagonal
            float2 o1[NT], o2[NT];
            float od[NT];
        } o;
    };
    float2 ring[32];   // the black cells just outside the tile, once computed (ring_cell)
};
DEV int rslot(int lx, int ly) { return (ly + RH) * RW + lx + RH; }
__constant__ int RSTEP[4] = {-1, 1, -RW, RW};

// The cells of a tile by colour for the smoothing passes: threads 0 .. 127 take the red
// cells ((x + y) even; tiles start at even coordinates), 128 .. 255 the black ones, eight to
// a row, so that no warp holds both the short red formula and the long black one.
DEV int2 colour_cell() {
    const int c = threadIdx.x & 127, ly = c >> 3;
    return make_int2(2 * (c & 7) + ((ly & 1) ^ (threadIdx.x < 128 ? 0 : 1)), ly);
}
// The 32 black cells just outside a tile that its red border cells touch: slot j of side
// s = r / 8: (-1, 2j), (16, 2j + 1), (2j, -1), (2j + 1, 16); and the slot of such a cell.
DEV int2 ring_cell(int r) {
    const int j = r & 7;
    switch (r >> 3) {
        case 0: return make_int2(-1, 2 * j);
        case 1: return make_int2(16, 2 * j + 1);
        case 2: return make_int2(2 * j, -1);
        default: return make_int2(2 * j + 1, 16);
    }
}
DEV int ring_of(int lnx, int lny) {
    if (lnx < 0) return lny >> 1;
    if (lnx > 15) return 8 + (lny >> 1);
    if (lny < 0) return 16 + (lnx >> 1);
    return 24 + (lnx >> 1);
}

// The slots of a region that thread threadIdx.x copies and makes final: k = threadIdx.x +
// j NT (j < RJ), at cell (ox - RH + k % RW, oy - RH + k / RW) of the level.
constexpr int RJ = (RN + NT - 1) / NT;

// This block's work items through the pipeline of solve_common.cuh with kDepth regions:
// stage(it, rg) issues item it's copies into a region, finish(it, rg) computes it.
constexpr int kDepth = 2;
template <class I, class S, class F>
DEV void pipe_tiles(uint32_t cnt, I&& item, Region* rg, S&& stage, F&& finish) {
    pipeline<kDepth>(cnt, item, [&](uint32_t it, int b) { stage(it, rg[b]); }, [&](uint32_t it, int b) { finish(it, rg[b]); });
}

template <class M>
DEV float2 coarse_z(const DevScene& d, const Zc& zc, int mx, int my) {
    const int k = (my >> 1) * zc.w + (mx >> 1);
    return zc.s ? zc.s[k] : M::Z(d, zc.off + k);
}

// mg_down.comp on tile t of level l, copies: the diagonal, the couplings, the right-hand
// side (level 0: the residual before the update, and q when R.q) over the region; with
// `update` (level 0 fused with cg_update.comp) the tile's own p, x and operator diagonal.
template <class M>
DEV void stage_down(const DevScene& d, const Lv& F, int t, const Rsrc<M>& R, bool update, const float2* p, Region& rg) {
    const int2 og = tile_origin(F, t);
    const int ox = og.x, oy = og.y;
    const float2* r = R.r ? R.r : d.mgr;
#pragma unroll
    for (int j = 0; j < RJ; j++) {
        const int k = threadIdx.x + j * NT;
        if (k >= RN) break;
        const int x = ox - RH + k % RW, y = oy - RH + k / RW;
        const bool in = l_inside(F, x, y);
        const int i = in ? l_at(F, x, y) : 0;
        cp_async<4>(&rg.dg[k], M::Dptr(d) + i, in);
        cp_async<M::kABytes>(&rg.a[k], M::Araw(d, i), in);
        cp_async<8>(&rg.u[k], r + i, in);
        if (R.q) cp_async<8>(&rg.v[k], R.q + i, in);
    }
    if (update) {
        const int cx = ox + (threadIdx.x & 15), cy = oy + (threadIdx.x >> 4);
        const bool in = l_inside(F, cx, cy);
        const int i = in ? l_at(F, cx, cy) : 0;
        cp_async<4>(&rg.o.od[threadIdx.x], d.mgd + i, in);
        cp_async<8>(&rg.o.o1[threadIdx.x], p + i, in);
        cp_async<8>(&rg.o.o2[threadIdx.x], d.pres + i, in);
    }
}

// ... and its arithmetic. On level 0 with `r_out` it also applies cg_update.comp: x +=
// alpha p and the residual update into r_out. The staged slots are read as the shader reads
// its fields: a diagonal that is not positive as zero (dg), the right-hand side with the fused
// update (rhs). Every neighbour's values are read before the terms are summed, in the
// shader's order, each kept or not by a select.
template <class M>
DEV void finish_down(const DevScene& d, const Lv& F, const Lv& C, int t, const Rsrc<M>& R, float2* r_out, float2* sz,
                     Region& rg) {
    const int2 og = tile_origin(F, t);
    const int ox = og.x, oy = og.y;
    __syncthreads();   // (every thread's copies have landed)
    const bool fused = R.q != nullptr;
    auto dg = [&](int k) {
        const float v = rg.dg[k];
        return v > 0.0f ? v : 0.0f;
    };
    auto rhs = [&](int k) {   // R.at: r - alpha q
        float2 v = rg.u[k];
        if (fused) {
            const float2 qq = rg.v[k];
            v.x = v.x - R.ax * qq.x;
            v.y = v.y - R.ay * qq.y;
        }
        return v;
    };
    // the value of black slot k after the half-sweep from zero (mg_down black())
    auto black = [&](int k) {
        const float4 w = M::Aslot(rg.a[k]);
        float2 sum = rhs(k);
        const float d0 = dg(k - 1), d1 = dg(k + 1), d2 = dg(k - RW), d3 = dg(k + RW);
        const float2 r0 = rhs(k - 1), r1 = rhs(k + 1), r2 = rhs(k - RW), r3 = rhs(k + RW);
        const float t0x = M::quotp(w.x * r0.x, d0), t0y = M::quotp(w.x * r0.y, d0);
        const float t1x = M::quotp(w.y * r1.x, d1), t1y = M::quotp(w.y * r1.y, d1);
        const float t2x = M::quotp(w.z * r2.x, d2), t2y = M::quotp(w.z * r2.y, d2);
        const float t3x = M::quotp(w.w * r3.x, d3), t3y = M::quotp(w.w * r3.y, d3);
        if (d0 > 0.0f) { sum.x += t0x; sum.y += t0y; }
        if (d1 > 0.0f) { sum.x += t1x; sum.y += t1y; }
        if (d2 > 0.0f) { sum.x += t2x; sum.y += t2y; }
        if (d3 > 0.0f) { sum.x += t3x; sum.y += t3y; }
        return M::quot(sum, dg(k));
    };
    // one cell's z (mg_down: red from zero, black after it), the CG update and mgx
    auto own = [&](int lx, int ly, bool red) {
        const int cell = ly * 16 + lx;
        const int cx = ox + lx, cy = oy + ly;
        const int k0 = rslot(lx, ly);
        float2 z = make_float2(0.0f, 0.0f);
        if (l_inside(F, cx, cy)) {
            const int i = l_at(F, cx, cy);
            const float D = dg(k0);
            if (D > 0.0f) {
                if (red) {
                    z = M::quot(rhs(k0), D);
                } else {
                    z = black(k0);
                }
            }
            if (r_out && rg.o.od[cell] > 0.0f) {
                // cg_update.comp: x += alpha p, r -= alpha q (unknowns of active tiles)
                const float2 pp = rg.o.o1[cell];
                float2 x = rg.o.o2[cell];
                x.x += R.ax * pp.x;
                x.y += R.ay * pp.y;
                d.pres[i] = x;
                r_out[i] = rhs(k0);
            }
            M::setX(d, i, z);
        }
        sz[cell] = z;
    };
    // warps 0-3: the 128 black cells; warp 4: the 32 black cells around the tile (ring_cell),
    // which the restriction needs; warps 5-7: the 128 red cells (the shorter formula), 96 + 32
    const int tid = threadIdx.x;
    if (tid < 128) {
        const int ly = tid >> 3;
        own(2 * (tid & 7) + 1 - (ly & 1), ly, false);
    } else if (tid < 160) {
        const int2 rc = ring_cell(tid - 128);
        const int kr = rslot(rc.x, rc.y);
        rg.ring[tid - 128] = dg(kr) > 0.0f ? black(kr) : make_float2(0.0f, 0.0f);
    } else {
        for (int c = tid - 160; c < 128; c += 96) {
            const int ly = c >> 3;
            own(2 * (c & 7) + (ly & 1), ly, true);
        }
    }
    __syncthreads();
    if (threadIdx.x < 64) {   // the restriction: aggregate (ax, ay), its red cells (0, 0) and (1, 1)
        const int ax = threadIdx.x & 7, ay = threadIdx.x >> 3;
        const int Cx = (ox >> 1) + ax, Cy = (oy >> 1) + ay;
        if (Cx < C.w && Cy < C.h) {
            float sx = 0.0f, sy = 0.0f;
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const int lqx = 2 * ax + k, lqy = 2 * ay + k;
                const int kq = rslot(lqx, lqy);
                const bool own = dg(kq) > 0.0f;
                const float4 w = M::Aslot(rg.a[kq]);
                float dn[4];
                float2 zb[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    dn[q] = dg(kq + RSTEP[q]);
                    const int lnx = lqx + NBX[q], lny = lqy + NBY[q];
                    const bool here = lnx >= 0 && lny >= 0 && lnx < 16 && lny < 16;
                    zb[q] = here ? sz[lny * 16 + lnx] : rg.ring[ring_of(lnx, lny)];
                }
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float wd = wcomp(w, q);
                    const float ux = wd * zb[q].x, uy = wd * zb[q].y;
                    if (own && dn[q] > 0.0f) {
                        sx += ux;
                        sy += uy;
                    }
                }
            }
            M::setR(d, l_at(C, Cx, Cy), make_float2(sx, sy));
        }
    }
    __syncthreads();
}

// mg_up.comp on tile t of level l, copies: the diagonal, the couplings, the right-hand side
// (u), the pre-smoothed values mgx (v) and each slot's coarse-grid value (w; from zc.s, this
// block's shared copy of the tail, in finish_up).
template <class M>
DEV void stage_up(const DevScene& d, const Lv& F, int t, const Rsrc<M>& rhs, const Zc& zc, Region& rg) {
    const int2 og = tile_origin(F, t);
    const int ox = og.x, oy = og.y;
    const float2* r = rhs.r ? rhs.r : d.mgr;
#pragma unroll
    for (int j = 0; j < RJ; j++) {
        const int k = threadIdx.x + j * NT;
        if (k >= RN) break;
        const int x = ox - RH + k % RW, y = oy - RH + k / RW;
        const bool in = l_inside(F, x, y);
        const int i = in ? l_at(F, x, y) : 0;
        cp_async<4>(&rg.dg[k], M::Dptr(d) + i, in);
        cp_async<M::kABytes>(&rg.a[k], M::Araw(d, i), in);
        cp_async<8>(&rg.u[k], r + i, in);
        cp_async<8>(&rg.v[k], d.mgx + i, in);
        if (!zc.s) cp_async<8>(&rg.w[k], d.mgz + (in ? zc.off + (y >> 1) * zc.w + (x >> 1) : 0), in);
    }
}

// ... and its arithmetic; on level 0 (flag) the tile's sums of r.z, r.r into part[t]. Read
// as finish_down reads its slots.
template <class M>
DEV void finish_up(const DevScene& d, const Lv& F, int t, bool flag, const Zc& zc, float2* sz, typename M::acc4* buf,
                   Region& rg) {
    using acc = typename M::acc;
    typename M::acc4* part = M::part(d);
    const int2 og = tile_origin(F, t);
    const int ox = og.x, oy = og.y;
    if (zc.s) {   // the coarse values from this block's copy of the tail
#pragma unroll
        for (int j = 0; j < RJ; j++) {
            const int k = threadIdx.x + j * NT;
            if (k >= RN) break;
            const int x = ox - RH + k % RW, y = oy - RH + k / RW;
            rg.w[k] = l_inside(F, x, y) ? coarse_z<M>(d, zc, x, y) : make_float2(0.0f, 0.0f);
        }
    }
    __syncthreads();
    auto dg = [&](int k) {
        const float v = rg.dg[k];
        return v > 0.0f ? v : 0.0f;
    };
    // the new value of black slot k after the coarse correction (mg_up black())
    auto black = [&](int k) {
        const float4 w = M::Aslot(rg.a[k]);
        float2 sum = rg.u[k];
        float dn[4];
        float2 xm[4], zcv[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int j = k + RSTEP[q];
            dn[q] = dg(j);
            xm[q] = rg.v[j];
            zcv[q] = rg.w[j];
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float wd = wcomp(w, q);
            const float ux = wd * (xm[q].x + MG_OMEGA * zcv[q].x), uy = wd * (xm[q].y + MG_OMEGA * zcv[q].y);
            if (dn[q] > 0.0f) {
                sum.x += ux;
                sum.y += uy;
            }
        }
        return M::quot(sum, dg(k));
    };
    const int2 lc = colour_cell();
    const int lx = lc.x, ly = lc.y, cell = ly * 16 + lx;
    const int cx = ox + lx, cy = oy + ly;
    const int k0 = rslot(lx, ly);
    const bool red = threadIdx.x < 128;
    const bool unk = dg(k0) > 0.0f;
    float2 z = make_float2(0.0f, 0.0f);
    if (unk && !red) z = black(k0);
    sz[cell] = z;
    if (threadIdx.x < 32) {   // (a red warp, idle here) the black cells around the tile
        const int2 rc = ring_cell(threadIdx.x);
        const int kr = rslot(rc.x, rc.y);
        rg.ring[threadIdx.x] = dg(kr) > 0.0f ? black(kr) : make_float2(0.0f, 0.0f);
    }
    __syncthreads();
    typename M::acc4 a4 = M::zero4();
    if (l_inside(F, cx, cy)) {
        const int i = l_at(F, cx, cy);
        if (unk) {
            const float2 r = rg.u[k0];
            if (red) {
                const float4 w = M::Aslot(rg.a[k0]);
                float dn[4];
                float2 zb[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    dn[q] = dg(k0 + RSTEP[q]);
                    const int lnx = lx + NBX[q], lny = ly + NBY[q];
                    const bool here = lnx >= 0 && lny >= 0 && lnx < 16 && lny < 16;
                    zb[q] = here ? sz[lny * 16 + lnx] : rg.ring[ring_of(lnx, lny)];
                }
                float sx = r.x, sy = r.y;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float wd = wcomp(w, q);
                    const float ux = wd * zb[q].x, uy = wd * zb[q].y;
                    if (dn[q] > 0.0f) {
                        sx += ux;
                        sy += uy;
                    }
                }
                z = M::quot(make_float2(sx, sy), dg(k0));
            }
            a4 = M::prod4(r.x, z.x, r.y, z.y, r.x, r.x, r.y, r.y);
        }
        M::setZ(d, i, z);
    }
    if (flag) {
        buf[cell] = a4;
        block_tree(buf);
        if (threadIdx.x == 0) part[t] = buf[0];
    }
    __syncthreads();
}

// mg_tail.comp mode 0, computed by EVERY block in its own shared memory: the V-cycle on the
// tail levels, right-hand side the first tail level's mgr, result left in tl.x (the first
// tail level's slots). Every block gets the same values; the way up of the level above
// reads them from its own copy, so no grid barrier follows the tail.
template <class M>
DEV void phase_tail(const DevScene& d, const Tail& tl, bool writer) {
    const int first = d.lv.tail, last = d.lv.n - 1;
    // Each level's first half-sweep starts from zero: its black cells are r / D, the rest 0.
    // It is taken where the level's right-hand side is made (here for the first tail level,
    // in the restriction for the others), which saves a pass and a barrier per level.
    auto from_zero = [&](const Lv& L, int t, float2 r) {
        const int y = qdiv(t, L.wm), x = t - y * L.w;
        const int s = L.off - tl.base + t;
        const float D = tl.dg[s];
        if (!(D <= 0.0f) && ((x + y) & 1) == 0) tl.x[s] = divz(r, D);
        else tl.x[s] = make_float2(0.0f, 0.0f);
    };
    {
        const Lv F = lev(d.lv, first);
        for (int s = threadIdx.x; s < tl.nf; s += NT) {
            const float2 r = M::R(d, tl.base + s);
            tl.r[s] = r;
            from_zero(F, s, r);
        }
    }
    __syncthreads();
    // a half-sweep: every slot's reads are issued before its terms are summed (neighbour
    // slots clamped into the level and kept or not by the mask), in the shader's order
    auto sweep = [&](const Lv& L, int colour) {
        const int o = L.off - tl.base, n = L.w * L.h;
        const int lo = o, hi = o + n - 1;
        for (int t = threadIdx.x; t < n; t += NT) {
            const int y = qdiv(t, L.wm), x = t - y * L.w;
            const int s = o + t;
            const float D = tl.dg[s];
            const float2 r = tl.r[s];
            const bool mine = !(D <= 0.0f) && ((x + y) & 1) == colour;
            const float4 w = tail_a<M>(d, tl, s);
            const uint32_t m = tl.m[s];
            const float2 x0 = tl.x[max(s - 1, lo)], x1 = tl.x[min(s + 1, hi)];
            const float2 x2 = tl.x[max(s - L.w, lo)], x3 = tl.x[min(s + L.w, hi)];
            float2 sum = r;
            if (m & 1u) { sum.x += w.x * x0.x; sum.y += w.x * x0.y; }
            if (m & 2u) { sum.x += w.y * x1.x; sum.y += w.y * x1.y; }
            if (m & 4u) { sum.x += w.z * x2.x; sum.y += w.z * x2.y; }
            if (m & 8u) { sum.x += w.w * x3.x; sum.y += w.w * x3.y; }
            if (mine) tl.x[s] = divz(sum, D);
        }
        __syncthreads();
    };
    for (int l = first; l < last; l++) {
        Lv L = lev(d.lv, l), C = lev(d.lv, l + 1);
        const int o = L.off - tl.base, oc = C.off - tl.base;
        sweep(L, 1);
        for (int t = threadIdx.x; t < C.w * C.h; t += NT) {
            const int ccy = qdiv(t, C.wm), ccx = t - ccy * C.w;
            float sumx = 0.0f, sumy = 0.0f;
            const int step[4] = {-1, 1, -L.w, L.w};
            for (int k = 0; k < 4; k++) {
                int cx = 2 * ccx + (k & 1), cy = 2 * ccy + (k >> 1);
                if (!l_inside(L, cx, cy)) continue;
                int s = o + cy * L.w + cx;
                const uint32_t m = tl.m[s];
                if (!(m & 16u)) continue;
                float4 w = tail_a<M>(d, tl, s);
                float Ds = tl.dg[s];
                float2 xs = tl.x[s];
                float azx = Ds * xs.x, azy = Ds * xs.y;
                for (int q = 0; q < 4; q++) {
                    if (m & (1u << q)) {
                        float wd = wcomp(w, q);
                        float2 xn = tl.x[s + step[q]];
                        azx -= wd * xn.x;
                        azy -= wd * xn.y;
                    }
                }
                float2 rh = tl.r[s];
                sumx += rh.x - azx;
                sumy += rh.y - azy;
            }
            tl.r[oc + t] = make_float2(sumx, sumy);
            from_zero(C, t, make_float2(sumx, sumy));
        }
        __syncthreads();
    }
    {
        Lv L = lev(d.lv, last);
        for (int s = 1; s < 9; s++) sweep(L, s & 1);
    }
    for (int l = last - 1; l >= first; l--) {
        Lv F = lev(d.lv, l), C = lev(d.lv, l + 1);
        const int o = F.off - tl.base, oc = C.off - tl.base;
        for (int t = threadIdx.x; t < F.w * F.h; t += NT) {
            const int y = qdiv(t, F.wm), x = t - y * F.w;
            if (((x + y) & 1) == 0) continue;
            int s = o + t;
            float D = tl.dg[s];
            if (D <= 0.0f) continue;
            float4 w = tail_a<M>(d, tl, s);
            float2 sum = tl.r[s];
            const uint32_t m = tl.m[s];
            for (int q = 0; q < 4; q++) {
                int nx = x + NBX[q], ny = y + NBY[q];
                if (!(m & (1u << q))) continue;
                float wd = wcomp(w, q);
                float2 xn = tl.x[o + ny * F.w + nx];
                float2 xc = tl.x[oc + (ny >> 1) * C.w + (nx >> 1)];
                sum.x += wd * (xn.x + MG_OMEGA * xc.x);
                sum.y += wd * (xn.y + MG_OMEGA * xc.y);
            }
            tl.x[s] = divz(sum, D);
        }
        __syncthreads();
        sweep(F, 0);
    }
    if (writer)   // the first tail level's result (for inspection; a batch's way up reads it)
        for (int s = threadIdx.x; s < tl.nf; s += NT) M::setZ(d, tl.base + s, tl.x[s]);
}

// The active-tile lists of levels 0 .. tail - 1 of scene d (one block), from ptile.
DEV void build_plists(const DevScene& d) {
    for (int l = 0; l < d.lv.tail; l++) {
        const Lv L = lev(d.lv, l);
        compact_flags(d.ptile + L.toff, tiles_x(L) * tiles_y(L), d.plist + L.toff, d.pcount + l);
    }
}

// Level-0 tiles without unknowns keep zero partial sums through the solve (their tile
// bodies are never run): set them once at its start, every half and precision.
template <class M>
DEV void zero_inactive_tile(const DevScene& d, int t) {
    if (threadIdx.x != 0 || d.ptile[t] != 0u) return;
    const int n = d.nwg;
    M::part(d)[t] = M::zero4();
    M::part(d)[n + t] = M::zero4();
    if (M::kMixed) d.partials64[t] = Dbl4{0.0, 0.0, 0.0, 0.0};
}

// This block's share of the active-tile lists, read once per solve into shared memory:
// entry k of level l is work item blockIdx.x + k x gridDim.x (a tile index; in a batch the
// scene in the high 16 bits), so a phase starts on its tiles without first waiting for
// global memory. Items past kCachePer, or on levels past kCacheLevels, are read as before.
constexpr int kCacheLevels = 8, kCachePer = 32;
struct TileCache {
    uint32_t cnt[kCacheLevels];
    uint32_t item[kCacheLevels][kCachePer];
};

DEV void fill_cache(const DevScene& d, TileCache& tc) {
    for (int l = 0; l < kCacheLevels && l < d.lv.tail; l++) {
        const uint32_t cnt = *(volatile uint32_t*)&d.pcount[l];
        const uint32_t* list = d.plist + d.lv.toff[l];
        if (threadIdx.x == 0) tc.cnt[l] = cnt;
        for (int k = threadIdx.x; k < kCachePer; k += NT) {
            const uint32_t j = blockIdx.x + (uint32_t)k * gridDim.x;
            if (j < cnt) tc.item[l][k] = list[j];
        }
    }
    __syncthreads();
}

// For every active tile of level l of scene d, in this block's share of the list.
template <class F>
DEV void for_active(const DevScene& d, int l, const TileCache& tc, F&& f) {
    const bool cached = l < kCacheLevels;
    const uint32_t cnt = cached ? tc.cnt[l] : *(volatile uint32_t*)&d.pcount[l];
    const uint32_t* list = d.plist + d.lv.toff[l];
    int k = 0;
    for (uint32_t j = blockIdx.x; j < cnt; j += gridDim.x, k++)
        f((int)((cached && k < kCachePer) ? tc.item[l][k] : list[j]));
}

// The same share through the two-region pipeline (stage / finish halves of a tile body).
template <class S, class F>
DEV void pipe_active(const DevScene& d, int l, const TileCache& tc, Region* rg, S&& stage, F&& finish) {
    const bool cached = l < kCacheLevels;
    const uint32_t cnt = cached ? tc.cnt[l] : *(volatile uint32_t*)&d.pcount[l];
    const uint32_t* list = d.plist + d.lv.toff[l];
    pipe_tiles(
        cnt, [&](int k) { return (cached && k < kCachePer) ? tc.item[l][k] : list[blockIdx.x + (uint32_t)k * gridDim.x]; },
        rg, [&](uint32_t t, Region& r) { stage((int)t, r); }, [&](uint32_t t, Region& r) { finish((int)t, r); });
}

// Whether this block computes the tail of scene d: it owns a tile of the level above the tail
// (whose way up reads the tail's result from the block's own copy), or it is block 0.
DEV bool tail_reader(const DevScene& d, const TileCache& tc) {
    const int l = d.lv.tail - 1;
    const uint32_t cnt = l < kCacheLevels ? tc.cnt[l] : *(volatile uint32_t*)&d.pcount[l];
    return blockIdx.x == 0 || blockIdx.x < cnt;
}

// One V-cycle of one scene: level 0's right-hand side through R (fused with the CG update
// when R.q is set), result in mgz of level 0, partials of r.z and r.r. Returns false on a
// barrier timeout.
template <class M>
DEV bool vcycle(const DevScene& d, const Tail& tl, const Rsrc<M>& R, float2* r_out, const float2* p, const float2* r_new,
                float2* sz, typename M::acc4* buf, Region* rg, const TileCache& tc) {
    const int tail = d.lv.tail;
    for (int l = 0; l < tail; l++) {
        Rsrc<M> Rl = R;
        if (l > 0) Rl = Rsrc<M>{nullptr, nullptr, 0.0f, 0.0f};
        float2* ro = l == 0 ? r_out : nullptr;
        const Lv F = lev(d.lv, l), C = lev(d.lv, l + 1);
        pipe_active(d, l, tc, rg, [&](int t, Region& r) { stage_down<M>(d, F, t, Rl, ro != nullptr, p, r); },
                    [&](int t, Region& r) { finish_down<M>(d, F, C, t, Rl, ro, sz, r); });
        if (!grid_sync(d.K)) return false;
    }
    // only the blocks with a tile of the level above the tail read the tail's result (from
    // their own copy); block 0 also stores it
    if (tail_reader(d, tc)) phase_tail<M>(d, tl, blockIdx.x == 0);
    for (int l = tail - 1; l >= 0; l--) {
        const Lv C = lev(d.lv, l + 1);
        const Zc zc{(l == tail - 1) ? tl.x : nullptr, C.off, C.w};
        const Rsrc<M> rhs = l == 0 ? Rsrc<M>{r_new, nullptr, 0.0f, 0.0f} : Rsrc<M>{nullptr, nullptr, 0.0f, 0.0f};
        const Lv F = lev(d.lv, l);
        pipe_active(d, l, tc, rg, [&](int t, Region& r) { stage_up<M>(d, F, t, rhs, zc, r); },
                    [&](int t, Region& r) { finish_up<M>(d, F, t, l == 0, zc, sz, buf, r); });
        if (!grid_sync(d.K)) return false;
    }
    return true;
}

// b - A x of a level-0 cell's pressure column, and of both columns, evaluated as float pairs:
// each product exact (fma), the sum compensated (about 48 significant bits, FP64's job here
// at a small fraction of FP64's cost on this GPU), rounded once to FP32 at the end
DEV float2 pair_prod(float a, float b) {
    const float p = a * b;
    return make_float2(p, fmaf(a, b, -p));
}
DEV float2 pair_acc(float2 s, float2 t) { return ff_add(s.x, s.y, t.x, t.y); }

// The true residual |b - A x| / |b| of the pressure column after a mixed-precision solve:
// the tile's sums of (b - A x)^2 and b^2 as float pairs into part[t].
DEV void true_residual_tile(const DevScene& d, int t, FF4* part, FF4* buf) {
    const Lv F = lev(d.lv, 0);
    if (d.ptile[F.toff + t] == 0u) {
        if (threadIdx.x == 0) part[t] = FF4{make_float4(0.0f, 0.0f, 0.0f, 0.0f), make_float4(0.0f, 0.0f, 0.0f, 0.0f)};
        return;
    }
    const int2 og = tile_origin(F, t);
    const int cx = og.x + (threadIdx.x & 15), cy = og.y + (threadIdx.x >> 4);
    FF4 a4{make_float4(0.0f, 0.0f, 0.0f, 0.0f), make_float4(0.0f, 0.0f, 0.0f, 0.0f)};
    if (l_inside(F, cx, cy)) {
        const int i = l_at(F, cx, cy);
        const float D = d.mgd[i];
        if (D > 0.0f) {
            const float4 w = d.mga[i];
            const float b = d.prhs[i].x;
            const float2 dx = pair_prod(D, d.pres[i].x);
            float2 r = pair_acc(make_float2(b, 0.0f), make_float2(-dx.x, -dx.y));
            for (int q = 0; q < 4; q++) {
                const int nx = cx + NBX[q], ny = cy + NBY[q];
                if (unknown_op(d, F, nx, ny)) r = pair_acc(r, pair_prod(wcomp(w, q), d.pres[l_at(F, nx, ny)].x));
            }
            const float rf = r.x + r.y;
            a4 = ff_prod4(rf, rf, b, b, 0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
    buf[threadIdx.x] = a4;
    block_tree(buf);
    if (threadIdx.x == 0) part[t] = buf[0];
    __syncthreads();
}

// The mixed solve's refinement (residual replacement: van der Vorst and Ye, "Residual
// replacement strategies for Krylov subspace iterative methods", SIAM J. Sci. Comput. 22,
// 2000). The recurrence r -= alpha q drifts from b - A x by rounding; at a few points of the
// convergence the true residual of the current iterate is evaluated (the products and sums of
// the FP32 values as float pairs, rounded once to FP32) and, where the drift is worth removing, it
// replaces the carried one; the iteration continues with its directions unchanged.
//
// check_tile: on level-0 tile t, the true residual b - A x of both columns into rt, and the
// tile's sums of |b - A x|^2 and of (eps |A| |x|)^2 of the pressure column into part[t]: the
// second is the size of the residual that rounding x to FP32 alone leaves (eps = 2^-24), below
// which a replacement would feed that rounding back into the recurrence instead of removing
// drift.
DEV void check_tile(const DevScene& d, int t, float2* rt, FF4* part, FF4* buf) {
    const Lv F = lev(d.lv, 0);
    const FF4 zero{make_float4(0.0f, 0.0f, 0.0f, 0.0f), make_float4(0.0f, 0.0f, 0.0f, 0.0f)};
    if (d.ptile[F.toff + t] == 0u) {
        if (threadIdx.x == 0) part[t] = zero;
        return;
    }
    const int2 og = tile_origin(F, t);
    const int cx = og.x + (threadIdx.x & 15), cy = og.y + (threadIdx.x >> 4);
    FF4 a4 = zero;
    if (l_inside(F, cx, cy)) {
        const int i = l_at(F, cx, cy);
        const float D = d.mgd[i];
        if (D > 0.0f) {
            const float4 w = d.mga[i];
            const float2 x = d.pres[i];
            const float4 b = d.prhs[i];
            const float2 dx = pair_prod(D, x.x), dy = pair_prod(D, x.y);
            float2 rx = pair_acc(make_float2(b.x, 0.0f), make_float2(-dx.x, -dx.y));
            float2 ry = pair_acc(make_float2(b.y, 0.0f), make_float2(-dy.x, -dy.y));
            float ax = fabsf(D * x.x);
            for (int q = 0; q < 4; q++) {
                const int nx = cx + NBX[q], ny = cy + NBY[q];
                if (unknown_op(d, F, nx, ny)) {
                    const float2 xn = d.pres[l_at(F, nx, ny)];
                    const float wq = wcomp(w, q);
                    rx = pair_acc(rx, pair_prod(wq, xn.x));
                    ry = pair_acc(ry, pair_prod(wq, xn.y));
                    ax += fabsf(wq * xn.x);
                }
            }
            const float rfx = rx.x + rx.y, rfy = ry.x + ry.y;
            rt[i] = make_float2(rfx, rfy);
            const float fl = ax * 0x1p-24f;
            a4 = ff_prod4(rfx, rfx, fl, fl, 0.0f, 0.0f, 0.0f, 0.0f);
        } else {
            rt[i] = make_float2(0.0f, 0.0f);
        }
    }
    buf[threadIdx.x] = a4;
    block_tree(buf);
    if (threadIdx.x == 0) part[t] = buf[0];
    __syncthreads();
}

// ... and, where it is adopted, the carried residual r of tile t replaced by it.
DEV void adopt_tile(const DevScene& d, int t, const float2* rt, float2* r) {
    const Lv F = lev(d.lv, 0);
    if (d.ptile[F.toff + t] == 0u) return;
    const int2 og = tile_origin(F, t);
    const int cx = og.x + (threadIdx.x & 15), cy = og.y + (threadIdx.x >> 4);
    if (!l_inside(F, cx, cy)) return;
    const int i = l_at(F, cx, cy);
    if (d.mgd[i] > 0.0f) r[i] = rt[i];
}

// When to check: each time the pressure column's carried r.r has fallen by kCheckDrop (its
// norm by 100) since the start or the last check, before the solve has converged, unless a
// check found the carried residual already near the rounding floor.
// Whether to adopt: the true residual is more than twice the carried one (drift worth
// removing) and more than ten times the rounding floor.
constexpr double kCheckDrop = 1e-4;
template <class T>
DEV bool want_check(const Solve<T>& K) {
    return K.done[0] == 0u && K.floor_hit == 0u && K.rr[0] > 0 && K.rr[0] <= (T)kCheckDrop * K.rmark;
}
// Decides from the check's totals (|b - A x|^2, floor^2); updates the marks. Returns adopt.
template <class T>
DEV bool decide_check(Solve<T>& K, const Dbl4& tot) {
    K.rmark = K.rr[0];
    const double carried = (double)K.rr[0];
    if (carried <= 100.0 * tot.y) K.floor_hit = 1u;
    const bool adopt = tot.x > 4.0 * carried && tot.x > 100.0 * tot.y;
    if (adopt) K.replaced += 1u;
    return adopt;
}

// cg_apply.comp on level-0 tile t: p = z + beta p_old, q = A p (the FP32 operator), the
// tile's sum of p.q into part[n + t]. Copies (one ring around the tile is enough): the
// operator's diagonal, z (u) and p_old (v, unless both betas are zero); the couplings of the
// tile's own cells.
DEV void stage_apply(const DevScene& d, const Lv& F, int t, bool nob, const float2* p_old, Region& rg) {
    const int2 og = tile_origin(F, t);
    const int ox = og.x, oy = og.y;
#pragma unroll
    for (int j = 0; j < RJ; j++) {
        const int k = threadIdx.x + j * NT;
        if (k >= RN) break;
        const int kx = k % RW, ky = k / RW;
        if (kx == 0 || ky == 0 || kx == RW - 1 || ky == RW - 1) continue;
        const int x = ox - RH + kx, y = oy - RH + ky;
        const bool in = l_inside(F, x, y);
        const int i = in ? l_at(F, x, y) : 0;
        cp_async<4>(&rg.dg[k], d.mgd + i, in);
        cp_async<8>(&rg.u[k], d.mgz + i, in);
        if (!nob) cp_async<8>(&rg.v[k], p_old + i, in);
    }
    const int cx = ox + (threadIdx.x & 15), cy = oy + (threadIdx.x >> 4);
    const bool in = l_inside(F, cx, cy);
    cp_async<16>(&rg.a[rslot(threadIdx.x & 15, threadIdx.x >> 4)], d.mga + (in ? l_at(F, cx, cy) : 0), in);
}

template <class M>
DEV void finish_apply(const DevScene& d, const Lv& F, int t, float b0, float b1, float2* p_new, typename M::acc4* buf,
                      Region& rg) {
    using acc = typename M::acc;
    const int n = d.nwg;
    typename M::acc4* part = M::part(d) + n;
    const bool nob = b0 == 0.0f && b1 == 0.0f;
    const int2 og = tile_origin(F, t);
    const int ox = og.x, oy = og.y;
    __syncthreads();   // (every thread's copies have landed)
    auto dg = [&](int k) {
        const float v = rg.dg[k];
        return v > 0.0f ? v : 0.0f;
    };
    auto dir = [&](int k) {   // the direction p = z + beta p_old
        const float2 z = rg.u[k];
        if (nob) return z;
        const float2 po = rg.v[k];
        return make_float2(b0 != 0.0f ? z.x + b0 * po.x : z.x, b1 != 0.0f ? z.y + b1 * po.y : z.y);
    };
    const int cx = ox + (threadIdx.x & 15), cy = oy + (threadIdx.x >> 4);
    const int k0 = rslot(threadIdx.x & 15, threadIdx.x >> 4);
    typename M::acc4 a4 = M::zero4();
    if (l_inside(F, cx, cy)) {
        const int i = l_at(F, cx, cy);
        const float D = dg(k0);
        if (D > 0.0f) {
            const float2 pp = dir(k0);
            const float4 w = rg.a[k0];
            float dn[4];
            float2 pn[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                dn[q] = dg(k0 + RSTEP[q]);
                pn[q] = dir(k0 + RSTEP[q]);
            }
            float qx = D * pp.x, qy = D * pp.y;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float wd = wcomp(w, q);
                const float ux = wd * pn[q].x, uy = wd * pn[q].y;
                if (dn[q] > 0.0f) {
                    qx -= ux;
                    qy -= uy;
                }
            }
            p_new[i] = pp;
            d.cgq[i] = make_float2(qx, qy);
            a4 = M::prod4(0.0f, 0.0f, 0.0f, 0.0f, pp.x, qx, pp.y, qy);
        } else {
            p_new[i] = make_float2(0.0f, 0.0f);
        }
    }
    buf[threadIdx.x] = a4;
    block_tree(buf);
    if (threadIdx.x == 0) part[t] = buf[0];
    __syncthreads();
}

template <class T>
DEV T mix_was(T a, T keep, uint32_t was) { return mixf(a, keep, (float)was); }
template <>
DEV double mix_was<double>(double a, double keep, uint32_t was) { return was ? keep : a; }

// The solve's scalar steps (reduce_tail.glsl:61-116), shared by the single-scene and batched
// kernels so that a scene's numbers do not depend on which one solved it.
// mode 0 / 8: the start, from the totals a = (r.z, r.r) and b = (b.b).
template <class T, class A4>
DEV void scal_start(Solve<T>& K, const A4& a, const A4& b, T tx, T ty, int second) {
    K.bb[0] = b.x;
    K.bb[1] = b.y;
    K.rz[0] = a.x;
    K.rz[1] = a.y;
    K.rr[0] = a.z;
    K.rr[1] = a.w;
    K.rmark = a.z;
    K.replaced = 0u;
    K.floor_hit = 0u;
    K.adopt = 0u;
    K.beta[0] = K.beta[1] = 0;
    K.alpha[0] = K.alpha[1] = 0;
    K.iters[0] = K.iters[1] = 0u;
    K.done[0] = a.z <= tx * tx * b.x ? 1u : 0u;
    K.done[1] = a.w <= ty * ty * b.y ? 1u : 0u;
    if (second) K.done[1] = 1u;
    // a non-finite right-hand side or residual: no iteration can converge, stop here
    K.bad = finite4(a) && finite4(b) ? 0u : 1u;
    if (K.bad) K.done[0] = K.done[1] = 1u;
}

// mode 1: the step lengths from p.q.
template <class T, class A4>
DEV void scal_alpha(Solve<T>& K, const A4& b) {
    T ax = 0, ay = 0;
    if (K.done[0] == 0u && b.z > 0) ax = K.rz[0] / b.z;
    if (K.done[1] == 0u && b.w > 0) ay = K.rz[1] / b.w;
    K.alpha[0] = ax;
    K.alpha[1] = ay;
}

// mode 2: convergence and the next direction's beta from the new (r.z, r.r).
template <class T, class A4>
DEV void scal_beta(Solve<T>& K, const A4& a, T tx, T ty) {
    uint32_t was0 = K.done[0], was1 = K.done[1];
    K.iters[0] += 1u - was0;
    K.iters[1] += 1u - was1;
    uint32_t now0 = a.z <= tx * tx * K.bb[0] ? 1u : 0u, now1 = a.w <= ty * ty * K.bb[1] ? 1u : 0u;
    uint32_t d0 = was0 > now0 ? was0 : now0, d1 = was1 > now1 ? was1 : now1;
    T bx = 0, by = 0;
    if (d0 == 0u && K.rz[0] > 0) bx = a.x / K.rz[0];
    if (d1 == 0u && K.rz[1] > 0) by = a.y / K.rz[1];
    K.beta[0] = bx;
    K.beta[1] = by;
    K.rz[0] = a.x;
    K.rz[1] = a.y;
    K.rr[0] = mix_was<T>(a.z, K.rr[0], was0);
    K.rr[1] = mix_was<T>(a.w, K.rr[1], was1);
    K.done[0] = d0;
    K.done[1] = d1;
    if (!finite4(a)) {
        K.bad = 1u;
        K.done[0] = K.done[1] = 1u;
    }
}

// mode 3 / 9: the statistics of the finished solve into the scene's SolveState.
template <class M, class T>
DEV void scal_stats(SolveState* G, const Solve<T>& K, int second, double true_rel) {
    if (true_rel >= 0.0) {
        G->p_true_res = (float)true_rel;
        G->p_true_res_max = maxf(G->p_true_res_max, (float)true_rel);
    }
    G->p_repl += K.replaced;
    for (int c = 0; c < 2; c++) {
        G->p_rz[c] = (float)K.rz[c];
        G->p_alpha[c] = (float)K.alpha[c];
        G->p_beta[c] = (float)K.beta[c];
        G->p_bb[c] = (float)K.bb[c];
        G->p_rr[c] = (float)K.rr[c];
        G->p_done[c] = K.done[c];
        if (!second) G->p_iters[c] = K.iters[c];
    }
    if (second) G->p2_iters = K.iters[0];
    G->solves += 1u;
    if (!second) {
        uint32_t m = K.iters[0] > K.iters[1] ? K.iters[0] : K.iters[1];
        if (m > G->p_it_max) G->p_it_max = m;
        if (K.done[0] == 0u) G->p_unconv += 1u;
        if (m > G->f_it[0]) G->f_it[0] = m;
        if (K.done[0] == 0u) G->f_un[0] += 1u;
    } else {
        if (K.iters[0] > G->p2_it_max) G->p2_it_max = K.iters[0];
        if (K.done[0] == 0u) G->p2_unconv += 1u;
        if (K.iters[0] > G->f_it[1]) G->f_it[1] = K.iters[0];
        if (K.done[0] == 0u) G->f_un[1] += 1u;
    }
    if (K.bad) atomicOr(&G->error, ERR_DIVERGED);
    const float rel = K.bb[0] > 0 ? (float)sqrt((double)K.rr[0] / (double)K.bb[0]) : 0.0f;
    G->p_res_max = maxf(G->p_res_max, M::kMixed ? rel : (K.bb[0] > 0 ? sqrtf((float)K.rr[0] / (float)K.bb[0]) : 0.0f));
}

}  // namespace

// The whole pressure solve. `second`: the solve after the implicit viscosity (cg_reduce
// mode 8/9: same matrix and hierarchy, density correction counted as solved).
template <class M>
__global__ void __launch_bounds__(NT, 2) k_mgpcg(DevScene d, int second, int scale_mode) {
    grid_begin();
    using acc = typename M::acc;
    using acc4 = typename M::acc4;
    __shared__ TileCache tc;
    __shared__ float2 sz[NT];
    // the block's tree buffer: float pairs in mixed precision (the refinement's checks), whose
    // bytes the dot products' trees use as acc4 in other phases
    __shared__ typename std::conditional<M::kMixed, FF4, acc4>::type buf_raw[NT];
    acc4* buf = reinterpret_cast<acc4*>(buf_raw);
    __shared__ Solve<acc> K;
    // dynamic: the staging regions, then the tail levels (matrices, iterates, masks: kept for
    // the whole solve); the tail's right-hand sides, live only in the tail phase, when no
    // tile is being staged, in the regions' bytes
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    Region* rg = reinterpret_cast<Region*>(dyn_smem);
    const DevParams* P = d.P;
    const int n = d.nwg;
    acc4* part = M::part(d);
    const Tail tl = make_tail(d, dyn_smem + kDepth * sizeof(Region), reinterpret_cast<float2*>(dyn_smem));
    if (!second) {
        for (int t = blockIdx.x; t < n; t += gridDim.x) cg_scale_tile<M>(d, t, scale_mode);
        for (int l = 1; l <= d.lv.tail; l++) {
            if (!grid_sync(d.K)) return;
            const int T = level_tiles(d, l);
            for (int t = blockIdx.x; t < T; t += gridDim.x) mg_build_tile<M>(d, l - 1, t);
        }
        if (!grid_sync(d.K)) return;
    }
    // the active-tile lists (ptile is final now) and the inactive tiles' zero partial sums
    if (blockIdx.x == 0) build_plists(d);
    for (int t = blockIdx.x; t < n; t += gridDim.x) zero_inactive_tile<M>(d, t);
    if (!grid_sync(d.K)) return;
    fill_cache(d, tc);
    if (tail_reader(d, tc)) tail_setup<M>(d, tl, blockIdx.x == 0);
    float2* r_cur = d.mgr;    // level 0 of mgr: the residual, double-buffered with mgr2
    float2* r_nxt = d.mgr2;
    for_active(d, 0, tc, [&](int t) { residual_tile<M>(d, t, r_cur, buf, false); });
    if (!grid_sync(d.K)) return;
    // b.b now, while nothing writes the second half of the partials: the first apply phase
    // after the V-cycle does, and a block can reach it before a slower one has summed them
    const auto b = M::fin(total(part + n, n, buf));
    if (!vcycle<M>(d, tl, Rsrc<M>{r_cur, nullptr, 0.0f, 0.0f}, nullptr, nullptr, r_cur, sz, buf, rg, tc)) return;
    const acc tx = (acc)P->tol[0], ty = (acc)P->tol[1];
    {
        const auto a = M::fin(total(part, n, buf));
        if (threadIdx.x == 0) scal_start<acc>(K, a, b, tx, ty, second);
        __syncthreads();
    }
    float2* p_old = d.cgp;
    float2* p_new = d.cgp2;
    const Lv L0 = lev(d.lv, 0);
    const uint32_t cap = d.K->cap[second ? 1 : 0];   // this frame's recorded iterations
    for (uint32_t it = 0; it < cap; it++) {
        if (K.done[0] && K.done[1]) break;
        if constexpr (M::kMixed) {
            // the refinement (the same decisions in every block: the same K); q is free until
            // the apply phase rewrites it, and the partials' second half until it sums p.q
            if (it > 0 && want_check(K)) {
                FF4* pc = reinterpret_cast<FF4*>(d.partials64) + n;
                for_active(d, 0, tc, [&](int t) { check_tile(d, t, d.cgq, pc, reinterpret_cast<FF4*>(buf_raw)); });
                if (!grid_sync(d.K)) return;
                const Dbl4 tot = to_dbl(total(pc, n, reinterpret_cast<FF4*>(buf_raw)));
                __shared__ int s_adopt;
                if (threadIdx.x == 0) s_adopt = decide_check(K, tot) ? 1 : 0;
                __syncthreads();
                if (s_adopt) {
                    for_active(d, 0, tc, [&](int t) { adopt_tile(d, t, d.cgq, r_cur); });
                    if (!grid_sync(d.K)) return;
                }
            }
        }
        const float b0 = (float)K.beta[0], b1 = (float)K.beta[1];
        const bool nob = b0 == 0.0f && b1 == 0.0f;
        pipe_active(d, 0, tc, rg, [&](int t, Region& r) { stage_apply(d, L0, t, nob, p_old, r); },
                    [&](int t, Region& r) { finish_apply<M>(d, L0, t, b0, b1, p_new, buf, r); });
        if (!grid_sync(d.K)) return;
        {
            const auto b = M::fin(total(part + n, n, buf));
            if (threadIdx.x == 0) scal_alpha<acc>(K, b);
            __syncthreads();
        }
        Rsrc<M> R{r_cur, d.cgq, (float)K.alpha[0], (float)K.alpha[1]};
        if (!vcycle<M>(d, tl, R, r_nxt, p_new, r_nxt, sz, buf, rg, tc)) return;
        {
            const auto a = M::fin(total(part, n, buf));
            if (threadIdx.x == 0) scal_beta<acc>(K, a, tx, ty);
            __syncthreads();
        }
        float2* t = p_old;
        p_old = p_new;
        p_new = t;
        t = r_cur;
        r_cur = r_nxt;
        r_nxt = t;
    }
    double true_rel = -1.0;
    if constexpr (M::kMixed) {
        FF4* pt = reinterpret_cast<FF4*>(d.partials64);
        for_active(d, 0, tc, [&](int t) { true_residual_tile(d, t, pt, reinterpret_cast<FF4*>(buf_raw)); });
        if (!grid_sync(d.K)) return;
        const Dbl4 t4 = to_dbl(total(pt, n, reinterpret_cast<FF4*>(buf_raw)));
        true_rel = t4.y > 0.0 ? sqrt(t4.x / t4.y) : 0.0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) scal_stats<M, acc>(d.K, K, second, true_rel);
    trace_launch_done(d.K);
}

// ---- many scenes in one persistent solve --------------------------------------------------
//
// The same solve for a batch of scenes of any sizes in one cooperative launch: every phase
// runs over a flattened list of (scene, tile) work items of its level, so the small levels
// of many scenes fill one pass instead of leaving most blocks idle, and one set of grid
// barriers serves them all. Each scene's tiles go through the same tile bodies as above and
// its scalars through the same steps, summed by one block over its own partials in the
// same order; so a scene's result is the same alone and in any batch, to the bit. The
// differences: a scene's tail is computed by one block into global memory (one more
// barrier per V-cycle), each reduction is a phase of its own followed by a barrier (the
// scalars then live in global memory), and a converged scene (or one at its iteration
// limit) simply drops out of the work lists.

namespace {

// The scene, tile and level of work item g of level l: o holds the ns + 1 prefix sums of
// the scenes' tile counts of level l.
DEV int scene_of(const int* o, int ns, int g) {
    int lo = 0, hi = ns;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (o[mid] <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <class F>
DEV void for_tiles(const BatchView& B, int l, F&& f) {
    const int* o = B.off + l * (B.ns + 1);
    const int N = o[B.ns];
    for (int g = blockIdx.x; g < N; g += gridDim.x) {
        const int s = scene_of(o, B.ns, g);
        f(s, B.scenes[s], g - o[s]);
    }
}

// For every active tile of level l over the batch's scenes (B.aoff: the prefix sums of the
// scenes' active-tile counts, built at the solve's start).
DEV uint32_t batch_item(const BatchView& B, int l, int g) {
    const int* o = B.aoff + l * (B.ns + 1);
    const int s = scene_of(o, B.ns, g);
    const DevScene& d = B.scenes[s];
    return ((uint32_t)s << 16) | d.plist[d.lv.toff[l] + (g - o[s])];
}

DEV void fill_cache_b(const BatchView& B, TileCache& tc) {
    for (int l = 0; l < kCacheLevels && l < B.max_tail; l++) {
        const int N = *(volatile const int*)&B.aoff[l * (B.ns + 1) + B.ns];
        if (threadIdx.x == 0) tc.cnt[l] = (uint32_t)N;
        for (int k = threadIdx.x; k < kCachePer; k += NT) {
            const int g = blockIdx.x + k * gridDim.x;
            if (g < N) tc.item[l][k] = batch_item(B, l, g);
        }
    }
    __syncthreads();
}

template <class F>
DEV void for_active_b(const BatchView& B, int l, const TileCache& tc, F&& f) {
    const bool cached = l < kCacheLevels;
    const int N = cached ? (int)tc.cnt[l] : *(volatile const int*)&B.aoff[l * (B.ns + 1) + B.ns];
    int k = 0;
    for (int g = blockIdx.x; g < N; g += gridDim.x, k++) {
        const uint32_t it = (cached && k < kCachePer) ? tc.item[l][k] : batch_item(B, l, g);
        const int s = (int)(it >> 16);
        f(s, B.scenes[s], (int)(it & 0xffffu));
    }
}

// The same through the two-region pipeline: stage(s, d, t, rg) / finish(s, d, t, rg).
template <class S, class F>
DEV void pipe_active_b(const BatchView& B, int l, const TileCache& tc, Region* rg, S&& stage, F&& finish) {
    const bool cached = l < kCacheLevels;
    const int N = cached ? (int)tc.cnt[l] : *(volatile const int*)&B.aoff[l * (B.ns + 1) + B.ns];
    pipe_tiles(
        (uint32_t)N,
        [&](int k) {
            return (cached && k < kCachePer) ? tc.item[l][k] : batch_item(B, l, (int)(blockIdx.x + (uint32_t)k * gridDim.x));
        },
        rg,
        [&](uint32_t it, Region& r) {
            const int s = (int)(it >> 16);
            stage(s, B.scenes[s], (int)(it & 0xffffu), r);
        },
        [&](uint32_t it, Region& r) {
            const int s = (int)(it >> 16);
            finish(s, B.scenes[s], (int)(it & 0xffffu), r);
        });
}

DEV float2* parity_r(const DevScene& d, int it) { return (it & 1) ? d.mgr2 : d.mgr; }
DEV float2* parity_p(const DevScene& d, int it) { return (it & 1) ? d.cgp2 : d.cgp; }

}  // namespace

static_assert(sizeof(Region) % 16 == 0, "regions laid end to end in dynamic shared memory");

// The batched solve's dynamic shared memory: the staging regions and, during the tail phase
// only, one scene's tail (a scene's tail is rebuilt and solved within that phase and its
// result stored to global memory, while no tile is being staged), in the same bytes.
size_t pressure_batch_smem(const Levels& lv) {
    return std::max(tail_bytes(tail_cells(lv), true, tail_first_cells(lv)), (size_t)kDepth * sizeof(Region));
}

template <class M>
__global__ void __launch_bounds__(NT, 4) k_mgpcg_batch(BatchView B, int second) {
    grid_begin();
    using acc = typename M::acc;
    using acc4 = typename M::acc4;
    __shared__ TileCache tc;
    __shared__ float2 sz[NT];
    // the block's tree buffer: float pairs in mixed precision (the refinement's checks), whose
    // bytes the dot products' trees use as acc4 in other phases
    __shared__ typename std::conditional<M::kMixed, FF4, acc4>::type buf_raw[NT];
    acc4* buf = reinterpret_cast<acc4*>(buf_raw);
    __shared__ int s_run;
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    Region* rg = reinterpret_cast<Region*>(dyn_smem);
    unsigned char* tail_smem = dyn_smem;
    Solve<acc>* KS = reinterpret_cast<Solve<acc>*>(B.scal);
    SolveState* BK = B.K;
    auto tol = [&](const DevScene& d, int c) { return (acc)d.P->tol[c]; };
    // a scene takes part in iteration it while neither converged nor at its limit
    auto running = [&](int s, int it) {
        const Solve<acc>& K = KS[s];
        return !(K.done[0] && K.done[1]) && (uint32_t)it < B.scenes[s].K->cap[second ? 1 : 0];
    };
    if (!second) {
        for_tiles(B, 0, [&](int s, const DevScene& d, int t) { cg_scale_tile<M>(d, t, B.scale[s]); });
        for (int l = 1; l <= B.max_tail; l++) {
            if (!grid_sync(BK)) return;
            for_tiles(B, l, [&](int s, const DevScene& d, int t) { mg_build_tile<M>(d, l - 1, t); });
        }
        if (!grid_sync(BK)) return;
    }
    // every scene's active-tile lists (one block each) and the inactive tiles' zero partials
    for (int s = blockIdx.x; s < B.ns; s += gridDim.x) build_plists(B.scenes[s]);
    for_tiles(B, 0, [&](int s, const DevScene& d, int t) { zero_inactive_tile<M>(d, t); });
    if (!grid_sync(BK)) return;
    // ... and their prefix sums per level over the scenes
    if (blockIdx.x == 0) {
        for (int l = threadIdx.x; l < B.max_tail; l += NT) {
            int* o = B.aoff + l * (B.ns + 1);
            int acc_ = 0;
            o[0] = 0;
            for (int k = 0; k < B.ns; k++) {
                const DevScene& d = B.scenes[k];
                acc_ += l < d.lv.tail ? (int)d.pcount[l] : 0;
                o[k + 1] = acc_;
            }
        }
    }
    if (!grid_sync(BK)) return;
    fill_cache_b(B, tc);
    for_active_b(B, 0, tc, [&](int s, const DevScene& d, int t) { residual_tile<M>(d, t, d.mgr, buf, false); });
    if (!grid_sync(BK)) return;
    // b.b of each scene (before the first apply phase reuses those partials)
    for (int s = blockIdx.x; s < B.ns; s += gridDim.x) {
        const DevScene& d = B.scenes[s];
        const auto b = M::fin(total(M::part(d) + d.nwg, d.nwg, buf));
        if (threadIdx.x == 0) {
            KS[s].bb[0] = b.x;
            KS[s].bb[1] = b.y;
            KS[s].done[0] = KS[s].done[1] = 0u;
        }
        __syncthreads();
    }
    // One V-cycle on every running scene; it < 0: the start (right-hand side the residual
    // of x0, no update); else the iteration's, fused with its update.
    auto vcycle_all = [&](int it) -> bool {
        const bool fused = it >= 0;
        const int ir = fused ? it : 0;
        for (int l = 0; l < B.max_tail; l++) {
            auto rsrc = [&](int s, const DevScene& d) {
                const Solve<acc>& K = KS[s];
                Rsrc<M> R{nullptr, nullptr, 0.0f, 0.0f};
                if (l == 0) R = fused ? Rsrc<M>{parity_r(d, ir), d.cgq, (float)K.alpha[0], (float)K.alpha[1]}
                                      : Rsrc<M>{parity_r(d, ir), nullptr, 0.0f, 0.0f};
                return R;
            };
            pipe_active_b(
                B, l, tc, rg,
                [&](int s, const DevScene& d, int t, Region& r) {
                    if (l >= d.lv.tail || (fused && !running(s, it))) return;
                    stage_down<M>(d, lev(d.lv, l), t, rsrc(s, d), l == 0 && fused, parity_p(d, ir + 1), r);
                },
                [&](int s, const DevScene& d, int t, Region& r) {
                    if (l >= d.lv.tail || (fused && !running(s, it))) return;
                    finish_down<M>(d, lev(d.lv, l), lev(d.lv, l + 1), t, rsrc(s, d), (l == 0 && fused) ? parity_r(d, ir + 1) : nullptr,
                                   sz, r);
                });
            if (!grid_sync(BK)) return false;
        }
        for (int s = blockIdx.x; s < B.ns; s += gridDim.x) {
            if (fused && !running(s, it)) continue;
            const DevScene& d = B.scenes[s];
            const Tail tl = make_tail(d, tail_smem, nullptr, true);
            tail_setup<M>(d, tl, false);
            phase_tail<M>(d, tl, true);
        }
        if (!grid_sync(BK)) return false;
        for (int l = B.max_tail - 1; l >= 0; l--) {
            auto zc_of = [&](const DevScene& d) {
                const Lv C = lev(d.lv, l + 1);
                return Zc{nullptr, C.off, C.w};
            };
            auto rhs_of = [&](const DevScene& d) {
                return l == 0 ? Rsrc<M>{parity_r(d, fused ? ir + 1 : 0), nullptr, 0.0f, 0.0f}
                              : Rsrc<M>{nullptr, nullptr, 0.0f, 0.0f};
            };
            pipe_active_b(
                B, l, tc, rg,
                [&](int s, const DevScene& d, int t, Region& r) {
                    if (l >= d.lv.tail || (fused && !running(s, it))) return;
                    stage_up<M>(d, lev(d.lv, l), t, rhs_of(d), zc_of(d), r);
                },
                [&](int s, const DevScene& d, int t, Region& r) {
                    if (l >= d.lv.tail || (fused && !running(s, it))) return;
                    finish_up<M>(d, lev(d.lv, l), t, l == 0, zc_of(d), sz, buf, r);
                });
            if (!grid_sync(BK)) return false;
        }
        return true;
    };
    if (!vcycle_all(-1)) return;
    for (int s = blockIdx.x; s < B.ns; s += gridDim.x) {
        const DevScene& d = B.scenes[s];
        const auto a = M::fin(total(M::part(d), d.nwg, buf));
        if (threadIdx.x == 0) {
            auto b = a;
            b.x = KS[s].bb[0];
            b.y = KS[s].bb[1];
            scal_start<acc>(KS[s], a, b, tol(d, 0), tol(d, 1), second);
        }
        __syncthreads();
    }
    if (!grid_sync(BK)) return;
    for (int it = 0;; it++) {
        if (threadIdx.x == 0) {
            int run = 0;
            for (int s = 0; s < B.ns && !run; s++) run = running(s, it) ? 1 : 0;
            s_run = run;
        }
        __syncthreads();
        if (!s_run) break;
        if constexpr (M::kMixed) {   // the refinement, as the single-scene solve takes it
            // a scene checks at iteration it when want_check holds at the top of the iteration;
            // one block decides (after the check's barrier) and leaves the outcome in KS[s].adopt
            auto chk = [&](int s) { return it > 0 && running(s, it) && want_check(KS[s]); };
            if (threadIdx.x == 0) {
                int any = 0;
                for (int s = 0; s < B.ns && !any; s++) any = chk(s) ? 1 : 0;
                s_run = any;
            }
            __syncthreads();
            if (s_run) {
                for_active_b(B, 0, tc, [&](int s, const DevScene& d, int t) {
                    if (chk(s)) check_tile(d, t, d.cgq, reinterpret_cast<FF4*>(d.partials64) + d.nwg, reinterpret_cast<FF4*>(buf_raw));
                });
                if (!grid_sync(BK)) return;
                // each scene's decision by one block (it alone writes KS[s] until the next barrier)
                for (int s = blockIdx.x; s < B.ns; s += gridDim.x) {
                    if (!chk(s)) continue;
                    const DevScene& d = B.scenes[s];
                    const Dbl4 tot = to_dbl(total(reinterpret_cast<FF4*>(d.partials64) + d.nwg, d.nwg, reinterpret_cast<FF4*>(buf_raw)));
                    if (threadIdx.x == 0) KS[s].adopt = decide_check(KS[s], tot) ? 1u : 0u;
                    __syncthreads();
                }
                if (!grid_sync(BK)) return;
                // every block reads the same decisions: without an adoption, the adopt pass
                // and its barrier are skipped by all of them
                if (threadIdx.x == 0) {
                    int adopt = 0;
                    for (int s = 0; s < B.ns && !adopt; s++) adopt = KS[s].adopt ? 1 : 0;
                    s_run = adopt;
                }
                __syncthreads();
                if (s_run) {
                    for_active_b(B, 0, tc, [&](int s, const DevScene& d, int t) {
                        if (KS[s].adopt) adopt_tile(d, t, d.cgq, parity_r(d, it));
                    });
                    if (!grid_sync(BK)) return;
                    for (int s = blockIdx.x; s < B.ns; s += gridDim.x)
                        if (threadIdx.x == 0) KS[s].adopt = 0u;
                }
            }
        }
        pipe_active_b(
            B, 0, tc, rg,
            [&](int s, const DevScene& d, int t, Region& r) {
                if (!running(s, it)) return;
                const float b0 = (float)KS[s].beta[0], b1 = (float)KS[s].beta[1];
                stage_apply(d, lev(d.lv, 0), t, b0 == 0.0f && b1 == 0.0f, parity_p(d, it), r);
            },
            [&](int s, const DevScene& d, int t, Region& r) {
                if (!running(s, it)) return;
                finish_apply<M>(d, lev(d.lv, 0), t, (float)KS[s].beta[0], (float)KS[s].beta[1], parity_p(d, it + 1), buf, r);
            });
        if (!grid_sync(BK)) return;
        for (int s = blockIdx.x; s < B.ns; s += gridDim.x) {
            if (!running(s, it)) continue;
            const DevScene& d = B.scenes[s];
            const auto b = M::fin(total(M::part(d) + d.nwg, d.nwg, buf));
            if (threadIdx.x == 0) scal_alpha<acc>(KS[s], b);
            __syncthreads();
        }
        if (!grid_sync(BK)) return;
        if (!vcycle_all(it)) return;
        for (int s = blockIdx.x; s < B.ns; s += gridDim.x) {
            if (!running(s, it)) continue;
            const DevScene& d = B.scenes[s];
            const auto a = M::fin(total(M::part(d), d.nwg, buf));
            if (threadIdx.x == 0) scal_beta<acc>(KS[s], a, tol(d, 0), tol(d, 1));
            __syncthreads();
        }
        if (!grid_sync(BK)) return;
    }
    if constexpr (M::kMixed) {
        for_active_b(B, 0, tc, [&](int s, const DevScene& d, int t) {
            true_residual_tile(d, t, reinterpret_cast<FF4*>(d.partials64), reinterpret_cast<FF4*>(buf_raw));
        });
        if (!grid_sync(BK)) return;
    }
    for (int s = blockIdx.x; s < B.ns; s += gridDim.x) {
        const DevScene& d = B.scenes[s];
        double true_rel = -1.0;
        if constexpr (M::kMixed) {
            const Dbl4 t4 = to_dbl(total(reinterpret_cast<FF4*>(d.partials64), d.nwg, reinterpret_cast<FF4*>(buf_raw)));
            true_rel = t4.y > 0.0 ? sqrt(t4.x / t4.y) : 0.0;
        }
        if (threadIdx.x == 0) scal_stats<M, acc>(d.K, KS[s], second, true_rel);
        __syncthreads();
    }
    trace_launch_done(BK);
}

size_t pressure_smem(const Levels& lv) {
    // the tail's first level has at most 1500 cells and each coarser level at most half the
    // one above, so a tail holds fewer than 3000 cells
    static_assert(kDepth * sizeof(Region) >= 4096 * sizeof(float2), "the tail's right-hand sides fit in the regions");
    return kDepth * sizeof(Region) + tail_bytes(tail_cells(lv), false);
}

namespace {
template <class M>
int blocks_max(int device, size_t smem) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    // Opt in to the dynamic shared memory the largest tank so far needs (static + dynamic
    // above 48 KB needs it). The attribute belongs to the kernel on the current device, so
    // it is tracked per device.
    static size_t opted[kMaxDevices] = {};
    if (device < 0 || device >= kMaxDevices || smem > opted[device]) {
        cudaFuncSetAttribute(k_mgpcg<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (device >= 0 && device < kMaxDevices) opted[device] = smem;
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mgpcg<M>, NT, smem);
    return sms * per;
}
}  // namespace

int pressure_blocks_max(int device, size_t smem, bool mixed) {
    return mixed ? blocks_max<Mixed>(device, smem) : blocks_max<Plain>(device, smem);
}

namespace {
template <class M>
int batch_blocks_max(int device, size_t smem) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    static size_t opted[kMaxDevices] = {};
    if (device < 0 || device >= kMaxDevices || smem > opted[device]) {
        cudaFuncSetAttribute(k_mgpcg_batch<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (device >= 0 && device < kMaxDevices) opted[device] = smem;
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mgpcg_batch<M>, NT, smem);
    return sms * per;
}
}  // namespace

int pressure_batch_blocks_max(int device, size_t smem, bool mixed) {
    return mixed ? batch_blocks_max<Mixed>(device, smem) : batch_blocks_max<Plain>(device, smem);
}

size_t pressure_batch_scalar_bytes() { return sizeof(Solve<double>); }

cudaError_t launch_pressure_batch(const BatchView& B, bool mixed, int blocks, size_t smem, cudaStream_t st, int second) {
    cudaMemsetAsync(&B.K->bar_count, 0, sizeof(uint32_t), st);
    void* args[] = {(void*)&B, &second};
    const void* fn = mixed ? (const void*)k_mgpcg_batch<Mixed> : (const void*)k_mgpcg_batch<Plain>;
    return cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(NT), args, smem, st);
}

// FluidSim::poll_readbacks' adaptation of a recorded iteration count (mod.rs:3100-3106):
// after a frame in which the solve ran out, half again plus two; otherwise the frame's most
// iterations plus the margin's share (truncated, as `as u32`) plus two, within [2, max].
DEV uint32_t adapt_rec(uint32_t rec, uint32_t used, uint32_t unconverged, uint32_t max, float margin) {
    if (unconverged > 0u) return min(rec + rec / 2u + 2u, max);
    const uint32_t v = used + (uint32_t)((float)used * margin) + 2u;
    return v < 2u ? 2u : (v > max ? max : v);
}

// The end of a frame (a step call): the recorded counts adapted from the frame's solves as
// the reference adapts them when the frame's read-back arrives (mod.rs:3093-3114: the second
// solve's follows the first's when it does not run; the viscosity solve's with margin 0.5),
// the next frame's limits, and the frame's statistics cleared.
DEV void frame_end(const DevScene& d) {
    const DevParams* P = d.P;
    SolveState* K = d.K;
    K->rec[0] = adapt_rec(K->rec[0], K->f_it[0], K->f_un[0], P->pressure_max_iters, P->iters_margin);
    if (P->visc_mode == 2 && P->viscous_projection != 0)
        K->rec[1] = adapt_rec(K->rec[1], K->f_it[1], K->f_un[1], P->pressure_max_iters, P->iters_margin);
    else
        K->rec[1] = K->rec[0];
    K->rec[2] = adapt_rec(K->rec[2], K->f_it[2], K->f_un[2], P->viscosity_max_iters, 0.5f);
    for (int k = 0; k < 3; k++) {
        K->cap[k] = recorded_limit(K->rec[k], k == 2, P->viscosity_precond != 0);
        K->f_it[k] = 0u;
        K->f_un[k] = 0u;
    }
}

__global__ void k_frame_end(DevScene d) { frame_end(d); }
__global__ void k_frame_end_many(const DevScene* scenes, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) frame_end(scenes[s]);
}

void launch_frame_end(const DevScene& d, cudaStream_t st) { k_frame_end<<<1, 1, 0, st>>>(d); }
void launch_frame_end_many(const DevScene* scenes, int n, cudaStream_t st) {
    if (n > 0) k_frame_end_many<<<(n + 127) / 128, 128, 0, st>>>(scenes, n);
}

cudaError_t launch_pressure(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st, int second) {
    // barrier counter back to zero (a solve left by a timeout may have stopped mid-barrier)
    cudaMemsetAsync(&d.K->bar_count, 0, sizeof(uint32_t), st);
    // cg_scale mode 1: with the viscosity between two solves, the first starts from last
    // substep's P1 alone (viscous_warm, mod.rs:2979-2983)
    int scale_mode = (!second && cfg.visc_mode == 2 && cfg.twice && cfg.viscous_warm) ? 1 : 0;
    void* args[] = {(void*)&d, &second, &scale_mode};
    const void* fn = cfg.mixed ? (const void*)k_mgpcg<Mixed> : (const void*)k_mgpcg<Plain>;
    const int blocks = cfg.mixed ? cfg.mg_blocks_mixed : cfg.mg_blocks;
    return cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(NT), args, pressure_smem(d.lv), st);
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
constexpr int kStaticMinSide = 16;           // and its narrowest side

// The most any accepted grid (both sides >= 16, at most kStaticMaxCells cells) needs of each
// part of the array: hierarchy cells, tiles of the levels down to the tail, level-0 tiles.
// For a given width every count grows with the height, so the tallest grid of each width is
// the one to check. Long thin grids need the most hierarchy: once a level is one cell high,
// each further level halves only the width.
struct StaticNeed {
    int total, tiles, nwg;
};
constexpr StaticNeed static_need() {
    StaticNeed m{0, 0, 0};
    for (int w = kStaticMinSide; w <= kStaticMaxCells / kStaticMinSide; w++) {
        const int h = kStaticMaxCells / w;
        const Levels L = make_levels(w, h);
        const int nwg = ((w + 15) / 16) * ((h + 15) / 16);
        if (L.total > m.total) m.total = L.total;
        if (L.tiles > m.tiles) m.tiles = L.tiles;
        if (nwg > m.nwg) m.nwg = nwg;
    }
    return m;
}
constexpr StaticNeed kStaticNeed = static_need();
constexpr size_t kStaticTotal = (size_t)kStaticNeed.total;
constexpr size_t kStaticTiles = (size_t)kStaticNeed.tiles;
constexpr size_t kStaticNwg = (size_t)kStaticNeed.nwg;
static_assert(kStaticTotal >= (size_t)kStaticMaxCells * 4 / 3, "the hierarchy holds at least 4/3 of the grid");
constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kStaticBytes =
    align256(sizeof(DevParams)) + align256(sizeof(StepState)) + align256(sizeof(SolveState)) +
    align256((size_t)kStaticMaxCells * sizeof(float4)) +          // rhs as the engine lays it out
    align256((size_t)kStaticMaxCells * sizeof(float)) +           // viscous part of the warm start
    align256(kStaticTiles * sizeof(uint32_t)) +                   // tile flags of every level
    align256(kStaticTiles * sizeof(uint32_t)) + align256(kMaxLevels * sizeof(uint32_t)) +   // active-tile lists
    align256(2 * kStaticNwg * sizeof(float4)) +                   // per-tile partial sums
    align256(kStaticTotal * sizeof(float4)) + align256(kStaticTotal * sizeof(float)) +
    3 * align256(kStaticTotal * sizeof(float2)) + 4 * align256((size_t)kStaticMaxCells * sizeof(float2));

static __device__ __align__(256) unsigned char g_solve_scratch[kStaticBytes];

namespace {

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
            const float D = mgd[i];
            d.mgd[i] = D;
            float2 b = rhs[i];
            d.prhs[i] = make_float4(b.x, b.y, 0.0f, 0.0f);
            d.p2keep[i] = 0.0f;
            // a cell that is no unknown leaves with zero potentials, also in tiles without
            // unknowns, which the solve itself never visits
            if (!(D > 0.0f)) d.pres[i] = make_float2(0.0f, 0.0f);
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
        K->cap[0] = K->cap[1] = max_iters;   // the caller's limit, not a recorded count
    }
}

struct StaticSlot {
    int ready;
    unsigned char* base;
};
StaticSlot g_slots[kMaxDevices];

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
    if (w < (uint32_t)kStaticMinSide || h < (uint32_t)kStaticMinSide || (size_t)w * h > (size_t)kStaticMaxCells) {
        sprout_internal_set_error("grid outside 16 x 16 .. 147,456 cells, the most the fixed solve array holds");
        return -3;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
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
    const Levels L = make_levels((int)w, (int)h);
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
    d.plist = reinterpret_cast<uint32_t*>(take(kStaticTiles * sizeof(uint32_t)));
    d.pcount = reinterpret_cast<uint32_t*>(take(kMaxLevels * sizeof(uint32_t)));
    d.partials = reinterpret_cast<float4*>(take(2 * kStaticNwg * sizeof(float4)));
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
    // (every accepted grid fits by construction of kStaticNeed; checked all the same)
    if ((size_t)(p - slot.base) > kStaticBytes || (size_t)L.total > kStaticTotal || (size_t)L.tiles > kStaticTiles ||
        (size_t)d.nwg > kStaticNwg) {
        sprout_internal_set_error("fixed solve array layout overflow");
        return -3;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_static_prep<<<128, 256, 0, st>>>(d, reinterpret_cast<const float4*>(mga), mgd, reinterpret_cast<const float2*>(rhs),
                                       tol_p, tol_psi, max_iters);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        sprout_internal_set_error(cudaGetErrorString(e));
        return -6;
    }
    const size_t smem = pressure_smem(L);
    int blocks = pressure_blocks_max(dev, smem, false);
    if (blocks > d.nwg) blocks = d.nwg;
    if (blocks < 1) blocks = 1;
    int second = 0, scale_mode = 0;
    void* args[] = {(void*)&d, &second, &scale_mode};
    e = cudaLaunchCooperativeKernel((const void*)k_mgpcg<Plain>, dim3(blocks), dim3(NT), args, smem, st);
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
        if (K.error & ERR_DIVERGED) {
            sprout_internal_set_error("the solve met a non-finite right-hand side or residual and stopped");
            return -4;
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

// The implicit viscosity solve on sm_103a, and the second pressure projection after it.
//
// Backward-Euler viscosity in the variational form (visc.glsl:39-56): A u = M u*, with
// A = M + G^T W G over the u and v faces of the active 16 x 16 tiles (cells within one cell
// of a diffusion number >= implicit_viscosity_min), solved by conjugate gradients
// preconditioned with an aggregation V-cycle whose smoother is red-black Gauss-Seidel over
// cells, u and v together (vmg.glsl). The weakly viscous tiles take the explicit step
// (visc_split.comp) and leave the system.
//
// Kernels:
//   k_visc_split        visc_split.comp: explicit step in the inactive tiles
//   k_visc_diag         visc_diag.comp: diagonal, warm start, level-0 matrix, clears
//   k_vmg_build         vmg_build.comp: Galerkin coarse level l from l - 1
//   k_visc_solve<NU>    the whole solve, ONE persistent cooperative kernel: strain of u*,
//                       start (visc_apply mode 0), warm start (visc_iter WARM), the first
//                       V-cycle, then per iteration the update fused with the way down on
//                       level 0 (visc_mgu.comp), the coarse levels down and up (vmg_down,
//                       vmg_up) and the way up on level 0 with A z and both step lengths
//                       (visc_mgz.comp). Phases are separated by the grid barrier of
//                       solve_common.cuh; every block evaluates the solve's scalars itself
//                       from the per-tile partial sums (reduce_tail.glsl modes 4, 10-13, 7),
//                       so the loop exits on the device as soon as the solve has converged.
//   k_rhs_visc          rhs_visc.comp: right-hand side of the second pressure solve
//   k_project_visc      project_visc.comp: subtracts the gradient of P2, keeps it
//
// Each smoothing pass holds a tile and 2 NU (+1 for A z) cells around it in shared memory and
// recomputes the ring around the tile that its neighbours also compute (vmg.glsl:142-147): a
// half-sweep over ring >= h leaves exactly the values that global half-sweeps would, so the
// result does not depend on the tiling.
#include <cuda_runtime.h>

#include "dev_common.cuh"
#include "kernels.h"
#include "solve_common.cuh"

namespace sprout {

namespace {

using namespace solve;

DEV bool v_live_u(const DevScene& d, int i) { return face_live(d.vel[i].z); }
DEV bool v_live_v(const DevScene& d, int i) { return face_live(d.vel[i].w); }
DEV bool v_closed_u(const DevScene& d, int i) { return face_closed(d.vel[i].z); }
DEV bool v_closed_v(const DevScene& d, int i) { return face_closed(d.vel[i].w); }
DEV bool in_grid(const DevScene& d, int x, int y) { return x >= 0 && y >= 0 && x < d.W && y < d.H; }
DEV bool interior(const DevScene& d, int x, int y) { return x >= 1 && y >= 1 && x < d.W - 1 && y < d.H - 1; }
DEV uint32_t tile_of(const DevScene& d, int x, int y) { return (uint32_t)((y >> 4) * ((d.W + 15) >> 4) + (x >> 4)); }
DEV float2 f2(float x, float y) { return make_float2(x, y); }
DEV float dot2(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
DEV float2 mask_of(float2 d) { return f2(d.x > 0.0f ? 1.0f : 0.0f, d.y > 0.0f ? 1.0f : 0.0f); }

// G^T of the weighted strain in vs at the faces of cell i (visc_split.comp:12-24).
DEV float2 gts_vs(const DevScene& d, int i) {
    const int W = d.W;
    float2 g = f2(0.0f, 0.0f);
    if (v_live_u(d, i)) {
        float c1 = v_closed_u(d, i - W) ? 1.0f : 0.5f, c2 = v_closed_u(d, i + W) ? -1.0f : -0.5f;
        g.x = d.vs[i - 1].x - d.vs[i].x + d.vs[i].z * c1 + d.vs[i + W].z * c2;
    }
    if (v_live_v(d, i)) {
        float d1 = v_closed_v(d, i - 1) ? 1.0f : 0.5f, d2 = v_closed_v(d, i + 1) ? -1.0f : -0.5f;
        g.y = d.vs[i - W].y - d.vs[i].y + d.vs[i].z * d1 + d.vs[i + 1].z * d2;
    }
    return g;
}

DEV void store_vel_xy(const DevScene& d, int i, float x, float y) {
    reinterpret_cast<float2*>(d.vel)[2 * i] = f2(x, y);
}

// ---- the passes before the solve -------------------------------------------------------

__global__ void __launch_bounds__(256) k_visc_split(DevScene d) {
    const int cx = blockIdx.x * 16 + threadIdx.x, cy = blockIdx.y * 16 + threadIdx.y;
    if (!in_grid(d, cx, cy) || d.tiles[blockIdx.y * gridDim.x + blockIdx.x] != 0u) return;
    if (!interior(d, cx, cy)) return;
    const int i = cy * d.W + cx;
    float2 g = gts_vs(d, i);
    float4 cf = d.coef[i];
    float4 v = d.vel[i];
    if (face_live(v.z)) v.x -= g.x / cf.z;
    if (face_live(v.w)) v.y -= g.y / cf.w;
    store_vel_xy(d, i, v.x, v.y);
}

// Strain weights as the implicit system sees them (visc_diag.comp:12-16).
DEV float2 wts(const DevScene& d, int x, int y, int i) {
    if (d.tiles[tile_of(d, x, y)] == 0u) return f2(0.0f, 0.0f);
    float4 w = d.vw[i];
    return f2(w.x, w.y);
}
DEV bool unk_u(const DevScene& d, int x, int y) { return interior(d, x, y) && d.tiles[tile_of(d, x, y)] != 0u && v_live_u(d, y * d.W + x); }
DEV bool unk_v(const DevScene& d, int x, int y) { return interior(d, x, y) && d.tiles[tile_of(d, x, y)] != 0u && v_live_v(d, y * d.W + x); }

// visc_diag.comp:23-52: the couplings of A at cell (cx, cy) as the multigrid stores them.
DEV void couplings(const DevScene& d, int cx, int cy, int i, float4& a, float4& b) {
    const int W = d.W;
    const bool u = unk_u(d, cx, cy), v = unk_v(d, cx, cy);
    a = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    b = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (u && unk_u(d, cx - 1, cy)) a.x = -wts(d, cx - 1, cy, i - 1).x;
    if (v && unk_v(d, cx, cy - 1)) a.w = -wts(d, cx, cy - 1, i - W).x;
    const float wn = wts(d, cx, cy, i).y;
    if (wn > 0.0f) {
        float ua = u ? (v_closed_u(d, i - W) ? 1.0f : 0.5f) : 0.0f;
        float ub = unk_u(d, cx, cy - 1) ? -(v_closed_u(d, i) ? 1.0f : 0.5f) : 0.0f;
        float va = v ? (v_closed_v(d, i - 1) ? 1.0f : 0.5f) : 0.0f;
        float vb = unk_v(d, cx - 1, cy) ? -(v_closed_v(d, i) ? 1.0f : 0.5f) : 0.0f;
        a.y = wn * ua * ub;
        a.z = wn * va * vb;
        b.x = wn * ua * va;
        b.y = wn * ua * vb;
    }
    const float wu = wts(d, cx, cy + 1, i + W).y;
    if (wu > 0.0f && u) {
        float ub = -(v_closed_u(d, i + W) ? 1.0f : 0.5f);
        float va = unk_v(d, cx, cy + 1) ? (v_closed_v(d, i + W - 1) ? 1.0f : 0.5f) : 0.0f;
        float vb = unk_v(d, cx - 1, cy + 1) ? -(v_closed_v(d, i + W) ? 1.0f : 0.5f) : 0.0f;
        b.z = wu * ub * va;
        b.w = wu * ub * vb;
    }
}

// visc_diag.comp:56-119, with the multigrid's level 0 (viscosity_precond 1).
__global__ void __launch_bounds__(256) k_visc_diag(DevScene d) {
    __shared__ uint32_t s_was;
    const uint32_t slot = blockIdx.y * gridDim.x + blockIdx.x;
    const int t = threadIdx.y * 16 + threadIdx.x;
    if (t == 0) s_was = d.vtile[slot];
    __syncthreads();
    if (t == 0) d.vtile[slot] = d.tiles[slot];
    const int cx = blockIdx.x * 16 + threadIdx.x, cy = blockIdx.y * 16 + threadIdx.y;
    if (!in_grid(d, cx, cy)) return;
    const int W = d.W;
    const int i = cy * W + cx;
    const bool on = d.tiles[slot] != 0u;
    float2 dg = f2(1.0f, 1.0f);
    const bool inner = interior(d, cx, cy);
    if (inner) {
        float4 cf = d.coef[i];
        float2 me = wts(d, cx, cy, i);
        if (v_live_u(d, i)) {
            float c1 = v_closed_u(d, i - W) ? 1.0f : 0.5f, c2 = v_closed_u(d, i + W) ? 1.0f : 0.5f;
            dg.x = cf.z + wts(d, cx - 1, cy, i - 1).x + me.x + me.y * c1 * c1 + wts(d, cx, cy + 1, i + W).y * c2 * c2;
        }
        if (v_live_v(d, i)) {
            float d1 = v_closed_v(d, i - 1) ? 1.0f : 0.5f, d2 = v_closed_v(d, i + 1) ? 1.0f : 0.5f;
            dg.y = cf.w + wts(d, cx, cy - 1, i - W).x + me.x + me.y * d1 * d1 + wts(d, cx + 1, cy, i + 1).y * d2 * d2;
        }
    }
    float4 o = d.vw[i];
    o.z = dg.x;
    o.w = dg.y;
    float2 dv = f2(0.0f, 0.0f);
    if (d.P->viscosity_warm != 0 && on && inner) {
        const float ratio = d.S->dt / d.S->dt_prev;
        float2 old = d.vd[i];
        dv = f2(old.x * ratio * (v_live_u(d, i) ? 1.0f : 0.0f), old.y * ratio * (v_live_v(d, i) ? 1.0f : 0.0f));
    }
    d.vd[i] = dv;
    const float2 zero = f2(0.0f, 0.0f);
    if (!on) {
        o.x = 0.0f;
        o.y = 0.0f;
        d.vs[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        d.vr[i] = zero;
        d.vp[i] = zero;
        d.vq[i] = zero;
    }
    if (on || s_was != 0u) {
        float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f), b = a;
        float2 dm = zero;
        if (on && inner) {
            couplings(d, cx, cy, i, a, b);
            dm = f2(dg.x * (v_live_u(d, i) ? 1.0f : 0.0f), dg.y * (v_live_v(d, i) ? 1.0f : 0.0f));
        }
        if (!on) {
            d.vmz[i] = zero;
            d.vaz[i] = zero;
            d.vr2[i] = zero;
            d.vq2[i] = zero;
        }
        d.vma[i] = a;
        d.vmb[i] = b;
        d.vmd[i] = dm;
    }
    // vw last: the couplings above read vw.xy of the neighbours, which this pass leaves as
    // they were wherever a tile is active (and wts() reads none in an inactive one)
    d.vw[i] = o;
}

// vmg_build.comp: level l of the viscosity multigrid from level l - 1. One block per coarse
// tile of level l.
__global__ void __launch_bounds__(256) k_vmg_build(DevScene d, int l) {
    __shared__ uint32_t s_state;
    const Lv F = lev(d.lv, l - 1), C = lev(d.lv, l);
    const int t = threadIdx.y * 16 + threadIdx.x;
    if (t == 0) {
        const int tfx = tiles_x(F), tfy = tiles_y(F);
        uint32_t on = 0u;
        for (int k = 0; k < 4; k++) {
            int fx = 2 * (int)blockIdx.x + (k & 1), fy = 2 * (int)blockIdx.y + (k >> 1);
            if (fx < tfx && fy < tfy) {
                uint32_t s = (uint32_t)(fy * tfx + fx);
                on |= (l - 1 == 0) ? d.tiles[s] : d.vtile[F.toff + s];
            }
        }
        uint32_t slot = (uint32_t)C.toff + blockIdx.y * gridDim.x + blockIdx.x;
        uint32_t was = d.vtile[slot];
        d.vtile[slot] = on != 0u ? 1u : 0u;
        s_state = (on != 0u ? 1u : 0u) | (was != 0u ? 2u : 0u);
    }
    __syncthreads();
    const uint32_t state = s_state;
    if (state == 0u) return;
    const int ccx = blockIdx.x * 16 + threadIdx.x, ccy = blockIdx.y * 16 + threadIdx.y;
    if (!l_inside(C, ccx, ccy)) return;
    const int o = l_at(C, ccx, ccy);
    if ((state & 1u) == 0u) {
        d.vma[o] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        d.vmb[o] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        d.vmd[o] = f2(0.0f, 0.0f);
        return;
    }
    const int UVX[4] = {0, -1, 0, -1}, UVY[4] = {0, 0, 1, 1};
    float2 D = f2(0.0f, 0.0f);
    float4 A = make_float4(0.0f, 0.0f, 0.0f, 0.0f), B = A;
    for (int k = 0; k < 4; k++) {
        const int abx = k & 1, aby = k >> 1;
        const int fx = 2 * ccx + abx, fy = 2 * ccy + aby;
        if (!l_inside(F, fx, fy)) continue;
        const int i = l_at(F, fx, fy);
        const float4 a = d.vma[i], b = d.vmb[i];
        const float2 dd = d.vmd[i];
        D.x += dd.x;
        D.y += dd.y;
        if (abx == 1) { D.x += 2.0f * a.x; D.y += 2.0f * a.z; }
        else { A.x += a.x; A.z += a.z; }
        if (aby == 1) { D.x += 2.0f * a.y; D.y += 2.0f * a.w; }
        else { A.y += a.y; A.w += a.w; }
        for (int m = 0; m < 4; m++) {
            const int rx = ((fx + UVX[m]) >> 1) - ccx, ry = ((fy + UVY[m]) >> 1) - ccy;
            const int s = (rx == 0 ? 0 : 1) + (ry == 0 ? 0 : 2);
            const float bm = m == 0 ? b.x : m == 1 ? b.y : m == 2 ? b.z : b.w;
            if (s == 0) B.x += bm; else if (s == 1) B.y += bm; else if (s == 2) B.z += bm; else B.w += bm;
        }
    }
    d.vma[o] = A;
    d.vmb[o] = B;
    d.vmd[o] = f2(maxf(D.x, 0.0f), maxf(D.y, 0.0f));
}

// ---- the persistent solve ----------------------------------------------------------------

template <int NU>
struct VCfg {
    static constexpr int HALO = 2 * NU;
    static constexpr int RHMAX = HALO + 1;            // the way up on level 0 forms A z too
    static constexpr int RWMAX = 16 + 2 * RHMAX;
    static constexpr int NMAX = RWMAX * RWMAX;
};

// One tile's copies, staged asynchronously (vmg.glsl:90-111 load_region and what the pass
// reads besides): the level's matrix (vma, vmb, vmd), the right-hand side (sr) and two more
// per-cell fields e1, e2 (the way up: the pre-smoothed values and the coarse values; the
// update: A z and the old q), zero-filled outside the level.
template <int NU>
struct VStage {
    static constexpr int N = VCfg<NU>::NMAX;
    float4 sa[N], sb[N];
    float2 sd[N], sr[N], e1[N], e2[N];
};

template <int NU>
struct VSmem {
    VStage<NU> st[2];
    float2 sx[VCfg<NU>::NMAX];   // the iterate of the tile being computed
    float2 sres[NT];
    float4 buf[NT];
};

// The solve's scalars (SolveBuf v_*, common.glsl:138-149), one copy per block.
struct VScal {
    float rz, alpha, beta, r0, rr, pq;
    uint32_t done, iters;
};

// One region of RH cells around a 16 x 16 tile: the matrix, right-hand side and extra fields
// in a staging buffer g, the iterate in sx.
template <int NU, int RH>
struct Region {
    static constexpr int RW = 16 + 2 * RH;
    static constexpr int N = RW * RW;
    static constexpr int PER = (N + NT - 1) / NT;
    VStage<NU>& g;
    float2* sx;
    VSmem<NU>& s;
    int ox, oy;   // first cell of the tile

    DEV int cell_x(int k) const { return ox - RH + k % RW; }
    DEV int cell_y(int k) const { return oy - RH + k / RW; }
    DEV static bool red(int k) { return (((k % RW) + (k / RW)) & 1) == 0; }   // ox, oy, 2 RH even
    DEV static int tile_slot(int t) { return ((t >> 4) + RH) * RW + (t & 15) + RH; }

    // offd of vmg.glsl:70-78 at slot k (x in sx)
    DEV float2 offd(int k) const {
        const float4 a = g.sa[k], b = g.sb[k];
        const float2 xl = sx[k - 1], xr = sx[k + 1], xd = sx[k - RW], xu = sx[k + RW];
        float u = a.x * xl.x + g.sa[k + 1].x * xr.x + a.y * xd.x + g.sa[k + RW].y * xu.x
                + b.x * sx[k].y + b.y * xl.y + b.z * xu.y + b.w * sx[k + RW - 1].y;
        float v = a.z * xl.y + g.sa[k + 1].z * xr.y + a.w * xd.y + g.sa[k + RW].w * xu.y
                + b.x * sx[k].x + g.sb[k + 1].y * xr.x + g.sb[k - RW].z * xd.x + g.sb[k + 1 - RW].w * sx[k + 1 - RW].x;
        return f2(u, v);
    }
    DEV float2 relax(int k) const {
        const float2 dd = g.sd[k];
        const float2 o = offd(k);
        const float2 rr = g.sr[k];
        const float sx_ = rr.x - o.x, sy_ = rr.y - o.y;
        return f2(divp(sx_, dd.x), divp(sy_, dd.y));
    }

    // The copies of the region: matrix, right-hand side rhs (an array of the level, offset
    // included), and e1 / e2 from arrays f1 / f2 (null: not copied); f2 may be read at the
    // coarse cell (x / 2, y / 2) of level LC.
    DEV void stage(const DevScene& d, const Lv& L, const float2* rhs, const float2* f1, const float2* f2_,
                   const Lv* LC) const {
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const int k = threadIdx.x + j * NT;
            if (k >= N) break;
            const int x = cell_x(k), y = cell_y(k);
            const bool in = l_inside(L, x, y);
            const int i = in ? l_at(L, x, y) : 0;
            cp_async<16>(&g.sa[k], d.vma + i, in);
            cp_async<16>(&g.sb[k], d.vmb + i, in);
            cp_async<8>(&g.sd[k], d.vmd + i, in);
            cp_async<8>(&g.sr[k], rhs + i, in);
            if (f1) cp_async<8>(&g.e1[k], f1 + i, in);
            if (f2_) cp_async<8>(&g.e2[k], f2_ + (in ? (LC ? l_at(*LC, x >> 1, y >> 1) : i) : 0), in);
        }
    }

    // half_sweep (vmg.glsl:121-134) over the slots of one colour in ring lo (w = RW - 2 lo
    // columns from lo, w / 2 of each colour per row): every new value from the old ones, then
    // stored.
    DEV void half_sweep(bool is_red, int lo) const {
        const int w = RW - 2 * lo, hw = w >> 1, cnt = w * hw;
        constexpr int PH = (N / 2 + NT - 1) / NT;
        float2 nv[PH];
        int kk[PH];
#pragma unroll
        for (int j = 0; j < PH; j++) {
            const int m = threadIdx.x + NT * j;
            kk[j] = -1;
            if (m < cnt) {
                const int ly = lo + m / hw;
                const int lx = lo + 2 * (m % hw) + ((ly + lo + (is_red ? 0 : 1)) & 1);
                kk[j] = ly * RW + lx;
                nv[j] = relax(kk[j]);
            }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PH; j++)
            if (kk[j] >= 0) sx[kk[j]] = nv[j];
        __syncthreads();
    }

    // way_down (vmg.glsl:145-168) on the staged region: pre-smoothing from zero, the tile's
    // values to vmx and, unless coarsest, its residual summed over 2 x 2 aggregates into
    // vmr of the next level. fix(k) first makes this thread's slot k of the right-hand side
    // final (its own copies have landed).
    template <class Fix>
    DEV void way_down(const DevScene& d, const Lv& L, const Lv* LC, Fix&& fix) const {
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const int k = threadIdx.x + j * NT;
            if (k >= N) break;
            fix(k);
            const float2 dd = g.sd[k], r = g.sr[k];
            const float2 x = f2(divp(r.x, dd.x), divp(r.y, dd.y));
            sx[k] = red(k) ? x : f2(0.0f, 0.0f);
        }
        __syncthreads();
#pragma unroll
        for (int h = 1; h < VCfg<NU>::HALO; h++) half_sweep((h & 1) == 0, h);
        const int t = threadIdx.x;
        const int k = tile_slot(t);
        const int cx = ox + (t & 15), cy = oy + (t >> 4);
        const float2 x = sx[k], dd = g.sd[k], r = g.sr[k];
        const float2 o = offd(k);
        const float2 m = mask_of(dd);
        const float2 res = f2((r.x - dd.x * x.x - o.x) * m.x, (r.y - dd.y * x.y - o.y) * m.y);
        if (l_inside(L, cx, cy)) d.vmx[l_at(L, cx, cy)] = x;
        if (LC) {
            s.sres[t] = res;
            __syncthreads();
            const int ccx = cx >> 1, ccy = cy >> 1;
            if (((t & 1) | ((t >> 4) & 1)) == 0 && l_inside(*LC, ccx, ccy)) {
                const float2 a0 = s.sres[t], a1 = s.sres[t + 1], a2 = s.sres[t + 16], a3 = s.sres[t + 17];
                d.vmr[l_at(*LC, ccx, ccy)] = f2(a0.x + a1.x + a2.x + a3.x, a0.y + a1.y + a2.y + a3.y);
            }
        }
        __syncthreads();
    }

    // the start of a way up (vmg_up.comp:37-46, visc_mgz.comp:33-38): x = vmx (e1) plus the
    // coarse values (e2, with LC), zero where a face is no unknown; then HALO half-sweeps,
    // black first.
    DEV void way_up(bool coarse) const {
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const int k = threadIdx.x + j * NT;
            if (k >= N) break;
            float2 v = g.e1[k];
            if (coarse) {
                const float2 zc = g.e2[k];
                v = f2(v.x + zc.x, v.y + zc.y);
            }
            const float2 m = mask_of(g.sd[k]);
            sx[k] = f2(v.x * m.x, v.y * m.y);
        }
        __syncthreads();
#pragma unroll
        for (int h = 1; h <= VCfg<NU>::HALO; h++) half_sweep((h & 1) == 0, h);
    }
};

// This block's share of the active-tile lists in shared memory (entry k of level l: list
// item blockIdx.x + k x gridDim.x), filled once per solve; items past kVCachePer are read from
// global memory.
constexpr int kVCacheLevels = 4, kVCachePer = 32;
struct VTileCache {
    uint32_t cnt[kVCacheLevels];
    uint32_t item[kVCacheLevels][kVCachePer];
};

template <int NU>
struct VSolve {
    const DevScene& d;
    VSmem<NU>& s;
    VScal& K;
    int n;   // level-0 tiles (partial slots per half)
    VTileCache& tc;

    DEV const uint32_t* list(int l) const { return d.vlist + d.lv.toff[l]; }

    DEV void fill_cache(int nlev) const {
        for (int l = 0; l < kVCacheLevels && l <= nlev; l++) {
            const uint32_t cnt = *(volatile uint32_t*)&d.vcount[l];
            if (threadIdx.x == 0) tc.cnt[l] = cnt;
            for (int k = threadIdx.x; k < kVCachePer; k += NT) {
                const uint32_t j = blockIdx.x + (uint32_t)k * gridDim.x;
                if (j < cnt) tc.item[l][k] = list(l)[j];
            }
        }
        __syncthreads();
    }
    // For every active tile of level l in this block's share.
    template <class F>
    DEV void each(int l, F&& f) const {
        const bool cached = l < kVCacheLevels;
        const uint32_t cnt = cached ? tc.cnt[l] : *(volatile uint32_t*)&d.vcount[l];
        int k = 0;
        for (uint32_t j = blockIdx.x; j < cnt; j += gridDim.x, k++)
            f((cached && k < kVCachePer) ? tc.item[l][k] : list(l)[j]);
    }

    // Every block sums one half of the partials in the shader's order (reduce_tail.glsl).
    DEV float4 sum(int half) const { return total(d.partials + half * n, n, s.buf); }

    // group_sum (reduce.glsl:5-14) of this thread's acc into the tile's slot of one half
    DEV void tile_sum(float4 acc, int half, uint32_t slot) const {
        s.buf[threadIdx.x] = acc;
        block_tree(s.buf);
        if (threadIdx.x == 0) d.partials[half * n + slot] = s.buf[0];
        __syncthreads();
    }

    // the compact lists of active tiles per level (block 0)
    DEV void build_lists(int nlev) const {
        __shared__ uint32_t wsum[NT / 32];
        __shared__ uint32_t s_base;
        for (int l = 0; l <= nlev; l++) {
            const Lv L = lev(d.lv, l);
            const int T = tiles_x(L) * tiles_y(L);
            const uint32_t* flags = l == 0 ? d.tiles : d.vtile + L.toff;
            uint32_t* out = d.vlist + L.toff;
            if (threadIdx.x == 0) s_base = 0u;
            __syncthreads();
            for (int b0 = 0; b0 < T; b0 += NT) {
                const int k = b0 + threadIdx.x;
                const bool on = k < T && flags[k] != 0u;
                const uint32_t bal = __ballot_sync(0xffffffffu, on);
                const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
                if (lane == 0) wsum[w] = __popc(bal);
                __syncthreads();
                uint32_t before = s_base;
                for (int j = 0; j < w; j++) before += wsum[j];
                before += __popc(bal & ((1u << lane) - 1u));
                if (on) out[before] = (uint32_t)k;
                __syncthreads();
                if (threadIdx.x == 0) {
                    uint32_t tot = 0;
                    for (int j = 0; j < NT / 32; j++) tot += wsum[j];
                    s_base += tot;
                }
                __syncthreads();
            }
            if (threadIdx.x == 0) d.vcount[l] = s_base;
            __syncthreads();
        }
    }

    // visc_strain.comp on level-0 tile tt (if active): the weighted strain of the current
    // velocities
    DEV void strain_tile(int tt) const {
        if (d.tiles[tt] == 0u) return;
        const Lv L0 = lev(d.lv, 0);
        const int W = d.W;
        const int2 og = tile_origin(L0, tt);
        const int cx = og.x + (threadIdx.x & 15), cy = og.y + (threadIdx.x >> 4);
        if (!in_grid(d, cx, cy)) return;
        const int i = cy * W + cx;
        const float4 w4 = d.vw[i];
        float4 o = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        auto vu = [&](int j) { float4 v = d.vel[j]; return face_live(v.z) ? v.x : 0.0f; };
        auto vv = [&](int j) { float4 v = d.vel[j]; return face_live(v.w) ? v.y : 0.0f; };
        if (w4.x > 0.0f) {
            o.x = w4.x * (vu(i + 1) - vu(i));
            o.y = w4.x * (vv(i + W) - vv(i));
        }
        if (w4.y > 0.0f) {
            float ua = vu(i), ub = vu(i - W), va = vv(i), vb = vv(i - 1);
            if (v_closed_u(d, i) && v_live_u(d, i - W)) ua = -ub;
            if (v_closed_u(d, i - W) && v_live_u(d, i)) ub = -ua;
            if (v_closed_v(d, i) && v_live_v(d, i - 1)) va = -vb;
            if (v_closed_v(d, i - 1) && v_live_v(d, i)) vb = -va;
            o.z = w4.y * 0.5f * ((ua - ub) + (va - vb));
        }
        d.vs[i] = o;
    }
    DEV void strain() const {
        for (int tt = blockIdx.x; tt < n; tt += gridDim.x) strain_tile(tt);
    }

    // visc_apply.comp mode 0 on level-0 tile tt: r = -G^T W G u*, z = r / diag in an active
    // tile, zero partials (both halves) in the others.
    DEV void start_tile(int tt) const {
        if (d.tiles[tt] == 0u) {
            if (threadIdx.x == 0) {
                d.partials[tt] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                d.partials[n + tt] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
            return;
        }
        const Lv L0 = lev(d.lv, 0);
        const int2 og = tile_origin(L0, tt);
        const int cx = og.x + (threadIdx.x & 15), cy = og.y + (threadIdx.x >> 4);
        float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (in_grid(d, cx, cy)) {
            const int i = cy * d.W + cx;
            if (interior(d, cx, cy)) {
                const float2 g = gts_vs(d, i);
                const float lu = v_live_u(d, i) ? 1.0f : 0.0f, lv = v_live_v(d, i) ? 1.0f : 0.0f;
                const float4 w4 = d.vw[i];
                const float2 r = f2(-g.x * lu, -g.y * lv);
                const float2 z = f2(divz(r.x, w4.z), divz(r.y, w4.w));
                d.vr[i] = r;
                d.vp[i] = z;
                acc = make_float4(dot2(r, z), dot2(r, r), 0.0f, 0.0f);
            } else {
                d.vr[i] = f2(0.0f, 0.0f);
                d.vp[i] = f2(0.0f, 0.0f);
            }
        }
        tile_sum(acc, 0, (uint32_t)tt);
    }
    DEV void start() const {
        for (int tt = blockIdx.x; tt < n; tt += gridDim.x) start_tile(tt);
    }

    // visc_iter.comp WARM at one interior cell: the step d of the warm start
    DEV float2 warm_dir(int x, int y) const {
        if (!in_grid(d, x, y) || !interior(d, x, y)) return f2(0.0f, 0.0f);
        return d.vd[y * d.W + x];
    }
    DEV float4 strain_dir(int cx, int cy) const {
        if (!in_grid(d, cx, cy)) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const int W = d.W, i = cy * W + cx;
        float4 o = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const float4 w = d.vw[i];
        auto U = [&](int x, int y, int j) { return v_live_u(d, j) ? warm_dir(x, y).x : 0.0f; };
        auto V = [&](int x, int y, int j) { return v_live_v(d, j) ? warm_dir(x, y).y : 0.0f; };
        if (w.x > 0.0f) {
            o.x = w.x * (U(cx + 1, cy, i + 1) - U(cx, cy, i));
            o.y = w.x * (V(cx, cy + 1, i + W) - V(cx, cy, i));
        }
        if (w.y > 0.0f) {
            float ua = U(cx, cy, i), ub = U(cx, cy - 1, i - W), va = V(cx, cy, i), vb = V(cx - 1, cy, i - 1);
            if (v_closed_u(d, i) && v_live_u(d, i - W)) ua = -ub;
            if (v_closed_u(d, i - W) && v_live_u(d, i)) ub = -ua;
            if (v_closed_v(d, i) && v_live_v(d, i - 1)) va = -vb;
            if (v_closed_v(d, i - 1) && v_live_v(d, i)) vb = -va;
            o.z = w.y * 0.5f * ((ua - ub) + (va - vb));
        }
        return o;
    }
    // visc_iter.comp WARM on active level-0 tile tt
    DEV void warm_tile(uint32_t tt, int half) const {
        const Lv L0 = lev(d.lv, 0);
        const int W = d.W;
        {
            const int2 og = tile_origin(L0, (int)tt);
            const int cx = og.x + (threadIdx.x & 15), cy = og.y + (threadIdx.x >> 4);
            float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (in_grid(d, cx, cy) && interior(d, cx, cy)) {
                const int i = cy * W + cx;
                float2 g = f2(0.0f, 0.0f);
                if (v_live_u(d, i)) {
                    float c1 = v_closed_u(d, i - W) ? 1.0f : 0.5f, c2 = v_closed_u(d, i + W) ? -1.0f : -0.5f;
                    const float4 sl = strain_dir(cx - 1, cy), sc = strain_dir(cx, cy), su = strain_dir(cx, cy + 1);
                    g.x = sl.x - sc.x + sc.z * c1 + su.z * c2;
                }
                if (v_live_v(d, i)) {
                    float d1 = v_closed_v(d, i - 1) ? 1.0f : 0.5f, d2 = v_closed_v(d, i + 1) ? -1.0f : -0.5f;
                    const float4 sd_ = strain_dir(cx, cy - 1), sc = strain_dir(cx, cy), sr_ = strain_dir(cx + 1, cy);
                    g.y = sd_.y - sc.y + sc.z * d1 + sr_.z * d2;
                }
                const float lu = v_live_u(d, i) ? 1.0f : 0.0f, lv = v_live_v(d, i) ? 1.0f : 0.0f;
                const float4 cf = d.coef[i];
                const float2 p = warm_dir(cx, cy);
                const float2 dd = f2(p.x * lu, p.y * lv);
                const float2 q = f2((cf.z * dd.x + g.x) * lu, (cf.w * dd.y + g.y) * lv);
                const float4 v = d.vel[i];
                store_vel_xy(d, i, v.x + dd.x, v.y + dd.y);
                const float2 r0 = d.vr[i];
                const float2 r = f2(r0.x - q.x, r0.y - q.y);
                d.vr[i] = r;
                const float4 w4 = d.vw[i];
                const float2 z = f2(divz(r.x, w4.z), divz(r.y, w4.w));
                acc = make_float4(dot2(r, z), dot2(r, r), 0.0f, 0.0f);
            }
            tile_sum(acc, half, tt);
        }
    }
    DEV void warm(int half) const {
        each(0, [&](uint32_t tt) { warm_tile(tt, half); });
    }

    // visc_iter.comp (not WARM), the Jacobi-preconditioned iteration on active level-0 tile
    // tt: the direction p = z + beta p_old (z = r / diag) on the tile and two cells around, its
    // weighted strain on the tile and one cell around (both in the shared staging area, which
    // this path does not otherwise use), then q = M p + G^T s on the tile into vq and p into
    // p_new; partial sums of p.q
    DEV void jac_iter_tile(uint32_t tt, const float2* p_old, float2* p_new, int half) const {
        constexpr int PW = 20, SW = 18;
        float2* sp = reinterpret_cast<float2*>(&s.st[0]);
        float4* ss = reinterpret_cast<float4*>(sp + PW * PW);
        const Lv L0 = lev(d.lv, 0);
        const int2 O = tile_origin(L0, (int)tt);
        const float b = K.beta;
        for (int k = threadIdx.x; k < PW * PW; k += NT) {
            const int x = O.x - 2 + k % PW, y = O.y - 2 + k / PW;
            float2 p = f2(0.0f, 0.0f);
            if (in_grid(d, x, y) && interior(d, x, y)) {
                const int i = y * d.W + x;
                const float4 w = d.vw[i];
                const float2 r = d.vr[i];
                const float2 z = f2(divz(r.x, w.z), divz(r.y, w.w));
                if (b == 0.0f) p = z;
                else {
                    const float2 po = p_old[i];
                    p = f2(z.x + b * po.x, z.y + b * po.y);
                }
            }
            sp[k] = p;
        }
        __syncthreads();
        auto pd = [&](int x, int y) { return sp[(y - O.y + 2) * PW + (x - O.x + 2)]; };
        auto U = [&](int x, int y, int j) { return v_live_u(d, j) ? pd(x, y).x : 0.0f; };
        auto Vv = [&](int x, int y, int j) { return v_live_v(d, j) ? pd(x, y).y : 0.0f; };
        const int W = d.W;
        for (int k = threadIdx.x; k < SW * SW; k += NT) {
            const int cx = O.x - 1 + k % SW, cy = O.y - 1 + k / SW;
            float4 o = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (in_grid(d, cx, cy)) {
                const int i = cy * W + cx;
                const float4 w = d.vw[i];
                if (w.x > 0.0f) {
                    o.x = w.x * (U(cx + 1, cy, i + 1) - U(cx, cy, i));
                    o.y = w.x * (Vv(cx, cy + 1, i + W) - Vv(cx, cy, i));
                }
                if (w.y > 0.0f) {
                    float ua = U(cx, cy, i), ub = U(cx, cy - 1, i - W), va = Vv(cx, cy, i), vb = Vv(cx - 1, cy, i - 1);
                    if (v_closed_u(d, i) && v_live_u(d, i - W)) ua = -ub;
                    if (v_closed_u(d, i - W) && v_live_u(d, i)) ub = -ua;
                    if (v_closed_v(d, i) && v_live_v(d, i - 1)) va = -vb;
                    if (v_closed_v(d, i - 1) && v_live_v(d, i)) vb = -va;
                    o.z = w.y * 0.5f * ((ua - ub) + (va - vb));
                }
            }
            ss[k] = o;
        }
        __syncthreads();
        auto sat = [&](int x, int y) { return ss[(y - O.y + 1) * SW + (x - O.x + 1)]; };
        const int cx = O.x + (threadIdx.x & 15), cy = O.y + (threadIdx.x >> 4);
        float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (in_grid(d, cx, cy)) {
            const int i = cy * W + cx;
            const float2 pn = pd(cx, cy);
            p_new[i] = pn;
            if (interior(d, cx, cy)) {
                float2 g = f2(0.0f, 0.0f);
                if (v_live_u(d, i)) {
                    const float c1 = v_closed_u(d, i - W) ? 1.0f : 0.5f, c2 = v_closed_u(d, i + W) ? -1.0f : -0.5f;
                    g.x = sat(cx - 1, cy).x - sat(cx, cy).x + sat(cx, cy).z * c1 + sat(cx, cy + 1).z * c2;
                }
                if (v_live_v(d, i)) {
                    const float d1 = v_closed_v(d, i - 1) ? 1.0f : 0.5f, d2 = v_closed_v(d, i + 1) ? -1.0f : -0.5f;
                    g.y = sat(cx, cy - 1).y - sat(cx, cy).y + sat(cx, cy).z * d1 + sat(cx + 1, cy).z * d2;
                }
                const float lu = v_live_u(d, i) ? 1.0f : 0.0f, lv = v_live_v(d, i) ? 1.0f : 0.0f;
                const float4 cf = d.coef[i];
                const float2 p = f2(pn.x * lu, pn.y * lv);
                const float2 q = f2((cf.z * p.x + g.x) * lu, (cf.w * p.y + g.y) * lv);
                d.vq[i] = q;
                acc = make_float4(0.0f, 0.0f, dot2(p, q), 0.0f);
            } else {
                d.vq[i] = f2(0.0f, 0.0f);
            }
        }
        tile_sum(acc, half, tt);
    }
    // visc_update.comp on active level-0 tile tt: u += alpha p, the warm-start step, r -= alpha
    // q; partial sums of r.z and r.r
    DEV void jac_update_tile(uint32_t tt, const float2* p_cur, int half) const {
        const Lv L0 = lev(d.lv, 0);
        const int2 O = tile_origin(L0, (int)tt);
        const int cx = O.x + (threadIdx.x & 15), cy = O.y + (threadIdx.x >> 4);
        float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (in_grid(d, cx, cy) && interior(d, cx, cy)) {
            const int i = cy * d.W + cx;
            const float a = K.alpha;
            float4 v = d.vel[i];
            const float2 p = p_cur[i];
            const bool lu = face_live(v.z), lv = face_live(v.w);
            if (lu) v.x += a * p.x;
            if (lv) v.y += a * p.y;
            store_vel_xy(d, i, v.x, v.y);
            const float2 dv = d.vd[i];
            d.vd[i] = f2(dv.x + a * (lu ? p.x : 0.0f), dv.y + a * (lv ? p.y : 0.0f));
            const float2 r0 = d.vr[i], q = d.vq[i];
            const float2 r = f2(r0.x - a * q.x, r0.y - a * q.y);
            d.vr[i] = r;
            const float4 w = d.vw[i];
            const float2 z = f2(divz(r.x, w.z), divz(r.y, w.w));
            acc = make_float4(dot2(r, z), dot2(r, r), 0.0f, 0.0f);
        }
        tile_sum(acc, half, tt);
    }

    // For every active tile of level l in this block's share, through the pipeline of two
    // staging buffers: stage(tt, g) issues the tile's copies, finish(tt, g) computes it.
    template <class S, class F>
    DEV void pipe(int l, S&& stage, F&& finish) const {
        const bool cached = l < kVCacheLevels;
        const uint32_t cnt = cached ? tc.cnt[l] : *(volatile uint32_t*)&d.vcount[l];
        pipeline<2>(
            cnt,
            [&](int k) {
                return (cached && k < kVCachePer) ? tc.item[l][k] : list(l)[blockIdx.x + (uint32_t)k * gridDim.x];
            },
            [&](uint32_t tt, int b) { stage(tt, s.st[b]); }, [&](uint32_t tt, int b) { finish(tt, s.st[b]); });
    }
    template <int RH>
    DEV Region<NU, RH> region(VStage<NU>& g, const Lv& L, uint32_t tt) const {
        const int2 og = tile_origin(L, (int)tt);
        return Region<NU, RH>{g, s.sx, s, og.x, og.y};
    }

    // vmg_down.comp on tile tt of level l (l = 0 at the start of a solve, right-hand side rhs0)
    DEV void down_stage(uint32_t tt, VStage<NU>& g, int l, const float2* rhs0) const {
        const Lv L = lev(d.lv, l);
        region<VCfg<NU>::HALO>(g, L, tt).stage(d, L, l == 0 ? rhs0 : d.vmr, nullptr, nullptr, nullptr);
    }
    DEV void down_finish(uint32_t tt, VStage<NU>& g, int l, int nlev) const {
        const Lv L = lev(d.lv, l), LC = lev(d.lv, l + 1);
        region<VCfg<NU>::HALO>(g, L, tt).way_down(d, L, l == nlev ? nullptr : &LC, [](int) {});
    }
    DEV void down(int l, int nlev, const float2* rhs0) const {
        pipe(
            l, [&](uint32_t tt, VStage<NU>& g) { down_stage(tt, g, l, rhs0); },
            [&](uint32_t tt, VStage<NU>& g) { down_finish(tt, g, l, nlev); });
    }

    // vmg_up.comp on tile tt of a coarse level l: the finished values to vmz
    DEV void up_stage(uint32_t tt, VStage<NU>& g, int l, int nlev) const {
        const Lv L = lev(d.lv, l), LC = lev(d.lv, l + 1);
        const bool coarse = l != nlev;
        region<VCfg<NU>::HALO>(g, L, tt).stage(d, L, d.vmr, d.vmx, coarse ? d.vmz : nullptr, coarse ? &LC : nullptr);
    }
    DEV void up_finish(uint32_t tt, VStage<NU>& g, int l, int nlev) const {
        const Lv L = lev(d.lv, l);
        const Region<NU, VCfg<NU>::HALO> R = region<VCfg<NU>::HALO>(g, L, tt);
        R.way_up(l != nlev);
        const int t = threadIdx.x;
        const int cx = R.ox + (t & 15), cy = R.oy + (t >> 4);
        if (l_inside(L, cx, cy)) d.vmz[l_at(L, cx, cy)] = s.sx[R.tile_slot(t)];
        __syncthreads();
    }
    DEV void up(int l, int nlev) const {
        pipe(
            l, [&](uint32_t tt, VStage<NU>& g) { up_stage(tt, g, l, nlev); },
            [&](uint32_t tt, VStage<NU>& g) { up_finish(tt, g, l, nlev); });
    }

    // visc_mgz.comp on level-0 tile tt: the way up with A z and the partial sums of r.z, z.A z,
    // z.q
    DEV void mgz_stage(uint32_t tt, VStage<NU>& g, const float2* rn) const {
        const Lv L = lev(d.lv, 0), LC = lev(d.lv, 1);
        region<VCfg<NU>::HALO + 1>(g, L, tt).stage(d, L, rn, d.vmx, d.vmz, &LC);
    }
    DEV void mgz_finish(uint32_t tt, VStage<NU>& g, const float2* qn, int half) const {
        const Lv L = lev(d.lv, 0);
        const Region<NU, VCfg<NU>::HALO + 1> R = region<VCfg<NU>::HALO + 1>(g, L, tt);
        const int t = threadIdx.x;
        const int cx = R.ox + (t & 15), cy = R.oy + (t >> 4);
        const bool in = l_inside(L, cx, cy);
        const float2 qi = in ? qn[l_at(L, cx, cy)] : f2(0.0f, 0.0f);   // (in flight meanwhile)
        R.way_up(true);
        const int k = R.tile_slot(t);
        float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (in) {
            const int i = l_at(L, cx, cy);
            const float2 z = s.sx[k], dd = g.sd[k];
            const float2 o = R.offd(k);
            const float2 az = f2(dd.x * z.x + o.x, dd.y * z.y + o.y);
            d.vmz[i] = z;
            d.vaz[i] = az;
            acc = make_float4(dot2(g.sr[k], z), dot2(z, az), dot2(z, qi), 0.0f);
        }
        tile_sum(acc, half, tt);
    }
    DEV void mgz(const float2* rn, const float2* qn, int half) const {
        pipe(
            0, [&](uint32_t tt, VStage<NU>& g) { mgz_stage(tt, g, rn); },
            [&](uint32_t tt, VStage<NU>& g) { mgz_finish(tt, g, qn, half); });
    }

    // visc_mgu.comp on level-0 tile tt: p, q, x, r of the iteration and the way down from the
    // new r. Copies: A z (e1), the old q (e2, unless beta is zero) and the old r (sr) over the
    // region; each slot's new r = r - alpha q, q = A z + beta q_old, made final in place.
    DEV void mgu_stage(uint32_t tt, VStage<NU>& g, const float2* ro, const float2* qo) const {
        const Lv L = lev(d.lv, 0);
        region<VCfg<NU>::HALO>(g, L, tt).stage(d, L, ro, d.vaz, K.beta != 0.0f ? qo : nullptr, nullptr);
    }
    DEV void mgu_finish(uint32_t tt, VStage<NU>& g, float2* rn, float2* qn, int half) const {
        const Lv L = lev(d.lv, 0), LC = lev(d.lv, 1);
        const float a = K.alpha, b = K.beta;
        auto new_q = [&](int k) {
            const float2 sq = g.e1[k];
            if (b == 0.0f) return sq;
            const float2 q = g.e2[k];
            return f2(sq.x + b * q.x, sq.y + b * q.y);
        };
        const Region<NU, VCfg<NU>::HALO> R = region<VCfg<NU>::HALO>(g, L, tt);
        const int t = threadIdx.x;
        const int cx = R.ox + (t & 15), cy = R.oy + (t >> 4);
        const bool own = cx < d.W && cy < d.H;
        const int i = own ? cy * d.W + cx : 0;
        const bool inner = own && interior(d, cx, cy);
        // this cell's z, p_old, velocity and step, in flight while the region is made final
        const float2 z = own ? d.vmz[i] : f2(0.0f, 0.0f);
        const float2 po = (own && b != 0.0f) ? d.vp[i] : f2(0.0f, 0.0f);
        float4 v = inner ? d.vel[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const float2 dv = inner ? d.vd[i] : f2(0.0f, 0.0f);
        const int ks = R.tile_slot(t);
        R.way_down(d, L, &LC, [&](int k) {
            const float2 q = new_q(k);
            const float2 r0 = g.sr[k];
            g.sr[k] = f2(r0.x - a * q.x, r0.y - a * q.y);
        });
        float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (own) {
            float2 p = z;
            if (b != 0.0f) p = f2(z.x + b * po.x, z.y + b * po.y);
            const float2 q = new_q(ks);
            const float2 r = g.sr[ks];
            if (inner) {
                if (face_live(v.z)) v.x += a * p.x;
                if (face_live(v.w)) v.y += a * p.y;
                store_vel_xy(d, i, v.x, v.y);
                d.vd[i] = f2(dv.x + a * p.x, dv.y + a * p.y);
            }
            d.vp[i] = p;
            qn[i] = q;
            rn[i] = r;
            acc = make_float4(0.0f, dot2(r, r), dot2(p, q), 0.0f);
        }
        tile_sum(acc, half, tt);
    }
    DEV void mgu(const float2* ro, const float2* qo, float2* rn, float2* qn, int half) const {
        pipe(
            0, [&](uint32_t tt, VStage<NU>& g) { mgu_stage(tt, g, ro, qo); },
            [&](uint32_t tt, VStage<NU>& g) { mgu_finish(tt, g, rn, qn, half); });
    }

    // record_visc_coarse (mod.rs:2838-2853): the coarse levels down, then up
    DEV bool coarse(int nlev) const {
        for (int l = 1; l <= nlev; l++) {
            down(l, nlev, nullptr);
            if (!grid_sync(d.K)) return false;
        }
        for (int l = nlev; l >= 1; l--) {
            up(l, nlev);
            if (!grid_sync(d.K)) return false;
        }
        return true;
    }
};

}  // namespace

// The whole viscosity solve (record_viscosity_solve, mod.rs:2867-2908, with the
// multigrid preconditioner). `restrain`: take the strain of u* again first (the first
// pressure solve changed the velocity since visc_setup).
template <int NU>
__global__ void __launch_bounds__(NT, 2) k_visc_solve(DevScene d, int restrain) {
    grid_begin();
    __shared__ VSmem<NU> sm;
    __shared__ VScal K;
    __shared__ VTileCache tc;
    const DevParams* P = d.P;
    const int nlev = P->visc_levels;
    VSolve<NU> V{d, sm, K, d.nwg, tc};
    const float tz = P->tol[2];
    if (blockIdx.x == 0) V.build_lists(nlev);
    if (restrain) V.strain();
    if (!grid_sync(d.K)) return;
    V.fill_cache(nlev);
    V.start();
    if (!grid_sync(d.K)) return;
    {   // cg_reduce mode 4
        const float4 a = V.sum(0);
        if (threadIdx.x == 0) {
            K.rz = a.x;
            K.r0 = a.y;
            K.rr = a.y;
            K.beta = 0.0f;
            K.alpha = 0.0f;
            K.pq = 0.0f;
            K.iters = 0u;
            K.done = (a.y <= 1e-30f || a.x <= 0.0f) ? 1u : 0u;
        }
        __syncthreads();
    }
    int half = 1;
    if (P->viscosity_warm != 0 && K.done == 0u) {
        V.warm(half);
        if (!grid_sync(d.K)) return;
        const float4 a = V.sum(half);   // mode 10
        if (threadIdx.x == 0) {
            K.rz = a.x;
            K.rr = a.y;
            K.beta = 0.0f;
            K.done = (a.y <= tz * tz * K.r0 || a.x <= 0.0f) ? 1u : 0u;
        }
        __syncthreads();
        half ^= 1;
    }
    if (P->viscosity_precond == 0) {
        // the Jacobi-preconditioned iteration (mod.rs:2909-2921): visc_iter with cg_reduce mode
        // 5, visc_update with mode 6; the directions alternate between vp and vr2 (free without
        // the multigrid) as vp / vp2 swap in the reference
        float2 *pa = d.vp, *pb = d.vr2;
        for (uint32_t k = 0; k < d.K->cap[2] && K.done == 0u; k++) {
            V.each(0, [&](uint32_t tt) { V.jac_iter_tile(tt, pa, pb, half); });
            if (!grid_sync(d.K)) return;
            {
                const float4 a = V.sum(half);   // mode 5
                if (threadIdx.x == 0) K.alpha = (K.done == 0u && a.z > 0.0f) ? K.rz / a.z : 0.0f;
                __syncthreads();
                half ^= 1;
            }
            V.each(0, [&](uint32_t tt) { V.jac_update_tile(tt, pb, half); });
            if (!grid_sync(d.K)) return;
            {
                const float4 a = V.sum(half);   // mode 6
                if (threadIdx.x == 0) {
                    const uint32_t was = K.done;
                    K.iters += 1u - was;
                    const uint32_t now = a.y <= tz * tz * K.r0 ? 1u : 0u;
                    const uint32_t done = was > now ? was : now;
                    K.beta = (done == 0u && K.rz > 0.0f) ? a.x / K.rz : 0.0f;
                    K.rz = a.x;
                    if (was == 0u) K.rr = a.y;
                    K.done = done;
                }
                __syncthreads();
                half ^= 1;
            }
            float2* t = pa;
            pa = pb;
            pb = t;
        }
    }
    // the two parities of the residual and of q: the current residual alternates between
    // vr and vr2 (visc_mgu.comp writes the other one)
    float2 *ra = d.vr, *rb = d.vr2, *qa = d.vq, *qb = d.vq2;
    if (K.done == 0u && P->viscosity_precond != 0) {
        V.down(0, nlev, ra);
        if (!grid_sync(d.K)) return;
        if (!V.coarse(nlev)) return;
        V.mgz(ra, qa, half);
        if (!grid_sync(d.K)) return;
        const float4 a = V.sum(half);   // mode 11
        if (threadIdx.x == 0) {
            K.rz = a.x;
            K.beta = 0.0f;
            K.pq = a.y;
            K.alpha = a.y > 0.0f ? a.x / a.y : 0.0f;
            if (a.x <= 0.0f || a.y <= 0.0f) K.done = 1u;
        }
        __syncthreads();
        half ^= 1;
    }
    for (uint32_t k = 0; k < d.K->cap[2] && K.done == 0u && P->viscosity_precond != 0; k++) {
        V.mgu(ra, qa, rb, qb, half);
        if (!grid_sync(d.K)) return;
        {
            const float4 a = V.sum(half);   // mode 12
            if (threadIdx.x == 0) {
                const uint32_t was = K.done;
                K.iters += 1u - was;
                const uint32_t now = a.y <= tz * tz * K.r0 ? 1u : 0u;
                if (was == 0u) K.rr = a.y;
                K.pq = a.z;
                K.done = was > now ? was : now;
            }
            __syncthreads();
            half ^= 1;
        }
        if (K.done != 0u) break;
        if (!V.coarse(nlev)) return;
        V.mgz(rb, qb, half);
        if (!grid_sync(d.K)) return;
        {
            const float4 a = V.sum(half);   // mode 13
            if (threadIdx.x == 0) {
                const float beta = (K.done == 0u && K.rz > 0.0f) ? a.x / K.rz : 0.0f;
                const float pq = a.y + 2.0f * beta * a.z + beta * beta * K.pq;
                K.beta = beta;
                K.alpha = (K.done == 0u && pq > 0.0f) ? a.x / pq : 0.0f;
                K.rz = a.x;
            }
            __syncthreads();
            half ^= 1;
        }
        float2* t = ra;
        ra = rb;
        rb = t;
        t = qa;
        qa = qb;
        qb = t;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {   // mode 7
        SolveState* G = d.K;
        if (K.iters > G->v_it_max) G->v_it_max = K.iters;
        if (K.done == 0u) G->v_unconv += 1u;
        if (K.iters > G->f_it[2]) G->f_it[2] = K.iters;
        if (K.done == 0u) G->f_un[2] += 1u;
        const float rel = K.r0 > 0.0f ? sqrtf(K.rr / K.r0) : 0.0f;
        G->v_res_max = maxf(G->v_res_max, rel);
        G->v_iters = K.iters;
        G->v_done = K.done;
        G->v_rr = K.rr;
        G->v_r0 = K.r0;
        if (!isfinite(K.rr) || !isfinite(K.r0)) atomicOr(&G->error, ERR_DIVERGED);
    }
    trace_launch_done(d.K);
}

// ---- many tanks' viscosity solves in one persistent solve -----------------------------------
//
// The same solve for a batch of tanks in one cooperative launch, over flattened (tank, tile)
// work lists per level, as k_mgpcg_batch does for the pressure: every tile goes through the
// same tile bodies as above and every tank's scalars through the same steps (reduce_tail
// modes 4, 10-13, 7), summed by one block over the tank's own partials in the same order; so a
// tank's result is the same alone and in any batch, to the bit. The differences: each
// reduction is a phase of its own followed by a barrier (the scalars live in global memory),
// and a tank whose solve has converged (or reached its iteration limit) drops out of the
// work lists.

namespace {

// per tank: its scalars, which half of the partials the next reduction reads, whether it
// takes part in the rest of the current iteration
struct VBatchScene {
    VScal K;
    int half, run2, pad0, pad1;
};

DEV int vscene_of(const int* o, int ns, int g) {
    int lo = 0, hi = ns;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (o[mid] <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

// work item g of level l's active tiles over the tanks: the tank in the high 16 bits
DEV uint32_t vbatch_item(const VBatchView& B, int l, int g) {
    const int* o = B.aoff + l * (B.ns + 1);
    const int s = vscene_of(o, B.ns, g);
    const DevScene& d = B.scenes[s];
    return ((uint32_t)s << 16) | d.vlist[d.lv.toff[l] + (g - o[s])];
}

DEV void vbatch_fill_cache(const VBatchView& B, VTileCache& tc) {
    for (int l = 0; l < kVCacheLevels && l <= B.max_lev; l++) {
        const int N = *(volatile const int*)&B.aoff[l * (B.ns + 1) + B.ns];
        if (threadIdx.x == 0) tc.cnt[l] = (uint32_t)N;
        for (int k = threadIdx.x; k < kVCachePer; k += NT) {
            const int g = blockIdx.x + k * gridDim.x;
            if (g < N) tc.item[l][k] = vbatch_item(B, l, g);
        }
    }
    __syncthreads();
}

}  // namespace

template <int NU>
__global__ void __launch_bounds__(NT, 2) k_visc_batch(VBatchView B) {
    grid_begin();
    __shared__ VSmem<NU> sm;
    __shared__ VTileCache tc;
    __shared__ int s_run;
    VBatchScene* S = reinterpret_cast<VBatchScene*>(B.scal);
    SolveState* BK = B.K;
    const int ns = B.ns;
    auto V = [&](int s) { return VSolve<NU>{B.scenes[s], sm, S[s].K, B.scenes[s].nwg, tc}; };
    auto nlev = [&](int s) { return B.scenes[s].P->visc_levels; };
    // every level-0 tile of every tank
    auto for_all0 = [&](auto&& f) {
        const int N = B.off0[ns];
        for (int g = blockIdx.x; g < N; g += gridDim.x) {
            const int s = vscene_of(B.off0, ns, g);
            f(s, g - B.off0[s]);
        }
    };
    // this block's share of level l's active tiles over the tanks, plain or through the pipeline
    auto count = [&](int l) {
        return l < kVCacheLevels ? tc.cnt[l] : (uint32_t)*(volatile const int*)&B.aoff[l * (ns + 1) + ns];
    };
    auto item = [&](int l, int k) {
        return (l < kVCacheLevels && k < kVCachePer) ? tc.item[l][k]
                                                      : vbatch_item(B, l, (int)(blockIdx.x + (uint32_t)k * gridDim.x));
    };
    auto for_active = [&](int l, auto&& f) {
        const uint32_t N = count(l);
        int k = 0;
        for (uint32_t g = blockIdx.x; g < N; g += gridDim.x, k++) {
            const uint32_t it = item(l, k);
            f((int)(it >> 16), it & 0xffffu);
        }
    };
    auto pipe = [&](int l, auto&& stage, auto&& finish) {
        pipeline<2>(
            count(l), [&](int k) { return item(l, k); },
            [&](uint32_t it, int b) { stage((int)(it >> 16), it & 0xffffu, sm.st[b]); },
            [&](uint32_t it, int b) { finish((int)(it >> 16), it & 0xffffu, sm.st[b]); });
    };
    // one V-cycle's coarse levels for the tanks run(s) says
    auto coarse = [&](auto&& run) -> bool {
        for (int l = 1; l <= B.max_lev; l++) {
            pipe(
                l, [&](int s, uint32_t tt, VStage<NU>& g) { if (l <= nlev(s) && run(s)) V(s).down_stage(tt, g, l, nullptr); },
                [&](int s, uint32_t tt, VStage<NU>& g) { if (l <= nlev(s) && run(s)) V(s).down_finish(tt, g, l, nlev(s)); });
            if (!grid_sync(BK)) return false;
        }
        for (int l = B.max_lev; l >= 1; l--) {
            pipe(
                l, [&](int s, uint32_t tt, VStage<NU>& g) { if (l <= nlev(s) && run(s)) V(s).up_stage(tt, g, l, nlev(s)); },
                [&](int s, uint32_t tt, VStage<NU>& g) { if (l <= nlev(s) && run(s)) V(s).up_finish(tt, g, l, nlev(s)); });
            if (!grid_sync(BK)) return false;
        }
        return true;
    };
    auto mgz = [&](auto&& run, int par) {
        pipe(
            0, [&](int s, uint32_t tt, VStage<NU>& g) {
                if (run(s)) V(s).mgz_stage(tt, g, (par & 1) ? B.scenes[s].vr2 : B.scenes[s].vr); },
            [&](int s, uint32_t tt, VStage<NU>& g) {
                if (run(s)) V(s).mgz_finish(tt, g, (par & 1) ? B.scenes[s].vq2 : B.scenes[s].vq, S[s].half); });
    };

    // the lists (one block per tank) and the strain of u* (every tank takes it again)
    for (int s = blockIdx.x; s < ns; s += gridDim.x) V(s).build_lists(nlev(s));
    for_all0([&](int s, int tt) { V(s).strain_tile(tt); });
    if (!grid_sync(BK)) return;
    // the prefix sums of the active tiles per level over the tanks, and the start
    if (blockIdx.x == 0) {
        for (int l = threadIdx.x; l <= B.max_lev; l += NT) {
            int* o = B.aoff + l * (ns + 1);
            int a = 0;
            o[0] = 0;
            for (int k = 0; k < ns; k++) {
                a += l <= nlev(k) ? (int)B.scenes[k].vcount[l] : 0;
                o[k + 1] = a;
            }
        }
    }
    for_all0([&](int s, int tt) { V(s).start_tile(tt); });
    if (!grid_sync(BK)) return;
    vbatch_fill_cache(B, tc);
    for (int s = blockIdx.x; s < ns; s += gridDim.x) {   // cg_reduce mode 4
        const float4 a = V(s).sum(0);
        if (threadIdx.x == 0) {
            VScal& K = S[s].K;
            K.rz = a.x;
            K.r0 = a.y;
            K.rr = a.y;
            K.beta = 0.0f;
            K.alpha = 0.0f;
            K.pq = 0.0f;
            K.iters = 0u;
            K.done = (a.y <= 1e-30f || a.x <= 0.0f) ? 1u : 0u;
            S[s].half = 1;
        }
        __syncthreads();
    }
    if (!grid_sync(BK)) return;
    // the warm start, for the tanks that take it and have not converged
    auto warm_on = [&](int s) { return B.scenes[s].P->viscosity_warm != 0 && S[s].K.done == 0u; };
    for_active(0, [&](int s, uint32_t tt) { if (warm_on(s)) V(s).warm_tile(tt, S[s].half); });
    if (!grid_sync(BK)) return;
    for (int s = blockIdx.x; s < ns; s += gridDim.x) {   // mode 10
        if (!warm_on(s)) continue;
        const float4 a = V(s).sum(S[s].half);
        if (threadIdx.x == 0) {
            VScal& K = S[s].K;
            const float tz = B.scenes[s].P->tol[2];
            K.rz = a.x;
            K.rr = a.y;
            K.beta = 0.0f;
            K.done = (a.y <= tz * tz * K.r0 || a.x <= 0.0f) ? 1u : 0u;
            S[s].half ^= 1;
        }
        __syncthreads();
    }
    if (!grid_sync(BK)) return;
    // the first V-cycle of the tanks not converged
    {
        auto run = [&](int s) { return S[s].K.done == 0u; };
        pipe(
            0, [&](int s, uint32_t tt, VStage<NU>& g) { if (run(s)) V(s).down_stage(tt, g, 0, B.scenes[s].vr); },
            [&](int s, uint32_t tt, VStage<NU>& g) { if (run(s)) V(s).down_finish(tt, g, 0, nlev(s)); });
        if (!grid_sync(BK)) return;
        if (!coarse(run)) return;
        mgz(run, 0);
        if (!grid_sync(BK)) return;
        for (int s = blockIdx.x; s < ns; s += gridDim.x) {   // mode 11
            if (!run(s)) continue;
            const float4 a = V(s).sum(S[s].half);
            if (threadIdx.x == 0) {
                VScal& K = S[s].K;
                K.rz = a.x;
                K.beta = 0.0f;
                K.pq = a.y;
                K.alpha = a.y > 0.0f ? a.x / a.y : 0.0f;
                if (a.x <= 0.0f || a.y <= 0.0f) K.done = 1u;
                S[s].half ^= 1;
            }
            __syncthreads();
        }
        if (!grid_sync(BK)) return;
    }
    for (uint32_t k = 0;; k++) {
        auto running = [&](int s) { return S[s].K.done == 0u && k < B.scenes[s].K->cap[2]; };
        if (threadIdx.x == 0) {
            int r = 0;
            for (int s = 0; s < ns && !r; s++) r = running(s) ? 1 : 0;
            s_run = r;
        }
        __syncthreads();
        if (!s_run) break;
        const int par = (int)(k & 1u);
        pipe(
            0, [&](int s, uint32_t tt, VStage<NU>& g) {
                const DevScene& d = B.scenes[s];
                if (running(s)) V(s).mgu_stage(tt, g, par ? d.vr2 : d.vr, par ? d.vq2 : d.vq); },
            [&](int s, uint32_t tt, VStage<NU>& g) {
                const DevScene& d = B.scenes[s];
                if (running(s)) V(s).mgu_finish(tt, g, par ? d.vr : d.vr2, par ? d.vq : d.vq2, S[s].half); });
        if (!grid_sync(BK)) return;
        for (int s = blockIdx.x; s < ns; s += gridDim.x) {   // mode 12
            const bool was_running = running(s);
            if (was_running) {
                const float4 a = V(s).sum(S[s].half);
                if (threadIdx.x == 0) {
                    VScal& K = S[s].K;
                    const float tz = B.scenes[s].P->tol[2];
                    const uint32_t was = K.done;
                    K.iters += 1u - was;
                    const uint32_t now = a.y <= tz * tz * K.r0 ? 1u : 0u;
                    if (was == 0u) K.rr = a.y;
                    K.pq = a.z;
                    K.done = was > now ? was : now;
                    S[s].half ^= 1;
                }
            }
            if (threadIdx.x == 0) S[s].run2 = (was_running && S[s].K.done == 0u) ? 1 : 0;
            __syncthreads();
        }
        if (!grid_sync(BK)) return;
        auto run2 = [&](int s) { return S[s].run2 != 0; };
        if (!coarse(run2)) return;
        mgz(run2, par ^ 1);
        if (!grid_sync(BK)) return;
        for (int s = blockIdx.x; s < ns; s += gridDim.x) {   // mode 13
            if (!run2(s)) continue;
            const float4 a = V(s).sum(S[s].half);
            if (threadIdx.x == 0) {
                VScal& K = S[s].K;
                const float beta = (K.done == 0u && K.rz > 0.0f) ? a.x / K.rz : 0.0f;
                const float pq = a.y + 2.0f * beta * a.z + beta * beta * K.pq;
                K.beta = beta;
                K.alpha = (K.done == 0u && pq > 0.0f) ? a.x / pq : 0.0f;
                K.rz = a.x;
                S[s].half ^= 1;
            }
            __syncthreads();
        }
        if (!grid_sync(BK)) return;
    }
    for (int s = blockIdx.x; s < ns; s += gridDim.x) {   // mode 7
        if (threadIdx.x == 0) {
            const VScal& K = S[s].K;
            SolveState* G = B.scenes[s].K;
            if (K.iters > G->v_it_max) G->v_it_max = K.iters;
            if (K.done == 0u) G->v_unconv += 1u;
            if (K.iters > G->f_it[2]) G->f_it[2] = K.iters;
            if (K.done == 0u) G->f_un[2] += 1u;
            const float rel = K.r0 > 0.0f ? sqrtf(K.rr / K.r0) : 0.0f;
            G->v_res_max = maxf(G->v_res_max, rel);
            G->v_iters = K.iters;
            G->v_done = K.done;
            G->v_rr = K.rr;
            G->v_r0 = K.r0;
            if (!isfinite(K.rr) || !isfinite(K.r0)) atomicOr(&G->error, ERR_DIVERGED);
        }
    }
    trace_launch_done(BK);
}

namespace {

// rhs_visc.comp
__global__ void __launch_bounds__(256) k_rhs_visc(DevScene d) {
    const int cx = blockIdx.x * 16 + threadIdx.x, cy = blockIdx.y * 16 + threadIdx.y;
    if (cx >= d.W || cy >= d.H) return;
    const int W = d.W;
    const int i = cy * W + cx;
    const float D = d.mgd[i];
    if (D <= 0.0f) {
        d.prhs[i].z = 0.0f;
        return;
    }
    const float4 w = d.mga[i];
    const float p1 = d.prhs[i].z;
    float ap = D * p1;
    if (d.mgd[i - 1] > 0.0f) ap -= w.x * d.prhs[i - 1].z;
    if (d.mgd[i + 1] > 0.0f) ap -= w.y * d.prhs[i + 1].z;
    if (d.mgd[i - W] > 0.0f) ap -= w.z * d.prhs[i - W].z;
    if (d.mgd[i + W] > 0.0f) ap -= w.w * d.prhs[i + W].z;
    const float aL = __ldg(&d.solid[i]).x, aB = __ldg(&d.solid[i]).y, aR = __ldg(&d.solid[i + 1]).x, aT = __ldg(&d.solid[i + W]).y;
    const float4 vme = d.vel[i];
    const float div = aR * d.vel[i + 1].x - aL * vme.x + aT * d.vel[i + W].y - aB * vme.y;
    const float4 r = d.prhs[i];
    d.prhs[i] = make_float4(ap - div, r.y, p1, 0.0f);
    if (d.P->viscous_warm != 0) d.pres[i].x = p1 + d.p2keep[i] * (d.S->dt / d.S->dt_prev);
}

// project_visc.comp
DEV float p2_of(const DevScene& d, int i) { return d.mgd[i] > 0.0f ? d.pres[i].x - d.prhs[i].z : 0.0f; }

__global__ void __launch_bounds__(256) k_project_visc(DevScene d) {
    const int cx = blockIdx.x * 16 + threadIdx.x, cy = blockIdx.y * 16 + threadIdx.y;
    float m = 0.0f;
    if (cx >= 1 && cy >= 1 && cx < d.W && cy < d.H) {
        const int i = cy * d.W + cx;
        const float pc = p2_of(d, i);
        d.p2keep[i] = pc;
        const float4 cf = d.coef[i];
        float4 me = d.vel[i];
        const bool lu = face_live(me.z) && cf.x != 0.0f, lv = face_live(me.w) && cf.y != 0.0f;
        if (lu || lv) {
            if (lu) me.x -= cf.x * (pc - p2_of(d, i - 1));
            if (lv) me.y -= cf.y * (pc - p2_of(d, i - d.W));
            store_vel_xy(d, i, me.x, me.y);
        }
        if (lu) m = fabsf(me.x);
        if (lv) m = maxf(m, fabsf(me.y));
    }
    report_max(&d.S->umax_grid, m);
}

template <int NU>
int visc_blocks_max_nu(int device) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_visc_solve<NU>, NT, 0);
    return sms * per;
}

}  // namespace

size_t viscosity_batch_scalar_bytes() { return sizeof(VBatchScene); }

cudaError_t launch_viscosity_batch(const VBatchView& B, int sweeps, int blocks, cudaStream_t st) {
    cudaMemsetAsync(&B.K->bar_count, 0, sizeof(uint32_t), st);
    void* args[] = {(void*)&B};
    const void* fn = sweeps >= 2 ? (const void*)k_visc_batch<2> : (const void*)k_visc_batch<1>;
    return cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(NT), args, 0, st);
}

int viscosity_blocks_max(int device, int sweeps) {
    return sweeps >= 2 ? visc_blocks_max_nu<2>(device) : visc_blocks_max_nu<1>(device);
}

void launch_viscosity_setup(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st) {
    dim3 blk(16, 16);
    dim3 grd((d.W + 15) / 16, (d.H + 15) / 16);
    k_visc_split<<<grd, blk, 0, st>>>(d);
    k_visc_diag<<<grd, blk, 0, st>>>(d);
    for (int l = 1; l <= cfg.visc_levels; l++) {
        dim3 g((d.lv.w[l] + 15) / 16, (d.lv.h[l] + 15) / 16);
        k_vmg_build<<<g, blk, 0, st>>>(d, l);
    }
}

cudaError_t launch_viscosity(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st, int restrain) {
    cudaMemsetAsync(&d.K->bar_count, 0, sizeof(uint32_t), st);
    void* args[] = {(void*)&d, &restrain};
    const void* fn = cfg.visc_sweeps >= 2 ? (const void*)k_visc_solve<2> : (const void*)k_visc_solve<1>;
    return cudaLaunchCooperativeKernel(fn, dim3(cfg.visc_blocks), dim3(NT), args, 0, st);
}

void launch_second_projection_rhs(const DevScene& d, cudaStream_t st) {
    dim3 blk(16, 16);
    dim3 grd((d.W + 15) / 16, (d.H + 15) / 16);
    k_rhs_visc<<<grd, blk, 0, st>>>(d);
}

void launch_second_projection(const DevScene& d, cudaStream_t st) {
    dim3 blk(16, 16);
    dim3 grd((d.W + 15) / 16, (d.H + 15) / 16);
    k_project_visc<<<grd, blk, 0, st>>>(d);
}

}  // namespace sprout

// Particle side of the substep on sm_103a:
//   k_step      the substep length on the device (step.comp:22-51)
//   k_advance   G2P gather, tool, speed cap, midpoint advection, path walk with SDF
//               collisions, crowd jitter (particles.comp:98-949); float4 particle loads;
//               emits the particle's new cell and its arrival rank there
//   scan        exclusive scan of the per-cell counts
//   k_place / k_cell_sort / k_crowd_sort / k_cell_gather
//               a stable counting sort by cell (ties by slot), the permutation the
//               reference's sort.comp:83-119 defines up to its within-cell atomic order:
//               ranks by arrival, each cell's few entries put in slot order, then one thread
//               per slot copies its particle (coalesced); dead slots go to the end and are
//               cleared
//   k_p2g       P2G as a per-tile gather over the sorted particles: each 16 x 16 tile of
//               nodes accumulates the fixed-point mass / momentum / channel sums of the
//               particles of its 19 x 19 cell neighbourhood in shared memory (integer
//               atomics only, so the sums are exact and order-free) and writes its nodes
//               once; no zero fill and no global atomics (deposit, particles.comp:997-1062)
#include <cuda_runtime.h>

#include "dev_common.cuh"
#include "kernels.h"
#include "sample.cuh"

namespace sprout {

constexpr uint32_t DEAD_KEY = 0xffffffffu;

__global__ void k_step(DevScene d) {
    const DevParams* P = d.P;
    StepState* S = d.S;
    float u = maxf(minf(__uint_as_float(S->umax_grid), P->ext[0]), __uint_as_float(S->umax_part));
    u = maxf(maxf(u, P->ext_speed), S->emit_speed);
    float dt_cfl = P->cfl / (u + sqrtf(5.0f * maxf(P->gravity, 0.0f)) + 1e-6f);
    float dt;
    if (P->dt_fixed > 0.0f) {
        dt = P->dt_fixed;
    } else {
        uint32_t left = S->batch_steps > S->batch_done ? S->batch_steps - S->batch_done : 1u;
        dt = minf(minf(dt_cfl, P->dt_max), maxf(S->frame_left, 0.0f) / (float)left);
    }
    dt = maxf(dt, 1e-6f);
    S->dt_prev = S->dt > 0.0f ? S->dt : dt;
    S->dt = dt;
    S->dt_cfl = minf(dt_cfl, P->dt_max);
    S->umax_seen = u;
    S->frame_left -= dt;
    float lo = __uint_as_float(S->pad0);
    float y = dt - lo;
    float t = S->advanced + y;
    S->pad0 = __float_as_uint((t - S->advanced) - y);
    S->advanced = t;
    S->batch_done += 1u;
    S->substeps += 1u;
    S->umax_grid = 0u;
    S->umax_part = 0u;
    S->region_air = 0u;
    S->corr_gain = minf(1.0f - sp_expf(-dt / P->tol[3]), P->density_k);
}

// ---- G2P and advection ------------------------------------------------------------------

DEV bool collide(const Grid& g, float wall_margin, float& x, float& y, float& vx, float& vy, bool beyond) {
    float nx, ny;
    float d = sample_sdf(g, x, y, &nx, &ny);
    if (d < wall_margin) {
        float l = len2(nx, ny);
        if (l > 1e-5f) {
            nx = nx / l;
            ny = ny / l;
            float push = wall_margin - d + (beyond ? maxf(-d, 0.0f) : 0.0f);
            x += nx * push;
            y += ny * push;
            float vn = vx * nx + vy * ny;
            if (vn < 0.0f) {
                vx -= vn * nx;
                vy -= vn * ny;
            }
            return true;
        }
    }
    return false;
}


DEV float2 tool_target(const DevParams* P, float dx, float dy) {
    float l = len2(dx, dy);
    if (P->tool_mode == 3) {
        float q = maxf(l, 0.15f * P->tool_radius);
        return make_float2(-dx / q * P->tool_vel[0], -dy / q * P->tool_vel[0]);
    }
    if (P->tool_mode == 4) return make_float2(P->tool_vel[0], P->tool_vel[1]);
    if (P->tool_mode == 7) {
        float q = maxf(l, 0.4f * P->tool_radius);
        return make_float2(dy / q * P->tool_vel[0] + dx * 2.0f, -dx / q * P->tool_vel[0] + dy * 2.0f);
    }
    if (P->tool_mode == 8) return make_float2(0.0f, 0.0f);
    return make_float2(P->tool_vel[0] + dx * 4.0f, P->tool_vel[1] + dy * 4.0f);
}

// APIC gather on one face grid: u faces (axis 0) at (i, j + 0.5), v faces (axis 1) at
// (i + 0.5, j). Returns whether any live face was near; writes velocity, correction
// velocity and the two affine entries.
template <int AXIS>
DEV bool gather_face(const Grid& g, float px, float py, float& vel_out, float& corr_out, float& c0, float& c1) {
    float gx = AXIS == 0 ? px - 0.0f : px - 0.5f;
    float gy = AXIS == 0 ? py - 0.5f : py - 0.0f;
    int bx = (int)floorf(gx - 0.5f), by = (int)floorf(gy - 0.5f);
    float fx = gx - (float)bx, fy = gy - (float)by;
    float wx[3], wy[3];
    bspline(fx, fy, wx, wy);
    float sw = 0.0f, su = 0.0f, sc = 0.0f, sdx = 0.0f, sdy = 0.0f, sudx = 0.0f, sudy = 0.0f;
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int a = 0; a < 3; a++) {
            float4 q = g.v(bx + a, by + b);
            float st = AXIS == 0 ? q.z : q.w;
            float val = AXIS == 0 ? q.x : q.y;
            if (face_live(st)) {
                float wt = wx[a] * wy[b];
                float ddx = (float)a - fx, ddy = (float)b - fy;
                sw += wt;
                su += wt * val;
                sc += wt * st;
                sdx += wt * ddx;
                sdy += wt * ddy;
                sudx += wt * val * ddx;
                sudy += wt * val * ddy;
            }
        }
    if (sw > 1e-4f) {
        float u = su / sw;
        vel_out = u;
        corr_out = sc / sw;
        c0 = 4.0f * (sudx - u * sdx) / sw;
        c1 = 4.0f * (sudy - u * sdy) / sw;
        return true;
    }
    return false;
}

DEV float f4c(float4 v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }
// The group that leads among shares f (the first of equals).
DEV int lead4(float4 f) { return f.x >= maxf(f.y, maxf(f.z, f.w)) ? 0 : f.y >= maxf(f.z, f.w) ? 1 : f.z >= f.w ? 2 : 3; }

// Drift between immiscible phase groups (particles.comp:374-476): the terminal velocity of a
// droplet of the unresolved size (sep_tau cells) of the particle's group, against the others'
// local mean density, in the continuous phase that leads around it, times the others' share;
// held back where a resolved interface (a clear gradient of the smoothed share of the pair's
// later group) has interfacial tension enough to keep droplets from shedding (cell Bond
// number below 1). Returns the vertical slip (cells / s).
DEV float group_drift(const DevScene& d, const DevMat* mats, uint32_t row, float ps, int grp, float px, float py,
                      int bx, int by, const float wx[3], const float wy[3], float sw, float fg, float others,
                      float sgx, float sgy, float sgz, float dt) {
    const DevParams* P = d.P;
    float4 sgr = make_float4(0.0f, 0.0f, 0.0f, 0.0f), snu = sgr, snw = sgr;   // share x density; viscosity of the majority group and its weight
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int ci = (by + b) * d.W + bx + a;
            const float4 q = __ldg(&d.comp[ci]);
            if (q.x <= 0.0f) continue;
            const float wt = wx[a] * wy[b];
            const float4 gr = __ldg(&d.grho[ci]);
            sgr.x += wt * gr.x;
            sgr.y += wt * gr.y;
            sgr.z += wt * gr.z;
            sgr.w += wt * gr.w;
            const float4 ax = __ldg(&d.aux[ci]);
            const float4 fc = make_float4(1.0f - q.y - ax.z - ax.w, q.y, ax.z, ax.w);
            const float top = maxf(maxf(fc.x, fc.y), maxf(fc.z, fc.w));
            float4 oh = make_float4(fc.x == top ? 1.0f : 0.0f, fc.y == top ? 1.0f : 0.0f, fc.z == top ? 1.0f : 0.0f, fc.w == top ? 1.0f : 0.0f);
            const float on = maxf(oh.x + oh.y + oh.z + oh.w, 1.0f);
            oh = make_float4(oh.x / on, oh.y / on, oh.z / on, oh.w / on);
            const float wn = wt * ax.x;
            snu.x += wn * oh.x;
            snu.y += wn * oh.y;
            snu.z += wn * oh.z;
            snu.w += wn * oh.w;
            snw.x += wt * oh.x;
            snw.y += wt * oh.y;
            snw.z += wt * oh.z;
            snw.w += wt * oh.w;
        }
    sgr = make_float4(sgr.x / sw, sgr.y / sw, sgr.z / sw, sgr.w / sw);
    const float rho_g = fg > 1e-4f ? f4c(sgr, grp) / fg : row_density(mats, row, ps);
    const float rho_o = (sgr.x + sgr.y + sgr.z + sgr.w - f4c(sgr, grp)) / others;
    const float drho = rho_g - rho_o;
    const int W = d.W;
    const int k = clampi((int)py, 1, d.H - 2) * W + clampi((int)px, 1, W - 2);
    const float4 fsv = make_float4(1.0f - sgx - sgy - sgz, sgx, sgy, sgz);
    const int G = lead4(fsv);
    const float rho_c = f4c(sgr, G) / maxf(f4c(fsv, G), 1e-4f);
    const float nu_c = f4c(snw, G) > 1e-6f ? f4c(snu, G) / f4c(snw, G) : __ldg(&d.aux[k]).x;
    const float vt = terminal(drho, rho_c, nu_c, P->sep_tau, P->gravity);
    const float sep_max = P->corr[2] > 0.0f ? P->cfl / dt : 1e30f;
    float slip = -minf(vt, sep_max) * signf(drho) * others;
    float4 fs = fsv;
    if (grp == 0) fs.x = -1.0f;
    else if (grp == 1) fs.y = -1.0f;
    else if (grp == 2) fs.z = -1.0f;
    else fs.w = -1.0f;
    const int h = lead4(fs);
    const float bond = fabsf(drho) * P->gravity / maxf(P->pair[grp][h], 1e-9f);
    const float hold = clampf(1.0f - bond, 0.0f, 1.0f);
    if (slip != 0.0f && hold > 0.0f) {
        const int hi = max(grp, h);
        float gx, gy;
        if (hi == 1) {
            gx = 0.5f * (__ldg(&d.surf[k + 1]).y - __ldg(&d.surf[k - 1]).y);
            gy = 0.5f * (__ldg(&d.surf[k + W]).y - __ldg(&d.surf[k - W]).y);
        } else if (hi == 2) {
            gx = 0.5f * (__ldg(&d.surf2[k + 1]).x - __ldg(&d.surf2[k - 1]).x);
            gy = 0.5f * (__ldg(&d.surf2[k + W]).x - __ldg(&d.surf2[k - W]).x);
        } else {
            gx = 0.5f * (__ldg(&d.surf2[k + 1]).y - __ldg(&d.surf2[k - 1]).y);
            gy = 0.5f * (__ldg(&d.surf2[k + W]).y - __ldg(&d.surf2[k - W]).y);
        }
        const float resolved = 1.0f - clampf((0.12f - len2(gx, gy)) / (0.12f - 0.04f), 0.0f, 1.0f);
        slip *= 1.0f - hold * resolved;
    }
    return slip;
}

// XTRA: the tank has concentration families, several phase groups, settling or currents.
// Without them the pass is compiled without that code (64 registers against ~90, so twice
// the resident warps for its latency-bound gathers); the launcher picks the instantiation.
template <bool XTRA>
__global__ void __launch_bounds__(256) k_advance(DevScene d) {
    const DevParams* P = d.P;
    const StepState* S = d.S;
    uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    float report = 0.0f;
    uint32_t key = DEAD_KEY;
    if (id < P->n_slots) {
        float4 q0 = d.part[3 * id + 0], q1 = d.part[3 * id + 1], q2 = d.part[3 * id + 2];
        uint32_t kind = __float_as_uint(q2.y);
        if (kind != KIND_DEAD && (kind & 255u) != 0u) {
            const DevMat* mats = d.mats;
            float dt = S->dt;
            uint32_t row = (kind & 255u) - 1u;
            int ia1 = mats[row].ia[1];
            bool thermal = P->thermal != 0;
            float px = q0.x, py = q0.y;
            float pvx = q0.z, pvy = q0.w;
            float4 C = q1;
            float ps = q2.x, pt = q2.w;
            uint32_t pid = __float_as_uint(q2.z);
            // viscoelastic stress (upper-convected Maxwell): a particle that has not run a substep
            // yet starts unstressed; the slot keeps what it held unless the pass updates it
            // (particles.comp:152-156, 250-279)
            // frozen, or too viscous to flow: part of a rigid body (particles.comp:144-151)
            const bool rigid_cap = XTRA && (P->caps & CAP_RIGID) != 0u;
            bool frozen = false;
            if (rigid_cap) {
                const float2 ph = thermal ? phase_of(pt, thermal_of(mats, row, ps)) : make_float2(P->heat[0], 0.0f);
                frozen = ph.y > 0.5f || row_lnu(mats, row, ps, ph.x, thermal) >= P->heat2[0];
            }
            bool held = false;
            const bool elastic = XTRA && (P->caps & CAP_ELASTIC) != 0u;
            const float4 held_tau = elastic ? d.pstress[id] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            float4 tau = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (elastic && (kind & KIND_FRESH) == 0u && mats[row].el[0] > 0.0f) tau = held_tau;
            float4 tau_store = held_tau;
            bool alive = true;
            if (S->gather) {
                Grid g{d.vel, d.sdf, d.W, d.H};
                float vx = pvx, vy = pvy, corrx = 0.0f, corry = 0.0f;
                float slip = 0.0f;   // vertical drift relative to the mixture (cells / s)
                float crowd = 0.0f;
                gather_face<0>(g, px, py, vx, corrx, C.x, C.y);
                gather_face<1>(g, px, py, vy, corry, C.z, C.w);
                if (rigid_cap) {
                    // a frozen particle, a yield-stress plug's particle in a sparse cell, or any
                    // particle in a rigid cell moves exactly with the body around it
                    // (particles.comp:222-248)
                    const int pcx = clampi((int)px, 0, d.W - 1), pcy = clampi((int)py, 0, d.H - 1);
                    const bool plug = (mats[row].rheo[0] > 0.0f || mats[row].temp[3] > 0.0f) && d.cell[pcy * d.W + pcx].w <= 0.0f;
                    const int c0x = clampi((int)px, 1, d.W - 2), c0y = clampi((int)py, 1, d.H - 2);
                    const bool in_body = row != 57u && d.rl[c0y * d.W + c0x].x >= 0;
                    if (frozen || plug || in_body) {
                        const int ox[9] = {0, -1, 1, 0, 0, -1, 1, -1, 1}, oy[9] = {0, 0, 0, -1, 1, -1, -1, 1, 1};
                        for (int k = 0; k < 9 && !held; k++) {
                            const int root = d.rl[(c0y + oy[k]) * d.W + c0x + ox[k]].x;
                            if (root < 0 || d.rl[root].y < 0) continue;
                            float3 u;
                            if (body_motion(d, d.rl[root].y, root, px, py, u)) {
                                vx = u.x;
                                vy = u.y;
                                C = make_float4(0.0f, -u.z, u.z, 0.0f);
                                held = true;
                            }
                        }
                    }
                }
                if (elastic) {
                    const float G = mats[row].el[0];
                    if (G > 0.0f) {
                        // L = [[du/dx, du/dy], [dv/dx, dv/dy]] (the APIC matrix); at most
                        // elastic_step_max of deformation per substep enters the stress
                        float l00 = C.x, l01 = C.y, l10 = C.z, l11 = C.w;
                        const float lnorm = sqrtf(C.x * C.x + C.y * C.y + C.z * C.z + C.w * C.w) * dt;
                        if (P->elastic[3] > 0.0f && lnorm > P->elastic[3]) {
                            const float k = P->elastic[3] / lnorm;
                            l00 *= k;
                            l01 *= k;
                            l10 *= k;
                            l11 *= k;
                        }
                        const float t00 = tau.x, t01 = tau.z, t10 = tau.z, t11 = tau.y;
                        // D = L T + T L^T + G (L + L^T), each entry summed in that order
                        const float d00 = ((l00 * t00 + l01 * t10) + (t00 * l00 + t01 * l01)) + G * (l00 + l00);
                        const float d01 = ((l00 * t01 + l01 * t11) + (t00 * l10 + t01 * l11)) + G * (l01 + l10);
                        const float d10 = ((l10 * t00 + l11 * t10) + (t10 * l00 + t11 * l01)) + G * (l10 + l01);
                        const float d11 = ((l10 * t01 + l11 * t11) + (t10 * l10 + t11 * l11)) + G * (l11 + l11);
                        const float lam = maxf(mats[row].el[1], 1e-4f);
                        const float den = 1.0f + dt / lam;
                        const float n00 = (t00 + dt * d00) / den, n01 = (t01 + dt * d01) / den;
                        const float n10 = (t10 + dt * d10) / den, n11 = (t11 + dt * d11) / den;
                        tau = make_float4(n00, n11, 0.5f * (n01 + n10), 0.0f);
                        const float tn = sqrtf(tau.x * tau.x + tau.y * tau.y + tau.z * tau.z);
                        if (P->elastic[2] > 0.0f && tn > P->elastic[2] * G) {
                            const float k = P->elastic[2] * G / tn;
                            tau = make_float4(tau.x * k, tau.y * k, tau.z * k, tau.w * k);
                        }
                        // no liquid around (spray, a torn-off droplet): no stress the grid can carry
                        const int c1x = clampi((int)px, 1, d.W - 2), c1y = clampi((int)py, 1, d.H - 2);
                        float around = 0.0f;
                        for (int b = -1; b <= 1; b++)
                            for (int a = -1; a <= 1; a++) around += minf(d.cell[(c1y + b) * d.W + c1x + a].x, 1.0f);
                        if (around < 1.0f) tau = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    }
                    tau_store = tau;
                }
                if (P->apic_clamp > 0.0f) {
                    float lim = P->apic_clamp / dt;
                    C.x = clampf(C.x, -lim, lim);
                    C.y = clampf(C.y, -lim, lim);
                    C.z = clampf(C.z, -lim, lim);
                    C.w = clampf(C.w, -lim, lim);
                }
                if (P->corr[0] > 0.0f) {
                    float cl = len2(corrx, corry), cmax = P->corr[0] / dt;
                    if (cl > cmax) {
                        corrx *= cmax / cl;
                        corry *= cmax / cl;
                    }
                }
                // composition: occupancy around the particle and the heat it takes
                {
                    float gx = px - 0.5f, gy = py - 0.5f;
                    int bx = (int)floorf(gx - 0.5f), by = (int)floorf(gy - 0.5f);
                    float fx = gx - (float)bx, fy = gy - (float)by;
                    float wx[3], wy[3];
                    bspline(fx, fy, wx, wy);
                    // with concentration families: sw, the weight of the cells holding liquid;
                    // sfw, sfs, the weight and concentration of those that hold the particle's
                    // own family (a diluent's: family 0)
                    int fam = mats[row].ib[0];
                    const int nmix = P->n_fam - 1;
                    const bool fams = XTRA && P->n_fam > 0;
                    // with several phase groups: sg, the shares of groups 1 - 3 around the
                    // particle; with a group that sorts its materials, sbg, share x base density
                    // of the particle's group
                    const int grp = mats[row].ia[0];
                    const uint32_t gm = P->group_mask;
                    const bool groups = XTRA && (gm & (gm - 1u)) != 0u, more = XTRA && (gm & 12u) != 0u;
                    const bool sorts = XTRA && grp > 0 && ((P->sorts >> grp) & 1u) != 0u;
                    const bool gather = fams || groups || sorts;
                    float sw = 0.0f, sfw = 0.0f, sfs = 0.0f, sg0 = 0.0f, sg1 = 0.0f, sg2 = 0.0f, sbg = 0.0f;
#pragma unroll
                    for (int b = 0; b < 3; b++)
#pragma unroll
                        for (int a = 0; a < 3; a++) {
                            const int ci = (by + b) * d.W + bx + a;
                            const float4 q = __ldg(&d.comp[ci]);
                            const float wt = wx[a] * wy[b];
                            crowd += wt * q.w;
                            if (gather && q.x > 0.0f) {
                                sw += wt;
                                sg0 += wt * q.y;
                                if (more) {
                                    const float4 ax = __ldg(&d.aux[ci]);
                                    sg1 += wt * ax.z;
                                    sg2 += wt * ax.w;
                                }
                                if (sorts) sbg += wt * f4c(__ldg(&d.gbase[ci]), grp - 1);
                            }
                            if (fams && q.x > 0.0f) {
                                const float sb = fam > 0 ? d.mixb[(size_t)ci * nmix + fam - 1] : q.z;
                                if (sb >= 0.0f) {
                                    sfw += wt;
                                    sfs += wt * sb;
                                }
                            }
                        }
                    if (XTRA && (P->caps & CAP_SETTLE) != 0u) {
                        // Settling hands each cell a change of its family's concentration, taken
                        // with the scatter's weights; the first row, as the primary family's
                        // diluent, takes part at concentration 0 (particles.comp:331-352).
                        const bool dil0 = fam < 0 && P->primary >= 0 && P->fams[0][1] == (int)row;
                        const int sf = dil0 ? 0 : fam;
                        if (sf >= 0 && (kind & KIND_FRESH) == 0u && mats[dil0 ? (uint32_t)P->primary : row].b[2] > 0.0f) {
                            float dsx = 0.0f, dsy = 0.0f;
#pragma unroll
                            for (int b = 0; b < 3; b++)
#pragma unroll
                                for (int a = 0; a < 3; a++) {
                                    const float2 v = d.dsettle[(size_t)((by + b) * d.W + bx + a) * P->n_fam + sf];
                                    const float wt = wx[a] * wy[b];
                                    dsx += wt * v.x;
                                    dsy += wt * v.y;
                                }
                            const float s0 = dil0 ? 0.0f : ps;
                            const float s1 = clampf(s0 + (1.0f - s0) * dsx - s0 * dsy, 0.0f, 1.0f);
                            const float c0 = thermal ? thermal_of(mats, row, ps).w : 0.0f;
                            if (dil0 && s1 > 0.0f) {
                                row = (uint32_t)P->primary;
                                ia1 = mats[row].ia[1];
                                fam = 0;
                                kind = (kind & ~255u) | (row + 1u);
                            }
                            if (!dil0 || s1 > 0.0f) ps = s1;
                            if (thermal) pt = keep_heat(pt, c0, thermal_of(mats, row, ps).w);
                        }
                    }
                    if (thermal && (kind & KIND_FRESH) == 0u) {
                        float dT = 0.0f;
#pragma unroll
                        for (int b = 0; b < 3; b++)
#pragma unroll
                            for (int a = 0; a < 3; a++) dT += wx[a] * wy[b] * d.dheat[(by + b) * d.W + bx + a].x;
                        int ox = clampi((int)floorf(px), 0, d.W - 1), oy = clampi((int)floorf(py), 0, d.H - 1);
                        float4 own = d.dheat[oy * d.W + ox];
                        if (own.y > 0.0f) {
                            float4 th = thermal_of(mats, row, ps);
                            float tb = ia1 >= 0 ? mixf(mats[ia1].th2[2], mats[row].th2[2], ps) : mats[row].th2[2];
                            int2 hq = heat_quanta(th.w, minf(phase_of(pt, th).x, tb));
                            dT += own.y * (own.z - (float)hq.y / (float)hq.x) * T_SCALE;
                        }
                        pt += dT;
                    }
                    if (gather && sw > 1e-4f) {
                        const float sgx = sg0 / sw, sgy = sg1 / sw, sgz = sg2 / sw;
                        const int gnow = mats[row].ia[0];   // the group of the row as settling left it
                        const float fg = gnow == 0 ? 1.0f - sgx - sgy - sgz : (gnow == 1 ? sgx : gnow == 2 ? sgy : sgz);
                        const float others = 1.0f - fg;
                        if (others > 1e-4f && groups && !held)
                            slip = group_drift(d, mats, row, ps, gnow, px, py, bx, by, wx, wy, sw, fg, others, sgx, sgy, sgz, dt);
                        if (sorts && !held) {
                            // drift within the particle's own group against its local mean base
                            // density (particles.comp:478-502)
                            const float fgi = groups ? (gnow == 1 ? sgx : gnow == 2 ? sgy : sgz) : 1.0f;
                            if (fgi > 1e-4f) {
                                const float rmean = sbg / sw / fgi;
                                const float drho = mats[row].a[0] - rmean;
                                const int pcx = clampi((int)px, 0, d.W - 1), pcy = clampi((int)py, 0, d.H - 1);
                                const float4 cq = __ldg(&d.cell[pcy * d.W + pcx]);
                                const float nu_c = cq.y > 0.0f ? cq.z / cq.y : __ldg(&d.aux[pcy * d.W + pcx]).x;
                                const float vt = terminal(drho, rmean, nu_c, P->sep_tau, P->gravity);
                                const float sep_max = P->corr[2] > 0.0f ? P->cfl / dt : 1e30f;
                                slip -= minf(vt, sep_max) * signf(drho);
                            }
                        }
                    }
                    if (fams && sw > 1e-4f) {
                        // Miscible exchange: the concentration relaxes towards its family's
                        // local mean; the first row, the diluent of the primary family, takes
                        // part as concentration 0 and becomes a particle of the family when it
                        // gains any (particles.comp:519-543).
                        const bool dil0 = fam < 0 && P->primary >= 0 && P->fams[0][1] == (int)row;
                        if ((fam >= 0 || dil0) && sfw > 1e-4f) {
                            const float s0 = dil0 ? 0.0f : ps;
                            const float rate = mats[dil0 ? (uint32_t)P->primary : row].a[3];
                            const float s1 = clampf(s0 + (sfs / sfw - s0) * (1.0f - sp_expf(-rate * dt)), 0.0f, 1.0f);
                            const float c0 = thermal ? thermal_of(mats, row, ps).w : 0.0f;
                            if (!dil0) {
                                ps = s1;
                            } else if (s1 > 0.0f) {
                                row = (uint32_t)P->primary;
                                ia1 = mats[row].ia[1];
                                kind = (kind & ~255u) | (row + 1u);
                                ps = s1;
                            }
                            if (thermal) pt = keep_heat(pt, c0, thermal_of(mats, row, ps).w);
                        }
                        // A pure diluent next to another of its concentrates joins that family
                        // at concentration 0 (the same liquid): the primary family if it gained
                        // some above, else the first family in table order found around it
                        // (particles.comp:544-569).
                        if (fam < 0 && (kind & 255u) - 1u == row && mats[row].ib[0] < 0) {
                            for (int j = P->primary >= 0 ? 1 : 0; j < P->n_fam; j++) {
                                if (P->fams[j][1] != (int)row) continue;
                                float found = 0.0f;
                                if (j == 0) {
                                    found = sfw;
                                } else {
                                    for (int b = 0; b < 3; b++)
                                        for (int a = 0; a < 3; a++)
                                            if (d.mixb[(size_t)((by + b) * d.W + bx + a) * nmix + j - 1] >= 0.0f) found += wx[a] * wy[b];
                                }
                                if (found > 1e-4f) {
                                    row = (uint32_t)P->fams[j][0];
                                    ia1 = mats[row].ia[1];
                                    kind = (kind & ~255u) | (row + 1u);
                                    ps = 0.0f;
                                    break;
                                }
                            }
                        }
                    }
                }
                if (held && crowd <= REST_PHI + maxf(P->corr[1], 0.05f)) {   // particles.comp:576
                    corrx = 0.0f;
                    corry = 0.0f;
                }
                // drains: a zone with a negative rate removes each particle in it with probability
                // -rate (1 - 0.75 r^2) dt per substep (particles.comp:577-594)
                const int ncur = XTRA ? (int)P->ext[3] : 0;
                for (int c = 0; c < ncur && alive; c++) {
                    const float* z = P->current_zone[c];
                    if (z[3] >= 0.0f) continue;
                    const float dzx = px - z[0], dzy = py - z[1];
                    const float r2 = (dzx * dzx + dzy * dzy) / (z[2] * z[2]);
                    if (r2 < 1.0f) {
                        const float u = (float)(hash32(pid * 2246822519u + S->substeps * 3266489917u + (uint32_t)c) >> 8) / 16777216.0f;
                        if (u < -z[3] * (1.0f - 0.75f * r2) * dt) alive = false;
                    }
                }
                bool pushed = false;
                if (alive && P->tool_mode != 0) {
                    float dx = P->tool_pos[0] - px, dy = P->tool_pos[1] - py;
                    float r2 = (dx * dx + dy * dy) / (P->tool_radius * P->tool_radius);
                    if (r2 < 1.0f) {
                        float fall = 1.0f - r2;
                        if (P->tool_mode == 2) {
                            alive = false;
                        } else if (P->tool_mode == 5 || P->tool_mode == 6) {
                            if (thermal) {
                                float e = P->heat2[1] * fall * dt;
                                float Cc = thermal_of(mats, row, ps).w;
                                if (P->tool_mode == 6) e = minf(e, maxf(phase_of(pt, thermal_of(mats, row, ps)).x + 150.0f, 0.0f) * Cc);
                                pt += (P->tool_mode == 5 ? e : -e) / Cc;
                                ledger_add(d.ledger, P->tool_mode == 5 ? 4 : 5, e * P->inv_ppc);
                            }
                        } else {
                            float k = clampf(P->tool_strength * fall * dt, 0.0f, 1.0f);
                            if (P->tool_crowd_max > 0.0f && P->tool_mode != 4)
                                k *= clampf((P->tool_crowd_max - crowd) / (0.25f * P->tool_crowd_max), 0.0f, 1.0f);
                            float2 tt = tool_target(P, dx, dy);
                            vx = mixf(vx, tt.x, k);
                            vy = mixf(vy, tt.y, k);
                            pushed = true;
                        }
                    }
                }
                if (alive) {
                    if (thermal && mats[row].rx[2] > 0.0f) {
                        float e = mats[row].rx[2] * mats[row].th[0] * (ia1 >= 0 ? ps : 1.0f) * dt * P->heat[1];
                        pt += e / thermal_of(mats, row, ps).w;
                        ledger_add(d.ledger, 7, e * P->inv_ppc);
                    }
                    // currents: raise the velocity along each towards its speed, never brake, and
                    // not in a crowd (particles.comp:809-835)
                    const float drive = P->tool_crowd_max > 0.0f ? clampf((P->tool_crowd_max - crowd) / (0.25f * P->tool_crowd_max), 0.0f, 1.0f) : 1.0f;
                    for (int c = 0; c < ncur && drive > 0.0f; c++) {
                        const float* z = P->current_zone[c];
                        if (z[3] <= 0.0f) continue;
                        const float dzx = px - z[0], dzy = py - z[1];
                        const float r2 = (dzx * dzx + dzy * dzy) / (z[2] * z[2]);
                        if (r2 < 1.0f) {
                            const float tx = P->current_vel[c][0], ty = P->current_vel[c][1];
                            const float speed = len2(tx, ty);
                            const float dx = tx / maxf(speed, 1e-6f), dy = ty / maxf(speed, 1e-6f);
                            const float fall = (1.0f - r2) * (1.0f - r2);
                            const float gap = maxf(speed - (vx * dx + vy * dy), 0.0f);
                            const float e = 1.0f - sp_expf(-z[3] * fall * dt);
                            vx += dx * gap * e * drive;
                            vy += dy * gap * e * drive;
                        }
                    }
                    float vcap = P->ext[0];
                    {
                        float sp = len2(vx, vy);
                        if (sp > vcap) {
                            vx *= vcap / sp;
                            vy *= vcap / sp;
                        }
                    }
                    float vax = vx, vay = vy;
                    if (P->ext[1] >= 2.0f && !pushed && !held) {
                        float xmx = clampf(px + 0.5f * dt * (vx + corrx + 0.0f), 2.01f, (float)d.W - 2.01f);
                        float xmy = clampf(py + 0.5f * dt * (vy + corry + slip), 2.01f, (float)d.H - 2.01f);
                        float2 here = sample_vel(g, px, py, make_float2(vx, vy));
                        float2 there = sample_vel(g, xmx, xmy, here);
                        vax = vx + there.x - here.x;
                        vay = vy + there.y - here.y;
                        float sp = len2(vax, vay);
                        if (sp > vcap) {
                            vax *= vcap / sp;
                            vay *= vcap / sp;
                        }
                        if (crowd < LIQUID_THR && (vax * vax + vay * vay) < 0.01f * (vx * vx + vy * vy)) {
                            vx = vax;
                            vy = vay;
                        }
                    }
                    float dispx = vax + corrx + 0.0f, dispy = vay + corry + slip;
                    {
                        float mine = len2(dispx, dispy);
                        if (crowd < LIQUID_THR) mine /= P->ext[2];
                        report = mine;
                    }
                    float sx = dt * dispx, sy = dt * dispy;
                    int pieces = clampi((int)ceilf(len2(sx, sy)), 1, 32);
                    sx /= (float)pieces;
                    sy /= (float)pieces;
                    float x = px, y = py;
                    float wm = P->wall_margin;
                    for (int k = 1; k < pieces; k++) {
                        x += sx;
                        y += sy;
                        collide(g, wm, x, y, vx, vy, true);
                    }
                    x += sx;
                    y += sy;
                    float excess = clampf(crowd - 1.5f, 0.0f, 1.0f);
                    if (excess > 0.0f && P->crowd_jitter > 0.0f) {
                        uint32_t hh = hash32(pid ^ hash32(__float_as_uint(px) ^ S->substeps));
                        x += ((float)(hh & 0xffffu) / 65535.0f - 0.5f) * P->crowd_jitter * excess;
                        y += ((float)(hh >> 16) / 65535.0f - 0.5f) * P->crowd_jitter * excess;
                    }
                    collide(g, wm, x, y, vx, vy, true);
                    bool again = collide(g, wm, x, y, vx, vy, true);
                    if (again) {
                        float ggx, ggy;
                        if (sample_sdf(g, x, y, &ggx, &ggy) < -1.0f) collide(g, wm, x, y, vx, vy, false);
                    }
                    x = clampf(x, 2.01f, (float)d.W - 2.01f);
                    y = clampf(y, 2.01f, (float)d.H - 2.01f);
                    px = x;
                    py = y;
                    pvx = vx;
                    pvy = vy;
                    kind &= ~KIND_FRESH;
                }
            }
            if (alive) {
                if (thermal) {
                    float4 th = thermal_of(mats, row, ps);
                    float2 ph = phase_of(pt, th);
                    float tb = ia1 >= 0 ? mixf(mats[ia1].th2[2], mats[row].th2[2], ps) : mats[row].th2[2];
                    int hx = clampi((int)floorf(px), 0, d.W - 1), hy = clampi((int)floorf(py), 0, d.H - 1);
                    int2 hq = heat_quanta(th.w, minf(ph.x, tb));
                    atomicAdd(&d.hcell[hy * d.W + hx].x, hq.x);
                    atomicAdd(&d.hcell[hy * d.W + hx].y, hq.y);
                }
                int cx = clampi((int)px, 0, d.W - 1), cy = clampi((int)py, 0, d.H - 1);
                key = (uint32_t)(cy * d.W + cx);
                d.part2[3 * id + 0] = make_float4(px, py, pvx, pvy);
                d.part2[3 * id + 1] = C;
                d.part2[3 * id + 2] = make_float4(ps, __uint_as_float(kind), __uint_as_float(pid), pt);
                if (elastic) {
                    d.pstress2[id] = tau_store;
                    d.pdep[id] = tau;
                }
            }
        }
    }
    report_max(&d.S->umax_part, report);
    if (id < P->n_slots) {
        d.pkey[id] = key;
        d.prank[id] = key != DEAD_KEY ? atomicAdd(&d.count[key], 1u) : 0u;
    }
}

// ---- the sort ---------------------------------------------------------------------------

constexpr int SCAN_BLOCK = 1024;

// Block-wise exclusive scan of count[0..n) into start, block totals into tmp.
__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_blocks(const uint32_t* count, uint32_t* start, uint32_t* tmp, int n) {
    __shared__ uint32_t warp_sums[SCAN_BLOCK / 32];
    int i = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    uint32_t v = i < n ? count[i] : 0u;
    uint32_t x = v;
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warp_sums[lane] = s;
    }
    __syncthreads();
    uint32_t base = wid > 0 ? warp_sums[wid - 1] : 0u;
    if (i < n) start[i] = base + x - v;
    if (threadIdx.x == SCAN_BLOCK - 1) tmp[blockIdx.x] = base + x;
}

// Exclusive scan of the block totals (one block, any count); the grand total is the
// number of live particles.
__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_top(uint32_t* tmp, int nb, StepState* S) {
    __shared__ uint32_t warp_sums[SCAN_BLOCK / 32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0u;
    __syncthreads();
    for (int b0 = 0; b0 < nb; b0 += SCAN_BLOCK) {
        int i = b0 + threadIdx.x;
        uint32_t v = i < nb ? tmp[i] : 0u;
        uint32_t x = v;
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t s = warp_sums[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            warp_sums[lane] = s;
        }
        __syncthreads();
        uint32_t base = (wid > 0 ? warp_sums[wid - 1] : 0u) + carry;
        if (i < nb) tmp[i] = base + x - v;
        __syncthreads();
        if (threadIdx.x == SCAN_BLOCK - 1) carry = base + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) S->n_live = carry;
}

__global__ void k_scan_add(uint32_t* start, const uint32_t* tmp, int n) {
    int i = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    if (i < n) start[i] += tmp[blockIdx.x];
}

__global__ void k_place(DevScene d) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.P->n_slots) return;
    uint32_t key = d.pkey[i];
    if (key == DEAD_KEY) return;
    d.perm[d.start[key] + d.prank[i]] = i;
}

// Each cell's arrivals in slot order: the stable order of the counting sort (sort.comp keeps
// a cell's particles in arrival order, which atomics make arbitrary; slot order makes it
// deterministic). One thread per cell sorts up to 16 entries of perm in registers; a cell with
// more goes on the crowd list for k_crowd_sort (a thread's sort in place in global memory
// costs two dependent global accesses per step, and one cell of 60 took 0.25 ms).
constexpr int kCrowdMax = 4096;    // entries a block sorts in shared memory
constexpr int kCrowdBlocks = 152;  // k_crowd_sort's grid: one block per SM over the list
__global__ void __launch_bounds__(256) k_cell_sort(DevScene d) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.ncell) return;
    const uint32_t n = d.count[c];
    if (n < 2u) return;
    uint32_t* seg = d.perm + d.start[c];
    if (n <= 16u) {
        uint32_t v[16];
#pragma unroll
        for (int k = 0; k < 16; k++)
            if ((uint32_t)k < n) v[k] = seg[k];
        for (uint32_t k = 1; k < n; k++) {
            const uint32_t x = v[k];
            int j = (int)k - 1;
            while (j >= 0 && v[j] > x) {
                v[j + 1] = v[j];
                j--;
            }
            v[j + 1] = x;
        }
#pragma unroll
        for (int k = 0; k < 16; k++)
            if ((uint32_t)k < n) seg[k] = v[k];
    } else if (n <= (uint32_t)kCrowdMax) {
        const uint32_t at = atomicAdd(&d.crowd[0], 1u);   // at most ncell cells: the list holds them
        d.crowd[1 + at] = (uint32_t)c;
    } else {   // (more particles in one cell than a block sorts in shared memory)
        for (uint32_t k = 1; k < n; k++) {
            const uint32_t x = seg[k];
            int j = (int)k - 1;
            while (j >= 0 && seg[j] > x) {
                seg[j + 1] = seg[j];
                j--;
            }
            seg[j + 1] = x;
        }
    }
}

// The crowded cells, a block each: the entries (distinct slots) into shared memory, each
// entry's place = how many entries are smaller, written back in that order.
__global__ void __launch_bounds__(256) k_crowd_sort(DevScene d) {
    __shared__ uint32_t in[kCrowdMax], out[kCrowdMax];
    const uint32_t cells = d.crowd[0];
    for (uint32_t b = blockIdx.x; b < cells; b += gridDim.x) {
        const uint32_t c = d.crowd[1 + b];
        const uint32_t n = d.count[c];
        uint32_t* seg = d.perm + d.start[c];
        for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) in[k] = seg[k];
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
            const uint32_t x = in[k];
            uint32_t r = 0;
            for (uint32_t j = 0; j < n; j++) r += in[j] < x ? 1u : 0u;
            out[r] = x;
        }
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) seg[k] = out[k];
        __syncthreads();
    }
}

// The particles in sorted order, one thread per slot: slot j < n_live takes the advanced
// particle perm[j] (consecutive slots write consecutive records), slots [n_live, n_slots)
// become dead (zero) slots.
__global__ void __launch_bounds__(256) k_cell_gather(DevScene d) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= d.P->n_slots) return;
    if (j < d.S->n_live) {
        const uint32_t src = d.perm[j];
        const float4 a = d.part2[3 * src + 0], b = d.part2[3 * src + 1], c = d.part2[3 * src + 2];
        d.part[3 * j + 0] = a;
        d.part[3 * j + 1] = b;
        d.part[3 * j + 2] = c;
        if (d.pstress) d.pstress[j] = d.pstress2[src];   // the stress moves with its particle (sort.comp:66)
        if (d.plook) d.plook2[j] = d.plook[src];          // and the look's state (sort.comp's plook)
    } else {
        const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        d.part[3 * j + 0] = z;
        d.part[3 * j + 1] = z;
        d.part[3 * j + 2] = z;
        if (d.pstress) d.pstress[j] = z;
        if (d.plook) d.plook2[j] = make_uint4(0u, 0u, 0u, 0u);
    }
}

// The look's state back from the sort's target, slot for slot.
__global__ void __launch_bounds__(256) k_look_back(DevScene d) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < d.P->n_slots) d.plook[j] = d.plook2[j];
}

// ---- P2G gather ------------------------------------------------------------------------

constexpr int P2G_T = 16;                 // nodes per tile edge
constexpr int P2G_HALO_ROWS = P2G_T + 3;  // particle cells [n0 - 2, n0 + 16]

DEV void sadd(int* sacc, int ps, int lx, int ly, int ch, int v) {
    if (lx >= 0 && ly >= 0 && lx < P2G_T && ly < P2G_T) atomicAdd(&sacc[(ly * P2G_T + lx) * ps + ch], v);
}

__global__ void __launch_bounds__(256) k_p2g(DevScene d) {
    extern __shared__ int sacc[];
    __shared__ uint32_t row_beg[P2G_HALO_ROWS], row_pre[P2G_HALO_ROWS + 1];
    const DevParams* P = d.P;
    const DevMat* mats = d.mats;
    const int stride = d.stride;
    const int pst = stride + 1;   // a node's channels padded by one word: nodes on distinct banks
    const int n0x = blockIdx.x * P2G_T, n0y = blockIdx.y * P2G_T;
    for (int k = threadIdx.x; k < P2G_T * P2G_T * pst; k += blockDim.x) sacc[k] = 0;
    if (threadIdx.x < P2G_HALO_ROWS) {
        int cy = n0y - 2 + threadIdx.x;
        uint32_t b = 0, e = 0;
        if (cy >= 0 && cy < d.H) {
            int x0 = max(n0x - 2, 0), x1 = min(n0x + P2G_T, d.W - 1);
            b = d.start[cy * d.W + x0];
            e = d.start[cy * d.W + x1 + 1];
        }
        row_beg[threadIdx.x] = b;
        row_pre[threadIdx.x + 1] = e - b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        row_pre[0] = 0;
        for (int r = 0; r < P2G_HALO_ROWS; r++) row_pre[r + 1] += row_pre[r];
    }
    __syncthreads();
    const uint32_t total = row_pre[P2G_HALO_ROWS];
    const float dt = d.S->dt;
    const bool thermal = P->thermal != 0;
    const int ct = thermal ? (int)P->heat2[2] : -1;
    // particle f of the tile's neighbourhood lies in row r: f only grows, so each thread's row
    // search continues from where its previous particle was found
    int r = 0;
    for (uint32_t f = threadIdx.x; f < total; f += blockDim.x) {
        while (row_pre[r + 1] <= f) r++;
        uint32_t pi = row_beg[r] + (f - row_pre[r]);
        float4 q0 = d.part[3 * pi + 0], q1 = d.part[3 * pi + 1], q2 = d.part[3 * pi + 2];
        uint32_t kind = __float_as_uint(q2.y);
        uint32_t row = (kind & 255u) - 1u;
        const int* ia = mats[row].ia;
        float ps = q2.x;
        float rho = row_density(mats, row, ps);
        float CT = 0.0f;
        int cg = -1;
        if (thermal) {
            float4 th = thermal_of(mats, row, ps);
            float2 ph = phase_of(q2.w, th);
            float tb = ia[1] >= 0 ? mixf(mats[ia[1]].th2[2], mats[row].th2[2], ps) : mats[row].th2[2];
            rho *= expansion_of(mats, row, ps, ph.x);
            if (ph.y > 0.0f) {
                float rs = ia[1] >= 0 ? mixf(mats[ia[1]].b[3], mats[row].b[3], ps) : mats[row].b[3];
                rho = mixf(rho, rs, ph.y);
            }
            CT = th.w * (minf(ph.x, tb) + 273.15f) / T_SCALE;
            cg = group_heat_chan(P, ia[0]);
        }
        const float px = q0.x, py = q0.y;
        const float vsx = q0.z * dt, vsy = q0.w * dt;
        const float csx = q1.x * dt, csy = q1.y * dt, csz = q1.z * dt, csw = q1.w * dt;
        const int cw = ia[2], cs = ia[3];
        // the stress it deposits (particles.comp:983-984, 1050-1055): only a stressed particle
        int ce = -1;
        float tex = 0.0f, tey = 0.0f, tez = 0.0f;
        if (d.pdep && (P->caps & CAP_ELASTIC) != 0u) {
            const float4 tau = d.pdep[d.perm[pi]];
            if (tau.x != 0.0f || tau.y != 0.0f || tau.z != 0.0f || tau.w != 0.0f) {
                ce = (int)P->elastic[0];
                tex = tau.x / P->elastic[1] * 65536.0f;
                tey = tau.y / P->elastic[1] * 65536.0f;
                tez = tau.z / P->elastic[1] * 65536.0f;
            }
        }
        float wx[3], wy[3];
        {   // u faces at (i, j + 0.5)
            float gx = px - 0.0f, gy = py - 0.5f;
            int bx = (int)floorf(gx - 0.5f), by = (int)floorf(gy - 0.5f);
            float fx = gx - (float)bx, fy = gy - (float)by;
            bspline(fx, fy, wx, wy);
#pragma unroll
            for (int b = 0; b < 3; b++)
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    int lx = bx + a - n0x, ly = by + b - n0y;
                    if (lx < 0 || ly < 0 || lx >= P2G_T || ly >= P2G_T) continue;
                    float m = wx[a] * wy[b] * rho;
                    float ddx = (float)a - fx, ddy = (float)b - fy;
                    sadd(sacc, pst, lx, ly, 0, (int)floorf(m * MASS_SCALE + 0.5f));
                    sadd(sacc, pst, lx, ly, 1, (int)floorf(m * (vsx + (csx * ddx + csy * ddy)) * MOM_SCALE + 0.5f));
                }
        }
        {   // v faces at (i + 0.5, j)
            float gx = px - 0.5f, gy = py - 0.0f;
            int bx = (int)floorf(gx - 0.5f), by = (int)floorf(gy - 0.5f);
            float fx = gx - (float)bx, fy = gy - (float)by;
            bspline(fx, fy, wx, wy);
#pragma unroll
            for (int b = 0; b < 3; b++)
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    int lx = bx + a - n0x, ly = by + b - n0y;
                    if (lx < 0 || ly < 0 || lx >= P2G_T || ly >= P2G_T) continue;
                    float m = wx[a] * wy[b] * rho;
                    float ddx = (float)a - fx, ddy = (float)b - fy;
                    sadd(sacc, pst, lx, ly, 2, (int)floorf(m * MASS_SCALE + 0.5f));
                    sadd(sacc, pst, lx, ly, 3, (int)floorf(m * (vsy + (csz * ddx + csw * ddy)) * MOM_SCALE + 0.5f));
                }
        }
        {   // cell centres
            float gx = px - 0.5f, gy = py - 0.5f;
            int bx = (int)floorf(gx - 0.5f), by = (int)floorf(gy - 0.5f);
            float fx = gx - (float)bx, fy = gy - (float)by;
            bspline(fx, fy, wx, wy);
#pragma unroll
            for (int b = 0; b < 3; b++)
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    int lx = bx + a - n0x, ly = by + b - n0y;
                    if (lx < 0 || ly < 0 || lx >= P2G_T || ly >= P2G_T) continue;
                    int wi = (int)floorf(wx[a] * wy[b] * MASS_SCALE + 0.5f);
                    sadd(sacc, pst, lx, ly, 4, wi);
                    if (cw >= 0) sadd(sacc, pst, lx, ly, cw, wi);
                    if (cs >= 0 && ps > 0.0f) sadd(sacc, pst, lx, ly, cs, (int)floorf(wx[a] * wy[b] * ps * MASS_SCALE + 0.5f));
                    if (ce >= 0) {
                        const float wab = wx[a] * wy[b];
                        sadd(sacc, pst, lx, ly, ce, (int)floorf(wab * tex + 0.5f));
                        sadd(sacc, pst, lx, ly, ce + 1, (int)floorf(wab * tey + 0.5f));
                        sadd(sacc, pst, lx, ly, ce + 2, (int)floorf(wab * tez + 0.5f));
                    }
                    if (ct >= 0) {
                        int hq = (int)floorf(wx[a] * wy[b] * CT * MASS_SCALE + 0.5f);
                        sadd(sacc, pst, lx, ly, ct, hq);
                        if (cg >= 0) sadd(sacc, pst, lx, ly, cg, hq);
                    }
                }
        }
    }
    __syncthreads();
    // write the tile's nodes: one row of the tile is 16 x stride contiguous ints
    for (int k = threadIdx.x; k < P2G_T * P2G_T * stride; k += blockDim.x) {
        int node = k / stride, ch = k - node * stride;
        int nx = n0x + (node % P2G_T), ny = n0y + node / P2G_T;
        if (nx < d.W && ny < d.H) d.acc[(ny * d.W + nx) * stride + ch] = sacc[node * pst + ch];
    }
}

// ---- launchers ------------------------------------------------------------------------

void launch_advance(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st) {
    k_step<<<1, 1, 0, st>>>(d);
    cudaMemsetAsync(d.count, 0, (size_t)(d.ncell + 1) * sizeof(uint32_t), st);
    if (cfg.thermal) cudaMemsetAsync(d.hcell, 0, (size_t)d.ncell * sizeof(int2), st);
    uint32_t nb = (cfg.n_slots + 255) / 256;
    if (nb == 0) nb = 1;
    if (cfg.xtra) k_advance<true><<<nb, 256, 0, st>>>(d);
    else k_advance<false><<<nb, 256, 0, st>>>(d);
}

void launch_sort(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st) {
    uint32_t nb = (cfg.n_slots + 255) / 256;
    if (nb == 0) nb = 1;
    int n = d.ncell + 1;
    int sb = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
    k_scan_blocks<<<sb, SCAN_BLOCK, 0, st>>>(d.count, d.start, d.scan_tmp, n);
    k_scan_top<<<1, SCAN_BLOCK, 0, st>>>(d.scan_tmp, sb, d.S);
    k_scan_add<<<sb, SCAN_BLOCK, 0, st>>>(d.start, d.scan_tmp, n);
    k_place<<<nb, 256, 0, st>>>(d);
    cudaMemsetAsync(d.crowd, 0, sizeof(uint32_t), st);
    k_cell_sort<<<(d.ncell + 255) / 256, 256, 0, st>>>(d);
    k_crowd_sort<<<kCrowdBlocks, 256, 0, st>>>(d);
    k_cell_gather<<<nb, 256, 0, st>>>(d);
    if (d.plook) k_look_back<<<nb, 256, 0, st>>>(d);
}

void launch_p2g(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st) {
    (void)cfg;
    dim3 tiles((d.W + P2G_T - 1) / P2G_T, (d.H + P2G_T - 1) / P2G_T);
    size_t smem = (size_t)P2G_T * P2G_T * (d.stride + 1) * sizeof(int);
    k_p2g<<<tiles, 256, smem, st>>>(d);
}

}  // namespace sprout

// Grid side of the substep on sm_103a, one thread per cell in 16 x 16 tiles:
//   k_grid_prep   accumulators -> face velocities (+ gravity), composition, density,
//                 viscosity, liquid / air level (grid_prep.comp:20-263)
//   k_coef        ghost-fluid face coefficients (grid_coef.comp:12-39)
//   k_smooth      5 x 5 binomial indicator smoothing (surf_smooth.comp:16-44)
//   k_curv        node-normal curvature with the contact angle (surf_curv.comp:67-165)
//   k_apply       ghost pressure jumps (surf_apply.comp:190-247)
//   k_heat        explicit energy-form conduction and in-cell exchange (heat.comp:81-198)
//   k_visc_*      explicit viscosity u -= M^-1 G^T W G u (visc_setup.comp, visc_apply.comp)
//   k_rhs         cut-cell matrix, divergence, density-correction RHS (rhs.comp:19-94)
//   k_project     pressure gradient, correction velocity, fastest face (project.comp:197-229)
// All of these are bandwidth-bound stencils: float4 loads of the per-cell records.
#include <cuda_runtime.h>

#include "dev_common.cuh"
#include "kernels.h"

namespace sprout {

#define CELL_XY                                            \
    const int cx = blockIdx.x * 16 + threadIdx.x;          \
    const int cy = blockIdx.y * 16 + threadIdx.y;          \
    const int W = d.W, H = d.H;                            \
    (void)H

DEV bool packed(const DevScene& d, int i) {
    float4 sol = __ldg(&d.solid[i]);
    float phi_f = (float)d.acc[i * d.stride + 4] / MASS_SCALE * d.P->inv_ppc;
    return sol.w > 0.02f && phi_f > 0.04f && phi_f + sol.z > LIQUID_THR;
}

__global__ void __launch_bounds__(256) k_grid_prep(DevScene d) {
    CELL_XY;
    const DevParams* P = d.P;
    const DevMat* mats = d.mats;
    uint32_t air_bits = 0u;
    if (cx < W && cy < H) {
        const int i = cy * W + cx;
        const int k = i * d.stride;
        const int um = d.acc[k], umom = d.acc[k + 1], vm = d.acc[k + 2], vmom = d.acc[k + 3];
        const int cw = d.acc[k + 4];
        const float4 sol = __ldg(&d.solid[i]);
        const float dt = d.S->dt;
        float4 o = make_float4(0.0f, 0.0f, FACE_EMPTY, FACE_EMPTY);
        if (sol.x <= 0.0f) o.z = FACE_CLOSED;
        else if (um >= MIN_FACE_MASS) {
            o.x = ((float)umom / MOM_SCALE) / ((float)um / MASS_SCALE) / dt;
            o.z = 0.0f;
        }
        if (sol.y <= 0.0f) o.w = FACE_CLOSED;
        else if (vm >= MIN_FACE_MASS) {
            o.y = ((float)vmom / MOM_SCALE) / ((float)vm / MASS_SCALE) / dt - P->gravity * dt;
            o.w = 0.0f;
        }
        d.vel[i] = o;
        d.vel0[i] = make_float2(o.x, o.y);
        const float phi_f = (float)cw / MASS_SCALE * P->inv_ppc;
        float f[kGroups] = {0.0f, 0.0f, 0.0f, 0.0f}, rg[kGroups] = {0.0f, 0.0f, 0.0f, 0.0f}, lg[kGroups] = {0.0f, 0.0f, 0.0f, 0.0f};
        float sigma = 0.0f, contx = 0.0f, conty = 0.0f, fam0 = -1.0f;
        float4 nn = make_float4(0.0f, -1.0f, 1.0f, 0.0f);   // the cell's non-Newtonian liquid: share, row, concentration, stiff
        float chi = 0.0f;   // the cell's liquid's susceptibility (share-weighted)
        float rho = 0.0f, mu = 0.0f, rho_c = 0.0f, nu_c = 0.0f;
        const bool thermal = P->thermal != 0;
        float T = P->heat[0], kappa = 0.0f, emis = 0.0f, frozen = 0.0f, Craw = 0.0f;
        int major = 0, top_row = -1;
        float top_share = 0.0f;
        const int nmix = P->n_fam - 1;
        for (int q = 0; q < nmix; q++) d.mixb[(size_t)i * nmix + q] = -1.0f;
        float bg[3] = {0.0f, 0.0f, 0.0f};   // share x base density of groups 1 - 3
        const bool settle = (P->caps & CAP_SETTLE) != 0u;
        if (settle)
            for (int q = 0; q < P->n_fam; q++) d.famocc[(size_t)i * P->n_fam + q] = 0.0f;
        if (cw > 0) {
            int others = 0;
            for (int j = 0; j < P->n_present; j++) {
                int ch = mats[P->present[j]].ia[2];
                if (ch >= 0) others += d.acc[k + ch];
            }
            float sh[kMaxPresent], scn[kMaxPresent];
            float Csh = 0.0f;
            float Cg[kGroups] = {0.0f, 0.0f, 0.0f, 0.0f};
            for (int j = 0; j < P->n_present; j++) {
                sh[j] = 0.0f;
                scn[j] = 1.0f;
                const int r = P->present[j];
                const int* ia = mats[r].ia;
                if (ia[2] < 0 && P->primary >= 0 && r != P->primary) continue;
                int wgt = ia[2] >= 0 ? d.acc[k + ia[2]] : max(cw - others, 0);
                if (wgt <= 0) continue;
                sh[j] = wgt >= cw ? 1.0f : clampf((float)wgt / (float)cw, 0.0f, 1.0f);
                if (ia[1] >= 0 && ia[3] >= 0) scn[j] = clampf((float)d.acc[k + ia[3]] / (float)wgt, 0.0f, 1.0f);
                if (thermal) {
                    float cr = sh[j] * thermal_of(mats, (uint32_t)r, scn[j]).w;
                    Csh += cr;
                    Cg[ia[0]] += cr;
                    float kp = mats[r].th[1];
                    kappa += sh[j] * (ia[1] >= 0 ? mixf(mats[ia[1]].th[1], kp, scn[j]) : kp);
                    float em = mats[r].th2[1];
                    emis += sh[j] * (ia[1] >= 0 ? mixf(mats[ia[1]].th2[1], em, scn[j]) : em);
                }
            }
            // the temperature of each phase group present (common.glsl:610-629)
            float Tg[kGroups] = {T, T, T, T};
            if (thermal && Csh > 0.0f) {
                int Htot = d.acc[k + (int)P->heat2[2]];
                T = (float)Htot * T_SCALE / (Csh * (float)cw) - 273.15f;
                for (int g = 0; g < kGroups; g++) Tg[g] = T;
                int rest = Htot, first = -1;
                for (int g = 0; g < kGroups; g++) {
                    int ch = group_heat_chan(P, g);
                    if (ch >= 0) {
                        int hh = d.acc[k + ch];
                        rest -= hh;
                        if (Cg[g] > 0.0f) Tg[g] = (float)hh * T_SCALE / (Cg[g] * (float)cw) - 273.15f;
                    } else if (first < 0 && (P->group_mask & (1u << (uint32_t)g)) != 0u) {
                        first = g;
                    }
                }
                if (first >= 0 && Cg[first] > 0.0f) Tg[first] = (float)rest * T_SCALE / (Cg[first] * (float)cw) - 273.15f;
            }
            for (int j = 0; j < P->n_present; j++) {
                const float share = sh[j];
                if (share <= 0.0f) continue;
                const int r = P->present[j];
                const int* ia = mats[r].ia;
                const float sc = scn[j];
                const float* ma = mats[r].a;
                float rho_m = ma[0], lnu = ma[1], sig = ma[2];
                const float Tm = Tg[ia[0]];
                if (thermal) lnu += temp_law(mats, r, Tm);
                const float xp = thermal ? expansion_of(mats, (uint32_t)r, sc, Tm) : 1.0f;
                float csx = mats[r].b[0], csy = mats[r].b[1];
                if (ia[1] >= 0) {
                    const float* da = mats[ia[1]].a;
                    rho_m = mixf(da[0], rho_m, sc);
                    // blend_share(s, e) = s: every concentrate here blends with exponent 1
                    lnu = mixf(thermal ? da[1] + temp_law(mats, ia[1], Tm) : da[1], lnu, sc);
                    sig = mixf(da[2], sig, sc);
                    csx = mixf(mats[ia[1]].b[0], csx, sc);
                    csy = mixf(mats[ia[1]].b[1], csy, sc);
                    const int fam = mats[r].ib[0];
                    if (fam == 0) fam0 = sc;
                    else if (fam > 0) d.mixb[(size_t)i * nmix + fam - 1] = sc;
                    if (settle && fam >= 0) d.famocc[(size_t)i * P->n_fam + fam] = share * phi_f;
                }
                rho_m *= xp;
                if (thermal) {
                    float4 th = thermal_of(mats, (uint32_t)r, sc);
                    float fs = th.y > -1e8f ? clampf((th.y - Tm) / maxf(th.y - th.x, 1e-3f), 0.0f, 1.0f) : 0.0f;
                    if (fs > 0.0f) {
                        lnu = mixf(lnu, maxf(lnu, P->heat2[0]), fs);
                        float rs = mats[r].b[3];
                        rho_m = mixf(rho_m, ia[1] >= 0 ? mixf(mats[ia[1]].b[3], rs, sc) : rs, fs);
                        frozen += share * fs;
                    }
                }
                if ((mats[r].ib[1] != 0 || mats[r].temp[3] > 0.0f || mats[r].gr[0] > 0.0f) && share > nn.x)
                    nn = make_float4(share, (float)r, sc, 0.0f);
                if (r != 57 && share > top_share) {
                    top_share = share;
                    top_row = r;
                }
                chi += share * mats[r].el[2];
                const int g = ia[0];
                if (g > 0) bg[g - 1] += share * ma[0];
                f[g] += share;
                rg[g] += share * rho_m;
                lg[g] += share * lnu;
                sigma += share * sig;
                contx += share * csx;
                conty += share * csy;
            }
            for (int g = 0; g < kGroups; g++) {
                if (f[g] <= 0.0f) continue;
                rho += rg[g];
                mu += rg[g] * sp_expf(lg[g] / f[g]);
                if (f[g] > f[major]) major = g;
            }
            if (f[major] > 0.0f) {
                rho_c = rg[major] / f[major];
                nu_c = sp_expf(lg[major] / f[major]);
            }
            Craw = Csh * (float)cw / MASS_SCALE;
        }
        const float phi_t = phi_f + sol.z;
        const bool has = phi_f > 0.04f && sol.w > 0.02f;
        float level = has ? phi_t - LIQUID_THR : -LIQUID_THR;
        if (has && level <= 0.0f && cx > 0 && cy > 0 && cx < W - 1 && cy < H - 1) {
            if ((packed(d, i - 1) && packed(d, i + 1)) || (packed(d, i - W) && packed(d, i + W))) level = 0.05f;
            else if (P->gravity > 0.0f && nn.x <= 0.0f && phi_t > 0.25f && packed(d, i - W)) level = 0.05f;
            else if ((P->caps & CAP_MAGNET) != 0u && nn.x <= 0.0f && phi_t > 0.25f && chi > 0.0f) {
                // with a magnet, lying on is towards gravity and the field's pull together
                // (grid_prep.comp:216-220, from the last substep's energy)
                const float km = chi / P->mag[1] / maxf(rho, 0.05f);
                const float pk = -km * 0.5f;
                const float pxl = pk * (d.magc[i + 1].y - d.magc[i - 1].y) - 0.0f;
                const float pyl = pk * (d.magc[i + W].y - d.magc[i - W].y) - P->gravity;
                const int toward = fabsf(pxl) > fabsf(pyl) ? (pxl > 0.0f ? i + 1 : i - 1) : (pyl > 0.0f ? i + W : i - W);
                if (packed(d, toward)) level = 0.05f;
            }
        }
        if (sol.w > 0.0f && level <= 0.0f) air_bits = 1u << (__ldg(&d.region[i]) & REGION_MASK);
        if ((P->caps & (CAP_RIGID | CAP_RHEO)) != 0u) {
            // the viscosity solve stops at rigid_viscosity; a cell that would need more is stiff
            const float cap = rho * sp_expf(P->heat2[0]);
            if (mu >= cap && level > 0.0f) nn.w = 1.0f;
            mu = minf(mu, cap);
            d.rh[i] = nn;
        }
        if ((P->caps & CAP_MAGNET) != 0u) d.magc[i].x = chi;
        if ((P->caps & CAP_ELASTIC) != 0u) {   // the deposited stress (grid_prep.comp:241-244)
            const int ce = (int)P->elastic[0];
            const float sc = P->elastic[1] * P->inv_ppc / 65536.0f;
            d.estr[i] = make_float4((float)d.acc[k + ce] * sc, (float)d.acc[k + ce + 1] * sc, (float)d.acc[k + ce + 2] * sc, 0.0f * sc);
        }
        d.cell[i] = make_float4(phi_f, rho, mu, level);
        d.comp[i] = make_float4(rho, f[1], fam0, phi_t);
        if (P->sorts != 0u) d.gbase[i] = make_float4(bg[0], bg[1], bg[2], 0.0f);
        if ((P->group_mask & (P->group_mask - 1u)) != 0u) {
            d.aux[i] = make_float4(nu_c, rho_c, f[2], f[3]);
            d.grho[i] = make_float4(rg[0], rg[1], rg[2], rg[3]);
        }
        d.sprop[i] = make_float4(sigma, contx, conty, (float)major + (float)(top_row + 1) / 128.0f);
        if (thermal) {
            d.therm[i] = make_float4(T, Craw, kappa, frozen);
            d.dheat[i] = make_float4(P->heat[1] > 0.0f ? emis : 0.0f, 0.0f, 0.0f, 0.0f);
        }
        if (level <= 0.0f) d.pres[i] = make_float2(0.0f, 0.0f);
    }
    air_bits = __reduce_or_sync(0xffffffffu, air_bits);
    if ((threadIdx.x & 31) == 0 && air_bits != 0u) atomicOr(&d.S->region_air, air_bits);
}

DEV void coef_face(float4 a, float4 b, float open, float& g, float& rho) {
    float wsum = a.x + b.x;
    rho = wsum > 1e-6f ? (a.x * a.y + b.x * b.y) / wsum : 1.0f;
    g = 0.0f;
    bool fa = a.w > 0.0f, fb = b.w > 0.0f;
    if (open <= 0.0f || !(fa || fb)) return;
    float theta = 1.0f;
    if (fa != fb) {
        float lf = fa ? a.w : b.w;
        float la = fa ? b.w : a.w;
        theta = clampf(lf / (lf - la), THETA_MIN, 1.0f);
    }
    g = 1.0f / (maxf(rho, 0.05f) * theta);
}

// Face coefficients and the smoothed indicators, both from the cells of grid_prep.
__global__ void __launch_bounds__(256) k_coef_smooth(DevScene d) {
    CELL_XY;
    if (cx >= W || cy >= H) return;
    const int i = cy * W + cx;
    const DevParams* P = d.P;
    float4 o = make_float4(0.0f, 0.0f, 1.0f, 1.0f);
    if (cx > 0 && cy > 0) {
        float4 me = d.cell[i];
        float4 sol = __ldg(&d.solid[i]);
        coef_face(me, d.cell[i - 1], sol.x, o.x, o.z);
        coef_face(me, d.cell[i - W], sol.y, o.y, o.w);
    }
    d.coef[i] = o;
    const float B5[5] = {1.0f, 4.0f, 6.0f, 4.0f, 1.0f};
    const bool more = (P->group_mask & 12u) != 0u;
    float sx = 0.0f, sy = 0.0f, s2x = 0.0f, s2y = 0.0f, wsum = 0.0f;
#pragma unroll
    for (int b = -2; b <= 2; b++)
#pragma unroll
        for (int a = -2; a <= 2; a++) {
            int nx = cx + a, ny = cy + b;
            if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
            int j = ny * W + nx;
            float open = __ldg(&d.solid[j]).w;
            if (open <= 0.02f) continue;
            float phi = clampf(d.cell[j].x / (REST_PHI * open), 0.0f, 1.0f);
            float w = B5[a + 2] * B5[b + 2];
            sx += w * phi;
            sy += w * (phi * d.comp[j].y);
            if (more) {
                float4 ax = d.aux[j];
                s2x += w * phi * ax.z;
                s2y += w * phi * ax.w;
            }
            wsum += w;
        }
    float2* surf_xy = reinterpret_cast<float2*>(d.surf);
    surf_xy[2 * i] = make_float2(wsum > 0.0f ? sx / wsum : 0.0f, wsum > 0.0f ? sy / wsum : 0.0f);
    if (more) {
        float2* s2 = reinterpret_cast<float2*>(d.surf2);
        s2[2 * i] = make_float2(wsum > 0.0f ? s2x / wsum : 0.0f, wsum > 0.0f ? s2y / wsum : 0.0f);
    }
}

DEV float surf_field(const DevScene& d, int x, int y, int k) {
    x = clampi(x, 0, d.W - 1);
    y = clampi(y, 0, d.H - 1);
    int i = y * d.W + x;
    const float2* sxy = reinterpret_cast<const float2*>(k < 2 ? d.surf : d.surf2);
    float2 v = sxy[2 * i];
    return (k == 0 || k == 2) ? v.x : v.y;
}

DEV float node_sdf(const DevScene& d, int x, int y) {
    x = clampi(x, 0, d.W);
    y = clampi(y, 0, d.H);
    return __ldg(&d.sdf[y * (d.W + 1) + x]);
}

DEV float2 contact_at(const DevScene& d, int nx, int ny) {
    int i0 = clampi(ny, 0, d.H - 1) * d.W + clampi(nx, 0, d.W - 1);
    float4 sp = d.sprop[i0];
    float csx = sp.y, csy = sp.z;
    if (csx * csx + csy * csy > 1e-12f) {
        float l = len2(csx, csy);
        return make_float2(csx / l, csy / l);
    }
    for (int b = -3; b <= 2; b++)
        for (int a = -3; a <= 2; a++) {
            int j = clampi(ny + b, 0, d.H - 1) * d.W + clampi(nx + a, 0, d.W - 1);
            float4 q = d.sprop[j];
            float cxv = d.cell[j].x;
            csx += q.y * cxv;
            csy += q.z * cxv;
        }
    if (csx * csx + csy * csy > 1e-12f) {
        float l = len2(csx, csy);
        return make_float2(csx / l, csy / l);
    }
    return make_float2(0.0f, 1.0f);
}

DEV float2 normal_node(const DevScene& d, int nx, int ny, int k, float& mag) {
    const float G_MIN = 0.05f, WALL_BAND = 0.5f;
    float a = surf_field(d, nx, ny, k), b = surf_field(d, nx - 1, ny, k), dd = surf_field(d, nx, ny - 1, k),
          e = surf_field(d, nx - 1, ny - 1, k);
    float gx = 0.5f * (a + dd - b - e), gy = 0.5f * (a + b - dd - e);
    mag = len2(gx, gy);
    if (mag < G_MIN) return make_float2(0.0f, 0.0f);
    float nnx = -gx / mag, nny = -gy / mag;
    if (k == 0) {
        float sd = node_sdf(d, nx, ny);
        if (sd < WALL_BAND) {
            float gwx = node_sdf(d, nx + 1, ny) - node_sdf(d, nx - 1, ny);
            float gwy = node_sdf(d, nx, ny + 1) - node_sdf(d, nx, ny - 1);
            if (len2(gwx, gwy) > 1e-4f) {
                float lw = len2(gwx, gwy);
                float nwx = gwx / lw, nwy = gwy / lw;
                float gd = gx * nwx + gy * nwy;
                float gtx = gx - gd * nwx, gty = gy - gd * nwy;
                float along = len2(gtx, gty);
                if (along > 0.5f * G_MIN) {
                    float tx = -gtx / along, ty = -gty / along;
                    float2 cs = contact_at(d, nx, ny);
                    float ncx = cs.x * nwx + cs.y * tx, ncy = cs.x * nwy + cs.y * ty;
                    float sm = smoothstepf(0.5f * G_MIN, G_MIN, along);
                    float mx = mixf(nnx, ncx, sm), my = mixf(nny, ncy, sm);
                    float lm = len2(mx, my);
                    if (lm > 1e-4f) {
                        nnx = mx / lm;
                        nny = my / lm;
                    } else {
                        nnx = ncx;
                        nny = ncy;
                    }
                }
            }
        }
    }
    return make_float2(nnx, nny);
}

DEV float curvature_at(const DevScene& d, int cx, int cy, int k, float kmax) {
    float m00, m10, m01, m11;
    float2 n00 = normal_node(d, cx, cy, k, m00);
    float2 n10 = normal_node(d, cx + 1, cy, k, m10);
    float2 n01 = normal_node(d, cx, cy + 1, k, m01);
    float2 n11 = normal_node(d, cx + 1, cy + 1, k, m11);
    if (0.25f * (m00 + m10 + m01 + m11) < 0.05f) return 0.0f;
    float kap = 0.5f * (n10.x + n11.x - n00.x - n01.x) + 0.5f * (n01.y + n11.y - n00.y - n10.y);
    return kmax > 0.0f ? clampf(kap, -kmax, kmax) : kap;
}

__global__ void __launch_bounds__(256) k_curv(DevScene d) {
    CELL_XY;
    if (cx >= W || cy >= H) return;
    const int i = cy * W + cx;
    const DevParams* P = d.P;
    float kmax = P->misc[0];
    float k0 = curvature_at(d, cx, cy, 0, kmax);
    float k1 = curvature_at(d, cx, cy, 1, kmax);
    float2* szw = reinterpret_cast<float2*>(d.surf);
    szw[2 * i + 1] = make_float2(k0, k1);
    if ((P->group_mask & 12u) != 0u) {
        float2* s2 = reinterpret_cast<float2*>(d.surf2);
        s2[2 * i + 1] = make_float2((P->group_mask & 4u) != 0u ? curvature_at(d, cx, cy, 2, kmax) : 0.0f,
                                    (P->group_mask & 8u) != 0u ? curvature_at(d, cx, cy, 3, kmax) : 0.0f);
    }
}

DEV float air_jump(const DevScene& d, int a, int b) {
    bool la = d.cell[a].w > 0.0f;
    int liq = la ? a : b, air = la ? b : a;
    float lf = d.cell[liq].w, lgv = d.cell[air].w;
    float theta = clampf(lf / (lf - lgv), THETA_MIN, 1.0f);
    float kl = d.surf[liq].z, kg = d.surf[air].z;
    float kap = kg != 0.0f ? mixf(kl, kg, theta) : kl;
    return d.S->dt * d.sprop[liq].x * kap;
}

DEV float share_of(const DevScene& d, int i, int g) {
    if (g == 1) return d.comp[i].y;
    if (g == 2) return d.aux[i].z;
    if (g == 3) return d.aux[i].w;
    return 1.0f - d.comp[i].y - d.aux[i].z - d.aux[i].w;
}

DEV float curv_of(const DevScene& d, int i, int g) { return g == 1 ? d.surf[i].w : g == 2 ? d.surf2[i].z : d.surf2[i].w; }

DEV float pair_jump(const DevScene& d, int c, int n) {
    int gc = (int)d.sprop[c].w, gn = (int)d.sprop[n].w;
    if (gc == gn) return 0.0f;
    int hi = max(gc, gn), lo = min(gc, gn);
    float dc = share_of(d, c, hi) - share_of(d, c, lo), dn = share_of(d, n, hi) - share_of(d, n, lo);
    if (dc * dn >= 0.0f) return 0.0f;
    float theta = -dn / (dc - dn);
    float kc = curv_of(d, c, hi), kn = curv_of(d, n, hi);
    float kap = kc == 0.0f ? kn : kn == 0.0f ? kc : mixf(kn, kc, theta);
    float j = d.S->dt * d.P->pair[hi][lo] * kap;
    return gc == hi ? j : -j;
}

DEV float face_jump(const DevScene& d, int c, int n, float open) {
    if (open <= 0.0f) return 0.0f;
    bool lc = d.cell[c].w > 0.0f, ln = d.cell[n].w > 0.0f;
    if (lc != ln) return air_jump(d, c, n);
    if (lc && ln) return pair_jump(d, c, n);
    return 0.0f;
}

__global__ void __launch_bounds__(256) k_apply(DevScene d) {
    CELL_XY;
    if (cx >= W || cy >= H) return;
    const int i = cy * W + cx;
    float2 pj = make_float2(0.0f, 0.0f);
    if (cx > 0 && cy > 0) {
        float4 sol = __ldg(&d.solid[i]);
        pj.x = face_jump(d, i, i - 1, sol.x);
        pj.y = face_jump(d, i, i - W, sol.y);
    }
    d.pjump[i] = pj;
}

// ---- heat ----------------------------------------------------------------------------

DEV float y_sat(float T) {
    T = clampf(T, -40.0f, 99.0f);
    float p = 0.61078f * sp_expf(17.27f * T / (T + 237.3f));
    return 0.622f * p / (101.325f - 0.378f * p);
}

DEV float2 centre_vel(const DevScene& d, int i) {
    int last = d.W * d.H - 1;
    float4 v = d.vel[i], vr = d.vel[min(i + 1, last)], vt = d.vel[min(i + d.W, last)];
    float ax = face_live(v.z) ? v.x : 0.0f, ay = face_live(v.w) ? v.y : 0.0f;
    float bx = face_live(vr.z) ? vr.x : 0.0f, by = face_live(vt.w) ? vt.y : 0.0f;
    return make_float2(0.5f * (ax + bx), 0.5f * (ay + by));
}

DEV int lead_of(float w) {
    float fr = w - floorf(w);
    return (int)(fr * 128.0f + 0.5f);
}

__global__ void __launch_bounds__(256) k_heat(DevScene d) {
    CELL_XY;
    if (cx >= W || cy >= H) return;
    const int i = cy * W + cx;
    const DevParams* P = d.P;
    const DevMat* mats = d.mats;
    float4 me = d.therm[i];
    float emis = d.dheat[i].x;
    float phi = d.cell[i].x;
    float k = d.S->dt * P->heat[1];
    int2 hsum = d.hcell[i];
    float ownx = 0.0f, owny = 0.0f;
    if (hsum.x > 0 && me.y > 0.0f && phi > 0.0f) {
        float rate = 5.78f * me.z * 3.14159265f / (P->inv_ppc * me.y * P->inv_ppc / phi);
        ownx = 1.0f - sp_expf(-k * rate);
        owny = (float)hsum.y / (float)hsum.x;
    }
    if (phi <= 0.04f || me.y <= 0.0f || cx < 1 || cy < 1 || cx >= W - 1 || cy >= H - 1) {
        d.dheat[i] = make_float4(0.0f, ownx, owny, 0.0f);
        return;
    }
    phi = minf(phi, 1.0f);
    const int nb[4] = {i - 1, i + 1, i - W, i + W};
    const float open[4] = {d.solid[i].x, d.solid[i + 1].x, d.solid[i].y, d.solid[i + W].y};
    float Tk = me.x + 273.15f, Ta = P->heat[0] + 273.15f;
    float cond = 0.0f, air = 0.0f, wall = 0.0f, contact = 0.0f;
    float cpc = me.y * P->inv_ppc;
    float hc = P->heat2[3];
    int lead = lead_of(d.sprop[i].w);
    float eddy_l2 = P->heat3[0] * P->heat3[0] / 0.85f;
    bool eddy = eddy_l2 > 0.0f && me.w < 0.5f;
    float2 u_me = eddy ? centre_vel(d, i) : make_float2(0.0f, 0.0f);
    float eddy_max = 0.2f / maxf(k, 1e-9f);
    float per_rate = 1.0f / maxf(P->heat[1], 1e-6f);
    float evap = 0.0f;
    for (int q = 0; q < 4; q++) {
        int n = nb[q];
        float a = open[q];
        float pn = d.cell[n].x;
        float4 o = d.therm[n];
        if (a > 0.0f) {
            float pl = (pn > 0.04f && o.y > 0.0f) ? minf(pn, 1.0f) : 0.0f;
            if (pl > 0.0f) {
                float gc = 2.0f * me.z * o.z / maxf(me.z + o.z, 1e-12f);
                if (eddy && o.w < 0.5f && lead_of(d.sprop[n].w) == lead) {
                    float2 cn = centre_vel(d, n);
                    float strain = 1.4142f * len2(cn.x - u_me.x, cn.y - u_me.y);
                    float alpha = minf(eddy_l2 * strain * per_rate, eddy_max);
                    float c1 = cpc / phi, c2 = o.y * P->inv_ppc / pl;
                    gc += alpha * 2.0f * c1 * c2 / maxf(c1 + c2, 1e-12f);
                }
                cond += a * minf(phi, pl) * gc * (o.x - me.x);
                if (hc > 0.0f && lead_of(d.sprop[n].w) != lead) {
                    float g1 = maxf(2.0f * me.z, hc), g2 = maxf(2.0f * o.z, hc);
                    float gx = maxf(g1 * g2 / (g1 + g2) - gc, 0.0f) * a * minf(phi, pl);
                    float cn = o.y * P->inv_ppc;
                    float x = gx * k * (1.0f / cpc + 1.0f / cn);
                    contact += 0.25f * (1.0f - sp_expf(-4.0f * x)) * cpc * cn / (cpc + cn) * (o.x - me.x);
                }
            }
            float exposed = maxf(phi - pl, 0.0f);
            if (exposed > 0.0f && d.solid[n].w > 0.02f) {
                float hh = P->heat[2] + emis * P->heat[3] * (Ta * Ta + Tk * Tk) * (Ta + Tk);
                air += a * exposed * hh * (P->heat[0] - me.x);
                if (P->heat3[1] > 0.0f && lead > 0 && mats[lead - 1].ia[0] == 0 && mats[lead - 1].th2[2] < 150.0f && me.w < 0.5f)
                    evap += a * exposed * P->heat[2] * P->heat3[1] * maxf(y_sat(me.x) - y_sat(P->heat[0]), 0.0f);
            }
        }
        if (a < 1.0f) {
            float ts = maxf(d.solid_t[n], d.solid_t[i]);
            if (ts > 0.5f * NO_TEMP) wall += (1.0f - a) * phi * 2.0f * me.z * (ts - me.x);
        }
    }
    if (evap > 0.0f) air -= evap;
    air *= k;
    wall *= k;
    float lim = cpc * fabsf(P->heat[0] - me.x);
    air = clampf(air, -lim, lim);
    float e = k * cond + contact + air + wall;
    d.dheat[i] = make_float4(e / cpc, ownx, owny, 0.0f);
    if (air > 0.0f) ledger_add(d.ledger, 0, air); else ledger_add(d.ledger, 1, -air);
    if (wall > 0.0f) ledger_add(d.ledger, 2, wall); else ledger_add(d.ledger, 3, -wall);
}

// ---- explicit viscosity ----------------------------------------------------------------

DEV bool live_u(const DevScene& d, int i) { return face_live(d.vel[i].z); }
DEV bool live_v(const DevScene& d, int i) { return face_live(d.vel[i].w); }
DEV bool closed_u(const DevScene& d, int i) { return face_closed(d.vel[i].z); }
DEV bool closed_v(const DevScene& d, int i) { return face_closed(d.vel[i].w); }
DEV float vel_u(const DevScene& d, int i) { float4 v = d.vel[i]; return face_live(v.z) ? v.x : 0.0f; }
DEV float vel_v(const DevScene& d, int i) { float4 v = d.vel[i]; return face_live(v.w) ? v.y : 0.0f; }

__global__ void __launch_bounds__(256) k_visc_setup(DevScene d) {
    CELL_XY;
    if (cx >= W || cy >= H) return;
    const int i = cy * W + cx;
    const float dt = d.S->dt;
    float wc = 0.0f, wn = 0.0f;
    if (cx >= 1 && cy >= 1 && cx < W - 1 && cy < H - 1) {
        float4 me = d.cell[i];
        auto ok_u = [&](int j) { float z = d.vel[j].z; return face_live(z) || face_closed(z); };
        auto ok_v = [&](int j) { float w = d.vel[j].w; return face_live(w) || face_closed(w); };
        if (me.w > 0.0f && ok_u(i) && ok_u(i + 1) && ok_v(i) && ok_v(i + W)) wc = 2.0f * dt * me.z;
        const int cs[4] = {i - W - 1, i - W, i - 1, i};
        int nliq = 0;
        bool any_air = false;
        float mu = 0.0f;
        for (int k = 0; k < 4; k++) {
            float4 q = d.cell[cs[k]];
            if (q.w > 0.0f) {
                nliq++;
                mu += q.z;
            } else if (__ldg(&d.solid[cs[k]]).w > 0.02f) {
                any_air = true;
            }
        }
        if (nliq > 0 && !any_air && ok_u(i) && ok_u(i - W) && ok_v(i) && ok_v(i - 1))
            wn = 4.0f * dt * (mu / (float)nliq) * ((float)nliq / 4.0f);
    }
    float4 w = d.vw[i];
    w.x = wc;
    w.y = wn;
    d.vw[i] = w;
    float4 o = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (wc > 0.0f) {
        o.x = wc * (vel_u(d, i + 1) - vel_u(d, i));
        o.y = wc * (vel_v(d, i + W) - vel_v(d, i));
    }
    if (wn > 0.0f) {
        float ua = vel_u(d, i), ub = vel_u(d, i - W), va = vel_v(d, i), vb = vel_v(d, i - 1);
        if (closed_u(d, i) && live_u(d, i - W)) ua = -ub;
        if (closed_u(d, i - W) && live_u(d, i)) ub = -ua;
        if (closed_v(d, i) && live_v(d, i - 1)) va = -vb;
        if (closed_v(d, i - 1) && live_v(d, i)) vb = -va;
        o.z = wn * 0.5f * ((ua - ub) + (va - vb));
    }
    d.vs[i] = o;
    // the tiles that need the implicit solve: within one cell of a cell whose diffusion
    // number reaches implicit_viscosity_min (visc_setup.comp:49-56)
    if (d.P->visc_mode == 2) {
        const float4 me = d.cell[i];
        if (me.w > 0.0f && dt * me.z / maxf(me.y, 0.05f) >= d.P->corr[3]) {
            const int tw = (W + 15) >> 4;
            for (int b = -1; b <= 1; b++)
                for (int a = -1; a <= 1; a++) {
                    const int nx = clampi(cx + a, 0, W - 1), ny = clampi(cy + b, 0, H - 1);
                    const int t = (ny >> 4) * tw + (nx >> 4);
                    if (d.tiles[t] == 0u) atomicOr(&d.tiles[t], 1u);
                }
        }
    }
}

__global__ void __launch_bounds__(256) k_visc_explicit(DevScene d) {
    CELL_XY;
    if (cx < 1 || cy < 1 || cx >= W - 1 || cy >= H - 1) return;
    const int i = cy * W + cx;
    float4 v = d.vel[i];
    float gx = 0.0f, gy = 0.0f;
    bool lu = face_live(v.z), lv = face_live(v.w);
    if (lu) {
        float c1 = closed_u(d, i - W) ? 1.0f : 0.5f, c2 = closed_u(d, i + W) ? -1.0f : -0.5f;
        gx = d.vs[i - 1].x - d.vs[i].x + d.vs[i].z * c1 + d.vs[i + W].z * c2;
    }
    if (lv) {
        float d1 = closed_v(d, i - 1) ? 1.0f : 0.5f, d2 = closed_v(d, i + 1) ? -1.0f : -0.5f;
        gy = d.vs[i - W].y - d.vs[i].y + d.vs[i].z * d1 + d.vs[i + 1].z * d2;
    }
    float4 cf = d.coef[i];
    if (lu) v.x -= gx / cf.z;
    if (lv) v.y -= gy / cf.w;
    float2* vxy = reinterpret_cast<float2*>(d.vel);
    vxy[2 * i] = make_float2(v.x, v.y);
}

// ---- pressure system ---------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_rhs(DevScene d) {
    CELL_XY;
    const DevParams* P = d.P;
    bool mark = false;
    if (cx < W && cy < H) {
        const int i = cy * W + cx;
        float4 me = d.cell[i];
        if (me.w <= 0.0f || cx == 0 || cy == 0 || cx == W - 1 || cy == H - 1) {
            d.mga[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            d.mgd[i] = 0.0f;
            d.prhs[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else {
            const StepState* S = d.S;
            float dt = S->dt;
            float4 sol = __ldg(&d.solid[i]);
            float4 cf = d.coef[i];
            float aL = sol.x, aB = sol.y, aR = __ldg(&d.solid[i + 1]).x, aT = __ldg(&d.solid[i + W]).y;
            float4 w = make_float4(aL * cf.x, aR * d.coef[i + 1].x, aB * cf.y, aT * d.coef[i + W].y);
            float diag = w.x + w.y + w.z + w.w;
            uint32_t rg = __ldg(&d.region[i]);
            uint32_t rair = S->region_air;
            if ((rg & REGION_VENT) != 0u && (rair & (1u << (rg & REGION_MASK))) == 0u && P->misc[1] > 0.0f)
                diag += 1.0f / maxf(me.y, 0.05f);
            float4 vme = d.vel[i];
            float div = aR * d.vel[i + 1].x - aL * vme.x + aT * d.vel[i + W].y - aB * vme.y;
            bool lR = d.cell[i + 1].w > 0.0f, lT = d.cell[i + W].w > 0.0f;
            bool lL = d.cell[i - 1].w > 0.0f, lB = d.cell[i - W].w > 0.0f;
            float2 pjm = d.pjump[i];
            float pjr = d.pjump[i + 1].x, pjt = d.pjump[i + W].y;
            float jump = w.x * pjm.x + w.y * (lR ? -pjr : pjr) + w.z * pjm.y + w.w * (lT ? -pjt : pjt);
            float err = clampf(d.comp[i].w - REST_PHI, -0.5f, 0.5f);
            {
                bool interior = (aL <= 0.0f || lL) && (aR <= 0.0f || lR) && (aB <= 0.0f || lB) && (aT <= 0.0f || lT);
                bool pressed = d.pres[i].x * (dt / S->dt_prev) > 0.5f * me.y * P->gravity * dt;
                if (interior && !pressed) err = maxf(err - P->corr[1], 0.0f);
                else if (!interior && err < 0.0f) err = 0.0f;
            }
            float s = S->corr_gain * err;
            if ((rair & (1u << (rg & REGION_MASK))) == 0u && P->misc[1] > 0.0f) s = 0.0f;
            mark = diag > 1e-9f;
            d.mga[i] = mark ? w : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            d.mgd[i] = mark ? diag : 0.0f;
            d.prhs[i] = make_float4(-div + jump, s / dt, 0.0f, 0.0f);
        }
    }
    // the level-0 tile flag of this 16 x 16 tile: non-zero where it holds unknowns
    int any = __syncthreads_or(mark);
    if (threadIdx.x == 0 && threadIdx.y == 0) d.ptile[blockIdx.y * gridDim.x + blockIdx.x] = any ? 1u : 0u;
}

DEV float p_difference(bool lc, bool ln, float pc, float pn, float j) {
    if (lc && ln) return pc - pn - j;
    return (lc ? pc : j) - (ln ? pn : j);
}

__global__ void __launch_bounds__(256) k_project(DevScene d) {
    CELL_XY;
    float m = 0.0f;
    if (cx >= 1 && cy >= 1 && cx < W && cy < H) {
        const int i = cy * W + cx;
        float4 cf = d.coef[i];
        float4 me = d.vel[i];
        if (d.mgd[i] > 0.0f) d.prhs[i].z = d.pres[i].x;
        if (cf.x != 0.0f || cf.y != 0.0f) {
            float2 p = d.pres[i];
            bool liq = d.cell[i].w > 0.0f;
            if (face_live(me.z) && cf.x != 0.0f) {
                int n = i - 1;
                me.x -= cf.x * p_difference(liq, d.cell[n].w > 0.0f, p.x, d.pres[n].x, d.pjump[i].x);
                me.z = -cf.x * (p.y - d.pres[n].y);
            }
            if (face_live(me.w) && cf.y != 0.0f) {
                int n = i - W;
                me.y -= cf.y * p_difference(liq, d.cell[n].w > 0.0f, p.x, d.pres[n].x, d.pjump[i].y);
                me.w = -cf.y * (p.y - d.pres[n].y);
            }
            d.vel[i] = me;
        }
        if (face_live(me.z) && cf.x != 0.0f) m = fabsf(me.x);
        if (face_live(me.w) && cf.y != 0.0f) m = maxf(m, fabsf(me.y));
    }
    report_max(&d.S->umax_grid, m);
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) d.S->gather = 1u;
}

// The shear rate |D| sqrt(2) of cell i from its faces' velocities, gravity's last increment
// taken back out when `pre` (common.glsl:527-540).
DEV float shear_rate(const DevScene& d, int i, bool pre) {
    const int W = d.W;
    const float gv = pre ? d.P->gravity * d.S->dt : 0.0f;
    auto U = [&](int k) { const float4 v = d.vel[k]; return face_live(v.z) ? v.x : 0.0f; };
    auto V = [&](int k) { const float4 v = d.vel[k]; return face_live(v.w) ? v.y + gv : 0.0f; };
    const float dxx = U(i + 1) - U(i);
    const float dyy = V(i + W) - V(i);
    const float duy = 0.25f * (U(i + W) + U(i + 1 + W) - U(i - W) - U(i + 1 - W));
    const float dvx = 0.25f * (V(i + 1) + V(i + 1 + W) - V(i - 1) - V(i - 1 + W));
    const float dxy = 0.5f * (duy + dvx);
    return sqrtf(2.0f * (dxx * dxx + dyy * dyy + 2.0f * dxy * dxy));
}

// The non-Newtonian factor F on the viscosity and the yield stress tau of the cell's liquid q
// (rh: share, row, concentration) at shear rate g: Carreau, Herschel-Bulkley, thickening;
// friction and skin add to tau; both scale with the liquid's share (common.glsl:546-571).
DEV void nn_eval(const DevScene& d, int i, float4 q, float g, float& F, float& tau) {
    const DevMat& m = d.mats[(int)q.y];
    const float* rp = m.rheo;
    const int model = m.ib[1];
    F = 1.0f;
    tau = 0.0f;
    if (model == 1) {
        F = rp[3] + (1.0f - rp[3]) * sp_powf(1.0f + (rp[2] * g) * (rp[2] * g), 0.5f * (rp[1] - 1.0f));
    } else if (model == 2) {
        F = sp_powf(maxf(g, 1e-6f), rp[1] - 1.0f);
        tau = rp[0] * q.z;
    } else if (model == 3) {
        F = minf(sp_powf(1.0f + (rp[2] * g) * (rp[2] * g), 0.5f * (rp[1] - 1.0f)), rp[3]);
    }
    const float fr = m.gr[0];
    if (fr > 0.0f) tau += fr * q.z * q.z * q.z * maxf(d.pres[i].x, 0.0f) / maxf(d.S->dt, 1e-6f);
    const int W = d.W;
    const float skin = m.temp[3];
    if (skin > 0.0f && (d.cell[i - 1].w <= 0.0f || d.cell[i + 1].w <= 0.0f || d.cell[i - W].w <= 0.0f || d.cell[i + W].w <= 0.0f))
        tau += skin;
    F = 1.0f + q.x * (F - 1.0f);
    tau *= q.x;
}

// rheo.comp: the viscosity of a cell holding a non-Newtonian liquid at its shear rate, capped
// at rigid_viscosity; a skinned surface cell too slow to yield turns stiff.
__global__ void __launch_bounds__(256) k_rheo(DevScene d) {
    CELL_XY;
    if (cx < 1 || cy < 1 || cx >= W - 1 || cy >= H - 1) return;
    const int i = cy * W + cx;
    float4 me = d.cell[i];
    float4 q = d.rh[i];
    if (me.w <= 0.0f || q.x <= 0.0f) return;
    const float g = shear_rate(d, i, true);
    float F, tau;
    nn_eval(d, i, q, g, F, tau);
    const float eff = me.z * F + tau / maxf(g, 1e-6f);
    const float cap = me.y * sp_expf(d.P->heat2[0]);
    const float skin = q.x * d.mats[(int)q.y].temp[3];
    if (skin > 0.0f && me.y * g * g < skin &&
        (d.cell[i - 1].w <= 0.0f || d.cell[i + 1].w <= 0.0f || d.cell[i - W].w <= 0.0f || d.cell[i + W].w <= 0.0f)) {
        q.w = 1.0f;
        d.rh[i] = q;
    }
    me.z = minf(eff, cap);
    d.cell[i] = me;
}

// The shear stress at node i (the cell corner at its lower left): the four cells' mean.
DEV float txy_node(const DevScene& d, int i) {
    const int W = d.W;
    return 0.25f * (d.estr[i].z + d.estr[i - 1].z + d.estr[i - W].z + d.estr[i - W - 1].z);
}

// elastic.comp: the divergence of the particles' deposited stress accelerates the faces.
__global__ void __launch_bounds__(256) k_elastic(DevScene d) {
    CELL_XY;
    if (cx >= W - 1 || cy >= H - 1 || cx < 2 || cy < 2) return;
    const int i = cy * W + cx;
    float4 q = d.vel[i];
    const float4 a = d.cell[i], l = d.cell[i - 1], b = d.cell[i - W];
    const float dt = d.S->dt;
    if (face_live(q.z)) {
        const float rho = (a.x * a.y + l.x * l.y) / maxf(a.x + l.x, 1e-6f);
        const float f = (d.estr[i].x - d.estr[i - 1].x) + (txy_node(d, i + W) - txy_node(d, i));
        q.x += dt * f / maxf(rho, 0.05f);
    }
    if (face_live(q.w)) {
        const float rho = (a.x * a.y + b.x * b.y) / maxf(a.x + b.x, 1e-6f);
        const float f = (d.estr[i].y - d.estr[i - W].y) + (txy_node(d, i + 1) - txy_node(d, i));
        q.y += dt * f / maxf(rho, 0.05f);
    }
    d.vel[i] = q;
}

// The settling flux of family f between an upper cell and a lower one at terminal velocity vt:
// concentrate leaving the upper cell into the diluent of the lower one, bounded by what either
// holds (settle.comp:8-16).
DEV float settle_flux(const DevScene& d, int up, int dn, int f, float vt) {
    const int nf = d.P->n_fam;
    const float ou = d.famocc[(size_t)up * nf + f], od = d.famocc[(size_t)dn * nf + f];
    if (ou <= 1e-3f || od <= 1e-3f) return 0.0f;
    const float su = f == 0 ? d.comp[up].z : d.mixb[(size_t)up * (nf - 1) + f - 1];
    const float sd = f == 0 ? d.comp[dn].z : d.mixb[(size_t)dn * (nf - 1) + f - 1];
    if (su <= 0.0f || sd < 0.0f) return 0.0f;
    const float F = vt * su * (1.0f - sd) * minf(ou, od);
    return minf(F, minf(su * ou, (1.0f - sd) * od) / d.S->dt);
}

// settle.comp: per cell and family with grains, the rates at which its particles gain
// concentrate from the cell above (or below, for grains lighter than the diluent) and lose it
// to the next, as fractions of what they can take or give this substep.
__global__ void __launch_bounds__(256) k_settle(DevScene d) {
    CELL_XY;
    if (cx >= W || cy >= H) return;
    const int i = cy * W + cx;
    const DevParams* P = d.P;
    const int nf = P->n_fam;
    const bool thermal = (P->caps & CAP_THERMAL) != 0u;
    for (int f = 0; f < nf; f++) {
        const int row = P->fams[f][0], dl = P->fams[f][1];
        const float gd = d.mats[row].b[2];
        const float occ = d.famocc[(size_t)i * nf + f];
        float2 ds = make_float2(0.0f, 0.0f);
        if (gd > 0.0f && occ > 1e-3f && cy > 0 && cy < H - 1) {
            const float drho = d.mats[row].a[0] - d.mats[dl].a[0];
            const float T = thermal ? d.therm[i].x : P->heat[0];
            // row_lnu of the (plain) diluent at concentration 1
            const float lnu = d.mats[dl].a[1] + (thermal ? temp_law(d.mats, dl, T) : 0.0f);
            const float vt = terminal(drho, d.mats[dl].a[0], sp_expf(lnu), gd, P->gravity);
            const float gain = drho > 0.0f ? settle_flux(d, i + W, i, f, vt) : settle_flux(d, i - W, i, f, vt);
            const float loss = drho > 0.0f ? settle_flux(d, i, i - W, f, vt) : settle_flux(d, i, i + W, f, vt);
            const float sv = f == 0 ? d.comp[i].z : d.mixb[(size_t)i * (nf - 1) + f - 1];
            const float dt = d.S->dt;
            ds = make_float2(dt * (gain / maxf(occ * (1.0f - sv), 1e-6f)), dt * (loss / maxf(occ * sv, 1e-6f)));
        }
        d.dsettle[(size_t)i * nf + f] = ds;
    }
}

// magnet.comp mode 0: the magnetic energy density of pure magnetic liquid in each cell
// (Langevin-like saturation, a demagnetising factor from the liquid's surface).
__global__ void __launch_bounds__(256) k_magnet_energy(DevScene d) {
    CELL_XY;
    if (cx >= W || cy >= H) return;
    const int i = cy * W + cx;
    const DevParams* P = d.P;
    const float MU0 = 1.25663706e-6f;
    const float2 B = magnet_field(P, (float)cx + 0.5f, (float)cy + 0.5f);
    const float Bl = len2(B.x, B.y);
    const float Hf = Bl / MU0;
    float psi = 0.0f;
    const float chi = P->mag[1];
    if (Hf > 0.0f && chi > 0.0f) {
        float N = 1.0f / 3.0f;
        if (P->heat3[3] > 0.0f) {
            float gx = 0.0f, gy = 0.0f;
            if (cx > 0 && cy > 0 && cx < W - 1 && cy < H - 1) {
                gx = 0.5f * (d.surf[i + 1].x - d.surf[i - 1].x);
                gy = 0.5f * (d.surf[i + W].x - d.surf[i - W].x);
            }
            const float gl = len2(gx, gy);
            const float nh = gl > 1e-6f ? (gx / gl) * (B.x / Bl) + (gy / gl) * (B.y / Bl) : 0.0f;
            N = mixf(1.0f / 3.0f, nh * nh, clampf(gl / 0.25f, 0.0f, 1.0f) * P->heat3[3]);
        }
        const float ce = chi / (1.0f + N * chi);
        const float Ms = P->mag[2] / MU0;
        const float xs = ce * Hf / Ms;
        const float f = xs < 0.02f ? xs * xs * (0.5f - xs * (1.0f / 3.0f - 0.25f * xs)) : xs - sp_logf(1.0f + xs);
        psi = -MU0 * Ms * Ms / ce * f * P->mag[3];
    }
    d.magc[i].y = psi;
}

DEV float magnet_face_force(const DevScene& d, int i, int n, float rho) {
    const bool li = d.cell[i].w > 0.0f, ln = d.cell[n].w > 0.0f;
    const float sc = (li == ln ? 0.5f * (d.magc[i].x + d.magc[n].x) : li ? d.magc[i].x : d.magc[n].x) / d.P->mag[1];
    return -d.S->dt * sc * (d.magc[i].y - d.magc[n].y) / maxf(rho, 0.05f);
}

// magnet.comp mode 1: the force of the energy's gradient on the liquid's faces.
__global__ void __launch_bounds__(256) k_magnet_force(DevScene d) {
    CELL_XY;
    if (cx >= W || cy >= H || cx < 1 || cy < 1) return;
    const int i = cy * W + cx;
    float4 me = d.vel[i];
    const float4 cf = d.coef[i];
    if (face_live(me.z) && cf.x != 0.0f) me.x += magnet_face_force(d, i, i - 1, cf.z);
    if (face_live(me.w) && cf.y != 0.0f) me.y += magnet_face_force(d, i, i - W, cf.w);
    d.vel[i] = me;
}

// ---- rigid bodies (rigid.comp) ---------------------------------------------------------
// Whether liquid cell i moves rigidly: frozen, stiff, or a non-Newtonian liquid that has not
// yielded or has jammed (rigid.comp:10-25).
DEV bool cell_rigid(const DevScene& d, int cx, int cy, int i) {
    const float4 me = d.cell[i];
    if (me.w <= 0.0f) return false;
    const DevParams* P = d.P;
    if ((P->caps & CAP_THERMAL) != 0u && d.therm[i].w > 0.5f) return true;
    const float4 q = d.rh[i];
    if (q.w > 0.5f) return true;
    if ((P->caps & CAP_RHEO) == 0u || q.x <= 0.0f || cx < 1 || cy < 1 || cx >= d.W - 1 || cy >= d.H - 1) return false;
    const float g = shear_rate(d, i, false);
    float F, tau;
    nn_eval(d, i, q, g, F, tau);
    if (tau > 0.0f && me.z * g < tau) return true;
    return d.mats[(int)q.y].ib[1] == 3 && me.z * F >= me.y * sp_expf(P->heat2[0]);
}

DEV float rigid_sdf(const DevScene& d, float x, float y, float& gx_out, float& gy_out) {
    const float gx = clampf(x, 0.0f, (float)d.W - 0.001f), gy = clampf(y, 0.0f, (float)d.H - 0.001f);
    const int ix = (int)gx, iy = (int)gy;
    const float fx = gx - (float)ix, fy = gy - (float)iy;
    const int w1 = d.W + 1, k = iy * w1 + ix;
    const float d00 = d.sdf[k], d10 = d.sdf[k + 1], d01 = d.sdf[k + w1], d11 = d.sdf[k + w1 + 1];
    gx_out = mixf(d10 - d00, d11 - d01, fy);
    gy_out = mixf(d01 - d00, d11 - d10, fx);
    return mixf(mixf(d00, d10, fx), mixf(d01, d11, fx), fy);
}

DEV int rl_root(const DevScene& d, int i) {
    int l = d.rl[i].x;
    for (int guard = 0; guard < (1 << 20) && l != i; guard++) {
        i = l;
        l = d.rl[i].x;
    }
    return i;
}

// mode 0: label each rigid cell with itself
__global__ void __launch_bounds__(256) k_rigid_label(DevScene d) {
    CELL_XY;
    if (cx >= W || cy >= H) return;
    const int i = cy * W + cx;
    d.rl[i] = make_int2(cell_rigid(d, cx, cy, i) ? i : -1, -1);
    if (i == 0) *d.nbodies = 0u;
}

// mode 1: join rigid neighbours (left, below, and the two below diagonals); each link takes
// the smaller root, so every body ends with its smallest cell as root whatever the order
__global__ void __launch_bounds__(256) k_rigid_unite(DevScene d) {
    CELL_XY;
    if (cx >= W || cy >= H) return;
    const int i = cy * W + cx;
    if (d.rl[i].x < 0) return;
    const int nb[4] = {cx > 0 ? i - 1 : -1, cy > 0 ? i - W : -1, (cy > 0 && cx > 0) ? i - W - 1 : -1,
                       (cy > 0 && cx < W - 1) ? i - W + 1 : -1};
    for (int q = 0; q < 4; q++) {
        if (nb[q] < 0 || d.rl[nb[q]].x < 0) continue;
        int a = i, b = nb[q];
        bool done = false;
        for (int guard = 0; guard < 4096 && !done; guard++) {
            a = rl_root(d, a);
            b = rl_root(d, b);
            if (a < b) {
                const int old = atomicMin(&d.rl[b].x, a);
                done = old == b;
                b = old;
            } else if (b < a) {
                const int old = atomicMin(&d.rl[a].x, b);
                done = old == a;
                a = old;
            } else {
                done = true;
            }
        }
    }
}

// mode 2: every cell points at its root; each root takes a body
__global__ void __launch_bounds__(256) k_rigid_bodies(DevScene d) {
    CELL_XY;
    if (cx >= W || cy >= H) return;
    const int i = cy * W + cx;
    if (d.rl[i].x < 0) return;
    const int r = rl_root(d, i);
    d.rl[i].x = r;
    if (r == i) {
        const uint32_t b = atomicAdd(d.nbodies, 1u);
        if (b < (uint32_t)kMaxBodies) {
            for (int k = 0; k < 16; k++) d.rbody[(size_t)b * 16 + k] = 0ull;
            d.rl[i].y = (int)b;
        }
    }
}

DEV void add64(unsigned long long* w, float x) {
    x = floorf(x + 0.5f);
    atomicAdd(w, (unsigned long long)(long long)x);
}

// mode 3: each body's mass, moments and contacts with the solids, in 64-bit fixed point
__global__ void __launch_bounds__(256) k_rigid_sums(DevScene d) {
    CELL_XY;
    if (cx >= W || cy >= H) return;
    const int i = cy * W + cx;
    const int l = d.rl[i].x;
    if (l < 0) return;
    const int b = d.rl[l].y;
    if (b < 0) return;
    unsigned long long* o = d.rbody + (size_t)b * 16;
    const float m = d.cell[i].y * minf(d.cell[i].x, 1.0f) * RIGID_FIX;
    const float dx = (float)(cx - l % W), dy = (float)(cy - l / W);
    const float4 q = d.vel[i];
    const float ur = cx < W - 1 ? d.vel[i + 1].x : 0.0f, ut = cy < H - 1 ? d.vel[i + W].y : 0.0f;
    const float ux = 0.5f * (q.x + ur), uy = 0.5f * (q.y + ut);
    add64(&o[0], m);
    add64(&o[1], m * dx);
    add64(&o[2], m * dy);
    add64(&o[3], m * ux);
    add64(&o[4], m * uy);
    add64(&o[5], m * (dx * uy - dy * ux));
    add64(&o[6], m * ((dx * dx + dy * dy) + 1.0f / 6.0f));
    if (d.P->misc[3] >= 0.0f) {
        float gx, gy;
        const float dist = rigid_sdf(d, (float)cx + 0.5f, (float)cy + 0.5f, gx, gy);
        if (dist < 1.0f && gx * gx + gy * gy > 1e-8f) {
            const float gl = len2(gx, gy);
            const float nx = gx / gl, ny = gy / gl;
            add64(&o[7], RIGID_FIX);
            add64(&o[8], RIGID_FIX * nx);
            add64(&o[9], RIGID_FIX * ny);
            add64(&o[10], RIGID_FIX * dx);
            add64(&o[11], RIGID_FIX * dy);
            add64(&o[12], RIGID_FIX * dx * dx);
            add64(&o[13], RIGID_FIX * dy * dy);
            add64(&o[14], RIGID_FIX * dx * dy);
        }
    }
}

// mode 4: the faces inside a body move with it
__global__ void __launch_bounds__(256) k_rigid_faces(DevScene d) {
    CELL_XY;
    if (cx >= W || cy >= H) return;
    const int i = cy * W + cx;
    const int l = d.rl[i].x;
    float4 q = d.vel[i];
    bool changed = false;
    const float clump = REST_PHI + maxf(d.P->corr[1], 0.05f);
    const bool cl = d.cell[i].x > clump;
    float3 u;
    if (l >= 0 && cx > 0 && d.rl[i - 1].x == l && face_live(q.z) && d.rl[l].y >= 0 &&
        body_motion(d, d.rl[l].y, l, (float)cx, (float)cy + 0.5f, u)) {
        q.x = u.x;
        if (!cl && d.cell[i - 1].x <= clump) q.z = 0.0f;
        changed = true;
    }
    if (l >= 0 && cy > 0 && d.rl[i - W].x == l && face_live(q.w) && d.rl[l].y >= 0 &&
        body_motion(d, d.rl[l].y, l, (float)cx + 0.5f, (float)cy, u)) {
        q.y = u.y;
        if (!cl && d.cell[i - W].x <= clump) q.w = 0.0f;
        changed = true;
    }
    if (changed) d.vel[i] = q;
}

void launch_rigid(const DevScene& d, cudaStream_t st) {
    dim3 blk(16, 16);
    dim3 grd((d.W + 15) / 16, (d.H + 15) / 16);
    k_rigid_label<<<grd, blk, 0, st>>>(d);
    k_rigid_unite<<<grd, blk, 0, st>>>(d);
    k_rigid_bodies<<<grd, blk, 0, st>>>(d);
    k_rigid_sums<<<grd, blk, 0, st>>>(d);
    k_rigid_faces<<<grd, blk, 0, st>>>(d);
}

void launch_grid(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st) {
    dim3 blk(16, 16);
    dim3 grd((d.W + 15) / 16, (d.H + 15) / 16);
    k_grid_prep<<<grd, blk, 0, st>>>(d);
    if (cfg.rheo) k_rheo<<<grd, blk, 0, st>>>(d);
    if (cfg.elastic) k_elastic<<<grd, blk, 0, st>>>(d);
    if (cfg.settle) k_settle<<<grd, blk, 0, st>>>(d);
    k_coef_smooth<<<grd, blk, 0, st>>>(d);
    k_curv<<<grd, blk, 0, st>>>(d);
    k_apply<<<grd, blk, 0, st>>>(d);
    if (cfg.magnet) {
        k_magnet_energy<<<grd, blk, 0, st>>>(d);
        k_magnet_force<<<grd, blk, 0, st>>>(d);
    }
    if (cfg.heat) k_heat<<<grd, blk, 0, st>>>(d);
    if (cfg.visc_mode == 1) {
        k_visc_setup<<<grd, blk, 0, st>>>(d);
        k_visc_explicit<<<grd, blk, 0, st>>>(d);
    } else if (cfg.visc_mode == 2) {
        // record_viscosity_split (mod.rs:2812-2836), and the solve itself here unless it
        // runs between two pressure solves (record_viscosity, mod.rs:2805-2808)
        cudaMemsetAsync(d.tiles, 0, (size_t)d.nwg * sizeof(uint32_t), st);
        k_visc_setup<<<grd, blk, 0, st>>>(d);
        launch_viscosity_setup(d, cfg, st);
        if (!cfg.twice) launch_viscosity(d, cfg, st, 0);
    }
    k_rhs<<<grd, blk, 0, st>>>(d);
}

void launch_project(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st) {
    (void)cfg;
    dim3 blk(16, 16);
    dim3 grd((d.W + 15) / 16, (d.H + 15) / 16);
    k_project<<<grd, blk, 0, st>>>(d);
}

}  // namespace sprout

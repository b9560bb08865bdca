// The render side's per-cell passes on the device, into a headless buffer of layers
// (FluidSim::record_cell_optics, mod.rs:1626-1660): cell_optics.comp (what the liquid in each
// cell looks like, 20 layers), light.comp (the key light from above through the liquid) and
// optics_blur.comp (the 3 x 3 binomial smoothing and the light's sideways spread). Layers are
// RGBA16F as the reference's image array holds them: IEEE half, rounded to nearest even, and
// read back as such by the later passes. exp / log / pow are the engine's own (sp_expf,
// sp_logf, sp_powf), the same arithmetic as the oracle's, where GLSL leaves their precision to
// the implementation.
//
// Then sss.comp (the light under the surface, layers 20-23 of the smoothed buffer, warm-started
// from the last call), flow_map.comp (how far the liquid has moved since its patterns
// restarted, four layers) and glow.comp (the emission blurred at half resolution).
//
// Not computed here: the film map's tile flags (no film map).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "dev_common.cuh"
#include "kernels.h"
#include "optics.h"

namespace sprout {

namespace {

constexpr int kLayers = 20;
constexpr float kDiluentFade = 24.0f;   // optics.glsl: DILUENT_FADE
constexpr float kGlowRef = 1300.0f;     // cell_optics.comp: GLOW_REF
constexpr float kLightPath = 0.35f;     // light.comp: LIGHT_PATH
constexpr float kCellTau = 0.25f;       // light.comp: CELL_TAU
constexpr int kMaxStretch = 32;
constexpr int kLightSpread = 14;        // optics_blur.comp: LIGHT_SPREAD
constexpr float kLightSigma = 6.0f;

DEV float4 f4(float x, float y, float z, float w) { return make_float4(x, y, z, w); }
DEV float4 add(float4 a, float4 b) { return f4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
DEV float4 mul(float s, float4 a) { return f4(s * a.x, s * a.y, s * a.z, s * a.w); }
DEV float4 mul(float4 a, float s) { return f4(a.x * s, a.y * s, a.z * s, a.w * s); }
DEV float4 mix4(float4 a, float4 b, float t) { return f4(mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t), mixf(a.w, b.w, t)); }
DEV float4 ld4(const float v[4]) { return f4(v[0], v[1], v[2], v[3]); }

// an RGBA16F texel: IEEE half, round to nearest even
DEV ushort4 to_half4(float4 v) {
    return make_ushort4(__half_as_ushort(__float2half_rn(v.x)), __half_as_ushort(__float2half_rn(v.y)),
                        __half_as_ushort(__float2half_rn(v.z)), __half_as_ushort(__float2half_rn(v.w)));
}
DEV float4 from_half4(ushort4 h) {
    return f4(__half2float(__ushort_as_half(h.x)), __half2float(__ushort_as_half(h.y)), __half2float(__ushort_as_half(h.z)),
              __half2float(__ushort_as_half(h.w)));
}

// optics.glsl: to_srgb, deep_reflectance, film_colour, look_key
DEV float srgb1(float v) {
    v = clampf(v, 0.0f, 1.0f);
    return mixf(v * 12.92f, 1.055f * sp_powf(v, 1.0f / 2.4f) - 0.055f, v < 0.0031308f ? 0.0f : 1.0f);
}
DEV float4 look_key(float4 k) {
    const float film = 0.35f;
    float out[3];
    const float kk[3] = {k.x, k.y, k.z};
    for (int c = 0; c < 3; c++) {
        const float ext = kk[c] + k.w;
        const float tv = sp_expf(-2.0f * ext * film);
        const float w = k.w / maxf(kk[c] + k.w, 1e-6f);
        const float q = sqrtf(maxf(1.0f - w, 0.0f));
        const float refl = (1.0f - q) / (1.0f + q) * (1.0f - tv);
        out[c] = srgb1(refl + 0.75f * tv * sp_expf(-2.0f * kk[c] * film));
    }
    return f4(out[0], out[1], out[2], 1.0f);
}

// cell_optics.comp: glow (black-body colour and brightness of a grey body at T, deg C)
DEV float3 glow_of(float T) {
    const float K = T + 273.15f;
    if (K < 760.0f) return make_float3(0.0f, 0.0f, 0.0f);
    const float rel = sp_expf(23587.0f / kGlowRef - 23587.0f / K);
    const float level = minf(sp_logf(1.0f + 200.0f * rel) / sp_logf(201.0f), 1.6f);
    const float cr = 1.0f, cg = 1.677f * sp_expf(-2573.0f / K), cb = 3.89f * sp_expf(-7355.0f / K);
    const float m = maxf(cr, maxf(cg, cb));
    return make_float3(cr / m * level, cg / m * level, cb / m * level);
}

DEV bool in_grid2(const DevScene& d, int x, int y) { return x >= 0 && y >= 0 && x < d.W && y < d.H; }
DEV float occ_of(const DevScene& d, int x, int y) {
    if (!in_grid2(d, x, y)) return 0.0f;
    return minf((float)d.acc[(y * d.W + x) * d.stride + 4] / MASS_SCALE * d.P->inv_ppc, 1.0f);
}
DEV float sdf_cell(const DevScene& d, int x, int y) {
    x = min(max(x, 0), d.W - 1);
    y = min(max(y, 0), d.H - 1);
    const int w1 = d.W + 1, k = y * w1 + x;
    return 0.25f * (d.sdf[k] + d.sdf[k + 1] + d.sdf[k + w1] + d.sdf[k + w1 + 1]);
}
// the share of a cell's liquid that is aqueous (cell_optics.comp aq_share)
DEV float aq_share(const DevScene& d, int x, int y) {
    if (!in_grid2(d, x, y)) return 0.0f;
    const DevParams* P = d.P;
    const int kq = (y * d.W + x) * d.stride;
    const int cwq = d.acc[kq + 4];
    if (cwq <= 0) return 0.0f;
    int others = 0, aqw = 0;
    for (int j = 0; j < P->n_present; j++) {
        const int r = P->present[j];
        const int* ia = d.mats[r].ia;
        if (ia[2] < 0) continue;
        const int w = d.acc[kq + ia[2]];
        others += w;
        if (ia[0] == 0) aqw += w;
    }
    const int rest = max(cwq - others, 0);
    if (d.mats[P->present[0]].ia[0] == 0) aqw += rest;
    return clampf((float)aqw / (float)cwq, 0.0f, 1.0f);
}

// Ferrofluid spikes (cell_optics.comp:78-117): their height from the field where a
// magnetisable surface faces it past the Rosensweig threshold (mu0 M of a flat surface, N = 1),
// to kSpikeK of their spacing; and where along the surface they stand, as the cos and sin of
// the distance round the magnet whose field is strongest, in spacings / 4 (SPIKE_PHASE_DIV).
constexpr float kSpikeK = 0.85f;   // mod.rs SPIKE_HEIGHT
DEV float spike_height(const DevParams* P, float gap, float mc, float B) {
    if (gap <= 0.0f || P->mag[1] <= 0.0f) return 0.0f;
    const float chi = P->mag[1], ce = chi / (1.0f + chi);
    const float m = ce * B / (1.0f + ce * B / maxf(P->mag[2], 1e-6f));   // mu0 M, T
    const float over = m * m / maxf(mc * mc, 1e-12f) - 1.0f;
    return over > 0.0f ? kSpikeK * gap * (1.0f - sp_expf(-over)) : 0.0f;
}
DEV float2 spike_phase(const DevParams* P, float gap, float x, float y) {
    int best = 0;
    float bb = -1.0f;
    for (int k = 0; k < (int)P->mag[0]; k++) {
        const float* mg = P->magnet[k];
        const float r = maxf(len2(x - mg[0], y - mg[1]), mg[2]);
        const float b = mg[3] * sp_powf(mg[2] / r, 3.0f);
        if (b > bb) {
            bb = b;
            best = k;
        }
    }
    const float dx = x - P->magnet[best][0], dy = y - P->magnet[best][1];
    const float mx = P->magnet_dir[best][0], my = P->magnet_dir[best][1];
    const float ang = sp_atan2(mx * dy - my * dx, mx * dx + my * dy);
    const float ph = 6.2831853f * len2(dx, dy) * ang / (maxf(gap, 1e-3f) * 4.0f);
    float s, c;
    sp_sincos(ph, &s, &c);
    return make_float2(c, s);
}

__global__ void __launch_bounds__(256) k_cell_optics(DevScene d, const DevOptics* opt, float inv_speed, float spike_gap,
                                                    float spike_mc, const int* dfield, float dust, ushort4* raw) {
    const int cx = blockIdx.x * 16 + threadIdx.x, cy = blockIdx.y * 16 + threadIdx.y;
    if (cx >= d.W || cy >= d.H) return;
    const DevParams* P = d.P;
    const DevMat* mats = d.mats;
    const int i = cy * d.W + cx, k = i * d.stride;
    const int cw = d.acc[k + 4];
    const size_t nc = (size_t)d.W * d.H;
    float4 o[kLayers];
    for (int l = 0; l < kLayers; l++) o[l] = f4(0.0f, 0.0f, 0.0f, 0.0f);
    if (spike_gap > 0.0f) {   // in every cell: the spikes stand in the air
        const float px = (float)cx + 0.5f, py = (float)cy + 0.5f;
        const float2 B = magnet_field(P, px, py);
        const float b = len2(B.x, B.y), hgt = spike_height(P, spike_gap, spike_mc, b);
        o[13] = f4(b > 1e-9f ? B.x / b * hgt : 0.0f, b > 1e-9f ? B.y / b * hgt : 0.0f, 0.0f, spike_gap);
        const float2 ph = spike_phase(P, spike_gap, px, py);
        o[14].x = ph.x;
        o[14].y = ph.y;
    }
    if (cw > 0) {
        const bool thermal = P->thermal != 0;
        float T = thermal ? d.therm[i].x : P->heat[0];
        int others = 0;
        for (int j = 0; j < P->n_present; j++) {
            const int ch = mats[P->present[j]].ia[2];
            if (ch >= 0) others += d.acc[k + ch];
        }
        const int cl = max(cw, 1);   // (no steam in this engine's tanks: its weight is zero)
        const float occ = minf((float)cw / MASS_SCALE * P->inv_ppc, 1.0f);
        float Tg[kGroups];
        {
            float Csh = 0.0f;
            float Cg[kGroups] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (thermal) {
                for (int j = 0; j < P->n_present; j++) {
                    const int r = P->present[j];
                    const int* ia = mats[r].ia;
                    if (ia[2] < 0 && P->primary >= 0 && r != P->primary) continue;
                    const int w = ia[2] >= 0 ? d.acc[k + ia[2]] : max(cw - others, 0);
                    if (w <= 0) continue;
                    const float sh = w >= cw ? 1.0f : clampf((float)w / (float)cw, 0.0f, 1.0f);
                    const float s = (ia[1] >= 0 && ia[3] >= 0) ? clampf((float)d.acc[k + ia[3]] / (float)w, 0.0f, 1.0f) : 1.0f;
                    const float cr = sh * thermal_of(mats, (uint32_t)r, s).w;
                    Csh += cr;
                    Cg[ia[0]] += cr;
                }
            }
            // group_temperatures (common.glsl:610-629)
            for (int g = 0; g < kGroups; g++) Tg[g] = T;
            if (Csh > 0.0f) {
                const int Htot = d.acc[k + (int)P->heat2[2]];
                T = (float)Htot * T_SCALE / (Csh * (float)cw) - 273.15f;
                for (int g = 0; g < kGroups; g++) Tg[g] = T;
                int rest = Htot, first = -1;
                for (int g = 0; g < kGroups; g++) {
                    const int ch = group_heat_chan(P, g);
                    if (ch >= 0) {
                        const int h = d.acc[k + ch];
                        rest -= h;
                        if (Cg[g] > 0.0f) Tg[g] = (float)h * T_SCALE / (Cg[g] * (float)cw) - 273.15f;
                    } else if (first < 0 && (P->group_mask & (1u << (uint32_t)g)) != 0u) {
                        first = g;
                    }
                }
                if (first >= 0 && Cg[first] > 0.0f) Tg[first] = (float)rest * T_SCALE / (Cg[first] * (float)cw) - 273.15f;
            }
        }
        float4 aq = f4(0, 0, 0, 0), ot = f4(0, 0, 0, 0), op_sum = f4(0, 0, 0, 0), sty = f4(0, 0, 0, 0);
        float4 aq_plain = f4(0, 0, 0, 0), aq_conc = f4(0, 0, 0, 0);
        float c_aq = 0.0f;
        float4 iaq = f4(0, 0, 0, 0), iot = f4(0, 0, 0, 0), fx = f4(0, 0, 0, 0), fx2 = f4(0, 0, 0, 0);
        float3 lum = make_float3(0.0f, 0.0f, 0.0f);
        float ior_sum = 0.0f;
        const float4 vi = d.vel[i];
        const float vsx = face_live(vi.z) ? vi.x : 0.0f, vsy = face_live(vi.w) ? vi.y : 0.0f;
        const float stirred = smoothstepf(1.5f, 12.0f, sqrtf(vsx * vsx + vsy * vsy));
        float4 dense = f4(0, 0, 0, 0);
        float best_sh = 0.0f;
        int best_row = -1;
        float wden = 0.0f, fden = 0.0f, mag = 0.0f, fzx = 0.0f, fzy = 0.0f, waq = 0.0f, wot = 0.0f, skin = 0.0f;
        float3 em = make_float3(0.0f, 0.0f, 0.0f);
        const float waq_here = aq_share(d, cx, cy);
        for (int j = 0; j < P->n_present; j++) {
            const int r = P->present[j];
            const int* ia = mats[r].ia;
            if (ia[2] < 0 && P->primary >= 0 && r != P->primary) continue;
            const int w = ia[2] >= 0 ? d.acc[k + ia[2]] : max(cw - others, 0);
            if (w <= 0) continue;
            const float sh = clampf((float)w / (float)cl, 0.0f, 1.0f);
            const float s = (ia[1] >= 0 && ia[3] >= 0) ? clampf((float)d.acc[k + ia[3]] / (float)w, 0.0f, 1.0f) : 1.0f;
            const DevOptics& oo = opt[r];
            float4 absorb = ld4(oo.absorb);
            if (oo.thermo[1] > oo.thermo[0]) absorb = mix4(absorb, ld4(oo.hot), smoothstepf(oo.thermo[0], oo.thermo[1], Tg[ia[0]]));
            float4 lab = absorb, op = ld4(oo.opt), st = ld4(oo.sty), ef = ld4(oo.fx);
            float4 e2 = f4(oo.fx2[0], oo.fx2[1], absorb.w * oo.scat[0], absorb.w * oo.scat[2]);
            float4 lm = ld4(oo.lum);
            float3 labs = make_float3(oo.solid[0], oo.solid[1], oo.solid[2]);
            if (ia[1] >= 0) {
                const DevOptics& dd = opt[ia[1]];
                lab = mix4(ld4(dd.absorb), absorb, s);
                labs = make_float3(mixf(dd.solid[0], labs.x, s), mixf(dd.solid[1], labs.y, s), mixf(dd.solid[2], labs.z, s));
                op = mix4(ld4(dd.opt), op, s);
                st = mix4(ld4(dd.sty), st, s);
                ef = mix4(ld4(dd.fx), ef, s);
                e2 = mix4(f4(dd.fx2[0], dd.fx2[1], dd.absorb[3] * dd.scat[0], dd.absorb[3] * dd.scat[2]), e2, s);
                lm = mix4(ld4(dd.lum), lm, s);
            }
            // for light: a clear plain liquid's tint attenuates it without colour
            float4 kl = absorb;
            if (absorb.w <= 1e-3f && oo.opt[0] < 0.2f) {
                const float grey = kl.x * 0.3f + kl.y * 0.45f + kl.z * 0.25f;
                kl = f4(grey, grey, grey, kl.w);
            }
            if (ia[1] >= 0) {
                const DevOptics& dd = opt[ia[1]];
                float4 kd = ld4(dd.absorb);
                if (dd.absorb[3] <= 1e-3f && dd.opt[0] < 0.2f) {
                    const float grey = kd.x * 0.3f + kd.y * 0.45f + kd.z * 0.25f;
                    kd = f4(grey, grey, grey, kd.w);
                }
                kl = mix4(kd, absorb, s);
            }
            o[19] = add(o[19], mul(sh, kl));
            ior_sum += sh * (ia[1] >= 0 ? mixf(opt[ia[1]].opt2[0], oo.opt2[0], s) : oo.opt2[0]);
            fx2 = add(fx2, mul(sh, e2));
            const float sl = mixf(1.0f, stirred, lm.w);
            lum = make_float3(lum.x + sh * lm.x * sl, lum.y + sh * lm.y * sl, lum.z + sh * lm.z * sl);
            mag += sh * mats[r].el[2];
            const float Tm = Tg[ia[0]];
            float fs = 0.0f;
            if (thermal) {
                const float4 th = thermal_of(mats, (uint32_t)r, s);
                fs = th.y > -1e8f ? clampf((th.y - Tm) / maxf(th.y - th.x, 1e-3f), 0.0f, 1.0f) : 0.0f;
                op.w *= 1.0f - 0.6f * fs;
                op.x = mixf(op.x, maxf(op.x, 0.6f), fs);
            }
            if (oo.idx[1] == 0) {
                aq = add(aq, mul(sh, lab));
                if (ia[1] >= 0) {
                    aq_plain = add(aq_plain, mul(sh * (1.0f - s), ld4(opt[ia[1]].absorb)));
                    aq_conc = add(aq_conc, mul(sh * s, absorb));
                    c_aq += sh * s;
                } else {
                    aq_plain = add(aq_plain, mul(sh, absorb));
                }
                waq += sh;
                iaq = add(iaq, mul(sh * fs, f4(labs.x, labs.y, labs.z, 0.0f)));
                fzx += sh * fs;
            } else {
                if (oo.idx[1] == 1) {
                    ot = add(ot, mul(sh, lab));
                } else {
                    dense = add(dense, mul(sh, lab));
                    wden += sh;
                    fden += sh * fs;
                }
                wot += sh;
                iot = add(iot, mul(sh * fs, f4(labs.x, labs.y, labs.z, 0.0f)));
                fzy += sh * fs;
            }
            // the quenched skin of a melt that crusts, against the liquid and air beside it
            if (thermal && ia[0] == 3 && ef.w > 0.01f && Tm > 0.0f) {
                const float4 th = thermal_of(mats, (uint32_t)r, s);
                if (th.y > -1e8f) {
                    const float g = 2.0f * mats[r].th[1];
                    const float hc = P->heat2[3], Tw = minf(Tg[0], 100.0f);
                    const float Ta = P->heat[0] + 273.15f;
                    const float ts_w = (g * Tm + hc * Tw) / maxf(g + hc, 1e-12f);
                    float ts_a = Tm;
                    for (int it = 0; it < 4; it++) {
                        const float Kk = ts_a + 273.15f;
                        const float h = P->heat[2] + st.w * P->heat[3] * (Kk * Kk + Ta * Ta) * (Kk + Ta);
                        ts_a = (g * Tm + h * P->heat[0]) / maxf(g + h, 1e-12f);
                    }
                    const float range = maxf(th.y - th.x, 1e-3f);
                    const float sk_w = clampf((th.y - ts_w) / range, 0.0f, 1.0f);
                    const float sk_a = clampf((th.y - ts_a) / range, 0.0f, 1.0f);
                    float to_air = 0.0f, to_water = waq_here;
                    for (int q = 0; q < 4; q++) {
                        const int nx = cx + (q == 0 ? -1 : q == 1 ? 1 : 0), ny = cy + (q == 2 ? -1 : q == 3 ? 1 : 0);
                        if (sdf_cell(d, nx, ny) < 0.0f) continue;
                        const float on = occ_of(d, nx, ny);
                        to_air += 1.0f - on;
                        to_water += on * aq_share(d, nx, ny);
                    }
                    skin = maxf(skin, sh * maxf(sk_w * clampf(to_water, 0.0f, 1.0f), sk_a * clampf(to_air, 0.0f, 1.0f)));
                }
            }
            op_sum = add(op_sum, mul(sh, op));
            fx = add(fx, mul(sh, ef));
            if (sh > best_sh) {
                best_sh = sh;
                best_row = r;
            }
            sty = add(sty, mul(sh, st));
            const float3 gl = glow_of(Tm);
            em = make_float3(em.x + sh * gl.x * st.w, em.y + sh * gl.y * st.w, em.z + sh * gl.z * st.w);
        }
        const float speed = minf(sqrtf(vsx * vsx + vsy * vsy) * inv_speed, 1.5f);
        o[15] = mul(f4(aq_plain.x, aq_plain.y, aq_plain.z, maxf(waq - c_aq, 0.0f)), occ);
        if (waq > 0.0f) aq = add(mul(aq_plain, sp_expf(-kDiluentFade * c_aq / waq)), aq_conc);
        o[0] = mul(aq, occ);
        o[1] = mul(ot, occ);
        o[2] = mul(op_sum, occ);
        const float sk = 1.0f - 0.6f * clampf(skin, 0.0f, 1.0f);
        em = make_float3(em.x * sk, em.y * sk, em.z * sk);
        o[3] = mul(f4(em.x + lum.x, em.y + lum.y, em.z + lum.z, speed), occ);
        const float s_mean = aq.w + ot.w + dense.w;
        o[16] = f4(fx2.x * occ, fx2.y * occ, s_mean > 1e-5f ? fx2.z / s_mean : 1.0f, s_mean > 1e-5f ? fx2.w / s_mean : 1.0f);
        // the specks' share of the colour (spray.comp's dust field, laid down last frame), per
        // cell of the tank: over the occupancy per unit of liquid, premultiplied by it again
        if (dust > 0.0f && occ > 0.02f) {
            const float f = 1.0f / 1024.0f;   // DUST_FIX
            o[18] = f4((float)dfield[4 * i] * f, (float)dfield[4 * i + 1] * f, (float)dfield[4 * i + 2] * f,
                       (float)dfield[4 * i + 3] * f);
            const float cap = 200.0f * occ;
            o[18] = f4(minf(o[18].x, cap), minf(o[18].y, cap), minf(o[18].z, cap), minf(o[18].w, cap));
        }
        o[19] = add(mul(o[19], occ), o[18]);
        o[17] = mul(f4(lum.x, lum.y, lum.z, ior_sum), occ);
        o[4] = mul(f4(sty.x, sty.y, waq, waq + wot), occ);
        o[5] = mul(f4(iaq.x, iaq.y, iaq.z, wden), occ);
        o[6] = mul(f4(iot.x, iot.y, iot.z, fden), occ);
        o[11] = mul(dense, occ);
        const int last = d.W * d.H - 1;
        const float4 vr = d.vel[min(i + 1, last)], vt = d.vel[min(i + d.W, last)];
        const float ucx = 0.5f * (vsx + (face_live(vr.z) ? vr.x : 0.0f)), ucy = 0.5f * (vsy + (face_live(vt.w) ? vt.y : 0.0f));
        o[7] = mul(f4(fzx, fzy, ucx, ucy), occ);
        o[8] = mul(fx, occ);
        o[9] = mul(f4(0.0f, 0.0f, 0.0f, skin), occ);
        o[10] = f4(fx.y * occ, 0.0f, 0.0f, 0.0f);
        o[13].z = fx.x * occ;
        o[14].w = (float)(best_row + 1);
        const float wl = waq + wot;
        if (wl > 0.0f) {
            const float4 sum = add(add(aq, ot), dense);
            o[12] = mul(look_key(f4(sum.x / wl, sum.y / wl, sum.z / wl, sum.w / wl)), occ);
        }
        o[14].z = P->mag[1] > 0.0f ? mag / P->mag[1] * occ : 0.0f;
    }
    for (int l = 0; l < kLayers; l++) raw[(size_t)l * nc + i] = to_half4(o[l]);
}

// light.comp: one block per column, a thread per stretch of it from the top
__global__ void __launch_bounds__(64) k_light(DevScene d, ushort4* raw) {
    __shared__ float3 s_sum[64];
    const int x = blockIdx.x, t = threadIdx.x, H = d.H;
    const size_t nc = (size_t)d.W * d.H;
    const int stretch = min((H + 63) / 64, kMaxStretch);
    const int top = H - 1 - t * stretch;
    auto alpha_at = [&](int y) {
        const float4 k = from_half4(raw[(size_t)19 * nc + (size_t)y * d.W + x]);
        return make_float3(minf(sqrtf(maxf(k.x * (k.x + 3.0f * k.w), 0.0f)), kCellTau),
                           minf(sqrtf(maxf(k.y * (k.y + 3.0f * k.w), 0.0f)), kCellTau),
                           minf(sqrtf(maxf(k.z * (k.z + 3.0f * k.w), 0.0f)), kCellTau));
    };
    float3 sum = make_float3(0.0f, 0.0f, 0.0f);
    for (int k = 0; k < stretch; k++) {
        const int y = top - k;
        if (y < 0) break;
        const float3 a = alpha_at(y);
        sum = make_float3(sum.x + a.x, sum.y + a.y, sum.z + a.z);
    }
    s_sum[t] = sum;
    __syncthreads();
    float3 tau = make_float3(0.0f, 0.0f, 0.0f);
    for (int j = 0; j < t; j++) tau = make_float3(tau.x + s_sum[j].x, tau.y + s_sum[j].y, tau.z + s_sum[j].z);
    for (int k = 0; k < stretch; k++) {
        const int y = top - k;
        if (y < 0) break;
        const float3 a = alpha_at(y);
        ushort4* p = &raw[(size_t)10 * nc + (size_t)y * d.W + x];
        const float4 l10 = from_half4(*p);
        const float4 il = f4(l10.x, sp_expf(-kLightPath * (tau.x + 0.5f * a.x)), sp_expf(-kLightPath * (tau.y + 0.5f * a.y)),
                             sp_expf(-kLightPath * (tau.z + 0.5f * a.z)));
        *p = to_half4(il);
        tau = make_float3(tau.x + a.x, tau.y + a.y, tau.z + a.z);
    }
}

// optics_blur.comp: 3 x 3 binomial smoothing that leaves out neighbours behind a solid, and the
// light from above spread sideways by a Gaussian, into the smoothed layers
__global__ void __launch_bounds__(256) k_optics_blur(DevScene d, const ushort4* raw, ushort4* sm) {
    const int cx = blockIdx.x * 16 + threadIdx.x, cy = blockIdx.y * 16 + threadIdx.y;
    if (cx >= d.W || cy >= d.H) return;
    const size_t nc = (size_t)d.W * d.H;
    const float K[3] = {1.0f, 2.0f, 1.0f};
    float4 s[kLayers];
    for (int l = 0; l < kLayers; l++) s[l] = f4(0.0f, 0.0f, 0.0f, 0.0f);
    float wsum = 0.0f;
    const float hx = (float)cx + 0.5f, hy = (float)cy + 0.5f;
    for (int b = -1; b <= 1; b++) {
        for (int a = -1; a <= 1; a++) {
            const int qx = cx + a, qy = cy + b;
            if (qx < 0 || qy < 0 || qx >= d.W || qy >= d.H) continue;
            if (a != 0 || b != 0) {   // sdf_at(here + 0.5 (a, b)): the nearest node
                const int nx = min(max((int)rintf(hx + 0.5f * (float)a), 0), d.W);
                const int ny = min(max((int)rintf(hy + 0.5f * (float)b), 0), d.H);
                if (d.sdf[ny * (d.W + 1) + nx] < 0.0f) continue;
            }
            const float w = K[a + 1] * K[b + 1];
            wsum += w;
            const size_t q = (size_t)qy * d.W + qx;
            for (int l = 0; l < kLayers; l++)
                if (l != 10) s[l] = add(s[l], mul(w, from_half4(raw[(size_t)l * nc + q])));
        }
    }
    for (int l = 0; l < kLayers; l++) s[l] = f4(s[l].x / wsum, s[l].y / wsum, s[l].z / wsum, s[l].w / wsum);
    {
        float3 il = make_float3(0.0f, 0.0f, 0.0f);
        float iw = 0.0f;
        for (int a = -kLightSpread; a <= kLightSpread; a++) {
            const int qx = cx + a;
            if (qx < 0 || qx >= d.W) continue;
            const float w = sp_expf(-0.5f * (float)(a * a) / (kLightSigma * kLightSigma));
            const float4 l10 = from_half4(raw[(size_t)10 * nc + (size_t)cy * d.W + qx]);
            il = make_float3(il.x + w * l10.y, il.y + w * l10.z, il.z + w * l10.w);
            iw += w;
        }
        const float iv = maxf(iw, 1e-6f);
        s[9] = f4(il.x / iv * s[4].w, il.y / iv * s[4].w, il.z / iv * s[4].w, s[9].w);
    }
    const size_t i = (size_t)cy * d.W + cx;
    for (int l = 0; l < kLayers; l++)
        if (l != 10) sm[(size_t)l * nc + i] = to_half4(s[l]);
}

// sss.comp: the light under the surface by the diffusion approximation, per channel
// -div(D grad phi) + s phi = s E, Jacobi iterations warm-started from the last call's
// solution (layer 20). stage 0 prepares each cell (layer 22: E, D; 23: s, kind), stage 1
// iterates from layer src into the other of 20, 21.
constexpr float kEscape = 0.04f, kDMax = 1.6f, kDMin = 0.04f, kKindAir = -1.0f, kKindSolid = -2.0f;
__global__ void __launch_bounds__(256) k_sss(DevScene d, const ushort4* raw, ushort4* co, int stage, int src) {
    const int cx = blockIdx.x * 16 + threadIdx.x, cy = blockIdx.y * 16 + threadIdx.y;
    if (cx >= d.W || cy >= d.H) return;
    const size_t nc = (size_t)d.W * d.H, i = (size_t)cy * d.W + cx;
    auto L = [&](int l, size_t c) { return from_half4(co[(size_t)l * nc + c]); };
    if (stage == 0) {
        const float occ = L(4, i).w;
        const int w1 = d.W + 1, k = cy * w1 + cx;
        const float sdc = 0.25f * (d.sdf[k] + d.sdf[k + 1] + d.sdf[k + w1] + d.sdf[k + w1 + 1]);
        if (sdc < -0.3f) {
            co[(size_t)22 * nc + i] = to_half4(f4(0.0f, 0.0f, 0.0f, 0.0f));
            co[(size_t)23 * nc + i] = to_half4(f4(0.0f, 0.0f, 0.0f, kKindSolid));
            return;
        }
        if (occ < 0.05f) {
            const float4 r10 = from_half4(raw[(size_t)10 * nc + i]);
            co[(size_t)22 * nc + i] = to_half4(f4(r10.y, r10.z, r10.w, 0.0f));
            co[(size_t)23 * nc + i] = to_half4(f4(0.0f, 0.0f, 0.0f, kKindAir));
            co[(size_t)20 * nc + i] = to_half4(f4(r10.y, r10.z, r10.w, 0.0f));
            return;
        }
        const float4 k19 = L(19, i), l9 = L(9, i);
        const float4 kk = f4(k19.x / occ, k19.y / occ, k19.z / occ, k19.w / occ);
        const float ex = l9.x / occ, ey = l9.y / occ, ez = l9.z / occ;
        const float lum_a = kk.x * 0.3f + kk.y * 0.45f + kk.z * 0.25f;
        const float D = clampf(1.0f / (3.0f * (lum_a + kk.w) + 1e-4f), kDMin, kDMax);
        co[(size_t)22 * nc + i] = to_half4(f4(ex, ey, ez, D));
        co[(size_t)23 * nc + i] = to_half4(f4(kk.x + kEscape, kk.y + kEscape, kk.z + kEscape, occ));
        return;
    }
    const int dst = src == 20 ? 21 : 20;
    const float4 kc = L(23, i), ec = L(22, i);
    if (kc.w < 0.0f) {
        co[(size_t)dst * nc + i] = to_half4(kc.w == kKindAir ? f4(ec.x, ec.y, ec.z, 0.0f) : f4(0.0f, 0.0f, 0.0f, 0.0f));
        return;
    }
    float nx = kc.x * ec.x, ny = kc.y * ec.y, nz = kc.z * ec.z;
    float dx = kc.x, dy = kc.y, dz = kc.z;
    for (int q = 0; q < 4; q++) {
        const int qx = cx + (q == 0 ? -1 : q == 1 ? 1 : 0), qy = cy + (q == 2 ? -1 : q == 3 ? 1 : 0);
        if (qx < 0 || qy < 0 || qx >= d.W || qy >= d.H) continue;
        const size_t n = (size_t)qy * d.W + qx;
        const float kind = L(23, n).w;
        if (kind == kKindSolid) continue;
        const float Dn = kind == kKindAir ? ec.w : L(22, n).w;
        const float Df = 2.0f * ec.w * Dn / maxf(ec.w + Dn, 1e-6f);
        const float4 pn = L(src, n);
        nx += Df * pn.x;
        ny += Df * pn.y;
        nz += Df * pn.z;
        dx += Df;
        dy += Df;
        dz += Df;
    }
    co[(size_t)dst * nc + i] = to_half4(f4(nx / dx, ny / dy, nz / dz, 0.0f));
}

// glow.comp: the emission at half the grid's resolution (the mean of 2 x 2 cells of raw layer
// 3) blurred by one separable Gaussian, across (dir 0, into ga) then down (dir 1, into gb)
constexpr int kGlowR = 9;
constexpr float kGlowSigma = 3.0f;
__global__ void __launch_bounds__(256) k_glow(DevScene d, const ushort4* raw, ushort4* ga, ushort4* gb, int dir) {
    const int hx = blockIdx.x * 16 + threadIdx.x, hy = blockIdx.y * 16 + threadIdx.y;
    const int hw = (d.W + 1) / 2, hh = (d.H + 1) / 2;
    if (hx >= hw || hy >= hh) return;
    const size_t nc = (size_t)d.W * d.H;
    float4 sum = f4(0.0f, 0.0f, 0.0f, 0.0f);
    float norm = 0.0f;
    for (int t = -kGlowR; t <= kGlowR; t++) {
        const float w = sp_expf(-0.5f * (float)(t * t) / (kGlowSigma * kGlowSigma));
        norm += w;
        const int qx = hx + (dir == 0 ? t : 0), qy = hy + (dir == 0 ? 0 : t);
        if (qx < 0 || qy < 0 || qx >= hw || qy >= hh) continue;
        float4 v;
        if (dir == 0) {
            float4 s = f4(0.0f, 0.0f, 0.0f, 0.0f);
            for (int j = 0; j < 2; j++)
                for (int i = 0; i < 2; i++) {
                    const int cx = 2 * qx + i, cy = 2 * qy + j;
                    if (cx >= d.W || cy >= d.H) continue;
                    const float4 e = from_half4(raw[(size_t)3 * nc + (size_t)cy * d.W + cx]);
                    s = add(s, f4(e.x, e.y, e.z, 0.0f));
                }
            v = mul(0.25f, s);
        } else {
            v = from_half4(ga[(size_t)qy * hw + qx]);
        }
        sum = add(sum, mul(w, v));
    }
    sum = f4(sum.x / norm, sum.y / norm, sum.z / norm, sum.w / norm);
    (dir == 0 ? ga : gb)[(size_t)hy * hw + hx] = to_half4(sum);
}

// record_cell_optics' clock (mod.rs:1628-1641, 1674-1680): the time since the last call from
// the simulated time after the last substep (the compensated sum of the substeps' lengths,
// step.comp), clamped to 0 .. 0.25 s in double precision and then rounded to f32; zero on the
// first call on a new tank. The flow map runs when the call records (`changed`) and dt > 0,
// reading the copy that holds the map and leaving it in the other.
__global__ void k_render_clock(const StepState* S, RenderClock* c, int valid, int changed) {
    const double now = (double)S->advanced - (double)__uint_as_float(S->pad0);
    double dt = 0.0;
    if (valid) dt = fmin(fmax(now - c->stain, 0.0), 0.25);
    c->stain = now;
    c->dt = (float)dt;
    c->now = (float)now;
    c->src = c->parity;
    c->run = (changed && c->dt > 0.0f) ? 1u : 0u;
    if (c->run) c->parity = 1u - c->parity;
}

// flow_map.comp: how far the liquid at each cell has moved since its pattern last restarted,
// carried semi-Lagrangian by the smoothed velocity (layer 7 zw over the occupancy, layer 4 w)
// and grown by u dt; two copies per period half a period apart, each restarted (zero) as its
// weight in the composite reaches zero. Layers 2 copy + period (0 short, 1 long).
constexpr float kFlowSpeedMax = 30.0f;   // flow_map.comp: SPEED_MAX, cells/s
constexpr float kFlowPeriodShort = 4.0f;  // mod.rs FLOW_PERIOD_SHORT, s
constexpr float kFlowPeriodLong = 12.0f;  // mod.rs FLOW_PERIOD_LONG, s
__global__ void __launch_bounds__(256) k_flow_map(DevScene d, const ushort4* sm, ushort4* flow, const RenderClock* c) {
    if (!c->run) return;
    const int cx = blockIdx.x * 16 + threadIdx.x, cy = blockIdx.y * 16 + threadIdx.y;
    if (cx >= d.W || cy >= d.H) return;
    const size_t nc = (size_t)d.W * d.H, i = (size_t)cy * d.W + cx;
    const float dt = c->dt, now = c->now;
    const float occ = from_half4(sm[(size_t)4 * nc + i]).w;
    float ux = 0.0f, uy = 0.0f;
    if (occ > 0.02f) {
        const float4 v = from_half4(sm[(size_t)7 * nc + i]);
        ux = v.z / occ;
        uy = v.w / occ;
    }
    const float s = len2(ux, uy);
    if (s > kFlowSpeedMax) {
        const float k = kFlowSpeedMax / s;
        ux *= k;
        uy *= k;
    }
    const float fx = ((float)cx + 0.5f) - ux * dt, fy = ((float)cy + 0.5f) - uy * dt;
    // sample_at: bilinear at a cell-centred position, clamped to the grid
    const float qx = clampf(fx - 0.5f, 0.0f, (float)(d.W - 1)), qy = clampf(fy - 0.5f, 0.0f, (float)(d.H - 1));
    // a position that is not a number (a texel that overflowed half) samples cell 0
    const int i0x = qx == qx ? (int)floorf(qx) : 0, i0y = qy == qy ? (int)floorf(qy) : 0;
    const int i1x = min(i0x + 1, d.W - 1), i1y = min(i0y + 1, d.H - 1);
    const float tx = qx - (float)i0x, ty = qy - (float)i0y;
    const int src = 2 * (int)c->src, dst = 2 * (1 - (int)c->src);
    for (int k = 0; k < 2; k++) {
        const float period = k == 0 ? kFlowPeriodShort : kFlowPeriodLong;
        const ushort4* L = flow + (size_t)(src + k) * nc;
        const float4 a = mix4(from_half4(L[(size_t)i0y * d.W + i0x]), from_half4(L[(size_t)i0y * d.W + i1x]), tx);
        const float4 b = mix4(from_half4(L[(size_t)i1y * d.W + i0x]), from_half4(L[(size_t)i1y * d.W + i1x]), tx);
        const float4 sa = mix4(a, b, ty);
        float4 o = f4(sa.x + ux * dt, sa.y + uy * dt, sa.z + ux * dt, sa.w + uy * dt);
        // restarted(period, o): floor(now / period + o) != floor((now - dt) / period + o)
        const float before = now - dt;
        if (floorf(now / period + 0.0f) != floorf(before / period + 0.0f)) o.x = o.y = 0.0f;
        if (floorf(now / period + 0.5f) != floorf(before / period + 0.5f)) o.z = o.w = 0.0f;
        flow[(size_t)(dst + k) * nc + i] = to_half4(o);
    }
}

// look.comp: the orientation of the platelets each particle of a liquid with platelets stands
// for, the second moment A of their normals (A_xx, A_yy, A_xy), evolved by Jeffery's equation
// averaged over them with the quadratic closure (the shear part of the particle's velocity
// gradient only), relaxed towards isotropy by rotational diffusion, and kept at 10 bits each,
// rounded stochastically (pack_a). A slot whose stored id is not its particle's holds a new
// particle, which starts isotropic. The particles with platelets are listed for the look
// splat (the order of that list is the atomics'). The specks a new particle brings into
// spray.comp's pool are not made: there is no pool here (the reference's dust_cap = 0 case).
DEV float rnd24(uint32_t h) { return (float)(h >> 8) / 16777216.0f; }
DEV uint32_t quant10(float v, uint32_t h) {
    const float m = 1023.0f;
    return (uint32_t)clampf(floorf(clampf(v, 0.0f, 1.0f) * m + rnd24(h)), 0.0f, m);
}
DEV uint32_t pack_a(float ax, float ay, float az, uint32_t h) {
    return quant10(ax, hash32(h ^ 0x1b873593u)) | (quant10(ay, hash32(h ^ 0xcc9e2d51u)) << 10) |
           (quant10(az + 0.5f, hash32(h ^ 0xe6546b64u)) << 20);
}
__global__ void __launch_bounds__(128) k_look(DevScene d, const DevOptics* opt, const RenderClock* clk, uint32_t frame,
                                             uint32_t* count, uint32_t* list, uint32_t cap) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.P->n_slots) return;
    const float4 q0 = d.part[3 * i + 1], q1 = d.part[3 * i + 2];   // c; s, kind, id, t
    const uint32_t kind = __float_as_uint(q1.y), id = __float_as_uint(q1.z), low = kind & 255u;
    if (kind == KIND_DEAD || low == 0u || low > 96u) return;   // rows of the optics table
    const uint32_t row = low - 1u;
    const DevOptics& o = opt[row];
    const float2 lk = look_of(opt, row, q1.x);
    const float lx = lk.x, ly = lk.y;
    if (maxf(lx, ly) <= 0.0f) return;
    const uint4 st = d.plook[i];
    const bool fresh = st.x != id;
    const uint32_t h = hash32(id * 0x9e3779b1u ^ hash32(frame * 0x85ebca6bu + 0x165667b1u));
    const float third = 1.0f / 3.0f;
    if (lx <= 0.0f) {
        if (fresh) d.plook[i] = make_uint4(id, 0u, pack_a(third, third, 0.0f, h), 0u);
        return;
    }
    float ax = third, ay = third, az = 0.0f;
    if (!fresh) {
        ax = (float)(st.z & 1023u) / 1023.0f;
        ay = (float)((st.z >> 10) & 1023u) / 1023.0f;
        az = (float)((st.z >> 20) & 1023u) / 1023.0f - 0.5f;
        const float dt = clk->dt;
        if (dt > 0.0f) {
            const float Bc = o.opt2[2];
            const float w = 0.5f * (q0.z - q0.y);   // rotation rate, 1 / s
            const float dv = 0.5f * (q0.x + q0.w);
            const float exx = q0.x - dv, eyy = q0.w - dv, exy = 0.5f * (q0.y + q0.z);
            const float rate = fabsf(w) + fabsf(exx) + fabsf(eyy) + fabsf(exy);
            const float sf = ceilf(rate * dt / 0.15f);
            const int sub = sf >= 8.0f ? 8 : (sf >= 1.0f ? (int)sf : 1);
            const float h1 = dt / (float)sub;
            const float ezz = 0.0f;
            for (int k = 0; k < sub; k++) {
                const float a = ax, b = ay, c = az, z = 1.0f - a - b;
                const float AE = exx * a + eyy * b + 2.0f * exy * c + ezz * z;
                const float rx = -2.0f * w * c, ry = 2.0f * w * c, rz = w * (a - b);
                const float e2 = 2.0f * AE;
                const float sx = 2.0f * (exx * a + exy * c) - e2 * a;
                const float sy = 2.0f * (exy * c + eyy * b) - e2 * b;
                const float sz = c * (exx + eyy) + exy * (a + b) - e2 * c;
                ax = ax + h1 * (rx + Bc * sx);
                ay = ay + h1 * (ry + Bc * sy);
                az = az + h1 * (rz + Bc * sz);
            }
            const float t = 1.0f - sp_expf(-6.0f * o.opt2[1] * dt);   // rotational diffusion
            ax = mixf(ax, third, t);
            ay = mixf(ay, third, t);
            az = mixf(az, 0.0f, t);
            ax = clampf(ax, 0.0f, 1.0f);
            ay = clampf(ay, 0.0f, 1.0f);
            az = clampf(az, -0.5f, 0.5f);
        }
    }
    d.plook[i] = make_uint4(id, 0u, pack_a(ax, ay, az, h), 0u);
    const uint32_t k = atomicAdd(count, 1u);   // listed for the look splat
    if (k < cap) list[k] = i;
}

}  // namespace

void launch_look(const DevScene& d, const DevOptics* opt, const RenderClock* clock, uint32_t frame, uint32_t* count,
                 uint32_t* list, uint32_t cap, uint32_t n_slots, cudaStream_t st) {
    cudaMemsetAsync(count, 0, sizeof(uint32_t), st);
    if (n_slots > 0) k_look<<<(n_slots + 127) / 128, 128, 0, st>>>(d, opt, clock, frame, count, list, cap);
}

void launch_render_clock(const DevScene& d, RenderClock* clock, int valid, int changed, cudaStream_t st) {
    k_render_clock<<<1, 1, 0, st>>>(d.S, clock, valid, changed);
}

void launch_cell_optics(const DevScene& d, const DevOptics* opt, float inv_speed, float spike_gap, float spike_mc,
                        const int* dfield, float dust, int sss_iters, ushort4* raw, ushort4* smooth, ushort4* flow,
                        const RenderClock* clock, ushort4* glow_a, ushort4* glow_b, cudaStream_t st) {
    const dim3 tiles((d.W + 15) / 16, (d.H + 15) / 16), block(16, 16);
    k_cell_optics<<<tiles, block, 0, st>>>(d, opt, inv_speed, spike_gap, spike_mc, dfield, dust, raw);
    k_light<<<d.W, 64, 0, st>>>(d, raw);
    k_optics_blur<<<tiles, block, 0, st>>>(d, raw, smooth);
    // sss.comp (mod.rs:1666-1675): prepared, then an even number of iterations, ending in layer 20
    const int iters = (sss_iters + 1) / 2 * 2;
    if (iters > 0) {
        k_sss<<<tiles, block, 0, st>>>(d, raw, smooth, 0, 20);
        for (int k = 0; k < iters; k++) k_sss<<<tiles, block, 0, st>>>(d, raw, smooth, 1, k % 2 == 0 ? 20 : 21);
    }
    k_flow_map<<<tiles, block, 0, st>>>(d, smooth, flow, clock);   // mod.rs:1673-1680
    const dim3 half(((d.W + 1) / 2 + 15) / 16, ((d.H + 1) / 2 + 15) / 16);
    for (int dir = 0; dir < 2; dir++) k_glow<<<half, block, 0, st>>>(d, raw, glow_a, glow_b, dir);
}

}  // namespace sprout

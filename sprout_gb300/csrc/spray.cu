// spray.comp on the device (FluidSim::record_spray, mod.rs:1739-1773): bubbles, foam and
// spray, secondary particles the liquid makes and carries that do not push back on it (Ihmsen
// et al. 2012), each one entry of a pool of kDiffuseMax.
//
// Stage 0 makes them, per cell: where a liquid traps air between streams that close on each
// other, where its surface folds in, at a crest moving out of it (white water, by the liquid's
// `foam`), and where a liquid fizzes (dissolved gas, most on the solids it touches). Stage 1
// moves each entry as a bubble (carried, rising at its terminal velocity), foam (on the
// surface, spreading where it crowds, bursting after the liquid's froth time) or spray
// (ballistic), turns it from one to another by the liquid around it, counts the foam per cell
// for the next frame's crowding, and lists the live entries for the sprites.
//
// The pool is handed out deterministically. The reference's emitters take entries through
// atomics in whatever order the cells run (pool.glsl: the free stack first, then entries never
// used), and return freed ones in whatever order the entries finish. Here the emissions of a
// frame are ranked by cell, then by their order in the cell, and the k-th takes what the k-th
// take would get: the stack's top first, then the next unused entry. Freed entries go onto the
// stack in entry order, and live ones are listed in entry order. That is one of the orders the
// reference allows, and it makes every entry's slot, and so every bit of the pool,
// reproducible. Not made here: the specks (look.comp's part of the pool; this engine does not
// carry them), and the splat a droplet leaves on a solid (film_lay.glsl, the film map's intake:
// no film map). The droplet is still removed, as the reference removes it.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "dev_common.cuh"
#include "kernels.h"
#include "sample.cuh"

namespace sprout {

namespace {

constexpr uint32_t FREE = 0u, BUBBLE = 1u, FOAM = 2u, SPRAY = 3u;
constexpr float FOAM_RATE = 40.0f, CREST_RATE = 25.0f, FIZZ_RATE = 1.6f, FIZZ_WALL = 5.0f, FIZZ_GROW = 0.5e-3f;
constexpr int EMIT_MAX = 6;
constexpr float BUBBLE_OCC = 0.62f, FOAM_OCC = 0.10f, FOAM_SPREAD = 6.0f, FOAM_CROWD = 2.0f, FOAM_FULL = 5.0f;
constexpr float FOAM_FALL = 8.0f, FOAM_SAG = 1.5f, ENTRAIN_RATE = 30.0f, SPRAY_DRAG = 1.2f, SPRAY_LIFE = 1.5f;
constexpr float BUBBLE_LIFE = 40.0f;
constexpr uint32_t DUST = 8u;
constexpr int kScan = 1024;

DEV float rnd24(uint32_t h) { return (float)(h >> 8) / 16777216.0f; }
DEV float ramp(float x, float lo, float hi) { return clampf((x - lo) / (hi - lo), 0.0f, 1.0f); }
DEV float4 half4(ushort4 h) {
    return make_float4(__half2float(__ushort_as_half(h.x)), __half2float(__ushort_as_half(h.y)),
                       __half2float(__ushort_as_half(h.z)), __half2float(__ushort_as_half(h.w)));
}

// A speck's flake normal in hemi-octahedral form, 10 + 10 bits (look.comp pack_n, spray.comp
// unpack_n): a disc's normal and its opposite are one orientation.
DEV uint32_t quant10(float v, uint32_t h) {
    const float m = 1023.0f;
    return (uint32_t)clampf(floorf(clampf(v, 0.0f, 1.0f) * m + rnd24(h)), 0.0f, m);
}
DEV uint32_t pack_n(float nx, float ny, float nz, uint32_t h) {
    if (nz < 0.0f) {
        nx = -nx;
        ny = -ny;
        nz = -nz;
    }
    const float den = maxf(fabsf(nx) + fabsf(ny) + nz, 1e-6f);
    const float px = nx / den, py = ny / den;
    const float qx = (px + py) * 0.5f + 0.5f, qy = (px - py) * 0.5f + 0.5f;
    return quant10(qx, hash32(h)) | (quant10(qy, hash32(h ^ 0x68e31da4u)) << 10);
}
DEV void normalize3(float& x, float& y, float& z) {
    const float l = sqrtf(x * x + y * y + z * z);
    x = x / l;
    y = y / l;
    z = z / l;
}
DEV void unpack_n(uint32_t b, float& x, float& y, float& z) {
    const float qx = (float)(b & 1023u) / 1023.0f * 2.0f - 1.0f, qy = (float)((b >> 10) & 1023u) / 1023.0f * 2.0f - 1.0f;
    x = (qx + qy) * 0.5f;
    y = (qx - qy) * 0.5f;
    z = maxf(1.0f - fabsf(x) - fabsf(y), 0.0f);
    normalize3(x, y, z);
}
DEV float signf(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
constexpr float DUST_IN = 0.30f, DUST_DRY_LIFE = 30.0f, SHIELDS = 0.05f, BED_U = 8.0f, DUST_FIX = 1024.0f;

struct Spray {
    DevScene d;
    const ushort4* sm;     // the smoothed layers (optics_blur.comp)
    const DevOptics* opt;
    DevDiffuse* pool;
    uint32_t* stack;       // the free stack
    uint32_t* stack1;      // the specks' free stack
    uint32_t* list;        // the live entries for the sprites
    uint32_t* dcount;      // foam per cell, two copies
    uint32_t* counts;      // stage 0: emissions per cell, then their first rank
    uint32_t* flags;       // stage 1: per entry, bit 0 freed, bit 1 listed
    int* dfield;
    uint32_t* nspeck;      // look.comp's specks: per particle slot, ranked
    PoolState* ps;
    const RenderClock* clk;
    uint32_t frame, parity;
    float amount;
    int W, H;

    DEV size_t nc() const { return (size_t)W * H; }
    DEV float4 layer(int l, int i) const { return half4(sm[(size_t)l * nc() + i]); }
    DEV float occ_cell(int x, int y) const {
        if (x < 0 || y < 0 || x >= W || y >= H) return 0.0f;
        return clampf(d.cell[y * W + x].x, 0.0f, 1.5f);
    }
    DEV float occ_at(float px, float py) const {
        const float gx = px - 0.5f, gy = py - 0.5f;
        const int bx = (int)floorf(gx), by = (int)floorf(gy);
        const float fx = gx - (float)bx, fy = gy - (float)by;
        return mixf(mixf(occ_cell(bx, by), occ_cell(bx + 1, by), fx), mixf(occ_cell(bx, by + 1), occ_cell(bx + 1, by + 1), fx),
                    fy);
    }
    DEV float2 centre_vel(int i) const {
        const int n = W * H;
        const float4 v = d.vel[i];
        const float ux = face_live(v.z) ? v.x : 0.0f, uy = face_live(v.w) ? v.y : 0.0f;
        const float4 vr = d.vel[min(i + 1, n - 1)], vt = d.vel[min(i + W, n - 1)];
        return make_float2(0.5f * (ux + (face_live(vr.z) ? vr.x : 0.0f)), 0.5f * (uy + (face_live(vt.w) ? vt.y : 0.0f)));
    }
    // common.glsl's sample_vel at a pool entry: a face's cell read by its linear index as the
    // shader reads it, zeros where that index leaves the grid's buffer
    DEV float4 vel_lin(int x, int y) const {
        const long long k = (long long)y * W + x;
        return (k >= 0 && k < (long long)W * H) ? d.vel[k] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    DEV float2 sample_vel_at(float x, float y) const { return sample_vel_fb(x, y, make_float2(0.0f, 0.0f)); }
    DEV float2 sample_vel_fb(float x, float y, float2 fb) const {
        float2 o = fb;
        for (int comp = 0; comp < 2; comp++) {
            const float gx = comp == 0 ? x : x - 0.5f, gy = comp == 0 ? y - 0.5f : y;
            const int bx = (int)floorf(gx), by = (int)floorf(gy);
            const float fx = gx - (float)bx, fy = gy - (float)by;
            float sw = 0.0f, su = 0.0f;
            for (int b = 0; b < 2; b++)
                for (int a = 0; a < 2; a++) {
                    const float4 q = vel_lin(bx + a, by + b);
                    if (face_live(comp == 0 ? q.z : q.w)) {
                        const float wt = (a == 0 ? 1.0f - fx : fx) * (b == 0 ? 1.0f - fy : fy);
                        sw += wt;
                        su += wt * (comp == 0 ? q.x : q.y);
                    }
                }
            if (sw > 1e-3f) {
                if (comp == 0) o.x = su / sw;
                else o.y = su / sw;
            }
        }
        return o;
    }
    DEV float crowd_cell(int x, int y, uint32_t copy) const {
        x = min(max(x, 0), W - 1);
        y = min(max(y, 0), H - 1);
        return (float)dcount[(size_t)copy * nc() + (size_t)y * W + x];
    }
    // the row of the liquid that holds most of cell i (-1 none), as cell_optics.comp counts
    DEV int dominant_row(int i) const {
        const DevParams* P = d.P;
        const int k = i * d.stride, cw = d.acc[k + 4];
        if (cw <= 0) return -1;
        int others = 0;
        for (int j = 0; j < P->n_present; j++) {
            const int ch = d.mats[P->present[j]].ia[2];
            if (ch >= 0) others += d.acc[k + ch];
        }
        int best = -1, bw = 0;
        for (int j = 0; j < P->n_present; j++) {
            const int r = P->present[j];
            const int* ia = d.mats[r].ia;
            if (ia[2] < 0 && P->primary >= 0 && r != P->primary) continue;
            const int w = ia[2] >= 0 ? d.acc[k + ia[2]] : max(cw - others, 0);
            if (w > bw) {   // (no steam row in this engine's tanks)
                bw = w;
                best = r;
            }
        }
        return best;
    }

    // What make() decides for cell (cx, cy): the emissions of the trapped air and the crest
    // (n, from h) and of the dissolved gas (nf, from h2), with what they carry.
    struct Cell {
        int n = 0, nf = 0, row = -1;
        uint32_t h = 0u, h2 = 0u;
        float ux = 0.0f, uy = 0.0f, r0 = 0.0f, r0f = 0.0f;
    };
    DEV Cell make_cell(int cx, int cy) const {
        Cell e;
        const int i = cy * W + cx;
        const float occ = occ_cell(cx, cy);
        if (occ < 0.08f) return e;
        const float4 l4 = layer(4, i);
        if (l4.w < 0.02f) return e;
        const float foam_k = l4.y / l4.w;
        const float4 l16r = layer(16, i);
        const float fizz = l16r.y / l4.w;
        const float cs = d.P->misc[2];
        const float2 u = centre_vel(i);
        float ta = 0.0f, gx = 0.0f, gy = 0.0f;
        for (int q = 0; q < 4; q++) {
            const int dx = q == 0 ? -1 : q == 1 ? 1 : 0, dy = q == 2 ? -1 : q == 3 ? 1 : 0;
            const int nx = cx + dx, ny = cy + dy;
            const float on = occ_cell(nx, ny);
            gx += (float)dx * on;
            gy += (float)dy * on;
            if (on < 0.08f || nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
            const float2 un = centre_vel(ny * W + nx);
            const float dvx = u.x - un.x, dvy = u.y - un.y;
            const float m = len2(dvx, dvy);
            if (m < 1e-4f) continue;
            ta += m * (1.0f - (dvx / m * -(float)dx + dvy / m * -(float)dy));
        }
        const float ul = len2(u.x, u.y);
        const float speed = ul * cs;
        const float energy = ramp(speed, 0.6f, 3.0f);
        const float trapped = ramp(ta * cs, 1.0f, 5.0f);
        const float g = len2(gx, gy);
        float crest = 0.0f, plunge = 0.0f;
        if (g > 0.15f && speed > 0.05f) {
            const float nox = -gx / g, noy = -gy / g;
            const float along = u.x / ul * nox + u.y / ul * noy;
            crest = ramp(along, 0.6f, 0.95f) * ramp(speed, 1.0f, 3.5f);
            plunge = ramp(-along, 0.4f, 0.9f) * ramp(speed, 0.08f, 1.2f) * smoothstepf(0.15f, 0.6f, g);
        }
        const float tension = maxf(d.sprop[i].x, 0.0f) * cs * cs * cs / 7.2e-5f;
        e.r0 = clampf(1.2e-3f * sqrtf(clampf(tension, 0.05f, 4.0f)) / cs, 0.03f, 0.4f);
        e.h = hash32((uint32_t)i * 0x85ebca6bu ^ hash32(frame * 0x9e3779b1u + 0x3c6ef372u));
        const float rate = amount * (FOAM_RATE * trapped * energy + ENTRAIN_RATE * plunge + CREST_RATE * crest * foam_k);
        const float dt = clk->dt;
        const float fn = floorf(rate * dt + rnd24(e.h));
        e.n = fn >= (float)EMIT_MAX ? EMIT_MAX : (fn >= 1.0f ? (int)fn : 0);
        e.row = (e.n > 0 || fizz > 0.0f) ? dominant_row(i) : -1;
        e.ux = u.x;
        e.uy = u.y;
        if (fizz > 0.0f) {
            const int w1 = W + 1, kk = cy * w1 + cx;
            const float sd = 0.25f * (d.sdf[kk] + d.sdf[kk + 1] + d.sdf[kk + w1] + d.sdf[kk + w1 + 1]);
            const float wall = 1.0f - ramp(sd, 0.5f, 2.0f);
            const float fr = amount * FIZZ_RATE * fizz * minf(occ, 1.0f) * (1.0f + FIZZ_WALL * wall);
            e.h2 = hash32(e.h ^ 0x7feb352du);
            const float ff = floorf(fr * dt + rnd24(e.h2));
            e.nf = ff >= 2.0f ? 2 : (ff >= 1.0f ? (int)ff : 0);
            e.r0f = clampf(0.25e-3f / cs, 0.02f, 0.2f);
        }
        return e;
    }
    // pool.glsl pool_take for the emission of rank r: the stack's top first, then unused entries
    DEV int take(uint32_t r, uint32_t top0, uint32_t hw0) const {
        if (r < top0) return (int)stack[top0 - 1u - r];
        const uint32_t hw = hw0 + (r - top0);
        return hw < kDiffuseMax ? (int)hw : -1;
    }
    // emit(): emission k of a run (h, n) of cell (cx, cy)
    DEV DevDiffuse bubble(int cx, int cy, uint32_t h, int k, float r0, uint32_t grows, float ux, float uy, float spread,
                          int row) const {
        const uint32_t hk = hash32(h + (uint32_t)k * 0x9e3779b9u);
        DevDiffuse e;
        e.px = (float)cx + rnd24(hk);
        e.py = (float)cy + rnd24(hash32(hk ^ 0x51ed270bu));
        const float a = 6.2831853f * rnd24(hash32(hk ^ 0x2545f491u));
        float sn, cs;
        sp_sincos(a, &sn, &cs);
        const float j = rnd24(hash32(hk ^ 0x27d4eb2fu));
        e.vx = ux + spread * cs * j;
        e.vy = uy + spread * sn * j;
        const float s = rnd24(hash32(hk ^ 0x165667b1u));
        e.r = r0 * (0.45f + 1.1f * s * s);
        e.info = BUBBLE | grows | ((uint32_t)(row + 1) << 8) | (hash32(hk ^ 0x68e31da4u) & 0xffff8000u);
        e.life = BUBBLE_LIFE;
        e.z = rnd24(hash32(hk ^ 0xb5297a4du));
        return e;
    }

    // move_dust(): a speck, suspended (BUBBLE: settling at its terminal velocity, lagging the
    // flow by its response time, a flake turned by the flow's gradient), resting (FOAM: held by
    // a solid or the packed specks below it, until the flow over it passes the Shields
    // threshold; a flake lies flat; left dry, gone after DUST_DRY_LIFE s) or falling (SPRAY);
    // resting ones counted per cell, and its share of the liquid's colour into the dust field
    DEV uint32_t move_dust(uint32_t i, DevDiffuse e) const {
        uint32_t st = e.info & 3u;
        const DevParams* P = d.P;
        const uint32_t copy_in = 1u - parity, copy_out = parity;
        const int row = (int)((e.info >> 8) & 127u) - 1;
        if (row < 0) {
            pool[i].info = 0u;
            return 1u;
        }
        const DevOptics& o = opt[row];
        const float rho_p = o.dust2[1] / 998.0f;
        const float aspect = o.dust2[2];
        const float rr = e.r;
        const float d_eq = 2.0f * rr * (aspect < 0.6667f ? sp_powf(1.5f * maxf(aspect, 0.005f), 1.0f / 3.0f) : 1.0f);
        const float pack = maxf(o.dcol[3], 1.0f);
        const float Bc = (aspect * aspect - 1.0f) / (aspect * aspect + 1.0f);
        float nx, ny, nz;
        unpack_n(__float_as_uint(e.life), nx, ny, nz);
        const uint32_t h0 = hash32(e.info ^ hash32(frame * 0x9e3779b1u + i));
        const float dt = clk->dt;
        const float sf = ceilf(dt * 120.0f);
        const int steps = sf >= 8.0f ? 8 : (sf >= 1.0f ? (int)sf : 1);
        const float h = dt / (float)steps;
        const Grid g{d.vel, d.sdf, W, H};
        for (int k = 0; k < steps && st != FREE; k++) {
            const int cx = min(max((int)e.px, 0), W - 1), cy = min(max((int)e.py, 0), H - 1), ci = cy * W + cx;
            const float occ = occ_at(e.px, e.py);
            const float4 cf = d.cell[ci];
            const float rho = maxf(cf.y, 0.3f), nu = maxf(cf.z / rho, 1e-6f);
            const float drho = rho_p - rho;
            const float down = drho >= 0.0f ? 1.0f : -1.0f;
            const float ux_ = e.px - 0.0f, uy_ = e.py - down * (rr + 0.35f);
            float gux, guy;
            const float sd_u = sample_sdf(g, ux_, uy_, &gux, &guy);
            const int cux = min(max((int)ux_, 0), W - 1), cuy = min(max((int)uy_, 0), H - 1);
            const float packed = (float)dcount[(size_t)(2u + copy_in) * nc() + (size_t)cuy * W + cux];
            const bool held = sd_u < 0.0f || ((cux != cx || cuy != cy) && packed >= pack) || uy_ < 0.0f;
            const bool wet = occ > DUST_IN;
            const float2 uf = sample_vel_at(e.px, e.py);
            const float u_crit = BED_U * sqrtf(SHIELDS * fabsf(drho) * P->gravity * d_eq / rho);
            if (st == FOAM) {
                if (!held) st = wet ? BUBBLE : SPRAY;
                else if (wet && len2(uf.x, uf.y) > u_crit) {
                    st = BUBBLE;
                    e.vx = uf.x;
                    e.vy = uf.y;
                } else {   // at rest: a flake lies flat on what holds it
                    float bx = 0.0f, by = 1.0f, bz = 0.0f;
                    if (sd_u < 0.0f) {
                        bx = gux + 0.0f;
                        by = guy + 1e-4f;
                        const float l = sqrtf(bx * bx + by * by);
                        bx = bx / l;
                        by = by / l;
                    }
                    const float sg = signf(nx * bx + ny * by + nz * bz + 1e-4f);
                    const float t = 1.0f - sp_expf(-h / 0.3f);
                    nx = mixf(nx, bx * sg, t);
                    ny = mixf(ny, by * sg, t);
                    nz = mixf(nz, bz * sg, t);
                    normalize3(nx, ny, nz);
                    e.vx = wet ? 0.0f : e.vx + h;
                    e.vy = 0.0f;
                    if (e.vx > DUST_DRY_LIFE) st = FREE;
                    continue;
                }
            }
            if (st == SPRAY && wet) st = BUBBLE;
            if (st == BUBBLE && !wet) st = SPRAY;
            if (st == BUBBLE) {
                const float vt = terminal(drho, rho, nu, d_eq, P->gravity);
                const float tx = uf.x - 0.0f, ty = uf.y - down * vt;
                const float tau = clampf(rho_p * d_eq * d_eq / (18.0f * rho * nu), 0.004f, 0.5f);
                const float t = 1.0f - sp_expf(-h / tau);
                e.vx = mixf(e.vx, tx, t);
                e.vy = mixf(e.vy, ty, t);
                if (aspect < 0.6667f) {   // a flake turns with the flow (Jeffery)
                    const float2 ux1 = sample_vel_fb(e.px + 0.5f, e.py + 0.0f, uf), ux0 = sample_vel_fb(e.px - 0.5f, e.py - 0.0f, uf);
                    const float2 uy1 = sample_vel_fb(e.px + 0.0f, e.py + 0.5f, uf), uy0 = sample_vel_fb(e.px - 0.0f, e.py - 0.5f, uf);
                    const float gxx = ux1.x - ux0.x, gxy = ux1.y - ux0.y, gyx = uy1.x - uy0.x, gyy = uy1.y - uy0.y;
                    const float w = 0.5f * (gxy - gyx);
                    const float dv = 0.5f * (gxx + gyy);
                    const float exx = gxx - dv, eyy = gyy - dv, exy = 0.5f * (gyx + gxy);
                    const float wnx = -w * ny, wny = w * nx, wnz = 0.0f;
                    const float enx = exx * nx + exy * ny, eny = exy * nx + eyy * ny, enz = 0.0f;
                    const float ne = nx * enx + ny * eny + nz * enz;
                    nx = nx + h * (wnx + Bc * (enx - ne * nx));
                    ny = ny + h * (wny + Bc * (eny - ne * ny));
                    nz = nz + h * (wnz + Bc * (enz - ne * nz));
                    normalize3(nx, ny, nz);
                }
                if (held && (e.vx - uf.x) * 0.0f + (e.vy - uf.y) * -down >= 0.0f && len2(uf.x, uf.y) < u_crit) {
                    st = FOAM;
                    e.vx = 0.0f;
                    e.vy = 0.0f;
                }
            } else if (st == SPRAY) {
                e.vx += 0.0f - e.vx * SPRAY_DRAG * h;
                e.vy += -P->gravity * h - e.vy * SPRAY_DRAG * h;
            }
            e.px += e.vx * h;
            e.py += e.vy * h;
            float gsx, gsy;
            const float sd = sample_sdf(g, e.px, e.py, &gsx, &gsy);
            const float rim = rr + 0.05f;
            if (sd < rim) {   // kept out of the solids; landing on one, it rests there
                const float gl = maxf(len2(gsx, gsy), 1e-6f);
                const float nrx = gsx / gl, nry = gsy / gl;
                e.px += nrx * (rim - sd);
                e.py += nry * (rim - sd);
                const float vn = minf(e.vx * nrx + e.vy * nry, 0.0f);
                e.vx -= nrx * vn;
                e.vy -= nry * vn;
                if (st == SPRAY) {
                    st = FOAM;
                    e.vx = 0.0f;
                    e.vy = 0.0f;
                }
            }
            if (e.px < 0.0f || e.py < -1.0f || e.px >= (float)W || e.py >= (float)H) st = FREE;
        }
        e.life = __uint_as_float(pack_n(nx, ny, nz, h0));
        e.info = (e.info & ~3u) | st;
        pool[i] = e;
        if (st == FREE) return 1u;
        const int cx = min(max((int)e.px, 0), W - 1), cy = min(max((int)e.py, 0), H - 1), ci = cy * W + cx;
        if (st == FOAM) atomicAdd(&dcount[(size_t)(2u + copy_out) * nc() + ci], 1u);
        if (o.dust[3] > 0.0f && occ_cell(cx, cy) > 0.05f) {   // its share of the liquid's colour
            const int qx = (int)(o.dust[0] * DUST_FIX + 0.5f), qy = (int)(o.dust[1] * DUST_FIX + 0.5f);
            const int qz = (int)(o.dust[2] * DUST_FIX + 0.5f), qw = (int)(o.dust[3] * DUST_FIX + 0.5f);
            if (qx > 0) atomicAdd(&dfield[4 * ci], qx);
            if (qy > 0) atomicAdd(&dfield[4 * ci + 1], qy);
            if (qz > 0) atomicAdd(&dfield[4 * ci + 2], qz);
            atomicAdd(&dfield[4 * ci + 3], qw);
        }
        return 2u;
    }

    // move(): entry i for the frame's dt in up to 8 steps
    DEV uint32_t move(uint32_t i) const {
        DevDiffuse e = pool[i];
        uint32_t st = e.info & 3u;
        if (st == FREE) return 0u;
        if ((e.info & DUST) != 0u) return move_dust(i, e);
        const DevParams* P = d.P;
        const uint32_t copy_in = 1u - parity, copy_out = parity;
        const float cs = P->misc[2], dt = clk->dt;
        const float sf = ceilf(dt * 120.0f);
        const int steps = sf >= 8.0f ? 8 : (sf >= 1.0f ? (int)sf : 1);
        const float h = dt / (float)steps;
        const Grid g{d.vel, d.sdf, W, H};
        for (int k = 0; k < steps && st != FREE; k++) {
            const int cx = min(max((int)e.px, 0), W - 1), cy = min(max((int)e.py, 0), H - 1), ci = cy * W + cx;
            const float occ = occ_at(e.px, e.py);
            const float2 uf = sample_vel_at(e.px, e.py);
            const float crowd = crowd_cell(cx, cy, copy_in);
            const float gcx = crowd_cell(cx + 1, cy, copy_in) - crowd_cell(cx - 1, cy, copy_in);
            const float gcy = crowd_cell(cx, cy + 1, copy_in) - crowd_cell(cx, cy - 1, copy_in);
            const uint32_t want = occ > BUBBLE_OCC ? BUBBLE : (occ + 0.06f * crowd > FOAM_OCC ? FOAM : SPRAY);
            const float4 l4 = layer(4, ci);
            const float wl = maxf(l4.w, 1e-3f);
            if (want != st) {
                if (want == FOAM || (want == BUBBLE && st == SPRAY)) {
                    const float foam_k = l4.w > 0.02f ? l4.y / wl : 0.0f;
                    const float froth = l4.w > 0.02f ? layer(16, ci).x / wl : 0.0f;
                    if (st == SPRAY && foam_k < 0.05f) {
                        st = FREE;
                        break;
                    }
                    if (want == FOAM && st == BUBBLE && (crowd > FOAM_FULL || foam_k < 0.05f)) {
                        st = FREE;
                        break;
                    }
                    if (want == FOAM) {
                        e.life = maxf(froth, 0.05f) * (0.5f + rnd24(hash32(e.info ^ (uint32_t)k)));
                        e.z = e.life;
                    }
                    if (want == BUBBLE) e.life = BUBBLE_LIFE;
                }
                if (want == SPRAY) e.life = minf(e.life, SPRAY_LIFE);
                if (want == BUBBLE && st == FOAM) e.z = rnd24(hash32(e.info ^ 0xb5297a4du));
                st = want;
            }
            float tx, ty, tau;
            if (st == BUBBLE) {
                const float4 cf = d.cell[ci];
                const float rho = maxf(cf.y, 0.3f), nu = maxf(cf.z / rho, 1e-6f);
                const float vt = terminal(rho, rho, nu, 2.0f * e.r, P->gravity);
                tx = uf.x + 0.0f;
                ty = uf.y + vt;
                tau = 0.03f;
                if ((e.info & 4u) != 0u) e.r = minf(e.r + FIZZ_GROW / cs * h, 0.35f);
                e.life -= h;
            } else if (st == FOAM) {
                const float sub = clampf(occ * 2.0f, 0.0f, 1.0f);
                tx = uf.x * sub;
                ty = uf.y * sub;
                const float below = occ_at(e.px - 0.0f, e.py - 0.7f) + 0.25f * crowd_cell(cx, cy - 1, copy_in);
                const bool held = occ > 0.25f || below > 0.45f;
                const float push = ramp(crowd, FOAM_CROWD * 0.7f, FOAM_CROWD * 2.0f);
                const float gl = len2(gcx, gcy);
                if (gl > 1e-3f) {
                    const float spx = -gcx / gl * FOAM_SPREAD * push;
                    float spy = -gcy / gl * FOAM_SPREAD * push;
                    if (!held) spy = minf(spy, 0.0f);
                    tx += spx;
                    ty += spy;
                }
                ty -= held ? FOAM_SAG * (1.0f - ramp(occ, 0.1f, 0.4f)) : FOAM_FALL;
                if (occ > 0.45f) ty += 4.0f * (occ - 0.45f);
                tau = 0.06f;
                e.life -= h * (crowd < 2.0f ? 2.5f : 1.0f);
            } else {
                tx = e.vx + 0.0f - e.vx * SPRAY_DRAG * h;
                ty = e.vy + -P->gravity * h - e.vy * SPRAY_DRAG * h;
                tau = 0.0f;
                e.life -= h;
            }
            if (tau > 0.0f) {
                const float t = 1.0f - sp_expf(-h / tau);
                e.vx = mixf(e.vx, tx, t);
                e.vy = mixf(e.vy, ty, t);
            } else {
                e.vx = tx;
                e.vy = ty;
            }
            e.px += e.vx * h;
            e.py += e.vy * h;
            float gsx, gsy;
            const float sd = sample_sdf(g, e.px, e.py, &gsx, &gsy);
            const float rim = e.r + 0.1f;
            const int drow = (int)((e.info >> 8) & 127u) - 1;
            if (st == SPRAY && sd < rim && drow >= 0) {   // a droplet splats on the solid (no film map here)
                st = FREE;
                break;
            }
            if (sd < rim) {
                const float gl = maxf(len2(gsx, gsy), 1e-6f);
                const float nx = gsx / gl, ny = gsy / gl;
                e.px += nx * (rim - sd);
                e.py += ny * (rim - sd);
                const float vn = minf(e.vx * nx + e.vy * ny, 0.0f);
                e.vx -= nx * vn;
                e.vy -= ny * vn;
            }
            if (e.life <= 0.0f || e.px < 0.0f || e.py < 0.0f || e.px >= (float)W || e.py >= (float)H) st = FREE;
        }
        e.info = (e.info & ~3u) | st;
        pool[i] = e;
        if (st == FREE) return 1u;
        if (st == FOAM) {
            const int cx = min(max((int)e.px, 0), W - 1), cy = min(max((int)e.py, 0), H - 1);
            atomicAdd(&dcount[(size_t)copy_out * nc() + (size_t)cy * W + cx], 1u);
        }
        return 2u;
    }
};

__global__ void __launch_bounds__(256) k_spray_count(Spray s) {
    const int cx = blockIdx.x * 16 + threadIdx.x, cy = blockIdx.y * 16 + threadIdx.y;
    if (cx >= s.W || cy >= s.H) return;
    uint32_t n = 0u;
    if (s.clk->dt > 0.0f) {
        const Spray::Cell e = s.make_cell(cx, cy);
        n = (uint32_t)(e.n + e.nf);
    }
    s.counts[cy * s.W + cx] = n;
}

// exclusive scan of counts[0, n) in blocks of kScan; block totals into bsum
__global__ void __launch_bounds__(kScan) k_spray_scan1(uint32_t* counts, uint32_t* bsum, int n) {
    __shared__ uint32_t t[kScan];
    const int i = blockIdx.x * kScan + threadIdx.x;
    const uint32_t v = i < n ? counts[i] : 0u;
    t[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kScan; o <<= 1) {
        const uint32_t a = threadIdx.x >= (unsigned)o ? t[threadIdx.x - o] : 0u;
        __syncthreads();
        t[threadIdx.x] += a;
        __syncthreads();
    }
    if (i < n) counts[i] = t[threadIdx.x] - v;
    if (threadIdx.x == kScan - 1) bsum[blockIdx.x] = t[threadIdx.x];
}
__global__ void __launch_bounds__(kScan) k_spray_scan2(uint32_t* bsum, int nb, uint32_t* total) {
    __shared__ uint32_t t[kScan];
    uint32_t carry = 0u;
    for (int b0 = 0; b0 < nb; b0 += kScan) {
        const int i = b0 + (int)threadIdx.x;
        const uint32_t v = i < nb ? bsum[i] : 0u;
        t[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kScan; o <<= 1) {
            const uint32_t a = threadIdx.x >= (unsigned)o ? t[threadIdx.x - o] : 0u;
            __syncthreads();
            t[threadIdx.x] += a;
            __syncthreads();
        }
        if (i < nb) bsum[i] = carry + t[threadIdx.x] - v;
        const uint32_t tot = t[kScan - 1];
        __syncthreads();
        carry += tot;
    }
    if (threadIdx.x == 0) *total = carry;
}
__global__ void __launch_bounds__(kScan) k_spray_scan3(uint32_t* counts, const uint32_t* bsum, int n) {
    const int i = blockIdx.x * kScan + threadIdx.x;
    if (i < n) counts[i] += bsum[blockIdx.x];
}

__global__ void __launch_bounds__(256) k_spray_make(Spray s) {
    const int cx = blockIdx.x * 16 + threadIdx.x, cy = blockIdx.y * 16 + threadIdx.y;
    if (cx >= s.W || cy >= s.H || !(s.clk->dt > 0.0f)) return;
    const Spray::Cell e = s.make_cell(cx, cy);
    if (e.n + e.nf == 0) return;
    const uint32_t r0 = s.counts[cy * s.W + cx], top0 = s.ps->top, hw0 = s.ps->hw;
    for (int k = 0; k < e.n; k++) {
        const int slot = s.take(r0 + (uint32_t)k, top0, hw0);
        if (slot >= 0)
            s.pool[slot] = s.bubble(cx, cy, e.h, k, e.r0, 0u, e.ux, e.uy, 0.3f * len2(e.ux, e.uy), e.row);
    }
    for (int k = 0; k < e.nf; k++) {
        const int slot = s.take(r0 + (uint32_t)(e.n + k), top0, hw0);
        if (slot >= 0) s.pool[slot] = s.bubble(cx, cy, e.h2, k, e.r0f, 4u, e.ux, e.uy, 0.0f, e.row);
    }
}
// the takes' effect on the pool's counters (pool.glsl: the stack popped, the rest unused entries)
__global__ void k_spray_taken(PoolState* ps, const RenderClock* clk) {
    if (!(clk->dt > 0.0f)) return;
    const uint32_t n = ps->total, top = ps->top;
    ps->top = n < top ? top - n : 0u;
    ps->hw += n > top ? n - top : 0u;
}

__global__ void __launch_bounds__(256) k_spray_move(Spray s) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kPoolMax) return;
    s.flags[i] = s.move(i);
}

// freed entries onto their part's stack and live ones into the list, all in entry order
__global__ void __launch_bounds__(kScan) k_spray_returns(Spray s) {
    __shared__ uint32_t tf[kScan], tg[kScan], tl[kScan];
    constexpr uint32_t per = kPoolMax / kScan;
    static_assert(kPoolMax % kScan == 0, "whole chunks");
    const uint32_t b = threadIdx.x * per;
    uint32_t nf = 0u, ng = 0u, nl = 0u;
    for (uint32_t j = 0; j < per; j++) {
        const uint32_t f = s.flags[b + j];
        if (f == 1u) {
            if (b + j < kDiffuseMax) nf++;
            else ng++;
        }
        nl += f == 2u;
    }
    tf[threadIdx.x] = nf;
    tg[threadIdx.x] = ng;
    tl[threadIdx.x] = nl;
    __syncthreads();
    for (int o = 1; o < kScan; o <<= 1) {
        const uint32_t a = threadIdx.x >= (unsigned)o ? tf[threadIdx.x - o] : 0u;
        const uint32_t c = threadIdx.x >= (unsigned)o ? tg[threadIdx.x - o] : 0u;
        const uint32_t e = threadIdx.x >= (unsigned)o ? tl[threadIdx.x - o] : 0u;
        __syncthreads();
        tf[threadIdx.x] += a;
        tg[threadIdx.x] += c;
        tl[threadIdx.x] += e;
        __syncthreads();
    }
    const uint32_t top = s.ps->top, top1 = s.ps->top1;
    uint32_t pf = top + tf[threadIdx.x] - nf, pg = top1 + tg[threadIdx.x] - ng, pl = tl[threadIdx.x] - nl;
    for (uint32_t j = 0; j < per; j++) {
        const uint32_t f = s.flags[b + j];
        if (f == 1u) {
            if (b + j < kDiffuseMax) s.stack[pf++] = b + j;
            else s.stack1[pg++] = b + j;
        } else if (f == 2u) s.list[pl++] = b + j;
    }
    __syncthreads();
    if (threadIdx.x == kScan - 1) {
        s.ps->top = top + tf[kScan - 1];
        s.ps->top1 = top1 + tg[kScan - 1];
        s.ps->listed = tl[kScan - 1];
    }
}

// look.comp's specks: how many each slot's particle brings in (a new particle of a liquid with
// specks: floor(drawn specks per cell / particles per cell + a draw), at most 8), before the
// look pass marks it seen
__global__ void __launch_bounds__(256) k_speck_count(Spray s, uint32_t n_slots) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n_slots) return;
    uint32_t n = 0u;
    if (i < n_slots) {
        const float4 q1 = s.d.part[3 * i + 2];
        const uint32_t kind = __float_as_uint(q1.y), id = __float_as_uint(q1.z), low = kind & 255u;
        if (kind != KIND_DEAD && low != 0u && low <= 96u) {
            const float2 lk = look_of(s.opt, low - 1u, q1.x);
            if (maxf(lk.x, lk.y) > 0.0f && s.d.plook[i].x != id && lk.y > 0.0f) {
                const uint32_t h = hash32(id * 0x9e3779b1u ^ hash32(s.frame * 0x85ebca6bu + 0x165667b1u));
                const float e = lk.y * s.d.P->inv_ppc;
                const float fn = floorf(e + rnd24(hash32(h ^ 0x2545f491u)));
                n = fn >= 8.0f ? 8u : (fn >= 1.0f ? (uint32_t)fn : 0u);
            }
        }
    }
    s.nspeck[i] = n;
}
// ... and brings them in: speck k of the slot takes what the take of its rank gets
__global__ void __launch_bounds__(256) k_speck_emit(Spray s, uint32_t n_slots) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_slots) return;
    const uint32_t r0 = s.nspeck[i], n = s.nspeck[i + 1] - r0;
    if (n == 0u) return;
    const float4 q0 = s.d.part[3 * i], q1 = s.d.part[3 * i + 2];
    const uint32_t id = __float_as_uint(q1.z), row = (__float_as_uint(q1.y) & 255u) - 1u;
    const DevOptics& o = s.opt[row];
    const int src = o.fx2[2] > 0.0f ? (int)row : o.idx[0];
    const DevOptics& ds = s.opt[max(src, 0)];
    const uint32_t h = hash32(id * 0x9e3779b1u ^ hash32(s.frame * 0x85ebca6bu + 0x165667b1u));
    const uint32_t top1 = s.ps->top1, hw1 = s.ps->hw1;
    for (uint32_t k = 0; k < n; k++) {
        const uint32_t r = r0 + k;
        int slot;
        if (r < top1) slot = (int)s.stack1[top1 - 1u - r];
        else {
            const uint32_t hw = hw1 + (r - top1);
            slot = hw < kDustMax ? (int)(kDiffuseMax + hw) : -1;
        }
        if (slot < 0) break;
        const uint32_t hk = hash32(h + k * 0x9e3779b9u);
        const float u1 = rnd24(hash32(hk ^ 0x2c1b3c6du)), u2 = rnd24(hash32(hk ^ 0x297a2d39u));
        const float z = u1, a = 6.2831853f * u2, rr = sqrtf(maxf(1.0f - z * z, 0.0f));
        float sn, cs;
        sp_sincos(a, &sn, &cs);
        DevDiffuse e;
        e.px = q0.x + (rnd24(hash32(hk ^ 0x51ed270bu)) - 0.5f) * 0.9f;
        e.py = q0.y + (rnd24(hash32(hk ^ 0x7feb352du)) - 0.5f) * 0.9f;
        e.vx = q0.z;
        e.vy = q0.w;
        e.life = __uint_as_float(pack_n(rr * cs, rr * sn, z, hk));
        e.r = ds.dust2[0] / s.d.P->misc[2];
        e.info = BUBBLE | DUST | ((uint32_t)(max(src, 0) + 1) << 8) | (hash32(hk ^ 0x68e31da4u) & 0xffff8000u);
        e.z = rnd24(hash32(hk ^ 0xb5297a4du));
        s.pool[slot] = e;
    }
}
__global__ void k_speck_taken(PoolState* ps) {
    const uint32_t n = ps->total1, top = ps->top1;
    ps->top1 = n < top ? top - n : 0u;
    ps->hw1 += n > top ? n - top : 0u;
}

}  // namespace

void launch_spray(const DevScene& d, const ushort4* smooth, const DevOptics* opt, const SprayBufs& b,
                  const RenderClock* clock, uint32_t frame, uint32_t parity, float amount, bool makes, cudaStream_t st) {
    Spray s{d, smooth, opt, b.pool, b.stack, b.stack1, b.list, b.dcount, b.counts, b.flags, b.dfield, b.nspeck, b.ps, clock,
            frame, parity, amount, d.W, d.H};
    const int n = d.W * d.H;
    // this frame's foam and resting specks counted from nothing, the dust field laid anew
    // (mod.rs:1751-1754)
    cudaMemsetAsync(b.dcount + (size_t)parity * n, 0, (size_t)n * sizeof(uint32_t), st);
    cudaMemsetAsync(b.dcount + (size_t)(2 + parity) * n, 0, (size_t)n * sizeof(uint32_t), st);
    cudaMemsetAsync(b.dfield, 0, (size_t)4 * n * sizeof(int), st);
    const dim3 tiles((d.W + 15) / 16, (d.H + 15) / 16), block(16, 16);
    if (makes) {
        const int nb = (n + kScan - 1) / kScan;
        k_spray_count<<<tiles, block, 0, st>>>(s);
        k_spray_scan1<<<nb, kScan, 0, st>>>(b.counts, b.bsum, n);
        k_spray_scan2<<<1, kScan, 0, st>>>(b.bsum, nb, &b.ps->total);
        k_spray_scan3<<<nb, kScan, 0, st>>>(b.counts, b.bsum, n);
        k_spray_make<<<tiles, block, 0, st>>>(s);
        k_spray_taken<<<1, 1, 0, st>>>(b.ps, clock);
    }
    k_spray_move<<<(kPoolMax + 255) / 256, 256, 0, st>>>(s);
    k_spray_returns<<<1, kScan, 0, st>>>(s);
}

void launch_specks(const DevScene& d, const DevOptics* opt, const SprayBufs& b, uint32_t frame, uint32_t n_slots,
                   cudaStream_t st) {
    Spray s{d, nullptr, opt, b.pool, b.stack, b.stack1, b.list, b.dcount, b.counts, b.flags, b.dfield, b.nspeck, b.ps,
            nullptr, frame, 0u, 0.0f, d.W, d.H};
    const int n = (int)n_slots + 1, nb = (n + kScan - 1) / kScan;
    k_speck_count<<<(n + 255) / 256, 256, 0, st>>>(s, n_slots);
    k_spray_scan1<<<nb, kScan, 0, st>>>(b.nspeck, b.bsum, n);
    k_spray_scan2<<<1, kScan, 0, st>>>(b.bsum, nb, &b.ps->total1);
    k_spray_scan3<<<nb, kScan, 0, st>>>(b.nspeck, b.bsum, n);
    k_speck_emit<<<(n_slots + 255) / 256, 256, 0, st>>>(s, n_slots);
    k_speck_taken<<<1, 1, 0, st>>>(b.ps);
}

}  // namespace sprout

// The brush's emitters on the device: World::emit's sources (src/world.rs:609-727) with the
// geometry of src/brush.rs, computed, checked against the solids and admitted where the
// particles are, and queued into the particle slots without anything read back to the host.
//
// The reference runs these on the CPU: it builds the candidate positions (brush::Stream,
// brush::stroke, the rain cloud), reads back the live particles per cell of a window around
// the stroke (FluidSim::cell_counts, a blocking download, mod.rs:3350-3387), admits the
// candidates one by one against that room (brush::Admission) and queues what it admits
// (FluidSim::spawn). Here one kernel lays out the candidates in the reference's order, one
// block admits them in that order against the counts taken on the device, and a placement
// pass puts them into particle slots; the ids, the generator World::rand and the per-step
// cap of queued particles live on the device, so the host never waits.
//
// What the host still computes: the window (Admission::window), the stream's range of
// lattice indices and the paint lattice's bounds (a few scalar expressions), and an upper
// bound of what an emission can admit, for which it reserves fresh slots; reserved slots
// that no admitted particle takes are left dead, and what overflows the fresh slots takes
// dead slots as claim.comp hands them out (admission.cu).
#include <cuda_runtime.h>

#include <cstdint>

#include "dev_common.cuh"
#include "kernels.h"

namespace sprout {

namespace {

constexpr int EMIT_T = 1024;
constexpr double GOLDEN = 0.6180339887498949;   // brush.rs:58: 1 / golden ratio
constexpr float SPRAY_SPEED = 260.0f;           // brush.rs:121
constexpr float SPRAY_SPREAD = 0.25f;           // brush.rs:198
constexpr float SPRAY_SPEED_SPREAD = 0.25f;     // brush.rs:200
constexpr float RAIN_SPEED = 200.0f;            // brush.rs:129

// World::rand (world.rs:738-743): xorshift32, the top 24 bits as a fraction
DEV float world_rand(uint32_t& s) {
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    return (float)(s >> 8) / 16777216.0f;
}

// hypotf as the host's libm computes it: the double-precision sum of squares, rounded once
DEV float hyp(float a, float b) { return (float)sqrt((double)a * (double)a + (double)b * (double)b); }

// World::solid_distance (world.rs:208-220): the node field interpolated bilinearly
DEV float solid_distance(const float* sdf, int W, int H, float px, float py) {
    const int nw = W + 1;
    const float x = fminf(fmaxf(px, 0.0f), (float)W - 1e-3f);
    const float y = fminf(fmaxf(py, 0.0f), (float)H - 1e-3f);
    const int i = (int)x, j = (int)y;
    const float fx = x - (float)i, fy = y - (float)j;
    const float bottom = sdf[j * nw + i] * (1.0f - fx) + sdf[j * nw + i + 1] * fx;
    const float top = sdf[(j + 1) * nw + i] * (1.0f - fx) + sdf[(j + 1) * nw + i + 1] * fx;
    return bottom * (1.0f - fy) + top * fy;
}

// brush.rs:155-164: the offset of p from the nearest point of the segment from-to
DEV float2 offset_from_stroke(float px, float py, const EmitArgs& a, float length2) {
    const float dx = a.to[0] - a.from[0], dy = a.to[1] - a.from[1];
    float t = 0.0f;
    if (length2 > 0.0f) t = fminf(fmaxf(((px - a.from[0]) * dx + (py - a.from[1]) * dy) / length2, 0.0f), 1.0f);
    return make_float2(px - a.from[0] - t * dx, py - a.from[1] - t * dy);
}

// sin and cos of |x| <= SPRAY_SPREAD from their Taylor series in FP64 (terms to x^15, far
// below FP32's resolution there), each rounded once to FP32; the tests' restatement
// evaluates the same terms in the same order
DEV void sincos_spread(float xf, float* s, float* c) {
    const double x = (double)xf, x2 = x * x;
    double sn = 1.0 / 1307674368000.0;   // 1 / 15!
    sn = 1.0 / 6227020800.0 - x2 * sn;   // 1 / 13!
    sn = 1.0 / 39916800.0 - x2 * sn;
    sn = 1.0 / 362880.0 - x2 * sn;
    sn = 1.0 / 5040.0 - x2 * sn;
    sn = 1.0 / 120.0 - x2 * sn;
    sn = 1.0 / 6.0 - x2 * sn;
    sn = x - x * x2 * sn;
    double cs = 1.0 / 20922789888000.0;   // 1 / 16!
    cs = 1.0 / 87178291200.0 - x2 * cs;   // 1 / 14!
    cs = 1.0 / 479001600.0 - x2 * cs;
    cs = 1.0 / 3628800.0 - x2 * cs;
    cs = 1.0 / 40320.0 - x2 * cs;
    cs = 1.0 / 720.0 - x2 * cs;
    cs = 1.0 / 24.0 - x2 * cs;
    cs = 0.5 - x2 * cs;
    cs = 1.0 - x2 * cs;
    *s = (float)sn;
    *c = (float)cs;
}

// Candidate positions in the reference's order, flag 1 where the candidate exists:
// - stream (brush.rs:86-115): lattice index k0 + m; it exists where it appears during the frame;
// - paint (brush.rs:134-153): lattice point m of the stroke's bounds, row by row; it exists
//   inside the swept disk.
__global__ void k_emit_candidates(EmitArgs a, float2* cand, uint8_t* flag) {
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= a.ncand) return;
    float2 p = make_float2(0.0f, 0.0f);
    uint8_t on = 0;
    if (a.mode == EMIT_STREAM) {
        const uint64_t k = a.k0 + m;
        const float half = 0.5f * a.width;
        const float across = ((float)((double)k * GOLDEN - floor((double)k * GOLDEN)) - 0.5f) * a.width;
        const float arc = sqrtf(fmaxf(half * half - across * across, 0.0f));
        const double appears = ((double)k + 0.5) / a.rate + (double)((half - arc) / a.speed);
        if (!(appears < a.start || appears >= a.end)) {
            const float t = (float)((appears - a.start) / (a.end - a.start));
            const float along = (float)(a.end - appears) * a.speed - arc;
            const float sx = -a.dir[1], sy = a.dir[0];
            p.x = a.from[0] + (a.to[0] - a.from[0]) * t + sx * across + a.dir[0] * along;
            p.y = a.from[1] + (a.to[1] - a.from[1]) * t + sy * across + a.dir[1] * along;
            on = 1;
        }
    } else if (a.mode == EMIT_PAINT) {
        const int nx = a.lat_hi[0] - a.lat_lo[0];
        const int x = a.lat_lo[0] + (int)(m % (uint32_t)nx), y = a.lat_lo[1] + (int)(m / (uint32_t)nx);
        p = make_float2(((float)x + 0.5f) * a.spacing, ((float)y + 0.5f) * a.spacing);
        const float dx = a.to[0] - a.from[0], dy = a.to[1] - a.from[1];
        const float2 d = offset_from_stroke(p.x, p.y, a, dx * dx + dy * dy);
        on = d.x * d.x + d.y * d.y <= a.radius * a.radius ? 1 : 0;
    }
    cand[m] = p;
    flag[m] = on;
}

// The admission, in one block: the room of each window cell (Admission::new, brush.rs:213-
// 217) from the live particles counted in it, then the candidates in order by one thread
// (each takes room in its cell, brush.rs:227-238, after the solid test and the spray's or the
// rain's draws of World::rand, as World::paint / rain / stream take them), the admitted ones
// written to the queue q with the next ids; the state's generator, ids, queue count and
// fastest admitted speed advanced.
__global__ void __launch_bounds__(EMIT_T) k_emit_admit(EmitArgs a, const float2* cand, const uint8_t* flag,
                                                      uint32_t* room, const float* sdf, float4* q, EmitState* st,
                                                      StepState* S) {
    const int nwin = a.win_size[0] * a.win_size[1];
    const uint32_t full = (uint32_t)((float)a.ppc * 1.5f);   // STREAM_FILL, brush.rs:11
    for (int c = threadIdx.x; c < nwin; c += EMIT_T) {
        const uint32_t n = room[c];   // the counts, turned into room in place
        room[c] = a.mode == EMIT_STREAM ? (full > n ? full - n : 0u) : (n == 0u ? (uint32_t)a.ppc : 0u);
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    uint32_t rng = st->rng;
    const uint32_t queued = st->queued;
    // room left in the queue this step (FluidSim::spawn, mod.rs:2028)
    const uint32_t cap = a.limit > queued ? a.limit - queued : 0u;
    uint32_t nq = 0;
    float fastest = 0.0f;
    auto admit = [&](float px, float py) {
        const int cx = (int)floorf(px) - a.win_lo[0], cy = (int)floorf(py) - a.win_lo[1];
        if (cx < 0 || cy < 0 || cx >= a.win_size[0] || cy >= a.win_size[1]) return false;
        uint32_t& r = room[cy * a.win_size[0] + cx];
        if (r == 0u) return false;
        r -= 1u;
        return true;
    };
    auto push = [&](float px, float py, float vx, float vy) {
        // Particle::new + FluidSim::spawn's settle_spawn (the template) and the engine's
        // position range; KIND_FRESH
        float4* o = q + 3 * (size_t)nq;
        const float x = fminf(fmaxf(px, 2.01f), (float)a.W - 2.01f), y = fminf(fmaxf(py, 2.01f), (float)a.H - 2.01f);
        o[0] = make_float4(x, y, vx, vy);
        o[1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        o[2] = make_float4(a.s, __uint_as_float(a.kind | KIND_FRESH), __uint_as_float(st->next_id + nq), a.t);
        fastest = fmaxf(fastest, hyp(vx, vy));
        nq++;
    };
    if (a.mode == EMIT_STREAM) {
        // the candidates that exist, of which the last `keep` (Stream::advance's limit)
        uint32_t exist = 0;
        for (uint32_t m = 0; m < a.ncand; m++) exist += flag[m];
        uint32_t skip = exist > a.keep ? exist - a.keep : 0u;
        for (uint32_t m = 0; m < a.ncand && nq < cap; m++) {
            if (!flag[m]) continue;
            if (skip) {
                skip--;
                continue;
            }
            const float2 p = cand[m];
            if (solid_distance(sdf, a.W, a.H, p.x, p.y) > 0.4f && admit(p.x, p.y)) push(p.x, p.y, a.vel[0], a.vel[1]);
        }
    } else if (a.mode == EMIT_PAINT) {
        // the lattice points inside the stroke as a list of their indices (after the window's
        // room in the same buffer)
        uint32_t* list = reinterpret_cast<uint32_t*>(room + nwin);
        uint32_t n = 0;
        for (uint32_t m = 0; m < a.ncand; m++)
            if (flag[m]) list[n++] = m;
        // World::paint's shuffle (world.rs:651-656)
        for (uint32_t i = n; i-- > 1;) {
            const uint32_t j = min((uint32_t)(world_rand(rng) * (float)(i + 1)), i);
            const uint32_t tmp = list[i];
            list[i] = list[j];
            list[j] = tmp;
        }
        const float dx = a.to[0] - a.from[0], dy = a.to[1] - a.from[1];
        const float length2 = dx * dx + dy * dy;
        for (uint32_t k = 0; k < n && nq < a.count && nq < cap; k++) {
            float2 p = cand[list[k]];
            if (a.spray) {
                const float jx = world_rand(rng), jy = world_rand(rng);
                p.x = p.x + (jx - 0.5f) * 0.6f * a.spacing;
                p.y = p.y + (jy - 0.5f) * 0.6f * a.spacing;
            }
            if (solid_distance(sdf, a.W, a.H, p.x, p.y) <= 0.4f) continue;
            float vx = 0.0f, vy = 0.0f;
            if (a.spray) {
                const float j0 = world_rand(rng), j1 = world_rand(rng);
                // brush::spray_velocity (brush.rs:177-193)
                const float2 off = offset_from_stroke(p.x, p.y, a, length2);
                const float dist = hyp(off.x, off.y);
                if (dist < a.radius * 0.7f || dist < 1e-4f) continue;
                float sn, cs;
                sincos_spread((j0 * 2.0f - 1.0f) * SPRAY_SPREAD, &sn, &cs);
                const float speed = SPRAY_SPEED * (1.0f + (j1 * 2.0f - 1.0f) * SPRAY_SPEED_SPREAD);
                const float nx = off.x / dist, ny = off.y / dist;
                vx = (nx * cs - ny * sn) * speed;
                vy = (nx * sn + ny * cs) * speed;
            }
            if (!admit(p.x, p.y)) continue;
            push(p.x, p.y, vx, vy);
        }
    } else {   // EMIT_RAIN (world.rs:689-710)
        for (uint32_t k = 0; k < a.count && nq < cap; k++) {
            const float rx = world_rand(rng), ry = world_rand(rng);
            const float px = a.at[0] + (rx * 2.0f - 1.0f) * a.half, py = a.at[1] + (ry * 2.0f - 1.0f) * 2.0f;
            if (solid_distance(sdf, a.W, a.H, px, py) <= 0.4f || !admit(px, py)) continue;
            const float speed = RAIN_SPEED * (0.8f + 0.4f * world_rand(rng));
            const float vx = (world_rand(rng) - 0.5f) * 12.0f;
            push(px, py, vx, -speed);
        }
    }
    st->rng = rng;
    st->next_id += nq;
    st->queued = queued + nq;
    st->count = nq;
    st->total += nq;
    // FluidSim::spawn's spawn_speed: the next step call's CFL limit takes it (mod.rs:2300)
    if (nq) S->emit_speed = fmaxf(S->emit_speed, fastest);
}

// The placement: queue entry r goes to fresh slot base + r while r < fresh, the rest of the
// fresh slots reserved for this emission are left dead; entries past `fresh` go to dead
// slots (k_emit_claim).
__global__ void k_emit_fresh(float4* part, uint32_t base, uint32_t fresh, const float4* q, const EmitState* st) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= fresh) return;
    float4* o = part + 3 * (size_t)(base + r);
    if (r < st->count) {
        o[0] = q[3 * (size_t)r + 0];
        o[1] = q[3 * (size_t)r + 1];
        o[2] = q[3 * (size_t)r + 2];
    } else {
        o[0] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        o[1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        o[2] = make_float4(0.0f, __uint_as_float(KIND_DEAD), 0.0f, 0.0f);
    }
}

// Ids of particles queued by the host (FluidSim::spawn's next_id + k), once the device holds
// the ids: the n particles at part[base ..] (fresh slots) and q[0 ..] (entries that claim dead
// slots) take next_id + k in queue order; the state's next_id and queue count advance.
__global__ void k_spawn_ids(float4* part, uint32_t base, uint32_t fresh, float4* q, uint32_t n, EmitState* st) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t id0 = st->next_id;
    if (k < n) {
        float4* o = k < fresh ? part + 3 * (size_t)(base + k) : q + 3 * (size_t)(k - fresh);
        o[2].z = __uint_as_float(id0 + k);
    }
}
__global__ void k_spawn_ids_done(EmitState* st, uint32_t n) {
    st->next_id += n;
    st->queued += n;
}

}  // namespace

void launch_emit(const EmitArgs& a, float2* cand, uint8_t* flag, uint32_t* room, const float* sdf, float4* q,
                 EmitState* st, StepState* S, cudaStream_t s) {
    if (a.ncand) k_emit_candidates<<<(a.ncand + 255) / 256, 256, 0, s>>>(a, cand, flag);
    k_emit_admit<<<1, EMIT_T, 0, s>>>(a, cand, flag, room, sdf, q, st, S);
}

void launch_emit_fresh(float4* part, uint32_t base, uint32_t fresh, const float4* q, const EmitState* st,
                       cudaStream_t s) {
    if (fresh) k_emit_fresh<<<(fresh + 255) / 256, 256, 0, s>>>(part, base, fresh, q, st);
}

void launch_spawn_ids(float4* part, uint32_t base, uint32_t fresh, float4* q, uint32_t n, EmitState* st,
                      cudaStream_t s) {
    if (!n) return;
    k_spawn_ids<<<(n + 255) / 256, 256, 0, s>>>(part, base, fresh, q, n, st);
    k_spawn_ids_done<<<1, 1, 0, s>>>(st, n);
}

}  // namespace sprout

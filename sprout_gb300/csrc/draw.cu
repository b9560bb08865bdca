// The renderer's particle fields (Renderer::render, src/render.rs:886-1075) and the wet map
// (render.rs:640-668, shaders/wet.frag) as kernels into headless device images, for one view
// (centre, zoom in pixels per cell, extent in pixels):
//   k_splat       splat.vert + splat.frag (the sharp field: each phase group's weight times
//                 the kernel), splat.vert + tint.frag (the tint field: absorption and
//                 scattering, concentrate share, aqueous and other weight), and look.vert +
//                 look.frag (the look field of the particles look.comp listed: their
//                 platelets' sheen, carried scalar, which way they lie, and weight)
//   k_fields_out  the texel sums to RGBA16F, the sums cleared for the next draw
//   k_down        down.frag: the box filter of bilinear taps into the wide field
//   k_blur        blur.frag: one direction of the 13-tap Gaussian of the wide field
//   k_wet         wet.frag: the liquid that last lay against a solid, per cell
// The reference rasterises one triangle per particle and blends additively into RGBA16F
// targets, in an order the hardware picks. Here a thread takes a particle, finds the texels
// whose centres lie inside its kernel from the same affine map the triangle interpolates
// (uv = the position's coordinates along the particle's path and across it, in kernel radii),
// and adds kernel x weight to 64-bit fixed-point texel sums (2^-32, integer atomics): the sum
// is the same whatever order the particles land in, and is rounded to half once.
#include <cuda_fp16.h>

#include <climits>

#include "dev_common.cuh"
#include "kernels.h"

namespace sprout {

namespace {

constexpr float kFix = 4294967296.0f;   // 2^32
constexpr double kUnfix = 1.0 / 4294967296.0;
constexpr uint32_t kRowSteam = 57u;     // common.glsl ROW_STEAM
constexpr float kStreakMax = 1.5f;      // splat.vert STREAK_MAX, kernel radii
constexpr float kReach = 1.75f;         // wet.frag REACH, cells
constexpr float kWetting = 0.3f;        // wet.frag WETTING

DEV int clampi_(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
DEV float minf_(float a, float b) { return a < b ? a : b; }
DEV float maxf_(float a, float b) { return a > b ? a : b; }
DEV float clampf_(float v, float lo, float hi) { return minf_(maxf_(v, lo), hi); }
DEV long long fix(float v) { return __float2ll_rn(v * kFix); }
DEV void add_fix(long long* p, float v) {
    const long long q = fix(v);
    if (q != 0) atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)q);
}
DEV float unfix(long long s) { return (float)((double)s * kUnfix); }
DEV ushort4 half4(float a, float b, float c, float d) {
    return make_ushort4(__half_as_ushort(__float2half_rn(a)), __half_as_ushort(__float2half_rn(b)),
                        __half_as_ushort(__float2half_rn(c)), __half_as_ushort(__float2half_rn(d)));
}
DEV float4 unhalf4(ushort4 v) {
    return make_float4(__half2float(__ushort_as_half(v.x)), __half2float(__ushort_as_half(v.y)),
                       __half2float(__ushort_as_half(v.z)), __half2float(__ushort_as_half(v.w)));
}

// The bilinear sample of a used region of w x h texels at (x, y) in texel units (a texel's
// centre at i + 0.5), clamped to its edge: (1 - fy) ((1 - fx) t00 + fx t10) + fy ((1 - fx) t01
// + fx t11), channel by channel in that order.
DEV float4 bilinear(const ushort4* img, int w, int h, float x, float y) {
    const float xs = x - 0.5f, ys = y - 0.5f;
    const float xf = floorf(xs), yf = floorf(ys);
    const float fx = xs - xf, fy = ys - yf;
    const int x0 = clampi_((int)xf, 0, w - 1), x1 = clampi_((int)xf + 1, 0, w - 1);
    const int y0 = clampi_((int)yf, 0, h - 1), y1 = clampi_((int)yf + 1, 0, h - 1);
    const float4 a = unhalf4(img[(size_t)y0 * w + x0]), b = unhalf4(img[(size_t)y0 * w + x1]);
    const float4 c = unhalf4(img[(size_t)y1 * w + x0]), e = unhalf4(img[(size_t)y1 * w + x1]);
    const float gx = 1.0f - fx, gy = 1.0f - fy;
    return make_float4(gy * (gx * a.x + fx * b.x) + fy * (gx * c.x + fx * e.x),
                       gy * (gx * a.y + fx * b.y) + fy * (gx * c.y + fx * e.y),
                       gy * (gx * a.z + fx * b.z) + fy * (gx * c.z + fx * e.z),
                       gy * (gx * a.w + fx * b.w) + fy * (gx * c.w + fx * e.w));
}

// splat.vert + splat.frag / tint.frag for particle slot id. A texel (i, j) of the image sits at
// (cx + ((i + 0.5) div - half_w) / zoom, cy - ((j + 0.5) div - half_h) / zoom) in cells (the
// view's map, y up); its uv is the position relative to the kernel's centre along the path
// over `along` and across it over the radius; inside the unit disc it takes (1 - |uv|^2)^2.
struct Splat {
    float ex, ey, dx, dy, along, ialong;
    int i0, i1, j0, j1;   // the texels it may reach (empty: i1 < i0)
    int ch0, nch;
    float c[7];           // what it lays down per unit kernel, channels ch0 ..
};

DEV Splat splat_of(const DevScene& d, const DevOptics* opt, uint32_t id, const DrawPass& v) {
    Splat sp;
    sp.i0 = 0, sp.i1 = -1, sp.j0 = 0, sp.j1 = -1, sp.ch0 = 0, sp.nch = 0;
    const float4 q0 = d.part[3 * id + 0], q2 = d.part[3 * id + 2];
    const uint32_t kind = __float_as_uint(q2.y), low = kind & 255u;
    // look.vert draws every listed slot as a disc about the particle (no streak)
    const bool look = v.mode == 2;
    if (!look && (low == 0u || (v.mode == 1 && low - 1u == kRowSteam))) return sp;
    const uint32_t row = low - 1u;
    const float speed = look ? 0.0f : sqrtf(q0.z * q0.z + q0.w * q0.w);
    sp.dx = speed > 1e-3f ? q0.z / speed : 1.0f;
    sp.dy = speed > 1e-3f ? q0.w / speed : 0.0f;
    const float streak = minf_(speed * v.exposure, kStreakMax * v.radius);
    sp.along = v.radius + 0.5f * streak;
    sp.ialong = 1.0f / sp.along;
    sp.ex = q0.x - sp.dx * (0.5f * streak);
    sp.ey = q0.y - sp.dy * (0.5f * streak);
    // the texels whose centres can lie within `along` of the centre (none farther is inside)
    const float tx0 = ((sp.ex - sp.along - v.cx) * v.zoom + v.half_w) / v.div, tx1 = ((sp.ex + sp.along - v.cx) * v.zoom + v.half_w) / v.div;
    const float ty0 = (-(sp.ey + sp.along - v.cy) * v.zoom + v.half_h) / v.div, ty1 = (-(sp.ey - sp.along - v.cy) * v.zoom + v.half_h) / v.div;
    if (!(tx1 >= -1.0f && ty1 >= -1.0f && tx0 <= (float)v.w + 1.0f && ty0 <= (float)v.h + 1.0f)) return sp;
    sp.i0 = (int)maxf_(floorf(tx0) - 1.0f, 0.0f), sp.i1 = (int)minf_(ceilf(tx1) + 1.0f, (float)(v.w - 1));
    sp.j0 = (int)maxf_(floorf(ty0) - 1.0f, 0.0f), sp.j1 = (int)minf_(ceilf(ty1) + 1.0f, (float)(v.h - 1));
    if (look) {
        // the platelets' sheen H.A.H over their packed second moment A, the carried scalar,
        // which way they lie in the plane (A_xx - A_yy about 0.5), and the weight
        const uint4 st = d.plook[id];
        const float ax = (float)(st.z & 1023u) / 1023.0f, ay = (float)((st.z >> 10) & 1023u) / 1023.0f;
        const float az = (float)((st.z >> 20) & 1023u) / 1023.0f - 0.5f;
        const float sheen = v.hx * v.hx * ax + v.hy * v.hy * ay + 2.0f * v.hx * v.hy * az + v.hz * v.hz * (1.0f - ax - ay);
        const float phi = (float)(st.w & 0xffffu) / 65535.0f;
        const float lie = clampf_(0.5f + (ax - ay), 0.0f, 1.0f);
        sp.nch = 4;
        sp.c[0] = sheen * v.weight;
        sp.c[1] = phi * v.weight;
        sp.c[2] = lie * v.weight;
        sp.c[3] = 1.0f * v.weight;
    } else if (v.mode == 0) {
        sp.ch0 = clampi_(d.mats[row].ia[0], 0, 3);
        sp.nch = 1;
        sp.c[0] = v.weight;
    } else {
        const DevOptics& o = opt[row];
        const float s = o.idx[0] >= 0 ? clampf_(q2.x, 0.0f, 1.0f) : 0.0f;
        const float* kc = o.absorb;
        const float* kp = o.idx[0] >= 0 ? opt[o.idx[0]].absorb : o.absorb;
        const float w = row == kRowSteam ? 0.0f : v.weight;
        if (o.idx[1] == 0) {
            sp.c[0] = (s * kc[0]) * w;
            sp.c[1] = (s * kc[1]) * w;
            sp.c[2] = (s * kc[2]) * w;
            sp.c[3] = (s * kc[3] + (1.0f - s) * kp[3]) * w;
            sp.c[4] = s * w;
            sp.c[5] = 1.0f * w;
            sp.c[6] = 0.0f * w;
        } else {
            sp.c[0] = kc[0] * w;
            sp.c[1] = kc[1] * w;
            sp.c[2] = kc[2] * w;
            sp.c[3] = kc[3] * w;
            sp.c[4] = 0.0f * w;
            sp.c[5] = 0.0f * w;
            sp.c[6] = w;
        }
        sp.nch = 7;
    }
    return sp;
}

// A 64-bit sum in shared memory as two 32-bit words (low, high), added to with the native
// 32-bit atomics: the low word's carry goes to the high word (mod 2^64, as a 64-bit add).
DEV void add_fix_shared(uint32_t* w, float v) {
    const unsigned long long u = (unsigned long long)fix(v);
    if (u == 0ull) return;
    const uint32_t lo = (uint32_t)u, hi = (uint32_t)(u >> 32);
    const uint32_t old = atomicAdd(w, lo);
    const uint32_t up = hi + ((uint32_t)(old + lo) < old ? 1u : 0u);
    if (up != 0u) atomicAdd(w + 1, up);
}
DEV void add_fix(uint32_t* w, float v) { add_fix_shared(w, v); }

// The particle's kernel x payload into sums laid out as `pitch` texels a row from texel
// (oi, oj), `stride` sums a texel: 64-bit words in global memory, or word pairs in shared.
template <class Acc, int kWords>
DEV void splat_into(const Splat& sp, const DrawPass& v, Acc* acc, int oi, int oj, int pitch, int stride, int ch0) {
    for (int j = sp.j0; j <= sp.j1; j++) {
        const float py = v.cy - (((float)j + 0.5f) * v.div - v.half_h) * v.izoom;
        for (int i = sp.i0; i <= sp.i1; i++) {
            const float px = v.cx + (((float)i + 0.5f) * v.div - v.half_w) * v.izoom;
            const float rx = px - sp.ex, ry = py - sp.ey;
            const float u = (rx * sp.dx + ry * sp.dy) * sp.ialong, w2 = (ry * sp.dx - rx * sp.dy) * v.iradius;
            const float r2 = u * u + w2 * w2;
            if (r2 >= 1.0f) continue;
            const float k = (1.0f - r2) * (1.0f - r2);
            Acc* t = acc + (((size_t)(j - oj) * pitch + (i - oi)) * stride + ch0) * kWords;
#pragma unroll
            for (int q = 0; q < 7; q++)
                if (q < sp.nch) add_fix(t + q * kWords, sp.c[q] * k);
        }
    }
}

// A block takes 256 consecutive slots. Sorted by cell, they mostly sit along a short run of
// cells, so the block sums them over the texels their kernels reach in shared memory first
// (one word a texel when they all lay down one channel, the sharp field of one phase group)
// and adds each texel's non-zero sums to the image's once; where that run of texels does not
// fit (a block across two rows of cells, a close view), each particle adds to the image
// directly. Integer sums: the same either way.
constexpr int kSplatSmemWords = 3072;   // 24 KB: five blocks of 256 threads still fit an SM
__global__ void __launch_bounds__(256) k_splat(DevScene d, const DevOptics* opt, uint32_t n_slots, DrawPass v,
                                               const uint32_t* list, long long* acc) {
    __shared__ uint32_t sacc[2 * kSplatSmemWords];
    __shared__ int box[6];
    const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    Splat sp;
    const uint32_t n = list ? list[0] : n_slots;
    if (id < n) sp = splat_of(d, opt, list ? list[1 + id] : id, v);
    else sp.i0 = 0, sp.i1 = -1, sp.j0 = 0, sp.j1 = -1, sp.ch0 = 0, sp.nch = 0;
    if (threadIdx.x == 0) box[0] = box[1] = box[4] = INT_MAX, box[2] = box[3] = box[5] = INT_MIN;
    __syncthreads();
    const bool any = sp.i1 >= sp.i0 && sp.j1 >= sp.j0;
    if (any) {
        atomicMin(&box[0], sp.i0);
        atomicMin(&box[1], sp.j0);
        atomicMax(&box[2], sp.i1);
        atomicMax(&box[3], sp.j1);
        atomicMin(&box[4], sp.ch0);
        atomicMax(&box[5], sp.ch0);
    }
    __syncthreads();
    if (box[2] < box[0]) return;   // nothing of the block's in view
    const int stride = v.mode == 1 ? 8 : 4;
    const bool one = v.mode == 0 && box[4] == box[5];
    const int sstride = one ? 1 : stride;
    const int bw = box[2] - box[0] + 1, bh = box[3] - box[1] + 1;
    const long long words = (long long)bw * bh * sstride;
    if (words > kSplatSmemWords) {
        if (any) splat_into<long long, 1>(sp, v, acc, 0, 0, v.w, stride, sp.ch0);
        return;
    }
    for (int k = threadIdx.x; k < 2 * (int)words; k += blockDim.x) sacc[k] = 0u;
    __syncthreads();
    if (any) splat_into<uint32_t, 2>(sp, v, sacc, box[0], box[1], bw, sstride, one ? 0 : sp.ch0);
    __syncthreads();
    for (int k = threadIdx.x; k < (int)words; k += blockDim.x) {
        const unsigned long long q = ((unsigned long long)sacc[2 * k + 1] << 32) | sacc[2 * k];
        if (q == 0ull) continue;
        const int t = k / sstride, c = one ? box[4] : k - t * sstride;
        const int ty = t / bw, tx = t - ty * bw;
        atomicAdd(reinterpret_cast<unsigned long long*>(acc + ((size_t)(box[1] + ty) * v.w + box[0] + tx) * stride + c),
                  q);
    }
}

// The texel sums of a pass to RGBA16F (the tint field's to its two images), cleared after.
__global__ void __launch_bounds__(256) k_fields_out(long long* acc, int n, int tint, ushort4* a, ushort4* b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    long long* s = acc + (size_t)i * (tint ? 8 : 4);
    a[i] = half4(unfix(s[0]), unfix(s[1]), unfix(s[2]), unfix(s[3]));
    if (tint) b[i] = half4(unfix(s[4]), unfix(s[5]), unfix(s[6]), 0.0f);
    for (int q = 0; q < (tint ? 8 : 4); q++) s[q] = 0;
}

// down.frag: wide texel (i, j) averages taps x taps bilinear samples of the sharp field around
// (i + 0.5, j + 0.5) x factor (its texels per wide texel), each held to the last used texel.
__global__ void __launch_bounds__(256) k_down(const ushort4* src, int sw, int sh, ushort4* dst, int dw, int dh,
                                              float factor, int taps) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= dw * dh) return;
    const int y = i / dw, x = i - y * dw;
    const float cx = ((float)x + 0.5f) * factor, cy = ((float)y + 0.5f) * factor;
    const float mx = (float)sw - 0.5f, my = (float)sh - 0.5f;
    float4 sum = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int tj = 0; tj < taps; tj++)
        for (int ti = 0; ti < taps; ti++) {
            const float ox = (((float)ti + 0.5f) / (float)taps - 0.5f) * factor;
            const float oy = (((float)tj + 0.5f) / (float)taps - 0.5f) * factor;
            const float4 s = bilinear(src, sw, sh, minf_(cx + ox, mx), minf_(cy + oy, my));
            sum.x += s.x;
            sum.y += s.y;
            sum.z += s.z;
            sum.w += s.w;
        }
    const float n = (float)(taps * taps);
    dst[i] = half4(sum.x / n, sum.y / n, sum.z / n, sum.w / n);
}

// blur.frag: one direction (vertical when vert) of the 13-tap Gaussian exp(-(k / 2)^2 / 2),
// taps `step` texels apart, each held inside the used texels (the liquid carries on past the
// edge of the view as it is at the edge).
__global__ void __launch_bounds__(256) k_blur(const ushort4* src, ushort4* dst, int w, int h, float step, int vert) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    const float G[7] = {1.0f, 0.8825f, 0.6065f, 0.3247f, 0.1353f, 0.0439f, 0.0111f};
    const int y = i / w, x = i - y * w;
    const float px = (float)x + 0.5f, py = (float)y + 0.5f;
    const float lo = 0.5f, hx = (float)w - 0.5f, hy = (float)h - 0.5f;
    const float4 c = bilinear(src, w, h, px, py);
    float4 sum = make_float4(G[0] * c.x, G[0] * c.y, G[0] * c.z, G[0] * c.w);
    float norm = G[0];
    for (int k = 1; k < 7; k++) {
        const float o = (float)k * step;
        const float4 a = vert ? bilinear(src, w, h, px, clampf_(py + o, lo, hy)) : bilinear(src, w, h, clampf_(px + o, lo, hx), py);
        const float4 b = vert ? bilinear(src, w, h, px, clampf_(py - o, lo, hy)) : bilinear(src, w, h, clampf_(px - o, lo, hx), py);
        sum.x += G[k] * (a.x + b.x);
        sum.y += G[k] * (a.y + b.y);
        sum.z += G[k] * (a.z + b.z);
        sum.w += G[k] * (a.w + b.w);
        norm += 2.0f * G[k];
    }
    dst[i] = half4(sum.x / norm, sum.y / norm, sum.z / norm, sum.w / norm);
}

// The wet map's clock: whether the simulated time moved since the map was last written (the
// reference writes it once per (tank, simulated time), render.rs:644-651).
__global__ void k_wet_clock(const StepState* S, WetClock* c) {
    const double now = (double)S->advanced - (double)__uint_as_float(S->pad0);
    c->run = (!c->valid || now != c->last) ? 1u : 0u;
    c->now = (float)now;
    c->last = now;
    c->valid = 1u;
}

// wet.frag: a cell close to a solid (the mean of its four nodes' distances at most REACH) and
// held by liquid (occupancy at least WETTING) records its leading material (table row + 1),
// family 0's concentration and the time; every other texel keeps what it had.
__global__ void __launch_bounds__(256) k_wet(DevScene d, const WetClock* c, float4* wet) {
    if (!c->run) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.W * d.H) return;
    const int y = i / d.W, x = i - y * d.W;
    const int w1 = d.W + 1, k = y * w1 + x;
    const float dist = 0.25f * (d.sdf[k] + d.sdf[k + 1] + d.sdf[k + w1] + d.sdf[k + w1 + 1]);
    if (dist > kReach || d.cell[i].x < kWetting) return;
    const float sw = d.sprop[i].w;
    const float code = floorf((sw - floorf(sw)) * 128.0f + 0.5f);
    if (code < 1.0f) return;
    wet[i] = make_float4(code, d.comp[i].z, c->now, 1.0f);
}

}  // namespace

void launch_draw(const DevScene& d, const DevOptics* opt, uint32_t n_slots, const DrawPass& sharp, const DrawPass* tint,
                 const DrawPass* look, const uint32_t* look_list, const DrawWide& wide, DrawBufs& b, cudaStream_t st) {
    const uint32_t nb = (n_slots + 255u) / 256u;
    if (n_slots > 0) k_splat<<<nb, 256, 0, st>>>(d, opt, n_slots, sharp, nullptr, b.acc);
    const int na = sharp.w * sharp.h;
    k_fields_out<<<(na + 255) / 256, 256, 0, st>>>(b.acc, na, 0, b.sharp, nullptr);
    if (look) {   // into the same sums, which k_fields_out left cleared
        if (n_slots > 0) k_splat<<<nb, 256, 0, st>>>(d, opt, n_slots, *look, look_list, b.acc);
        k_fields_out<<<(na + 255) / 256, 256, 0, st>>>(b.acc, na, 0, b.look, nullptr);
    }
    if (tint) {
        if (n_slots > 0) k_splat<<<nb, 256, 0, st>>>(d, opt, n_slots, *tint, nullptr, b.tacc);
        const int nt = tint->w * tint->h;
        k_fields_out<<<(nt + 255) / 256, 256, 0, st>>>(b.tacc, nt, 1, b.conc, b.share);
    }
    const int nw = wide.w * wide.h;
    k_down<<<(nw + 255) / 256, 256, 0, st>>>(b.sharp, sharp.w, sharp.h, b.wide0, wide.w, wide.h, wide.factor, wide.taps);
    k_blur<<<(nw + 255) / 256, 256, 0, st>>>(b.wide0, b.wide1, wide.w, wide.h, wide.step, 0);
    k_blur<<<(nw + 255) / 256, 256, 0, st>>>(b.wide1, b.wide0, wide.w, wide.h, wide.step, 1);
}

void launch_wet(const DevScene& d, WetClock* clock, float4* wet, cudaStream_t st) {
    k_wet_clock<<<1, 1, 0, st>>>(d.S, clock);
    const int n = d.W * d.H;
    k_wet<<<(n + 255) / 256, 256, 0, st>>>(d, clock, wet);
}

}  // namespace sprout

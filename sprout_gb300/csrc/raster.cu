// Scene::rasterize (src/scene.rs:215-470) on the device: node distances of the walls and
// shapes, the union depth inside the solids, open volumes, sealing of small enclosed pockets,
// face open fractions, smoothed solid occupancy, regions with their vents and the held
// temperatures. The arithmetic is the host restatement's (scene.cpp), expression for
// expression, so the fields are bit-identical to it; the structure is the device's own:
// - node and cell passes: one thread per node or cell;
// - union_depth's two chamfer sweeps: a diagonal wavefront, one thread per node row, node
//   (i, j) of the forward sweep at step i + 2 j (its left neighbour one step earlier, the
//   row below up to three steps earlier), so every relaxation reads the values the
//   sequential sweep reads; the backward sweep mirrored;
// - connected components (pockets, regions): union-find by atomicMin on labels, every
//   component rooted at its smallest cell index, which is the cell the host's sequential
//   fill starts it from; region ids are the roots' ranks in index order.
// Sealing a pocket lowers its corner nodes, which can close a face of a neighbouring
// component the host fills later: where a sealed pocket shares a node with another open
// component (rare: a pocket against the liquid side of a thin solid) the pockets are sealed
// by the host's sequential algorithm instead, run by one device thread.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "dev_common.cuh"
#include "kernels.h"
#include "scene.h"

namespace sprout {

namespace {

constexpr float kWallR = 3.0f;
constexpr float kNoTempR = -1e9f;
constexpr float kFar = 1e9f;
constexpr uint32_t kNone = 0xffffffffu;

struct DevShape {
    int kind;              // 0 circle, 1 box
    float cx, cy, hx, hy, r, sn, cs;
    int i0, i1, j0, j1;    // the nodes it touches (inclusive)
    int t0, t1, u0, u1;    // the cells it may hold at its temperature ([t0, t1) x [u0, u1))
    int held;
    float temp;
};

// std::min / std::max as the host evaluates them (the selects decide which zero comes back
// when +0 and -0 meet, where the fmin / fmax instructions may differ)
DEV float smin(float a, float b) { return b < a ? b : a; }
DEV float smax(float a, float b) { return a < b ? b : a; }

// hypotf as the host's libm computes it: the double-precision sum of squares, rounded once
// (checked against glibc's hypotf over 2e8 random pairs; the GPU test compares the fields)
DEV float hyp(float a, float b) { return (float)sqrt((double)a * (double)a + (double)b * (double)b); }

DEV float shape_sdf(const DevShape& s, float px, float py) {
    if (s.kind == 0) return hyp(px - s.cx, py - s.cy) - s.r;
    const float x = px - s.cx, y = py - s.cy;
    const float qx = s.cs * x + s.sn * y, qy = -s.sn * x + s.cs * y;
    const float dx = fabsf(qx) - s.hx, dy = fabsf(qy) - s.hy;
    return hyp(smax(dx, 0.0f), smax(dy, 0.0f)) + smin(smax(dx, dy), 0.0f);
}

__global__ void k_nodes(float* sdf, int nw, int nh, float W, float H, const DevShape* shapes, int ns) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nw * nh) return;
    const int i = k % nw, j = k / nw;
    const float x = (float)i, y = (float)j;
    float d = smin(smin(smin(x - kWallR, W - kWallR - x), y - kWallR), H - kWallR - y);
    for (int s = 0; s < ns; s++) {
        const DevShape& S = shapes[s];
        if (i >= S.i0 && i <= S.i1 && j >= S.j0 && j <= S.j1) d = smin(d, shape_sdf(S, x, y));
    }
    sdf[k] = d;
}

// union_depth: seeds (solid nodes next to an open one keep -sdf, deeper ones FAR, 0 outside)
__global__ void k_depth_seed(const float* sdf, float* depth, int nw, int nh) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nw * nh) return;
    const int i = k % nw, j = k / nw;
    if (!(sdf[k] < 0.0f)) {
        depth[k] = 0.0f;
        return;
    }
    bool edge = false;
    for (int di = -1; di <= 1 && !edge; di++)
        for (int dj = -1; dj <= 1; dj++) {
            if (di == 0 && dj == 0) continue;
            const int a = i + di, b = j + dj;
            if (a >= 0 && b >= 0 && a < nw && b < nh && !(sdf[b * nw + a] < 0.0f)) {
                edge = true;
                break;
            }
        }
    depth[k] = edge ? -sdf[k] : kFar;
}

// The two chamfer sweeps as wavefronts (one block; rows r = threadIdx.x, + blockDim.x, ...).
// Forward: node (i, j) at step i + 2 j relaxes from (i - 1, j), (i, j - 1), (i - 1, j - 1),
// (i + 1, j - 1), in the host's order. Backward: node (nw-1-i', nh-1-j') at step i' + 2 j'.
__global__ void __launch_bounds__(1024) k_depth_sweeps(float* depth, int nw, int nh) {
    const float Dg = 1.41421354f;
    auto relax = [&](int k, int n, float st) {
        const float c = depth[n] + st;
        if (c < depth[k]) depth[k] = c;
    };
    const int steps = (nw - 1) + 2 * (nh - 1) + 1;
    for (int t = 0; t < steps; t++) {
        for (int j = threadIdx.x; j < nh; j += blockDim.x) {
            const int i = t - 2 * j;
            if (i < 0 || i >= nw) continue;
            const int k = j * nw + i;
            if (depth[k] == 0.0f) continue;
            if (i > 0) relax(k, k - 1, 1.0f);
            if (j > 0) {
                relax(k, k - nw, 1.0f);
                if (i > 0) relax(k, k - nw - 1, Dg);
                if (i + 1 < nw) relax(k, k - nw + 1, Dg);
            }
        }
        __syncthreads();
    }
    for (int t = 0; t < steps; t++) {
        for (int jj = threadIdx.x; jj < nh; jj += blockDim.x) {
            const int ii = t - 2 * jj;
            if (ii < 0 || ii >= nw) continue;
            const int i = nw - 1 - ii, j = nh - 1 - jj;
            const int k = j * nw + i;
            if (depth[k] == 0.0f) continue;
            if (i + 1 < nw) relax(k, k + 1, 1.0f);
            if (j + 1 < nh) {
                relax(k, k + nw, 1.0f);
                if (i + 1 < nw) relax(k, k + nw + 1, Dg);
                if (i > 0) relax(k, k + nw - 1, Dg);
            }
        }
        __syncthreads();
    }
}

__global__ void k_depth_apply(float* sdf, const float* depth, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (sdf[k] < 0.0f && depth[k] < kFar) sdf[k] = smin(sdf[k], -depth[k]);
}

// Open volume per cell from four bilinear sub-samples (MIN_OPEN 0.1).
__global__ void k_open(const float* sdf, float* open, int w, int h) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= w * h) return;
    const int i = k % w, j = k / w, nw = w + 1;
    const float d0 = sdf[j * nw + i], d1 = sdf[j * nw + i + 1], d2 = sdf[(j + 1) * nw + i], d3 = sdf[(j + 1) * nw + i + 1];
    const float FX[4] = {0.25f, 0.75f, 0.25f, 0.75f}, FY[4] = {0.25f, 0.25f, 0.75f, 0.75f};
    float acc = 0.0f;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const float fx = FX[q], fy = FY[q];
        const float v = (d0 * (1.0f - fx) + d1 * fx) * (1.0f - fy) + (d2 * (1.0f - fx) + d3 * fx) * fy;
        acc += smin(smax(v / 0.5f + 0.5f, 0.0f), 1.0f);
    }
    open[k] = acc * 0.25f < 0.1f ? 0.0f : acc * 0.25f;
}

DEV float open_fraction(float d0, float d1) {
    float f;
    if (d0 > 0.0f && d1 > 0.0f) f = 1.0f;
    else if (d0 <= 0.0f && d1 <= 0.0f) f = 0.0f;
    else f = smax(d0, d1) / (smax(d0, d1) - smin(d0, d1));
    return f < 0.05f ? 0.0f : f;
}

// faces(i, j): the left and bottom faces' open fractions, open only between open cells
DEV float2 faces(const float* open, const float* sdf, int w, int i, int j) {
    const int nw = w + 1;
    const bool here = open[j * w + i] > 0.0f;
    const bool left = here && i > 0 && open[j * w + i - 1] > 0.0f;
    const bool below = here && j > 0 && open[(j - 1) * w + i] > 0.0f;
    return make_float2(left ? open_fraction(sdf[j * nw + i], sdf[(j + 1) * nw + i]) : 0.0f,
                       below ? open_fraction(sdf[j * nw + i], sdf[j * nw + i + 1]) : 0.0f);
}

// ---- connected components: union-find rooted at the smallest index ----------------------

DEV uint32_t find_root(uint32_t* label, uint32_t k) {
    uint32_t r = k;
    for (int guard = 0; guard < 64 && label[r] != r; guard++) r = label[r];
    return r;
}

// union of a and b: the larger root takes the smaller as its parent (bounded retries; the
// host repeats the pass until nothing changes)
DEV void unite(uint32_t* label, uint32_t a, uint32_t b, int* changed) {
    for (int guard = 0; guard < 64; guard++) {
        a = find_root(label, a);
        b = find_root(label, b);
        if (a == b) return;
        if (a > b) {
            const uint32_t t = a;
            a = b;
            b = t;
        }
        const uint32_t old = atomicMin(&label[b], a);
        *changed = 1;
        if (old == b) return;
        b = old;
    }
}

// mode 0: pockets (cells with open > 0 linked by faces() > 0); mode 1: regions (cells with
// open volume > 0 linked by the final face fractions)
__global__ void k_cc_init(uint32_t* label, const float* open, const float4* solid, int n, int mode) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float o = mode == 0 ? open[k] : solid[k].w;
    label[k] = o > 0.0f ? (uint32_t)k : kNone;
}

__global__ void k_cc_link(uint32_t* label, const float* open, const float* sdf, const float4* solid, int w, int h, int mode,
                          int* changed) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= w * h || label[k] == kNone) return;
    const int i = k % w, j = k / w;
    float2 f;
    if (mode == 0) f = faces(open, sdf, w, i, j);
    else f = make_float2(solid[k].x, solid[k].y);
    if (i > 0 && f.x > 0.0f && label[k - 1] != kNone) unite(label, (uint32_t)k, (uint32_t)(k - 1), changed);
    if (j > 0 && f.y > 0.0f && label[k - w] != kNone) unite(label, (uint32_t)k, (uint32_t)(k - w), changed);
}

__global__ void k_cc_flatten(uint32_t* label, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || label[k] == kNone) return;
    label[k] = find_root(label, (uint32_t)k);
}

__global__ void k_cc_size(const uint32_t* label, uint32_t* size, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || label[k] == kNone) return;
    atomicAdd(&size[label[k]], 1u);
}

// Pockets of fewer than 16 cells: their cells closed, their corner nodes at most -0.5 (all
// writers of a node store the same value). *contested is set where a sealed cell shares a node
// with a cell of a component that stays open: lowering that node could split it, and the
// host's order of fills would then decide what is sealed.
__global__ void k_seal(const uint32_t* label, const uint32_t* size, float* open, float* sdf, int w, int h, int* contested) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= w * h || label[k] == kNone || size[label[k]] >= 16u) return;
    const int i = k % w, j = k / w, nw = w + 1;
    for (int dj = -1; dj <= 1; dj++)
        for (int di = -1; di <= 1; di++) {
            const int a = i + di, b = j + dj;
            if (a < 0 || b < 0 || a >= w || b >= h) continue;
            const uint32_t lb = label[b * w + a];
            if (lb != kNone && lb != label[k] && size[lb] >= 16u) *contested = 1;
        }
    open[k] = 0.0f;
    const int nodes[4] = {j * nw + i, j * nw + i + 1, (j + 1) * nw + i, (j + 1) * nw + i + 1};
    for (int q = 0; q < 4; q++) sdf[nodes[q]] = smin(sdf[nodes[q]], -0.5f);
}

// seal_pockets exactly as the host runs it (scene.cpp), by one thread: flood fills in index
// order, each seeing the seals before it. stack and members hold w h entries each.
__global__ void k_seal_sequential(float* open, float* sdf, uint32_t* label, int* stack, int* members, int w, int h) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int n = w * h, nw = w + 1;
    for (int k = 0; k < n; k++) label[k] = kNone;
    for (int start = 0; start < n; start++) {
        if (open[start] == 0.0f || label[start] != kNone) continue;
        int sp = 0, nm = 0;
        label[start] = (uint32_t)start;
        stack[sp++] = start;
        while (sp > 0) {
            const int k = stack[--sp];
            members[nm++] = k;
            const int i = k % w, j = k / w;
            const float2 lb = faces(open, sdf, w, i, j);
            float right = 0.0f, above = 0.0f;
            if (i + 1 < w) right = faces(open, sdf, w, i + 1, j).x;
            if (j + 1 < h) above = faces(open, sdf, w, i, j + 1).y;
            const int nb[4] = {k - 1, k + 1, k - w, k + w};
            const float a[4] = {lb.x, right, lb.y, above};
            for (int q = 0; q < 4; q++)
                if (a[q] > 0.0f && label[nb[q]] == kNone) {
                    label[nb[q]] = (uint32_t)start;
                    stack[sp++] = nb[q];
                }
        }
        if (nm < 16) {
            for (int m = 0; m < nm; m++) {
                const int k = members[m];
                open[k] = 0.0f;
                const int i = k % w, j = k / w;
                const int nodes[4] = {j * nw + i, j * nw + i + 1, (j + 1) * nw + i, (j + 1) * nw + i + 1};
                for (int q = 0; q < 4; q++) sdf[nodes[q]] = smin(sdf[nodes[q]], -0.5f);
            }
        }
    }
}

// Kernel-smoothed solid occupancy, the face fractions and the open volume per cell.
__global__ void k_solid(const float* open, const float* sdf, float4* solid, int w, int h) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= w * h) return;
    const int i = k % w, j = k / w;
    const float K[3] = {1.0f / 6.0f, 2.0f / 3.0f, 1.0f / 6.0f};
    float occ = 0.0f;
    for (int b = 0; b < 3; b++)
        for (int a = 0; a < 3; a++) {
            const int ii = i + a - 1, jj = j + b - 1;
            const float sv = (ii < 0 || jj < 0 || ii >= w || jj >= h) ? 1.0f : 1.0f - open[jj * w + ii];
            occ += K[a] * K[b] * sv;
        }
    const float2 f = faces(open, sdf, w, i, j);
    solid[k] = make_float4(f.x, f.y, occ, open[k]);
}

// Region roots in index order: flags, then an exclusive scan by one block.
__global__ void k_root_flags(const uint32_t* label, uint32_t* rank, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    rank[k] = label[k] == (uint32_t)k ? 1u : 0u;
}

__global__ void __launch_bounds__(1024) k_scan_one_block(uint32_t* v, int n) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int b0 = 0; b0 < n; b0 += 1024) {
        const int i = b0 + threadIdx.x;
        const uint32_t x0 = i < n ? v[i] : 0u;
        uint32_t x = x0;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t s = warp_sums[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            warp_sums[lane] = s;
        }
        __syncthreads();
        const uint32_t base = (wid > 0 ? warp_sums[wid - 1] : 0u) + carry;
        if (i < n) v[i] = base + x - x0;
        __syncthreads();
        if (threadIdx.x == 1023) carry = base + x;
        __syncthreads();
    }
}

// the vent of a region: the leftmost cell of its top row (the largest key row w + w-1-col)
__global__ void k_vents(const uint32_t* label, uint32_t* vent, int w, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || label[k] == kNone) return;
    const int i = k % w, j = k / w;
    atomicMax(&vent[label[k]], (uint32_t)(j * w + (w - 1 - i)) + 1u);
}

__global__ void k_regions(const uint32_t* label, const uint32_t* rank, const uint32_t* vent, uint32_t* region, int w, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t r = label[k];
    if (r == kNone) {
        region[k] = 0u;
        return;
    }
    uint32_t id = min(rank[r], 31u);
    const uint32_t key = vent[r] - 1u;
    const int vj = (int)(key / (uint32_t)w), vi = w - 1 - (int)(key % (uint32_t)w);
    if (vj * w + vi == k) id |= 256u;
    region[k] = id;
}

// The cells in or against a held shape: the last such shape (in order) sets the temperature.
__global__ void k_temps(float* temp, int w, int h, const DevShape* shapes, int ns) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= w * h) return;
    const int i = k % w, j = k / w;
    float t = kNoTempR;
    for (int s = 0; s < ns; s++) {
        const DevShape& S = shapes[s];
        if (!S.held || i < S.t0 || i >= S.t1 || j < S.u0 || j >= S.u1) continue;
        if (shape_sdf(S, (float)i + 0.5f, (float)j + 0.5f) < 0.75f) t = S.temp;
    }
    temp[k] = t;
}

int grid_of(int n) { return (n + 255) / 256; }

// connected components into label (mode 0 pockets, 1 regions): link passes until none
// changes a label (bounded), then every label its root
cudaError_t components(uint32_t* label, const float* open, const float* sdf, const float4* solid, int w, int h, int mode,
                       int* d_changed, cudaStream_t st) {
    const int n = w * h;
    k_cc_init<<<grid_of(n), 256, 0, st>>>(label, open, solid, n, mode);
    for (int pass = 0; pass < 4096; pass++) {
        int changed = 0;
        cudaMemsetAsync(d_changed, 0, sizeof(int), st);
        k_cc_link<<<grid_of(n), 256, 0, st>>>(label, open, sdf, solid, w, h, mode, d_changed);
        k_cc_flatten<<<grid_of(n), 256, 0, st>>>(label, n);
        cudaError_t e = cudaMemcpyAsync(&changed, d_changed, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        if (!changed) return cudaGetLastError();
    }
    return cudaErrorUnknown;   // no convergence (cannot happen: every pass shortens the forest)
}

}  // namespace

// Rasterises `sc` into device buffers: sdf (w+1)(h+1), solid w h float4, region w h, temp w h
// (NO_TEMP where no held shape reaches; left untouched when no shape is held). *heated = any
// shape held. Scratch is allocated for the call and freed.
cudaError_t rasterize_device(const Scene& sc, float* sdf, float4* solid, uint32_t* region, float* temp, bool* heated,
                             cudaStream_t st) {
    const int w = sc.w, h = sc.h, nw = w + 1, nh = h + 1, n = w * h, nn = nw * nh;
    std::vector<DevShape> hs;
    bool any_held = false;
    for (const Shape& s : sc.shapes) {
        DevShape d{};
        d.kind = s.kind == Shape::Circle ? 0 : 1;
        d.cx = s.cx;
        d.cy = s.cy;
        d.hx = s.hx;
        d.hy = s.hy;
        d.r = s.r;
        d.sn = std::sin(s.angle);
        d.cs = std::cos(s.angle);
        const float bound = s.kind == Shape::Circle ? s.r : std::hypot(s.hx, s.hy);
        // the node box scene.cpp updates (REACH 6)
        const float r = bound + 6.0f;
        d.i0 = (int)std::max(std::floor(s.cx - r), 0.0f);
        const int i1 = std::min(std::max((int)std::ceil(s.cx + r), 0), nw - 1);
        d.j0 = (int)std::max(std::floor(s.cy - r), 0.0f);
        const int j1 = std::min(std::max((int)std::ceil(s.cy + r), 0), nh - 1);
        d.j1 = std::min(std::max(j1, d.j0), nh - 1);
        d.i1 = std::min(std::max(i1, d.i0), nw - 1);
        // the cell box of the held temperature (bound + 2)
        const float r2 = bound + 2.0f;
        d.t0 = (int)std::max(std::floor(s.cx - r2), 0.0f);
        d.t1 = std::min((int)std::max(std::ceil(s.cx + r2), 0.0f), w);
        d.u0 = (int)std::max(std::floor(s.cy - r2), 0.0f);
        d.u1 = std::min((int)std::max(std::ceil(s.cy + r2), 0.0f), h);
        d.held = s.held ? 1 : 0;
        d.temp = s.temp;
        any_held |= s.held;
        hs.push_back(d);
    }
    *heated = any_held;
    DevShape* dshapes = nullptr;
    float *depth = nullptr, *open = nullptr;
    uint32_t *label = nullptr, *size = nullptr, *rank = nullptr, *vent = nullptr;
    int *flags = nullptr, *stack = nullptr, *members = nullptr;
    cudaError_t e = cudaSuccess;
    auto A = [&](void** p, size_t b) {
        if (e == cudaSuccess) e = cudaMalloc(p, std::max<size_t>(b, 16));
    };
    A((void**)&dshapes, hs.size() * sizeof(DevShape));
    A((void**)&depth, (size_t)nn * sizeof(float));
    A((void**)&open, (size_t)n * sizeof(float));
    A((void**)&label, (size_t)n * sizeof(uint32_t));
    A((void**)&size, (size_t)n * sizeof(uint32_t));
    A((void**)&rank, (size_t)n * sizeof(uint32_t));
    A((void**)&vent, (size_t)n * sizeof(uint32_t));
    A((void**)&flags, 2 * sizeof(int));
    if (e == cudaSuccess && !hs.empty())
        e = cudaMemcpyAsync(dshapes, hs.data(), hs.size() * sizeof(DevShape), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        const int ns = (int)hs.size();
        k_nodes<<<grid_of(nn), 256, 0, st>>>(sdf, nw, nh, (float)w, (float)h, dshapes, ns);
        k_depth_seed<<<grid_of(nn), 256, 0, st>>>(sdf, depth, nw, nh);
        k_depth_sweeps<<<1, 1024, 0, st>>>(depth, nw, nh);
        k_depth_apply<<<grid_of(nn), 256, 0, st>>>(sdf, depth, nn);
        k_open<<<grid_of(n), 256, 0, st>>>(sdf, open, w, h);
        e = cudaGetLastError();
    }
    // pockets: components of the open cells, the small ones sealed
    if (e == cudaSuccess) e = components(label, open, sdf, nullptr, w, h, 0, flags, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(size, 0, (size_t)n * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(flags + 1, 0, sizeof(int), st);
    if (e == cudaSuccess) {
        k_cc_size<<<grid_of(n), 256, 0, st>>>(label, size, n);
        // a copy of the fields before sealing, in case the sequential path must redo it
        e = cudaMemcpyAsync(depth, sdf, (size_t)nn * sizeof(float), cudaMemcpyDeviceToDevice, st);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(rank, open, (size_t)n * sizeof(float), cudaMemcpyDeviceToDevice, st);
    int contested = 0;
    if (e == cudaSuccess) {
        k_seal<<<grid_of(n), 256, 0, st>>>(label, size, open, sdf, w, h, flags + 1);
        e = cudaMemcpyAsync(&contested, flags + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (e == cudaSuccess && contested) {
        // restore the unsealed fields and seal in the host's order
        A((void**)&stack, (size_t)n * sizeof(int));
        A((void**)&members, (size_t)n * sizeof(int));
        if (e == cudaSuccess) e = cudaMemcpyAsync(sdf, depth, (size_t)nn * sizeof(float), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(open, rank, (size_t)n * sizeof(float), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) {
            k_seal_sequential<<<1, 1, 0, st>>>(open, sdf, label, stack, members, w, h);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) {
        k_solid<<<grid_of(n), 256, 0, st>>>(open, sdf, solid, w, h);
        e = cudaGetLastError();
    }
    // regions: components through the final faces, ids by the roots' order, vents
    if (e == cudaSuccess) e = components(label, nullptr, nullptr, solid, w, h, 1, flags, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(vent, 0, (size_t)n * sizeof(uint32_t), st);
    if (e == cudaSuccess) {
        k_root_flags<<<grid_of(n), 256, 0, st>>>(label, rank, n);
        k_scan_one_block<<<1, 1024, 0, st>>>(rank, n);
        k_vents<<<grid_of(n), 256, 0, st>>>(label, vent, w, n);
        k_regions<<<grid_of(n), 256, 0, st>>>(label, rank, vent, region, w, n);
        if (any_held && temp) k_temps<<<grid_of(n), 256, 0, st>>>(temp, w, h, dshapes, (int)hs.size());
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    for (void* p : {(void*)dshapes, (void*)depth, (void*)open, (void*)label, (void*)size, (void*)rank, (void*)vent,
                    (void*)flags, (void*)stack, (void*)members})
        if (p) cudaFree(p);
    return e;
}


}  // namespace sprout

// Device helpers shared by the persistent solver kernels (pressure.cu, viscosity.cu): the
// multigrid level geometry, the grid-wide barrier of a cooperative launch with its bounded
// wait, and the work-group trees and strided totals of reduce.glsl / reduce_tail.glsl that
// every block evaluates in the same order (so every block gets the same scalars).
#pragma once

#include <cuda_runtime.h>

#include "dev_common.cuh"

namespace sprout {
namespace solve {

constexpr int NT = 256;                // threads per block: one 16 x 16 tile at a time
constexpr uint32_t SPIN_LIMIT = 1u << 24;

struct Lv {
    int off, w, h, toff;
};

DEV Lv lev(const Levels& L, int l) { return Lv{L.off[l], L.w[l], L.h[l], L.toff[l]}; }
DEV bool l_inside(const Lv& L, int x, int y) { return x >= 0 && y >= 0 && x < L.w && y < L.h; }
DEV int l_at(const Lv& L, int x, int y) { return L.off + y * L.w + x; }
DEV int tiles_x(const Lv& L) { return (L.w + 15) >> 4; }
DEV int tiles_y(const Lv& L) { return (L.h + 15) >> 4; }
DEV float wcomp(float4 w, int k) { return k == 0 ? w.x : k == 1 ? w.y : k == 2 ? w.z : w.w; }

// Grid-wide barrier over the co-resident blocks of a cooperative launch. Thread 0 of each
// block arrives on a counter and waits on a generation word with a bounded spin; the last
// to arrive resets the counter and advances the generation. Returns false (and every block
// leaves) once any wait has run out.
DEV bool grid_sync(SolveState* K) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile uint32_t* vgen = &K->bar_gen;
        volatile uint32_t* verr = &K->error;
        if (*verr != 0u) {
            ok = 0;
        } else {
            uint32_t g = *vgen;
            __threadfence();
            uint32_t arrived = atomicAdd(&K->bar_count, 1u) + 1u;
            if (arrived == gridDim.x) {
                atomicExch(&K->bar_count, 0u);
                __threadfence();
                atomicAdd(&K->bar_gen, 1u);
            } else {
                uint32_t spins = 0;
                while (*vgen == g) {
                    if (*verr != 0u) { ok = 0; break; }
                    __nanosleep(32);
                    if (++spins > SPIN_LIMIT) {
                        if (atomicExch(&K->error, 1u) == 0u) {
                            K->err_arrived = *(volatile uint32_t*)&K->bar_count;
                            K->err_blocks = gridDim.x;
                        }
                        ok = 0;
                        break;
                    }
                }
            }
            __threadfence();
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

DEV float4 add4(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
DEV Dbl4 add4(Dbl4 a, Dbl4 b) { return Dbl4{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }

// Work-group tree of reduce.glsl:5-14 over the 256 values in buf; result in buf[0].
template <class T>
DEV void block_tree(T* buf) {
    const int t = threadIdx.x;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (t < s) buf[t] = add4(buf[t], buf[t + s]);
        __syncthreads();
    }
}

// total() of reduce_tail.glsl:28-41: thread t sums partials t, t + 256, ... in order,
// then the tree. Every block calls it and gets the same value.
template <class T>
DEV T total(const T* part, int n, T* buf) {
    const int t = threadIdx.x;
    T s{};
    for (int k = t; k < n; k += NT) s = add4(s, part[k]);
    buf[t] = s;
    block_tree(buf);
    T r = buf[0];
    __syncthreads();
    return r;
}

}  // namespace solve
}  // namespace sprout

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
    uint32_t wm, tm;   // division constants of the width and the width in tiles (Levels)
};

DEV Lv lev(const Levels& L, int l) { return Lv{L.off[l], L.w[l], L.h[l], L.toff[l], L.wm[l], L.tm[l]}; }
// floor(t / d) from d's constant m = ceil(2^32 / d) (exact for t < 2^20, d < 2^11)
DEV int qdiv(int t, uint32_t m) { return (int)__umulhi((uint32_t)t, m); }
// the first cell (x, y) of tile t of a level
DEV int2 tile_origin(const Lv& L, int t) {
    const int ty = qdiv(t, L.tm);
    return make_int2((t - ty * ((L.w + 15) >> 4)) * 16, ty * 16);
}
DEV bool l_inside(const Lv& L, int x, int y) { return x >= 0 && y >= 0 && x < L.w && y < L.h; }
DEV int l_at(const Lv& L, int x, int y) { return L.off + y * L.w + x; }
DEV int tiles_x(const Lv& L) { return (L.w + 15) >> 4; }
DEV int tiles_y(const Lv& L) { return (L.h + 15) >> 4; }
DEV float wcomp(float4 w, int k) { return k == 0 ? w.x : k == 1 ? w.y : k == 2 ? w.z : w.w; }

// a / b with the same result for every a and b. A zero numerator over a positive divisor is
// the numerator itself (its sign kept) and skips the division: the IEEE division leaves its
// fast path for a zero numerator (about 240 cycles of latency on sm_103 against 48), and the
// smoothers meet one wherever a column's right-hand side or residual is exactly zero.
DEV float divz(float a, float b) {
    if (a == 0.0f && b > 0.0f) return a;
    return a / b;
}
DEV float2 divz(float2 a, float b) { return make_float2(divz(a.x, b), divz(a.y, b)); }
// a / b where the caller keeps the result only for b > 0 (zero otherwise, no division).
DEV float divp(float a, float b) {
    if (!(b > 0.0f)) return 0.0f;
    return divz(a, b);
}

DEV unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The number of grid barriers this block has passed in the current launch (one per block, in
// shared memory; grid_begin sets it to zero at the start of every persistent kernel).
DEV uint32_t& grid_epoch() {
    __shared__ uint32_t epoch;
    return epoch;
}
DEV void grid_begin() {
    if (threadIdx.x == 0) grid_epoch() = 0u;
    __syncthreads();
}

// Grid-wide barrier over the co-resident blocks of a cooperative launch: one arrival counter
// that only grows (zeroed before each launch). At its e-th barrier (e counted by the block
// itself) thread 0 of each block adds one without waiting for the old value and waits
// (bounded spin) until the counter reaches (e + 1) x blocks, which the last block to arrive
// makes true with its own add: releasing costs no store beyond the arrivals, and no block
// waits for its arrival's round trip before it starts to poll. Returns false (and every
// block leaves) once any wait has run out.
DEV bool grid_sync(SolveState* K) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile uint32_t* vcnt = &K->bar_count;
        volatile uint32_t* verr = &K->error;
        unsigned long long* trace = K->trace;
        const uint32_t epoch = grid_epoch();
        grid_epoch() = epoch + 1u;
        if (*verr != 0u) {
            ok = 0;
        } else {
            // failure injection (tests only, off unless set): this block arrives late, by a
            // wait bounded by the device clock (at most a second) and by a poll count
            const uint32_t stall = K->dbg_stall_ns;
            if (stall != 0u && blockIdx.x == K->dbg_block) {
                const unsigned long long t0 = global_ns();
                const unsigned long long lim = stall < 1000000000u ? stall : 1000000000u;
                for (uint32_t k = 0; k < (1u << 21) && global_ns() - t0 < lim; k++) __nanosleep(500);
            }
            const uint32_t spin_limit = K->dbg_spin_limit != 0u ? K->dbg_spin_limit : SPIN_LIMIT;
            const unsigned long long t_in = trace ? global_ns() : 0ull;
            const uint32_t base = trace ? *(volatile uint32_t*)&K->trace_base : 0u;
            // the arrival releases the block's writes (ordered before it by the block barrier
            // above; release is cumulative), the acquiring reads of the wait make the other
            // blocks' writes visible to this block after the block barrier below; this
            // thread's own add is ordered before its later loads of the same word
            asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&K->bar_count) : "memory");
            const uint32_t target = (epoch + 1u) * gridDim.x;
            unsigned long long* row = nullptr;
            if (trace && blockIdx.x + 1 < K->trace_cols) {
                row = trace + (size_t)((base + epoch) % K->trace_rows) * K->trace_cols;
                row[blockIdx.x] = t_in;
            }
            uint32_t spins = 0;
            for (;;) {
                uint32_t now;
                asm volatile("ld.acquire.gpu.u32 %0, [%1];" : "=r"(now) : "l"(&K->bar_count) : "memory");
                if (now >= target) break;
                if (*verr != 0u) { ok = 0; break; }
                if (++spins > spin_limit) {
                    if (atomicOr(&K->error, ERR_TIMEOUT) == 0u) {
                        K->err_arrived = *vcnt - epoch * gridDim.x;
                        K->err_blocks = gridDim.x;
                    }
                    ok = 0;
                    break;
                }
            }
            if (row && blockIdx.x == 0) row[K->trace_cols - 1] = global_ns();
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Asynchronous copies global -> shared (cp.async, N = 4, 8 or 16 bytes, both addresses
// N-aligned): when `ok` is false nothing is read and the N bytes are zero-filled (g must
// still be a valid address). A thread sees its own copies after cp_wait; other threads'
// after a __syncthreads that follows their cp_wait.
template <int N>
DEV void cp_async(void* s, const void* g, bool ok) {
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(s);
    const int src = ok ? N : 0;
    if constexpr (N == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(g), "r"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(sa), "l"(g), "n"(N), "r"(src) : "memory");
}
DEV void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// waits until at most N of this thread's committed groups are still in flight
template <int N>
DEV void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// This block's work items k = 0, 1, ... (item(k): the one at blockIdx.x + k gridDim.x of
// cnt) through a pipeline of D staging buffers: stage(it, b) issues item it's asynchronous
// copies into buffer b; finish(it, b) computes the item from them and ends with
// __syncthreads (so that the buffer can take a later item's copies). While item k computes,
// the copies of items k + 1 .. k + D - 1 are in flight (one commit group per item, empty
// past the last).
template <int D, class I, class S, class F>
DEV void pipeline(uint32_t cnt, I&& item, S&& stage, F&& finish) {
    if (blockIdx.x >= cnt) return;
    const uint32_t mine = (cnt - blockIdx.x + gridDim.x - 1) / gridDim.x;
    for (int k = 0; k < D - 1; k++) {
        if ((uint32_t)k < mine) stage(item(k), k);
        cp_commit();
    }
    for (uint32_t k = 0; k < mine; k++) {
        const uint32_t ahead = k + D - 1;
        if (ahead < mine) stage(item((int)ahead), (int)(ahead % D));
        cp_commit();
        cp_wait<D - 1>();
        finish(item((int)k), (int)(k % D));
    }
}

DEV float4 add4(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
DEV Dbl4 add4(Dbl4 a, Dbl4 b) { return Dbl4{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }

// Four sums each carried as an unevaluated pair of floats, hi + lo (about 48 significant
// bits): FP32 error-free transformations instead of FP64 arithmetic, which runs at a small
// fraction of the FP32 rate on this GPU. A product of two floats is exact as a pair (the FMA
// gives its rounding error); a sum of pairs keeps the rounding error of the high parts.
struct FF4 {
    float4 hi, lo;
};
DEV float2 ff_add(float ahi, float alo, float bhi, float blo) {
    const float s = ahi + bhi;
    const float bv = s - ahi;
    float e = (ahi - (s - bv)) + (bhi - bv);
    e += alo + blo;
    const float hi = s + e;
    return make_float2(hi, e - (hi - s));
}
DEV FF4 add4(FF4 a, FF4 b) {
    const float2 x = ff_add(a.hi.x, a.lo.x, b.hi.x, b.lo.x), y = ff_add(a.hi.y, a.lo.y, b.hi.y, b.lo.y);
    const float2 z = ff_add(a.hi.z, a.lo.z, b.hi.z, b.lo.z), w = ff_add(a.hi.w, a.lo.w, b.hi.w, b.lo.w);
    return FF4{make_float4(x.x, y.x, z.x, w.x), make_float4(x.y, y.y, z.y, w.y)};
}
// the exact products a0 b0 .. a3 b3 as pairs
DEV FF4 ff_prod4(float a0, float b0, float a1, float b1, float a2, float b2, float a3, float b3) {
    const float p0 = a0 * b0, p1 = a1 * b1, p2 = a2 * b2, p3 = a3 * b3;
    return FF4{make_float4(p0, p1, p2, p3),
               make_float4(fmaf(a0, b0, -p0), fmaf(a1, b1, -p1), fmaf(a2, b2, -p2), fmaf(a3, b3, -p3))};
}
DEV Dbl4 to_dbl(FF4 a) {
    return Dbl4{(double)a.hi.x + (double)a.lo.x, (double)a.hi.y + (double)a.lo.y, (double)a.hi.z + (double)a.lo.z,
                (double)a.hi.w + (double)a.lo.w};
}

// At the end of a persistent kernel (block 0, after its last barrier, which every block has
// reached): the trace rows of the next launch follow this one's.
DEV void trace_launch_done(SolveState* K) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && K->trace) K->trace_base += K->bar_count / gridDim.x;
}

DEV float4 shfl_down4(float4 v, int s) {
    return make_float4(__shfl_down_sync(0xffffffffu, v.x, s), __shfl_down_sync(0xffffffffu, v.y, s),
                       __shfl_down_sync(0xffffffffu, v.z, s), __shfl_down_sync(0xffffffffu, v.w, s));
}
DEV Dbl4 shfl_down4(Dbl4 v, int s) {
    return Dbl4{__shfl_down_sync(0xffffffffu, v.x, s), __shfl_down_sync(0xffffffffu, v.y, s),
                __shfl_down_sync(0xffffffffu, v.z, s), __shfl_down_sync(0xffffffffu, v.w, s)};
}
DEV FF4 shfl_down4(FF4 v, int s) { return FF4{shfl_down4(v.hi, s), shfl_down4(v.lo, s)}; }

// Work-group tree of reduce.glsl:5-14 over the 256 values in buf; result in buf[0]. The
// pairs are those of the tree (t with t + s, s = 128 .. 1): the three wide steps through
// shared memory, the last five inside the first warp by shuffles.
template <class T>
DEV void block_tree(T* buf) {
    const int t = threadIdx.x;
    __syncthreads();
    for (int s = 128; s >= 32; s >>= 1) {
        if (t < s) buf[t] = add4(buf[t], buf[t + s]);
        __syncthreads();
    }
    if (t < 32) {
        T v = buf[t];
        for (int s = 16; s > 0; s >>= 1) {
            const T o = shfl_down4(v, s);
            if (t < s) v = add4(v, o);
        }
        if (t == 0) buf[0] = v;
    }
    __syncthreads();
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

// One block compacts the nonzero flags[0 .. T) into out (their indices, in order) and
// stores how many into *count.
DEV void compact_flags(const uint32_t* flags, int T, uint32_t* out, uint32_t* count) {
    __shared__ uint32_t wsum[NT / 32];
    __shared__ uint32_t s_base;
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
    if (threadIdx.x == 0) *count = s_base;
    __syncthreads();
}

}  // namespace solve
}  // namespace sprout

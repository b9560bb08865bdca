// Admission of new liquid: the counts of live particles in a window of cells (count.comp,
// read back by FluidSim::cell_counts, mod.rs:3350-3387) and the recycling of dead particle
// slots by queued spawns once the buffer has no fresh slots left (claim.comp, with its
// dispatch in record, mod.rs:2486-2533).
//
// claim.comp hands the spawn entries to dead slots in the order in which its invocations win
// an atomic counter. Here the k-th dead slot in slot order takes the k-th entry: a block count,
// an exclusive scan of the block counts and a placement pass, so that the result does not
// depend on scheduling (one of the outcomes claim.comp allows).
#include <cuda_runtime.h>

#include <algorithm>

#include "dev_common.cuh"
#include "kernels.h"

namespace sprout {

namespace {

constexpr int CLAIM_BLOCK = 256;
constexpr int CLAIM_SCAN = 1024;

DEV uint32_t kind_of(const float4* part, uint32_t id) { return __float_as_uint(part[3 * id + 2].y); }

// Dead slots (kind == KIND_DEAD, claim.comp:13) per block of CLAIM_BLOCK slots.
__global__ void __launch_bounds__(CLAIM_BLOCK) k_claim_count(const float4* part, uint32_t n_slots, uint32_t* blk) {
    __shared__ uint32_t warp_n[CLAIM_BLOCK / 32];
    const uint32_t id = blockIdx.x * CLAIM_BLOCK + threadIdx.x;
    const bool dead = id < n_slots && kind_of(part, id) == KIND_DEAD;
    const uint32_t bal = __ballot_sync(0xffffffffu, dead);
    if ((threadIdx.x & 31) == 0) warp_n[threadIdx.x >> 5] = __popc(bal);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int w = 0; w < CLAIM_BLOCK / 32; w++) s += warp_n[w];
        blk[blockIdx.x] = s;
    }
}

// Exclusive scan of blk[0 .. nb) in place (one block).
__global__ void __launch_bounds__(CLAIM_SCAN) k_claim_scan(uint32_t* blk, int nb) {
    __shared__ uint32_t warp_sums[CLAIM_SCAN / 32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int b0 = 0; b0 < nb; b0 += CLAIM_SCAN) {
        const int i = b0 + threadIdx.x;
        const uint32_t v = i < nb ? blk[i] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t s = warp_sums[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            warp_sums[lane] = s;
        }
        __syncthreads();
        const uint32_t base = (wid > 0 ? warp_sums[wid - 1] : 0u) + carry;
        if (i < nb) blk[i] = base + x - v;
        __syncthreads();
        if (threadIdx.x == CLAIM_SCAN - 1) carry = base + x;
        __syncthreads();
    }
}

// The dead slot of rank r (in slot order) takes spawn entry r while r < claim (claim.comp:14-16).
__global__ void __launch_bounds__(CLAIM_BLOCK) k_claim_place(float4* part, uint32_t n_slots, const uint32_t* blk,
                                                             const float4* spawn, uint32_t claim) {
    __shared__ uint32_t warp_n[CLAIM_BLOCK / 32];
    const uint32_t id = blockIdx.x * CLAIM_BLOCK + threadIdx.x;
    const bool dead = id < n_slots && kind_of(part, id) == KIND_DEAD;
    const uint32_t bal = __ballot_sync(0xffffffffu, dead);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) warp_n[wid] = __popc(bal);
    __syncthreads();
    if (!dead) return;
    uint32_t r = blk[blockIdx.x] + __popc(bal & ((1u << lane) - 1u));
    for (int w = 0; w < wid; w++) r += warp_n[w];
    if (r >= claim) return;
    part[3 * id + 0] = spawn[3 * r + 0];
    part[3 * id + 1] = spawn[3 * r + 1];
    part[3 * id + 2] = spawn[3 * r + 2];
}

// k_claim_place with its entries counted on the device: entries skip .. st->count of spawn.
__global__ void __launch_bounds__(CLAIM_BLOCK) k_claim_place_dev(float4* part, uint32_t n_slots, const uint32_t* blk,
                                                                 const float4* spawn, const EmitState* st,
                                                                 uint32_t skip) {
    __shared__ uint32_t warp_n[CLAIM_BLOCK / 32];
    const uint32_t claim = st->count > skip ? st->count - skip : 0u;
    const uint32_t id = blockIdx.x * CLAIM_BLOCK + threadIdx.x;
    const bool dead = id < n_slots && kind_of(part, id) == KIND_DEAD;
    const uint32_t bal = __ballot_sync(0xffffffffu, dead);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) warp_n[wid] = __popc(bal);
    __syncthreads();
    if (!dead) return;
    uint32_t r = blk[blockIdx.x] + __popc(bal & ((1u << lane) - 1u));
    for (int w = 0; w < wid; w++) r += warp_n[w];
    if (r >= claim) return;
    const float4* e = spawn + 3 * (size_t)(skip + r);
    part[3 * id + 0] = e[0];
    part[3 * id + 1] = e[1];
    part[3 * id + 2] = e[2];
}

// count.comp:17-23: live particles (a material in the low byte of kind) per cell of the window
// at origin (ox, oy) of sw x sh cells, row by row. Integer atomics: the counts do not depend on
// the order of the adds.
__global__ void k_cell_counts(const float4* part, uint32_t n_slots, int ox, int oy, int sw, int sh, uint32_t* out) {
    const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n_slots) return;
    const float4 q0 = part[3 * id + 0];
    if ((kind_of(part, id) & 255u) == 0u) return;
    const int cx = (int)floorf(q0.x) - ox, cy = (int)floorf(q0.y) - oy;
    if (cx < 0 || cy < 0 || cx >= sw || cy >= sh) return;
    atomicAdd(&out[cy * sw + cx], 1u);
}

// stats.comp:14-42: the census of the particle slots: live particles, and per material row
// its particles and the sum of their concentrations in 1/256 of a particle, each particle's
// quantised as uint(clamp(s, 0, 1) * 256 + 0.5). The reference folds runs of 64 slots before
// its atomics; here every block first sums its slots per row in shared memory (integer adds,
// so the totals do not depend on the order), then adds each non-zero row once to the global
// counters: out[0] live, out[1 + m] count of row m, out[1 + kStatsRows + m] concentration.
constexpr int STATS_BLOCK = 256;
__global__ void __launch_bounds__(STATS_BLOCK) k_stats(const float4* part, uint32_t n_slots, uint32_t* out) {
    __shared__ uint32_t cnt[kStatsRows], conc[kStatsRows];
    __shared__ uint32_t live;
    for (int m = threadIdx.x; m < kStatsRows; m += STATS_BLOCK) cnt[m] = conc[m] = 0u;
    if (threadIdx.x == 0) live = 0u;
    __syncthreads();
    uint32_t mine = 0u;
    for (uint32_t id = blockIdx.x * STATS_BLOCK + threadIdx.x; id < n_slots; id += gridDim.x * STATS_BLOCK) {
        const float4 q2 = part[3 * id + 2];
        const uint32_t kind = __float_as_uint(q2.y) & 255u;
        if (kind == 0u || kind > (uint32_t)kStatsRows) continue;
        mine++;
        const float sc = fminf(fmaxf(q2.x, 0.0f), 1.0f);
        atomicAdd(&cnt[kind - 1u], 1u);
        atomicAdd(&conc[kind - 1u], (uint32_t)(sc * 256.0f + 0.5f));
    }
    // live particles of the block: a warp sum, then one shared add per warp
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, o);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(&live, mine);
    __syncthreads();
    for (int m = threadIdx.x; m < kStatsRows; m += STATS_BLOCK) {
        if (cnt[m]) atomicAdd(&out[1 + m], cnt[m]);
        if (conc[m]) atomicAdd(&out[1 + kStatsRows + m], conc[m]);
    }
    if (threadIdx.x == 0 && live) atomicAdd(&out[0], live);
}

}  // namespace

void launch_stats(const float4* part, uint32_t n_slots, uint32_t* out, cudaStream_t st) {
    cudaMemsetAsync(out, 0, stats_words() * sizeof(uint32_t), st);
    if (n_slots == 0) return;
    int sms = 152;
    const uint32_t want = (n_slots + STATS_BLOCK - 1) / STATS_BLOCK;
    const int blocks = (int)std::min<uint32_t>(want, (uint32_t)(4 * sms));
    k_stats<<<blocks, STATS_BLOCK, 0, st>>>(part, n_slots, out);
}

uint32_t claim_scratch_words(uint32_t n_slots) { return (n_slots + CLAIM_BLOCK - 1) / CLAIM_BLOCK + 1; }

void launch_claim(float4* part, uint32_t n_slots, const float4* spawn, uint32_t claim, uint32_t* scratch,
                  cudaStream_t st) {
    if (n_slots == 0 || claim == 0) return;
    const int nb = (int)((n_slots + CLAIM_BLOCK - 1) / CLAIM_BLOCK);
    k_claim_count<<<nb, CLAIM_BLOCK, 0, st>>>(part, n_slots, scratch);
    k_claim_scan<<<1, CLAIM_SCAN, 0, st>>>(scratch, nb);
    k_claim_place<<<nb, CLAIM_BLOCK, 0, st>>>(part, n_slots, scratch, spawn, claim);
}

void launch_claim_dev(float4* part, uint32_t n_slots, const float4* spawn, const EmitState* est, uint32_t skip,
                      uint32_t* scratch, cudaStream_t st) {
    if (n_slots == 0) return;
    const int nb = (int)((n_slots + CLAIM_BLOCK - 1) / CLAIM_BLOCK);
    k_claim_count<<<nb, CLAIM_BLOCK, 0, st>>>(part, n_slots, scratch);
    k_claim_scan<<<1, CLAIM_SCAN, 0, st>>>(scratch, nb);
    k_claim_place_dev<<<nb, CLAIM_BLOCK, 0, st>>>(part, n_slots, scratch, spawn, est, skip);
}

void launch_cell_counts(const float4* part, uint32_t n_slots, int ox, int oy, int sw, int sh, uint32_t* out,
                        cudaStream_t st) {
    cudaMemsetAsync(out, 0, (size_t)sw * sh * sizeof(uint32_t), st);
    if (n_slots == 0) return;
    k_cell_counts<<<(n_slots + 255) / 256, 256, 0, st>>>(part, n_slots, ox, oy, sw, sh, out);
}

}  // namespace sprout

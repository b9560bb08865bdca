// Launchers of the engine's kernels, one per stage of the substep. Each records its
// kernels on the given stream (so that a whole substep can be captured into a CUDA graph).
#pragma once

#include <cuda_runtime.h>

#include "dev_common.cuh"

namespace sprout {

// What the host decided for this configuration of the tank.
struct LaunchCfg {
    uint32_t n_slots = 0;
    bool thermal = false;
    bool heat = false;        // thermal and heat_rate > 0: heat.comp runs
    int visc_mode = 0;        // 0 none, 1 explicit, 2 implicit
    int mg_blocks = 0;        // blocks of the persistent pressure kernel
    int mg_threads = 256;
};

void launch_advance(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st);
void launch_sort(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st);
void launch_p2g(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st);
void launch_grid(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st);
cudaError_t launch_pressure(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st);
void launch_project(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st);
// Blocks of the persistent pressure kernel that fit on the device at once.
int pressure_blocks_max(int device, size_t smem);
// Dynamic shared memory of the persistent pressure kernel: the tail levels of each block.
size_t pressure_smem(const Levels& lv);

}  // namespace sprout

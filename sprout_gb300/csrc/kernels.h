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
    bool rheo = false;        // a non-Newtonian liquid is in the tank: rheo.comp runs
    bool settle = false;      // a family with grains settles: settle.comp runs
    bool elastic = false;     // a viscoelastic liquid: particles carry a stress, elastic.comp runs
    bool rigid = false;       // liquid can turn rigid: rigid.comp runs
    bool magnet = false;      // a magnet and a susceptible liquid: magnet.comp runs
    bool xtra = false;        // families, several phase groups, settling or currents: the particle pass's full form
    int visc_mode = 0;        // 0 none, 1 explicit, 2 implicit
    bool twice = false;       // implicit viscosity between two pressure solves
    bool viscous_warm = false;   // the first solve starts from last substep's P1 (cg_scale mode 1)
    int visc_levels = 0;      // levels below the grid in the viscosity V-cycle
    int visc_sweeps = 2;      // Gauss-Seidel sweeps per visit of a level (1 or 2)
    int visc_blocks = 0;      // blocks of the persistent viscosity kernel
    int mg_blocks = 0;        // blocks of the persistent pressure kernel
    int mg_threads = 256;
    bool mixed = false;       // the mixed-precision pressure solve
    int mg_blocks_mixed = 0;  // blocks of its persistent kernel
};

void launch_advance(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st);
void launch_sort(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st);
void launch_p2g(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st);
// Admission (admission.cu): queued spawns into dead slots, the k-th dead slot in slot order
// taking entry k < claim (scratch: claim_scratch_words(n_slots) words); live particles per
// cell of a window of sw x sh cells at (ox, oy) into out (zeroed first).
uint32_t claim_scratch_words(uint32_t n_slots);
void launch_claim(float4* part, uint32_t n_slots, const float4* spawn, uint32_t claim, uint32_t* scratch,
                  cudaStream_t st);
void launch_cell_counts(const float4* part, uint32_t n_slots, int ox, int oy, int sw, int sh, uint32_t* out,
                        cudaStream_t st);
// The same claim with the entry count on the device: entries spawn[skip ..] of *count.
struct EmitState;
void launch_claim_dev(float4* part, uint32_t n_slots, const float4* spawn, const EmitState* st, uint32_t skip,
                      uint32_t* scratch, cudaStream_t s);
// The brush's emitters on the device (emit.cu). EmitArgs: one emission as World::emit issues it
// (host-computed bounds and constants); EmitState: the emitters' device state (World::rand's
// generator, the next particle id, particles queued since the last step call, this
// emission's count and the running total).
constexpr int EMIT_STREAM = 0, EMIT_PAINT = 1, EMIT_RAIN = 2;
struct EmitArgs {
    int mode, W, H, ppc;
    float from[2], to[2];
    // stream: the spout and the frame's range of lattice indices [k0, k0 + ncand)
    float dir[2], speed, width, vel[2];
    double start, end, rate;
    uint64_t k0;
    uint32_t ncand, keep;
    // paint: the stroke's lattice bounds; rain: the cloud
    float radius, spacing, at[2], half;
    int lat_lo[2], lat_hi[2];
    uint32_t count, spray, limit;
    // the admission window [win_lo, win_lo + win_size)
    int win_lo[2], win_size[2];
    // the settled template particle
    float s, t;
    uint32_t kind;
};
struct EmitState {
    uint32_t rng, next_id, queued, count;
    unsigned long long total;
};
void launch_emit(const EmitArgs& a, float2* cand, uint8_t* flag, uint32_t* room, const float* sdf, float4* q,
                 EmitState* st, StepState* S, cudaStream_t s);
void launch_emit_fresh(float4* part, uint32_t base, uint32_t fresh, const float4* q, const EmitState* st,
                       cudaStream_t s);
void launch_spawn_ids(float4* part, uint32_t base, uint32_t fresh, float4* q, uint32_t n, EmitState* st,
                      cudaStream_t s);
// stats.comp: the census of the particle slots into out (stats_words() words, zeroed first):
// live particles, per material row its particles and their concentration in 1/256.
constexpr int kStatsRows = 96;   // the material table's rows (MAX_MATERIALS)
constexpr uint32_t stats_words() { return 1u + 2u * (uint32_t)kStatsRows; }
void launch_stats(const float4* part, uint32_t n_slots, uint32_t* out, cudaStream_t st);
void launch_grid(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st);
// rigid.comp's five modes at the end of a substep (tanks with CAP_RIGID)
void launch_rigid(const DevScene& d, cudaStream_t st);
// `second`: the pressure solve after the implicit viscosity (same matrix and hierarchy).
cudaError_t launch_pressure(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st, int second);
void launch_project(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st);
// The implicit viscosity: the passes before the solve (split, diagonal, multigrid levels),
// the solve itself (`restrain`: take the strain of u* again first), and the right-hand side
// and projection of the second pressure solve.
void launch_viscosity_setup(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st);
cudaError_t launch_viscosity(const DevScene& d, const LaunchCfg& cfg, cudaStream_t st, int restrain);
// The viscosity solves of a batch of tanks (all with the same sweep count) in one persistent
// kernel over their flattened active-tile lists.
struct VBatchView {
    const DevScene* scenes;   // ns tanks
    int ns;
    const int* off0;          // the ns + 1 prefix sums of the tanks' level-0 tile counts
    void* scal;               // per tank, the solve's scalars (viscosity_batch_scalar_bytes each)
    SolveState* K;            // the batch's grid barrier and error word
    int* aoff;                // per level 0 .. max_lev, the ns + 1 prefix sums of active tiles (filled)
    int max_lev;              // the most coarse levels over the tanks
};
size_t viscosity_batch_scalar_bytes();
cudaError_t launch_viscosity_batch(const VBatchView& B, int sweeps, int blocks, cudaStream_t st);
void launch_second_projection_rhs(const DevScene& d, cudaStream_t st);
void launch_second_projection(const DevScene& d, cudaStream_t st);
// Blocks of the persistent viscosity kernel that fit on the device at once.
int viscosity_blocks_max(int device, int sweeps);

// A batch of scenes for one persistent pressure solve over all of them (device arrays).
struct BatchView {
    const DevScene* scenes;   // ns scenes
    int ns;
    const int* off;           // level l: the ns + 1 prefix sums of the scenes' level-l tiles at l * (ns + 1)
                              // (a scene counts its levels 0 .. tail)
    void* scal;               // per scene, the solve's scalars (pressure_batch_scalar_bytes each)
    const int* scale;         // per scene, the warm-start mode of cg_scale (0 or 1)
    SolveState* K;            // the batch's grid barrier and error word
    int max_tail;             // the deepest tail level over the scenes
    int* aoff;                // the same prefix sums over the scenes' active tiles (the kernel fills it)
};
// The batched pressure solve: `second` for the solve after the implicit viscosity.
cudaError_t launch_pressure_batch(const BatchView& B, bool mixed, int blocks, size_t smem, cudaStream_t st, int second);
int pressure_batch_blocks_max(int device, size_t smem, bool mixed);
size_t pressure_batch_scalar_bytes();
// The render side's cell passes (optics.cu): cell_optics.comp into raw (20 layers of RGBA16F
// texels, layer-major), light.comp into raw's layer 10, optics_blur.comp into smooth's layers
// 0-19, sss.comp into its layers 20-23 (sss_iters Jacobi iterations, rounded up to even),
// flow_map.comp into flow (four layers: copy 0 short and long period, copy 1 short and long)
// when the clock says it runs, glow.comp into glow_a then glow_b (half resolution).
struct DevOptics;
struct RenderClock;
// spike_gap, spike_mc: the ferrofluid spikes' spacing (cells; 0: none) and Rosensweig
// threshold mu0 Mc (T), FluidSim::spike_params.
// dfield, dust: spray.comp's dust field (4 ints a cell: the specks' absorption and scattering
// x 1024) and whether it is read (a speck liquid in a tank whose pool has run).
void launch_cell_optics(const DevScene& d, const DevOptics* opt, float inv_speed, float spike_gap, float spike_mc,
                        const int* dfield, float dust, int sss_iters, ushort4* raw, ushort4* smooth, ushort4* flow,
                        const RenderClock* clock, ushort4* glow_a, ushort4* glow_b, cudaStream_t st);
// The clock of a render call (record_cell_optics, mod.rs:1628-1641, 1674-1680): `valid` 0 for
// the first call on a new tank (no step: the flow map does not run), `changed` 0 when the call
// records nothing (its key is the last call's); the time since the last call from the
// device's own simulated time.
// The end of a frame (a step call, or each substep of a profile): FluidSim's adaptation of the
// recorded iteration counts from the frame's solves (mod.rs:3093-3114) and the next limits.
void launch_frame_end(const DevScene& d, cudaStream_t st);
void launch_frame_end_many(const DevScene* scenes, int n, cudaStream_t st);   // a batch's members
void launch_render_clock(const DevScene& d, RenderClock* clock, int valid, int changed, cudaStream_t st);
// look.comp over the particle slots (d.plook must be allocated): the platelets' orientation of
// each particle of a liquid with a look, evolved by the clock's dt, and the slots listed for
// the look splat (*count of them, at most cap in list). `frame`: FluidSim's frame counter.
void launch_look(const DevScene& d, const DevOptics* opt, const RenderClock* clock, uint32_t frame, uint32_t* count,
                 uint32_t* list, uint32_t cap, uint32_t n_slots, cudaStream_t st);
// spray.comp's pool (spray.cu): an entry (the reference's Diffuse, 32 bytes), the pool's
// counters (entries never handed out so far, the free stack's height, the live entries listed,
// this frame's emissions), and its buffers.
constexpr uint32_t kDiffuseMax = 1u << 16;   // mod.rs DIFFUSE_MAX: bubbles, foam and spray
constexpr uint32_t kDustMax = 1u << 17;      // mod.rs DUST_MAX: the specks' part, after them
constexpr uint32_t kPoolMax = kDiffuseMax + kDustMax;
struct DevDiffuse {
    float px, py, vx, vy, life, r;
    uint32_t info;
    float z;
};
static_assert(sizeof(DevDiffuse) == 32, "Diffuse is 32 bytes");
struct PoolState {
    uint32_t hw, top, listed, total;   // bubbles' part (listed: both parts)
    uint32_t hw1, top1, total1, pad;   // the specks' part
};
struct SprayBufs {
    DevDiffuse* pool;                     // kPoolMax entries
    uint32_t *stack, *stack1, *list;      // free stacks of the two parts, the live entries
    uint32_t *dcount;                     // foam per cell (copies 0, 1), resting specks (2, 3)
    uint32_t *counts, *bsum, *flags;      // stage 0's ranks, scan partials, stage 1's flags
    uint32_t* nspeck;                     // per particle slot + 1: the specks it brings in, ranked
    int* dfield;                          // the dust field, 4 ints a cell
    PoolState* ps;
};
// look.comp's specks (lines 103-128): a new particle of a liquid with specks brings its share
// of them into the pool's second part, ranked in slot order (the engine's slot order is the
// oracle's); runs before launch_look, which marks the particles seen.
void launch_specks(const DevScene& d, const DevOptics* opt, const SprayBufs& b, uint32_t frame, uint32_t n_slots,
                   cudaStream_t st);
// record_spray: stage 0 (when `makes`, and the clock's dt > 0) and stage 1 of spray.comp, the
// foam counted into copy `parity` of dcount. `amount`: params.bubbles.
void launch_spray(const DevScene& d, const ushort4* smooth, const DevOptics* opt, const SprayBufs& b,
                  const RenderClock* clock, uint32_t frame, uint32_t parity, float amount, bool makes, cudaStream_t st);
// The renderer's particle fields for one view (draw.cu; Renderer::render, render.rs:886-1075).
// One splat pass: the view's map (centre, zoom in pixels per cell, texels of div pixels from
// the top-left of an extent of 2 half_w x 2 half_h pixels), its kernel and the used texels.
struct DrawPass {
    float cx, cy, zoom, div, half_w, half_h;
    float radius, weight, exposure;
    int w, h, mode;         // 0 the sharp field, 1 the tint field, 2 the look field
    float izoom, iradius;   // 1 / zoom, 1 / radius
    float hx, hy, hz;       // the look field: the half vector between the key light and the viewer
};
// The wide field's layout (WideLayout): used texels, bilinear taps per axis, sharp-field
// texels per wide texel, the blur's step (half a standard deviation) in texels.
struct DrawWide {
    int w, h, taps;
    float factor, step;
};
struct DrawBufs {
    long long *acc, *tacc;              // fixed-point texel sums (2^-32): 4 and 8 a texel
    ushort4 *sharp, *conc, *share;      // RGBA16F: the sharp field, the tint field's two images
    ushort4 *wide0, *wide1;             // the wide field (finished in wide0) and the blur's other image
    ushort4* look;                      // the look field (the sharp field's texels)
};
// splat (+ tint, + look over look_list = [count, slots ...] when given), then the wide field:
// down, blur across, blur down.
void launch_draw(const DevScene& d, const DevOptics* opt, uint32_t n_slots, const DrawPass& sharp, const DrawPass* tint,
                 const DrawPass* look, const uint32_t* look_list, const DrawWide& wide, DrawBufs& b, cudaStream_t st);
// The wet map (wet.frag) once per simulated time: the clock reads the time after the last
// substep on the device and lets the pass run when it moved.
struct WetClock {
    double last;
    float now;
    uint32_t run, valid, pad;
};
void launch_wet(const DevScene& d, WetClock* clock, float4* wet, cudaStream_t st);
// Scene::rasterize on the device (raster.cu): the tank's solid fields straight into device
// buffers, bit-identical to the host's Scene::rasterize (scene.cpp).
struct Scene;
cudaError_t rasterize_device(const Scene& sc, float* sdf, float4* solid, uint32_t* region, float* temp, bool* heated,
                             cudaStream_t st);
// Blocks of the persistent pressure kernel (plain or mixed precision) that fit on the
// device at once.
int pressure_blocks_max(int device, size_t smem, bool mixed);
// Dynamic shared memory of the persistent pressure kernel: the tail levels of each block.
size_t pressure_smem(const Levels& lv);
// ... and of the batched one, whose staging regions share it with the tail.
size_t pressure_batch_smem(const Levels& lv);

}  // namespace sprout

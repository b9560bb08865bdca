// The engine's host side: FluidSim's lifecycle (src/sim/mod.rs:862-3474) on one CUDA
// stream, and the C ABI of include/sprout_gpu.h.
//
// A substep is recorded once into a CUDA graph (sort + P2G, grid passes, the persistent
// pressure kernel, projection) and replayed; the per-call data (parameters, tool, the
// batch's target time) live in device memory the graph reads, so one graph serves every
// call until the tank's configuration (particle slots, capabilities, viscosity mode)
// changes. The step scalars stay on the device: the substep length is picked there
// (step.comp), and solve iterations end on the device (no host-recorded counts).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/sprout_gpu.h"
#include "dev_common.cuh"
#include "kernels.h"
#include "optics.h"
#include "params.h"
#include "scene.h"

using namespace sprout;

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& msg) {
    g_error = msg;
    return code;
}

#define CUDA_TRY(expr)                                                                          \
    do {                                                                                         \
        cudaError_t e_ = (expr);                                                                 \
        if (e_ != cudaSuccess) return fail(SPROUT_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

constexpr float kNominalDt = 1.0f / 240.0f;
static_assert(SPROUT_MATERIAL_ROWS == kStatsRows && kStatsRows == kMaxMaterials, "the census has a row per material");

// The autotuner's table (sprout_gb300/tune.py): per grid size, the block counts of the
// persistent solves that timed fastest; a sim of that size starts from them.
struct TunedLaunch {
    int w, h, pressure, pressure_mixed, viscosity;
};
constexpr TunedLaunch kTuned[] = {
#include "tuned_launch.inc"
    {0, 0, 0, 0, 0}};

SproutLaunch tuned_launch(int w, int h) {
    SproutLaunch l{};
    for (const TunedLaunch& t : kTuned)
        if (t.w == w && t.h == h) {
            l.pressure_blocks = (uint32_t)t.pressure;
            l.pressure_blocks_mixed = (uint32_t)t.pressure_mixed;
            l.viscosity_blocks = (uint32_t)t.viscosity;
        }
    return l;
}

}  // namespace

namespace sprout {
// Lets other translation units of the library report through sprout_last_error().
void sprout_internal_set_error(const char* msg) { g_error = msg ? msg : ""; }
}  // namespace sprout

struct SproutParams {
    SimParams p;
};

struct SproutScene {
    Scene s;
};

struct SproutSim {
    int W = 0, H = 0;
    uint32_t capacity = 0, n_slots = 0;
    SimParams params;
    Tank tank;
    bool thermal = false, solids_heated = false;
    uint32_t caps = 0;
    int visc_mode = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    DevScene d{};
    std::vector<void*> allocs;
    size_t bytes = 0;
    LaunchCfg cfg;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool graph_ok = false, use_graph = true;
    double sim_time = 0.0;
    float dt_est = kNominalDt;
    std::vector<float> solid_host;   // kept for nothing but the device copy's lifetime

    ~SproutSim() {
        if (stats_ev) cudaEventDestroy(stats_ev);
        if (h_stats) cudaFreeHost(h_stats);
        if (trace_buf) cudaFree(trace_buf);
        if (d_window) cudaFree(d_window);
        if (h_window) cudaFreeHost(h_window);
        for (void* p : emit_bufs) cudaFree(p);
        drop_part_graphs();
        if (cap_stream) cudaStreamDestroy(cap_stream);
        if (stage_params) cudaFreeHost(stage_params);
        if (stage_mats) cudaFreeHost(stage_mats);
        if (stage_done) cudaEventDestroy(stage_done);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (void* p : allocs) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }

    template <class T>
    int alloc(T** out, size_t n) {
        void* p = nullptr;
        size_t b = std::max<size_t>(n, 1) * sizeof(T);
        if (cudaMalloc(&p, b) != cudaSuccess) return fail(SPROUT_E_NOMEM, "device allocation of " + std::to_string(b) + " bytes failed");
        cudaMemset(p, 0, b);
        allocs.push_back(p);
        bytes += b;
        *out = static_cast<T*>(p);
        return SPROUT_OK;
    }

    // The implicit viscosity's buffers, allocated the first time a tank needs the solve.
    bool visc_alloc = false;
    int visc_max[2] = {0, 0};   // co-resident blocks of the viscosity kernel, 1 and 2 sweeps

    int ensure_visc_buffers() {
        if (visc_alloc) return SPROUT_OK;
        size_t nc = (size_t)W * H, tot = (size_t)d.lv.total;
        int rc = SPROUT_OK;
#define A(ptr, n) do { if ((rc = alloc(&(ptr), (n))) != SPROUT_OK) return rc; } while (0)
        A(d.vr, nc); A(d.vr2, nc); A(d.vp, nc); A(d.vq, nc); A(d.vq2, nc); A(d.vd, nc); A(d.vaz, nc);
        A(d.vma, tot); A(d.vmb, tot); A(d.vmd, tot); A(d.vmr, tot); A(d.vmx, tot); A(d.vmz, tot);
        A(d.tiles, (size_t)d.nwg);
        A(d.vtile, (size_t)d.lv.tiles);
        A(d.vlist, (size_t)d.lv.tiles);
        A(d.vcount, (size_t)kMaxLevels);
#undef A
        visc_max[0] = viscosity_blocks_max(device, 1);
        visc_max[1] = viscosity_blocks_max(device, 2);
        CUDA_TRY(cudaDeviceSynchronize());
        visc_alloc = true;
        // a new set of device pointers: the captured substep is stale
        graph_ok = false;
        return SPROUT_OK;
    }

    // The mixed-precision pressure solve: its BF16 matrices and FP64 partial sums,
    // allocated the first time it is asked for.
    bool mixed = false, mixed_alloc = false;

    int set_precision(int mode) {
        if (mode != 0 && mode != 1) return fail(SPROUT_E_ARG, "precision mode is 0 (plain FP32) or 1 (mixed)");
        if (mode == 1 && !mixed_alloc) {
            CUDA_TRY(cudaStreamSynchronize(stream));
            size_t tot = (size_t)d.lv.total;
            int rc = SPROUT_OK;
#define A(ptr, n) do { if ((rc = alloc(&(ptr), (n))) != SPROUT_OK) return rc; } while (0)
            A(d.hga, tot); A(d.hgd, tot); A(d.hgi, tot);
            A(d.partials64, 2 * (size_t)d.nwg);
#undef A
            mg_max_mixed = pressure_blocks_max(device, pressure_smem(d.lv), true);
            cfg.mg_blocks_mixed = pick_blocks(launch_req.pressure_blocks_mixed, mg_max_mixed, tuned.pressure_blocks_mixed);
            CUDA_TRY(cudaDeviceSynchronize());
            mixed_alloc = true;
            graph_ok = false;   // new device pointers: the captured substep is stale
        }
        mixed = mode == 1;
        return SPROUT_OK;
    }

    // The solvers' phase trace: rows > 0 turns it on (rows barrier generations kept, one
    // column per block of the widest persistent kernel plus block 0's leaving time), 0 off.
    unsigned long long* trace_buf = nullptr;
    uint32_t trace_rows = 0, trace_cols = 0;
    int trace_enable(uint32_t rows) {
        CUDA_TRY(cudaStreamSynchronize(stream));
        if (trace_buf) {
            cudaFree(trace_buf);
            trace_buf = nullptr;
        }
        trace_rows = rows;
        trace_cols = rows ? (uint32_t)std::max({cfg.mg_blocks, cfg.mg_blocks_mixed, cfg.visc_blocks, 1}) + 1 : 0;
        if (rows) {
            size_t b = (size_t)trace_rows * trace_cols * 8;
            if (cudaMalloc(&trace_buf, b) != cudaSuccess) return fail(SPROUT_E_NOMEM, "trace buffer");
            CUDA_TRY(cudaMemset(trace_buf, 0, b));
        }
        SolveState K0;
        CUDA_TRY(cudaMemcpy(&K0, d.K, sizeof K0, cudaMemcpyDeviceToHost));
        K0.trace = trace_buf;
        K0.trace_rows = trace_rows;
        K0.trace_cols = trace_cols;
        CUDA_TRY(cudaMemcpy(d.K, &K0, sizeof K0, cudaMemcpyHostToDevice));
        return SPROUT_OK;
    }

    // The viscosity treatment of the tank (FluidSim::viscosity_mode, mod.rs:2768-2792),
    // re-derived before every record as the reference does, and what this engine carries.
    int derive_viscosity() {
        visc_mode = viscosity_mode();
        if (visc_mode != 2) return SPROUT_OK;
        if (params.viscosity_precond != 0 && d.lv.tail < 1)
            return fail(SPROUT_E_UNSUPPORTED, "the multigrid-preconditioned viscosity solve needs a grid with at least one multigrid level below it");
        return ensure_visc_buffers();
    }

    int init(uint32_t w, uint32_t h, uint32_t cap, const SimParams& prm) {
        W = (int)w;
        H = (int)h;
        capacity = cap;
        params = prm;
        CUDA_TRY(cudaGetDevice(&device));
        CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        d.W = W;
        d.H = H;
        d.ncell = W * H;
        d.stride = 8;
        d.capacity = cap;
        d.lv = make_levels(W, H);
        d.nwg = ((W + 15) / 16) * ((H + 15) / 16);
        size_t nc = (size_t)W * H;
        int rc = SPROUT_OK;
#define A(ptr, n) do { if ((rc = alloc(&(ptr), (n))) != SPROUT_OK) return rc; } while (0)
        DevParams* P;
        DevMat* M;
        StepState* S;
        SolveState* K;
        A(P, 1);
        A(M, kMaxMaterials);
        A(S, 1);
        A(K, 1);
        d.P = P;
        d.mats = M;
        d.S = S;
        d.K = K;
        A(d.part, 3 * (size_t)cap);
        A(d.part2, 3 * (size_t)cap);
        A(d.pkey, cap);
        A(d.prank, cap);
        A(d.perm, cap);
        A(d.crowd, nc + 1);
        A(d.count, nc + 1);
        A(d.start, nc + 1);
        A(d.scan_tmp, (nc + 1 + 1023) / 1024 + 1);
        A(d.acc, nc * 32);
        A(d.vel, nc); A(d.cell, nc); A(d.comp, nc); A(d.coef, nc); A(d.sprop, nc); A(d.surf, nc);
        A(d.surf2, nc); A(d.aux, nc); A(d.grho, nc); A(d.gbase, nc); A(d.rh, nc); A(d.magc, nc); A(d.rl, nc); A(d.rbody, (size_t)kMaxBodies * 16); A(d.nbodies, 1); A(d.therm, nc); A(d.dheat, nc); A(d.vw, nc);
        A(d.vs, nc); A(d.prhs, nc); A(d.vel0, nc); A(d.pjump, nc); A(d.pres, nc); A(d.p2keep, nc);
        A(d.hcell, nc);
        float4* solid;
        float* sdf;
        uint32_t* region;
        float* solid_t;
        A(solid, nc);
        A(sdf, (size_t)(W + 1) * (H + 1));
        A(region, nc);
        A(solid_t, nc);
        d.solid = solid;
        d.sdf = sdf;
        d.region = region;
        d.solid_t = solid_t;
        A(d.ledger, 8);
        A(d.mga, (size_t)d.lv.total);
        A(d.mgd, (size_t)d.lv.total);
        A(d.mgx, (size_t)d.lv.total);
        A(d.mgz, (size_t)d.lv.total);
        A(d.mgr, (size_t)d.lv.total);
        A(d.mgr2, nc);
        A(d.cgp, nc);
        A(d.cgp2, nc);
        A(d.cgq, nc);
        A(d.ptile, (size_t)d.lv.tiles);
        A(d.plist, (size_t)d.lv.tiles);
        A(d.pcount, (size_t)kMaxLevels);
        A(d.partials, 2 * (size_t)d.nwg);
#undef A
        CUDA_TRY(cudaMemset(d.rl, 0xff, nc * sizeof(int2)));   // no cell rigid before the first rigid pass
        std::vector<float> nt(nc, NO_TEMP);
        CUDA_TRY(cudaMemcpy(solid_t, nt.data(), nc * sizeof(float), cudaMemcpyHostToDevice));
        tuned = tuned_launch(W, H);
        mg_max = pressure_blocks_max(device, pressure_smem(d.lv), false);
        cfg.mg_blocks = pick_blocks(launch_req.pressure_blocks, mg_max, tuned.pressure_blocks);
        CUDA_TRY(cudaDeviceSynchronize());
        return SPROUT_OK;
    }

    // The persistent solvers' block counts: the caller's request (0: one block per level-0
    // tile), at most what the device holds at once (mx).
    // tuned: the autotuner's counts for this grid size (0 where it has none).
    SproutLaunch launch_req{}, tuned{};
    int mg_max = 1, mg_max_mixed = 1;
    int pick_blocks(uint32_t want, int mx, uint32_t tuned_count) const {
        if (want == 0u) want = tuned_count;
        const int b = want != 0u ? (int)std::min<uint32_t>(want, (uint32_t)d.nwg) : d.nwg;
        return std::max(1, std::min(b, std::max(mx, 1)));
    }
    int set_launch(const SproutLaunch& l) {
        CUDA_TRY(cudaStreamSynchronize(stream));
        launch_req = l;
        cfg.mg_blocks = pick_blocks(l.pressure_blocks, mg_max, tuned.pressure_blocks);
        if (mixed_alloc) cfg.mg_blocks_mixed = pick_blocks(l.pressure_blocks_mixed, mg_max_mixed, tuned.pressure_blocks_mixed);
        graph_ok = false;   // the captured substep launches the old counts
        return SPROUT_OK;
    }
    void get_launch(SproutLaunch* out) const {
        *out = SproutLaunch{};
        out->pressure_blocks = (uint32_t)cfg.mg_blocks;
        out->pressure_blocks_mixed = mixed_alloc ? (uint32_t)cfg.mg_blocks_mixed : 0u;
        const int sw = (int)std::min(std::max(params.viscosity_mg_sweeps, 1u), 2u);
        out->viscosity_blocks =
            visc_alloc ? (uint32_t)pick_blocks(launch_req.viscosity_blocks, visc_max[sw - 1], tuned.viscosity_blocks) : 0u;
        out->batch_viscosity = launch_req.batch_viscosity;
    }

    // Failure injection for tests: the fields of SolveState the grid barrier reads.
    int debug_stall(uint32_t block, uint32_t stall_ns, uint32_t spin_limit) {
        CUDA_TRY(cudaStreamSynchronize(stream));
        SolveState K0;
        CUDA_TRY(cudaMemcpy(&K0, d.K, sizeof K0, cudaMemcpyDeviceToHost));
        K0.dbg_block = block;
        K0.dbg_stall_ns = stall_ns;
        K0.dbg_spin_limit = spin_limit;
        CUDA_TRY(cudaMemcpy(d.K, &K0, sizeof K0, cudaMemcpyHostToDevice));
        return SPROUT_OK;
    }

    float dt_limit() const {
        float dt = std::min(params.dt_max, params.dt_capillary(tank.rows));
        if (thermal) dt = std::min(dt, params.dt_thermal(tank.rows));
        return std::min(dt, params.dt_elastic(tank.rows));
    }

    int viscosity_mode() const {
        float dt = dt_limit();
        float dmax = 0.0f;
        for (int r : tank.rows) {
            const MatProps& m = params.mat[r];
            float cells = 1.0f / (params.cell_size * params.cell_size);
            float nu;
            if (!thermal) nu = m.viscosity_at(params.ambient_temp) * cells;
            else if (m.freezes() || m.temp_model != 0) nu = INFINITY;
            else nu = m.viscosity * cells;
            dmax = std::max(dmax, nu * dt);
        }
        if (dmax <= 0.0f) return 0;
        if (dmax <= 0.05f) return 1;
        return 2;
    }

    // The particles' stress buffers while the tank holds an elastic material (set_elastic,
    // mod.rs:2084-2110): zero-filled each time they are taken up again.
    bool elastic_on = false;
    int set_elastic(bool on) {
        if (on == elastic_on) return SPROUT_OK;
        if (on) {
            if (!d.pstress) {
                int rc = alloc(&d.pstress, (size_t)capacity);
                if (rc == SPROUT_OK) rc = alloc(&d.pstress2, (size_t)capacity);
                if (rc == SPROUT_OK) rc = alloc(&d.pdep, (size_t)capacity);
                if (rc == SPROUT_OK) rc = alloc(&d.estr, (size_t)W * H);
                if (rc != SPROUT_OK) return rc;
            } else {
                CUDA_TRY(cudaMemsetAsync(d.pstress, 0, (size_t)capacity * sizeof(float4), stream));
            }
            graph_ok = false;   // new device pointers: the captured substep is stale
        }
        elastic_on = on;
        return SPROUT_OK;
    }

    // Whether a family in the tank settles: a concentrate with grains under gravity (mod.rs:2139-2143).
    bool settles() const {
        if (!(params.gravity > 0.0f)) return false;
        for (int r : tank.rows)
            if (params.mat[r].diluent >= 0 && params.mat[r].grain > 0.0f) return true;
        return false;
    }

    // The settling buffers for `fams` families (mod.rs:2114-2136): new zero-filled ones when the
    // count grows or drops to none, the present ones otherwise.
    int settle_fams = 0;
    std::vector<Current> currents;   // set_currents: kept across resets, like the reference's
    std::vector<Magnet> magnets;     // set_magnets: likewise
    int set_settling(int fams) {
        if (fams == settle_fams || (fams > 0 && fams < settle_fams)) return SPROUT_OK;
        const size_t n = std::max<size_t>((size_t)W * H * (size_t)fams, 1);
        int rc = alloc(&d.famocc, n);
        if (rc == SPROUT_OK) rc = alloc(&d.dsettle, n);
        if (rc != SPROUT_OK) return rc;
        settle_fams = fams;
        graph_ok = false;   // new device pointers: the captured substep is stale
        return SPROUT_OK;
    }

    uint32_t compute_caps() const {
        uint32_t c = 0;
        if (tank.families > 0) c |= CAP_FAMILIES;
        if (settle_fams >= tank.families && tank.families > 0 && settles()) c |= CAP_SETTLE;
        if (tank.chan_e >= 0 && elastic_on) c |= CAP_ELASTIC;   // mod.rs:2746-2748
        if (thermal) c |= CAP_THERMAL;
        bool rigid = false;
        for (int r : tank.rows) {
            const MatProps& m = params.mat[r];
            const MatProps* dil = m.diluent >= 0 ? &params.mat[m.diluent] : nullptr;
            if (m.rheology != 0 || m.skin > 0.0f || m.friction > 0.0f) {
                c |= CAP_RHEO;
                rigid |= m.rheology == 2 || m.rheology == 3 || m.skin > 0.0f || m.friction > 0.0f;
            }
            if (thermal) rigid |= m.freezes() || (dil && dil->freezes()) || m.temp_model != 0 || (dil && dil->temp_model != 0);
            rigid |= m.viscosity_at(params.ambient_temp) >= params.rigid_viscosity || (!thermal && m.freezes() && params.ambient_temp < m.melt_hi);
            if (!magnets.empty() && m.susceptibility > 0.0f) c |= CAP_MAGNET;
            if (m.react_with >= 0 && m.react_rate > 0.0f && std::find(tank.rows.begin(), tank.rows.end(), m.react_with) != tank.rows.end()) c |= CAP_REACT;
            if (r == 57 && thermal) c |= CAP_STEAM;
        }
        if (rigid) c |= CAP_RIGID;
        return c;
    }

    // The parameters and material table in grid units, uploaded when they change (the
    // reference re-uploads its uniform every record and the table when it changed,
    // mod.rs:2512-2520). Pinned staging, so the copies stay asynchronous; a copy waits for
    // the previous one before its staging is rewritten.
    DevParams* stage_params = nullptr;
    DevMat* stage_mats = nullptr;
    cudaEvent_t stage_done = nullptr;
    DevParams last_params{};
    std::vector<DevMat> last_mats;
    size_t h2d_bytes = 0, d2h_bytes = 0;

    int upload_tables(const ToolState* tool) {
        if (!stage_params) {
            CUDA_TRY(cudaMallocHost(&stage_params, sizeof(DevParams)));
            CUDA_TRY(cudaMallocHost(&stage_mats, sizeof(DevMat) * kMaxMaterials));
            CUDA_TRY(cudaEventCreateWithFlags(&stage_done, cudaEventDisableTiming));
        }
        DevParams P;
        build_params(params, tank, thermal, caps, W, H, n_slots, dt_limit(), tool, &P, currents, magnets);
        P.ext_speed = std::max(P.ext_speed, spawn_speed);   // mod.rs:2300
        P.visc_mode = visc_mode;
        P.visc_levels = std::min(P.visc_levels, d.lv.tail);
        std::vector<DevMat> mats(kMaxMaterials);
        build_materials(params, tank, thermal, mats.data());
        bool pchg = std::memcmp(&P, &last_params, sizeof P) != 0 || last_mats.empty();
        bool mchg = last_mats.empty() || std::memcmp(mats.data(), last_mats.data(), sizeof(DevMat) * kMaxMaterials) != 0;
        if (!pchg && !mchg) return SPROUT_OK;
        enqueued = true;
        tables_gen++;
        CUDA_TRY(cudaEventSynchronize(stage_done));
        if (pchg) {
            *stage_params = P;
            CUDA_TRY(cudaMemcpyAsync(const_cast<DevParams*>(d.P), stage_params, sizeof P, cudaMemcpyHostToDevice, stream));
            h2d_bytes += sizeof P;
            last_params = P;
        }
        if (mchg) {
            std::memcpy(stage_mats, mats.data(), sizeof(DevMat) * kMaxMaterials);
            CUDA_TRY(cudaMemcpyAsync(const_cast<DevMat*>(d.mats), stage_mats, sizeof(DevMat) * kMaxMaterials, cudaMemcpyHostToDevice, stream));
            h2d_bytes += sizeof(DevMat) * kMaxMaterials;
            last_mats = mats;
        }
        CUDA_TRY(cudaEventRecord(stage_done, stream));
        return SPROUT_OK;
    }

    // Times `substeps` substeps with CUDA events on the sim's stream (blocking).
    int profile(uint32_t substeps, float* ms) {
        cudaEvent_t a, b;
        CUDA_TRY(cudaEventCreate(&a));
        CUDA_TRY(cudaEventCreate(&b));
        int rc = ensure_graph();
        if (rc != SPROUT_OK) return rc;
        CUDA_TRY(cudaEventRecord(a, stream));
        substeps_issued += substeps;
        for (uint32_t k = 0; k < substeps; k++) {   // each substep a frame of its own
            if (use_graph && graph_ok) CUDA_TRY(cudaGraphLaunch(exec, stream));
            else record_substep(stream);
            launch_frame_end(d, stream);
        }
        CUDA_TRY(cudaEventRecord(b, stream));
        CUDA_TRY(cudaEventSynchronize(b));
        CUDA_TRY(cudaEventElapsedTime(ms, a, b));
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        if ((rc = end_emit_call()) != SPROUT_OK) return rc;
        return check_device_error();
    }

    // One substep stage by stage, each bracketed by CUDA events (profile_passes, mod.rs:3120).
    int profile_passes(float* ms) {
        int rc = ensure_graph();
        if (rc != SPROUT_OK) return rc;
        cudaEvent_t ev[kStages + 1];
        for (auto& e : ev) CUDA_TRY(cudaEventCreate(&e));
        CUDA_TRY(cudaEventRecord(ev[0], stream));
        substeps_issued++;
        for (int k = 0; k < kStages; k++) {
            record_stage(k, stream);
            CUDA_TRY(cudaEventRecord(ev[k + 1], stream));
        }
        launch_frame_end(d, stream);
        CUDA_TRY(cudaEventSynchronize(ev[kStages]));
        for (int k = 0; k < kStages; k++) CUDA_TRY(cudaEventElapsedTime(&ms[k], ev[k], ev[k + 1]));
        for (auto& e : ev) cudaEventDestroy(e);
        if ((rc = end_emit_call()) != SPROUT_OK) return rc;
        return check_device_error();
    }

    // The stages of a substep, in order (profile_passes times each one). The last two run
    // only with the implicit viscosity between two pressure solves (viscous_projection).
    static constexpr int kStages = 8;
    void record_stage(int k, cudaStream_t st) {
        switch (k) {
        case 0: launch_advance(d, cfg, st); break;
        case 1: launch_sort(d, cfg, st); break;
        case 2: launch_p2g(d, cfg, st); break;
        case 3: launch_grid(d, cfg, st); break;
        case 4: launch_pressure(d, cfg, st, 0); break;
        case 5: launch_project(d, cfg, st); break;
        case 6:
            if (cfg.visc_mode == 2 && cfg.twice) launch_viscosity(d, cfg, st, 1);
            break;
        default:
            if (cfg.visc_mode == 2 && cfg.twice) {
                launch_second_projection_rhs(d, st);
                launch_pressure(d, cfg, st, 1);
                launch_second_projection(d, st);
            }
            if (cfg.rigid) launch_rigid(d, st);   // mod.rs:2701-2707
            break;
        }
    }

    void record_substep(cudaStream_t st) {
        for (int k = 0; k < kStages; k++) record_stage(k, st);
    }

    // A batch's subset stepping replays the tank's own stages from two small graphs: the
    // particle and grid stages (0-3) and the projection (5), captured on a private stream.
    cudaGraphExec_t part_exec[2] = {nullptr, nullptr};
    LaunchCfg part_cfg{};
    bool part_ok = false;
    cudaStream_t cap_stream = nullptr;
    void drop_part_graphs() {
        for (cudaGraphExec_t& e : part_exec)
            if (e) {
                cudaGraphExecDestroy(e);
                e = nullptr;
            }
        part_ok = false;
    }
    int ensure_part_graphs() {
        if (part_ok && std::memcmp(&part_cfg, &cfg, sizeof(LaunchCfg)) == 0 &&
            std::memcmp(&part_scene, &d, sizeof(DevScene)) == 0)
            return SPROUT_OK;
        drop_part_graphs();
        if (!cap_stream) CUDA_TRY(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
        for (int g = 0; g < 2; g++) {
            cudaGraph_t graph_ = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal));
            if (g == 0)
                for (int st = 0; st < 4; st++) record_stage(st, cap_stream);
            else
                record_stage(5, cap_stream);
            CUDA_TRY(cudaStreamEndCapture(cap_stream, &graph_));
            cudaError_t e = cudaGraphInstantiate(&part_exec[g], graph_, 0);
            cudaGraphDestroy(graph_);
            CUDA_TRY(e);
        }
        part_cfg = cfg;
        part_scene = d;
        part_ok = true;
        return SPROUT_OK;
    }
    DevScene part_scene{};

    // The launch configuration for the tank as it is now; true when it changed (a captured
    // substep is then stale).
    bool refresh_cfg() {
        LaunchCfg want = cfg;
        want.n_slots = n_slots;
        want.thermal = thermal;
        want.heat = thermal && params.heat_rate > 0.0f;
        want.rheo = (caps & CAP_RHEO) != 0u;
        want.settle = (caps & CAP_SETTLE) != 0u;
        want.magnet = (caps & CAP_MAGNET) != 0u;
        want.elastic = (caps & CAP_ELASTIC) != 0u;
        want.rigid = (caps & CAP_RIGID) != 0u;
        want.xtra = tank.families > 0 || (tank.group_mask & ~1u) != 0u || !currents.empty() || tank.chan_e >= 0 || (caps & CAP_RIGID) != 0u;
        want.visc_mode = visc_mode;
        want.twice = visc_mode == 2 && params.viscous_projection != 0;
        want.viscous_warm = params.viscous_warm != 0;
        want.visc_levels = std::min((int)std::max(params.viscosity_mg_levels, 1u), d.lv.tail);
        want.visc_sweeps = (int)std::min(std::max(params.viscosity_mg_sweeps, 1u), 2u);
        want.visc_blocks = pick_blocks(launch_req.viscosity_blocks, visc_max[want.visc_sweeps - 1], tuned.viscosity_blocks);
        want.mixed = mixed;
        bool same = want.n_slots == cfg.n_slots && want.thermal == cfg.thermal && want.heat == cfg.heat && want.rheo == cfg.rheo && want.settle == cfg.settle && want.magnet == cfg.magnet && want.elastic == cfg.elastic && want.rigid == cfg.rigid && want.xtra == cfg.xtra &&
                    want.visc_mode == cfg.visc_mode && want.twice == cfg.twice && want.viscous_warm == cfg.viscous_warm &&
                    want.visc_levels == cfg.visc_levels && want.visc_sweeps == cfg.visc_sweeps &&
                    want.visc_blocks == cfg.visc_blocks && want.mixed == cfg.mixed && d.stride == std::max(tank.stride, 8);
        cfg = want;
        d.stride = std::max(tank.stride, 8);
        return !same;
    }

    int ensure_graph() {
        const bool changed = refresh_cfg();
        if ((graph_ok && !changed) || !use_graph) return SPROUT_OK;
        if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
        if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
        graph_ok = false;
        if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            use_graph = false;
            return SPROUT_OK;
        }
        record_substep(stream);
        cudaError_t e = cudaStreamEndCapture(stream, &graph);
        if (e != cudaSuccess || graph == nullptr) {
            cudaGetLastError();
            use_graph = false;
            graph = nullptr;
            return SPROUT_OK;
        }
        if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphDestroy(graph);
            graph = nullptr;
            use_graph = false;
            return SPROUT_OK;
        }
        graph_ok = true;
        return SPROUT_OK;
    }

    // Particle::settle_spawn (params.rs:70-85) and the position range every substep leaves a
    // particle in, [2.01, size - 2.01] (particles.comp:912), so that the first gather's 3 x 3
    // stencils stay on the grid.
    int settle(SproutParticle& q, uint32_t k) const {
        if (!std::isfinite(q.pos[0]) || !std::isfinite(q.pos[1]))
            return fail(SPROUT_E_ARG, "particle " + std::to_string(k) + " has a non-finite position");
        q.pos[0] = std::min(std::max(q.pos[0], 2.01f), (float)W - 2.01f);
        q.pos[1] = std::min(std::max(q.pos[1], 2.01f), (float)H - 2.01f);
        uint32_t mat = q.kind & 255u;
        if (q.kind != 0u && mat != 0u) {
            const MatProps& def = params.mat[mat - 1u];
            if (q.t == -1.0e4f) {
                q.t = def.spawn_temp;
                q.kind |= 0x20000u;
            }
            if (q.s == -1.0f) q.s = def.diluent >= 0 ? std::min(std::max(def.load, 0.0f), 1.0f) : 1.0f;
            if (q.kind & 0x20000u) {
                q.kind &= ~0x20000u;
                q.t = params.enthalpy_temp((int)mat - 1, q.s, q.t);
            }
        }
        return SPROUT_OK;
    }

    // The materials of particles marked in present[], *th widened by their temperatures
    // (note_materials, mod.rs:2050-2060).
    void mark_materials(const SproutParticle* ps, uint32_t n, bool* present, bool* th) const {
        for (uint32_t k = 0; k < n; k++) {
            uint32_t m = ps[k].kind & 255u;
            if (m == 0u || ps[k].kind == 0u) continue;
            present[m - 1u] = true;
            *th |= std::fabs(ps[k].t - params.ambient_temp) > 0.05f || params.mat[m - 1u].self_heat > 0.0f;
        }
    }

    // The tank for the rows marked in present[] and the thermal flag (Tank::layout,
    // mod.rs:271-329) with the capabilities and viscosity treatment that follow. Changes
    // nothing unless every check passes: SPROUT_E_CAPACITY when the rows do not fit the
    // accumulator channels, SPROUT_E_UNSUPPORTED for what this engine does not carry.
    int set_tank(const bool* present, bool th) {
        std::vector<int> rows;
        for (int r = 0; r < kMaxMaterials; r++)
            if (present[r]) {
                if (params.mat[r].diluent >= 0 && !present[params.mat[r].diluent]) rows.push_back(params.mat[r].diluent);
                rows.push_back(r);
            }
        std::sort(rows.begin(), rows.end());
        rows.erase(std::unique(rows.begin(), rows.end()), rows.end());
        Tank t;
        if (!t.layout(rows, params, th)) return fail(SPROUT_E_CAPACITY, "the tank's materials do not fit the accumulator channels");
        const Tank old_tank = tank;
        const bool old_thermal = thermal;
        const uint32_t old_caps = caps;
        const int old_visc = visc_mode;
        tank = t;
        thermal = th;
        caps = compute_caps();
        int rc = SPROUT_OK;
        if (caps & (CAP_STEAM | CAP_REACT))
            rc = fail(SPROUT_E_UNSUPPORTED, "the tank needs steam / reaction passes, which this engine does not carry");
        for (int r : tank.rows) {
            const MatProps& m = params.mat[r];
            if (rc == SPROUT_OK && (m.volatility > 0.0f || (thermal && m.boil < 1e8f)))
                rc = fail(SPROUT_E_UNSUPPORTED, "evaporation and boiling are not carried by this engine");
        }
        if (rc == SPROUT_OK) rc = set_settling(settles() ? tank.families : 0);
        if (rc == SPROUT_OK) rc = set_elastic(tank.chan_e >= 0);
        if (rc == SPROUT_OK) caps = compute_caps();   // with the settling buffers in place
        if (rc == SPROUT_OK && tank.families > 1 && d.mixb == nullptr) {
            // the concentrations of families 1.. per cell, from the first tank that has them
            rc = alloc(&d.mixb, (size_t)W * H * (kMaxPresent - 1));
            graph_ok = false;   // new device pointers: the captured substep is stale
        }
        if (rc == SPROUT_OK) rc = derive_viscosity();
        if (rc != SPROUT_OK) {
            tank = old_tank;
            thermal = old_thermal;
            caps = old_caps;
            visc_mode = old_visc;
            return rc;
        }
        return SPROUT_OK;
    }

    int reset(const SproutParticle* in, uint32_t n) {
        if (n > capacity) n = capacity;
        std::vector<SproutParticle> ps(in, in + n);
        for (uint32_t k = 0; k < n; k++) {
            ps[k].id = k;
            int rc = settle(ps[k], k);
            if (rc != SPROUT_OK) return rc;
        }
        bool present[kMaxMaterials] = {};
        bool th = solids_heated;
        mark_materials(ps.data(), n, present, &th);
        if (std::fabs(params.ambient_temp - kTRef) > 0.05f) th = true;
        int rc = set_tank(present, th);
        if (rc != SPROUT_OK) return rc;
        n_slots = n;
        next_id = n;
        pending.clear();
        if (d_emit) {
            const uint32_t w2[2] = {n, 0u};   // next_id, queued
            CUDA_TRY(cudaMemcpyAsync(&d_emit->next_id, w2, sizeof w2, cudaMemcpyHostToDevice, stream));
            CUDA_TRY(cudaStreamSynchronize(stream));
        }
        spawn_speed = 0.0f;
        was_reset = true;
        d.stride = std::max(tank.stride, 8);
        CUDA_TRY(cudaStreamSynchronize(stream));
        size_t nc = (size_t)W * H;
        if (n > 0) CUDA_TRY(cudaMemcpy(d.part, ps.data(), (size_t)n * sizeof(SproutParticle), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemset(d.pres, 0, nc * sizeof(float2)));
        CUDA_TRY(cudaMemset(d.p2keep, 0, nc * sizeof(float)));
        CUDA_TRY(cudaMemset(d.S, 0, sizeof(StepState)));
        {
            SolveState K0;
            std::memset(&K0, 0, sizeof K0);
            // a new scene records the most until its frames say otherwise (mod.rs:2478-2483)
            K0.rec[0] = K0.rec[1] = params.pressure_max_iters;
            K0.rec[2] = params.viscosity_max_iters;
            for (int k = 0; k < 3; k++) K0.cap[k] = recorded_limit(K0.rec[k], k == 2, params.viscosity_precond != 0);
            K0.trace = trace_buf;
            K0.trace_rows = trace_rows;
            K0.trace_cols = trace_cols;
            CUDA_TRY(cudaMemcpy(d.K, &K0, sizeof K0, cudaMemcpyHostToDevice));
        }
        CUDA_TRY(cudaMemset(d.dheat, 0, nc * sizeof(float4)));
        CUDA_TRY(cudaMemset(d.ledger, 0, 8 * sizeof(unsigned long long)));
        sim_time = 0.0;
        dt_est = kNominalDt;
        resets++;
        stain_valid = false;
        return upload_tables(nullptr);
    }

    // FluidSim::spawn (mod.rs:2024-2046): particles queued for the next step call, at most
    // kSpawnMax queued; ids follow the last given; settle_spawn; KIND_FRESH. *accepted = 0
    // when their materials do not fit the tank (nothing changes then). Particles without a
    // material are not queued (reset drops them too, mod.rs:1994).
    static constexpr uint32_t kSpawnMax = 32768;   // mod.rs:63
    std::vector<SproutParticle> pending;
    uint32_t next_id = 0;
    float spawn_speed = 0.0f;
    bool was_reset = false;
    float4* d_spawn = nullptr;        // kSpawnMax particles: the entries that claim dead slots
    uint32_t* d_claim = nullptr;      // claim_scratch_words(capacity)
    uint32_t* d_window = nullptr;     // cell_counts' window
    size_t window_cap = 0;
    uint32_t* h_window = nullptr;     // pinned copy of the window

    int spawn(const SproutParticle* in, uint32_t n, uint32_t* accepted) {
        *accepted = 0;
        if (!was_reset) return fail(SPROUT_E_ARG, "spawn before reset");
        const uint32_t room = kSpawnMax - (uint32_t)pending.size();
        std::vector<SproutParticle> q;
        q.reserve(std::min(n, room));
        for (uint32_t k = 0; k < n && q.size() < room; k++) {
            const uint32_t mat = in[k].kind & 255u;
            if (in[k].kind == 0u || mat == 0u || mat > (uint32_t)kMaxMaterials) continue;
            SproutParticle p = in[k];
            p.id = next_id + (uint32_t)q.size();
            int rc = settle(p, k);
            if (rc != SPROUT_OK) return rc;
            q.push_back(p);
        }
        bool present[kMaxMaterials] = {};
        for (int r : tank.rows) present[r] = true;
        const size_t before = tank.rows.size();
        bool th = thermal;
        mark_materials(q.data(), (uint32_t)q.size(), present, &th);
        size_t after = 0;
        for (int r = 0; r < kMaxMaterials; r++) after += present[r] ? 1 : 0;
        if (after != before || th != thermal) {
            int rc = set_tank(present, th);
            if (rc == SPROUT_E_CAPACITY) return SPROUT_OK;   // they do not fit: none is accepted
            if (rc != SPROUT_OK) return rc;
        }
        for (SproutParticle& p : q) {
            spawn_speed = std::max(spawn_speed, std::hypot(p.vel[0], p.vel[1]));
            p.kind |= KIND_FRESH;
            pending.push_back(p);
        }
        next_id += (uint32_t)q.size();
        *accepted = (uint32_t)q.size();
        return SPROUT_OK;
    }

    // record (mod.rs:2486-2503, 2530-2534): the queue fills fresh slots while there are any,
    // then dead slots (admission.cu), on the sim's stream.
    int take_spawns() {
        if (pending.empty()) return SPROUT_OK;
        const uint32_t n = (uint32_t)pending.size();
        const uint32_t fresh = std::min(n, capacity - n_slots);
        const uint32_t base = n_slots;
        if (fresh > 0) {
            CUDA_TRY(cudaMemcpyAsync(d.part + 3 * (size_t)n_slots, pending.data(), (size_t)fresh * sizeof(SproutParticle),
                                     cudaMemcpyHostToDevice, stream));
            h2d_bytes += (size_t)fresh * sizeof(SproutParticle);
            n_slots += fresh;
        }
        if (n > fresh) {
            const uint32_t claim = n - fresh;
            if (!d_spawn) {
                int rc = alloc(&d_spawn, 3 * (size_t)kSpawnMax);
                if (rc == SPROUT_OK) rc = alloc(&d_claim, claim_scratch_words(capacity));
                if (rc != SPROUT_OK) return rc;
            }
            CUDA_TRY(cudaMemcpyAsync(d_spawn, pending.data() + fresh, (size_t)claim * sizeof(SproutParticle),
                                     cudaMemcpyHostToDevice, stream));
            h2d_bytes += (size_t)claim * sizeof(SproutParticle);
        }
        // once the device emitters have run, the device holds the next id: the queue takes
        // its ids there, in call order after what the emitters queued
        if (ids_on_device) launch_spawn_ids(d.part, base, fresh, d_spawn, n, d_emit, stream);
        if (n > fresh) {
            launch_claim(d.part, n_slots, d_spawn, n - fresh, d_claim, stream);
            CUDA_TRY(cudaGetLastError());
        }
        // the copies read the queue from pageable memory, which they have finished with on return
        pending.clear();
        return SPROUT_OK;
    }

    // ---- the brush's emitters on the device (emit.cu) ----
    static constexpr int kPPC = 4;   // sim::PPC
    EmitState* d_emit = nullptr;     // allocated by the first emission
    bool ids_on_device = false;
    float2* d_cand = nullptr;
    uint8_t* d_cflag = nullptr;
    size_t cand_cap = 0;
    uint32_t* d_room = nullptr;
    size_t room_cap = 0;
    std::vector<void*> emit_bufs;    // the grown buffers above, freed with the sim

    template <class T>
    int grow(T** p, size_t* cap, size_t n) {
        if (n <= *cap && *p) return SPROUT_OK;
        if (*p) {
            CUDA_TRY(cudaStreamSynchronize(stream));
            cudaFree(*p);
            emit_bufs.erase(std::remove(emit_bufs.begin(), emit_bufs.end(), (void*)*p), emit_bufs.end());
            *p = nullptr;
        }
        const size_t m = std::max<size_t>(n, 1024);
        if (cudaMalloc((void**)p, m * sizeof(T)) != cudaSuccess) return fail(SPROUT_E_NOMEM, "emitter buffers");
        emit_bufs.push_back((void*)*p);
        *cap = m;
        return SPROUT_OK;
    }

    // World::admission's window (world.rs:729-736): Admission::window (brush.rs:219-224)
    // clamped to the grid
    void window_of(const float from[2], const float to[2], float margin, EmitArgs& a) const {
        int lo[2], hi[2];
        for (int c = 0; c < 2; c++) {
            lo[c] = (int)std::floor(std::min(from[c], to[c]) - margin);
            hi[c] = (int)std::ceil(std::max(from[c], to[c]) + margin) + 1;
        }
        const int g[2] = {W, H};
        for (int c = 0; c < 2; c++) {
            lo[c] = std::min(std::max(lo[c], 0), g[c]);
            hi[c] = std::min(std::max(hi[c], lo[c]), g[c]);
            a.win_lo[c] = lo[c];
            a.win_size[c] = hi[c] - lo[c];
        }
    }

    // One emission: the template of the material (Particle::new + settle_spawn), the tank
    // taking the material's row as spawn does, the window's counts, the kernels, the
    // placement into `upper` fresh slots reserved for it (or dead ones). Nothing is read back.
    int emit(EmitArgs& a, uint32_t material, uint32_t upper, uint32_t* reserved) {
        if (reserved) *reserved = 0;
        if (!was_reset) return fail(SPROUT_E_ARG, "emit before reset");
        if (batch) return fail(SPROUT_E_ARG, "the sim belongs to a batch: emit into sims outside a batch");
        if (material >= (uint32_t)kMaxMaterials) return fail(SPROUT_E_ARG, "no such material row");
        SproutParticle p{};
        p.pos[0] = 0.5f * (float)W;
        p.pos[1] = 0.5f * (float)H;
        p.s = -1.0f;           // SPAWN_S
        p.t = -1.0e4f;         // SPAWN_TEMP
        p.kind = material + 1u;
        int rc = settle(p, 0);
        if (rc != SPROUT_OK) return rc;
        bool present[kMaxMaterials] = {};
        for (int r : tank.rows) present[r] = true;
        const size_t before = tank.rows.size();
        bool th = thermal;
        mark_materials(&p, 1, present, &th);
        size_t after = 0;
        for (int r = 0; r < kMaxMaterials; r++) after += present[r] ? 1 : 0;
        if (after != before || th != thermal) {
            rc = set_tank(present, th);
            if (rc == SPROUT_E_CAPACITY) return SPROUT_OK;   // the material does not fit: nothing is emitted
            if (rc != SPROUT_OK) return rc;
        }
        // what the host queued so far goes first (ids in call order)
        if ((rc = take_spawns()) != SPROUT_OK) return rc;
        if (!d_emit) {
            if ((rc = alloc(&d_emit, 1)) != SPROUT_OK) return rc;
            EmitState e{};
            e.rng = 0x12345678u;   // World::new (world.rs:181)
            CUDA_TRY(cudaMemcpyAsync(d_emit, &e, sizeof e, cudaMemcpyHostToDevice, stream));
            CUDA_TRY(cudaStreamSynchronize(stream));
        }
        if (!ids_on_device) {
            CUDA_TRY(cudaMemcpyAsync(&d_emit->next_id, &next_id, sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
            CUDA_TRY(cudaStreamSynchronize(stream));
            ids_on_device = true;
        }
        if (!d_spawn) {
            if ((rc = alloc(&d_spawn, 3 * (size_t)kSpawnMax)) != SPROUT_OK) return rc;
            if ((rc = alloc(&d_claim, claim_scratch_words(capacity))) != SPROUT_OK) return rc;
        }
        a.W = W;
        a.H = H;
        a.ppc = kPPC;
        a.s = p.s;
        a.t = p.t;
        a.kind = p.kind;
        a.limit = kSpawnMax;
        const size_t nwin = (size_t)a.win_size[0] * a.win_size[1];
        if ((rc = grow(&d_cand, &cand_cap, a.ncand)) != SPROUT_OK) return rc;
        size_t fcap = cand_cap;
        if ((rc = grow(&d_cflag, &fcap, a.ncand)) != SPROUT_OK) return rc;
        if ((rc = grow(&d_room, &room_cap, nwin + (a.mode == EMIT_PAINT ? a.ncand : 0))) != SPROUT_OK) return rc;
        launch_cell_counts(d.part, n_slots, a.win_lo[0], a.win_lo[1], a.win_size[0], a.win_size[1], d_room, stream);
        launch_emit(a, d_cand, d_cflag, d_room, d.sdf, d_spawn, d_emit, const_cast<StepState*>(d.S), stream);
        upper = std::min(upper, kSpawnMax);
        const uint32_t fresh = std::min(upper, capacity - n_slots);
        const uint32_t base = n_slots;
        launch_emit_fresh(d.part, base, fresh, d_spawn, d_emit, stream);
        n_slots += fresh;
        if (upper > fresh) launch_claim_dev(d.part, n_slots, d_spawn, d_emit, fresh, d_claim, stream);
        CUDA_TRY(cudaGetLastError());
        emitted = true;
        if (reserved) *reserved = fresh;
        return SPROUT_OK;
    }

    // ---- the render side's cell passes (optics.cu; FluidSim::record_cell_optics) ----
    static constexpr int kRenderLayers = 20, kSmoothLayers = 24, kFlowLayers = 4;
    DevOptics* d_optics = nullptr;
    ushort4* d_raw = nullptr;      // cell_optics.comp + light.comp
    ushort4* d_smooth = nullptr;   // optics_blur.comp (0-19), sss.comp (20-23)
    ushort4* d_flow = nullptr;     // flow_map.comp: two copies of (short, long period)
    ushort4* d_glow = nullptr;     // glow.comp: two half-resolution images
    RenderClock* d_clock = nullptr;
    size_t glow_texels() const { return (size_t)((W + 1) / 2) * ((H + 1) / 2); }
    std::vector<DevOptics> h_optics, last_optics;
    // The reference records nothing when nothing changed since its last call (optics_key:
    // substeps done, resets, table uploads, inv_speed), and keeps the time of the last call
    // for the tank it was made on (stain_at).
    uint64_t substeps_issued = 0, resets = 0, tables_gen = 0;
    uint64_t render_key[4] = {0, 0, 0, 0};
    bool render_key_set = false, stain_valid = false;
    // The optics table of the current parameters on the device (uploaded when it changed).
    int upload_optics() {
        if (!d_optics) {
            const int rc = alloc(&d_optics, kMaxMaterials);
            if (rc != SPROUT_OK) return rc;
        }
        h_optics.resize(kMaxMaterials);
        optics_table(params, h_optics.data());
        if (last_optics.size() != h_optics.size() ||
            std::memcmp(last_optics.data(), h_optics.data(), sizeof(DevOptics) * kMaxMaterials) != 0) {
            CUDA_TRY(cudaMemcpyAsync(d_optics, h_optics.data(), sizeof(DevOptics) * kMaxMaterials, cudaMemcpyHostToDevice,
                                     stream));
            last_optics = h_optics;
            tables_gen++;
        }
        return SPROUT_OK;
    }
    int render(float inv_speed) {
        if (!was_reset) return fail(SPROUT_E_ARG, "render before reset");
        int rc = upload_tables(nullptr);
        if (rc != SPROUT_OK) return rc;
        const size_t nc = (size_t)W * H;
        if (!d_raw) {
            if ((rc = alloc(&d_raw, kRenderLayers * nc)) != SPROUT_OK) return rc;
            if ((rc = alloc(&d_smooth, kSmoothLayers * nc)) != SPROUT_OK) return rc;
            if ((rc = alloc(&d_flow, kFlowLayers * nc)) != SPROUT_OK) return rc;
            if ((rc = alloc(&d_glow, 2 * glow_texels())) != SPROUT_OK) return rc;
            if ((rc = alloc(&d_clock, 1)) != SPROUT_OK) return rc;
            CUDA_TRY(cudaMemsetAsync(d_clock, 0, sizeof(RenderClock), stream));
        }
        if ((rc = upload_optics()) != SPROUT_OK) return rc;
        // a new tank: nothing carried (mod.rs:1631-1638)
        if (!stain_valid) CUDA_TRY(cudaMemsetAsync(d_flow, 0, sizeof(ushort4) * kFlowLayers * nc, stream));
        const uint64_t key[4] = {substeps_issued, resets, tables_gen, (uint64_t)__builtin_bit_cast(uint32_t, inv_speed)};
        const bool changed = !render_key_set || std::memcmp(key, render_key, sizeof key) != 0;
        launch_render_clock(d, d_clock, stain_valid ? 1 : 0, changed ? 1 : 0, stream);
        stain_valid = true;
        if (changed) {
            std::memcpy(render_key, key, sizeof key);
            render_key_set = true;
            float gap = 0.0f, mc = 0.0f;
            spike_params(&gap, &mc);
            bool makes = false, has_dust = false;
            for (int r : tank.rows) {
                makes |= params.bubbles > 0.0f && (params.mat[r].foam > 0.0f || params.mat[r].fizz > 0.0f);
                has_dust |= params.mat[r].dust > 0.0f;
            }
            // the dust field of the last frame's pool, once the pool has run (mod.rs:1653)
            const float dust = (diffuse_seen && has_dust && spray.dfield) ? 1.0f : 0.0f;
            launch_cell_optics(d, d_optics, inv_speed, gap, mc, spray.dfield, dust, (int)params.sss_iters, d_raw, d_smooth,
                               d_flow, d_clock, d_glow, d_glow + glow_texels(), stream);
            if ((makes || has_dust) && !spray.pool && (rc = alloc_spray()) != SPROUT_OK) return rc;
            if (look_live() && n_slots > 0) {   // record_look (mod.rs:1717-1729)
                if (!d.plook) {
                    if ((rc = alloc(&d.plook, (size_t)capacity)) != SPROUT_OK) return rc;
                    if ((rc = alloc(&d.plook2, (size_t)capacity)) != SPROUT_OK) return rc;
                    if ((rc = alloc(&d_look_list, (size_t)capacity + 1)) != SPROUT_OK) return rc;
                    CUDA_TRY(cudaMemsetAsync(d.plook, 0, (size_t)capacity * sizeof(uint4), stream));
                    graph_ok = false;   // the sort now carries the look's state: recapture
                }
                // a new particle of a liquid with specks brings them into the pool (look.comp)
                if (spray.pool) launch_specks(d, d_optics, spray, frames, n_slots, stream);
                launch_look(d, d_optics, d_clock, frames, d_look_list, d_look_list + 1, capacity, n_slots, stream);
            }
            // record_spray (mod.rs:1739-1773): once a liquid that foams, fizzes or carries specks
            // has been in the tank, the pool is moved every frame; new entries are made while one
            // that foams or fizzes is
            diffuse_seen |= makes || has_dust;
            if (diffuse_seen) {
                launch_spray(d, d_smooth, d_optics, spray, d_clock, frames, diffuse_parity, params.bubbles, makes, stream);
                diffuse_parity ^= 1u;
            }
        }
        CUDA_TRY(cudaGetLastError());
        return SPROUT_OK;
    }
    // FluidSim::spike_params (mod.rs:1885-1899): the spikes' spacing, the fastest growing wave
    // 2 pi sqrt(sigma / (rho g)) in cells (at least SPIKE_MIN_GAP = 3), and mu0 Mc of the most
    // susceptible liquid in the tank (the last of equals); none without a magnet.
    void spike_params(float* gap, float* mc) const {
        *gap = *mc = 0.0f;
        const MatProps* best = nullptr;
        for (int r : tank.rows) {
            const MatProps& m = params.mat[r];
            if (m.susceptibility > 0.0f && (!best || m.susceptibility >= best->susceptibility)) best = &m;
        }
        if (!best || magnets.empty()) return;
        const float g = std::max(params.gravity, 1.0f);
        const float rho = std::max(best->density, 1.0f), sigma = std::max(best->tension, 1e-4f);
        *gap = std::max(2.0f * 3.14159265f * std::sqrt(sigma / (rho * g)) / params.cell_size, 3.0f);
        const float mu0 = 1.2566371e-6f;
        *mc = std::sqrt(2.0f * mu0 * (1.0f + 1.0f / (1.0f + best->susceptibility)) * std::sqrt(rho * g * sigma));
    }
    // ---- the renderer's particle fields (draw.cu; Renderer::render, render.rs:886-1075) ----
    // render.rs's constants: SPLAT_RADIUS, ACCUM_KERNEL_TEXELS, ACCUM_MAX_DIV, SPLAT_MIN_TEXELS,
    // EXPOSURE, WIDE_SIGMA, WIDE_SIGMA_TEXELS, WIDE_MIN_FACTOR, WIDE_MAX_FACTOR, TINT_DIV
    static constexpr float kSplatRadius = 1.5f, kAccumKernelTexels = 2.8f, kAccumMaxDiv = 2.0f, kSplatMinTexels = 1.5f;
    static constexpr float kWideSigma = 2.0f, kWideSigmaTexels = 3.0f, kWideMinFactor = 2.0f, kWideMaxFactor = 64.0f;
    static constexpr uint32_t kTintDiv = 2u, kDrawMaxExtent = 16384u;
    static constexpr float kLookRadius = 1.0f;   // LOOK_RADIUS
    DrawBufs drawb{};
    size_t cap_acc = 0, cap_tacc = 0, cap_sharp = 0, cap_conc = 0, cap_share = 0, cap_w0 = 0, cap_w1 = 0, cap_look = 0;
    // used texels of the sharp field, the tint field's two images (0 x 0: never drawn), the
    // wide field, the look field
    uint32_t draw_dims[5][2] = {};
    float4* d_wet = nullptr;
    WetClock* d_wet_clock = nullptr;
    size_t wet_cells = 0;
    uint64_t wet_resets = ~0ull;
    // FluidSim::shares_a_group (mod.rs:1872-1878): two liquids of one phase group in the tank,
    // steam aside
    bool shares_a_group() const {
        uint32_t seen[8] = {};
        for (int r : tank.rows) {
            if (r == 57) continue;
            const uint32_t g = std::min<uint32_t>((uint32_t)params.mat[r].group, 7u);
            if (++seen[g] >= 2) return true;
        }
        return false;
    }
    // grow() for buffers that must start zeroed (the fixed-point texel sums)
    template <class T>
    int grow_zeroed(T** p, size_t* cap, size_t n) {
        T* before = *p;
        const int rc = grow(p, cap, n);
        if (rc != SPROUT_OK) return rc;
        if (*p != before) CUDA_TRY(cudaMemsetAsync(*p, 0, *cap * sizeof(T), stream));
        return SPROUT_OK;
    }
    // Renderer::render's passes 1, 1a and 2-4 (render.rs:889-1075) for a view of `ew` x `eh`
    // pixels centred on (cx, cy) cells at `zoom` pixels per cell, and the wet map
    // (render.rs:640-668), on the sim's stream (no wait).
    int draw(float cx, float cy, float zoom, uint32_t ew, uint32_t eh) {
        if (!was_reset) return fail(SPROUT_E_ARG, "draw before reset");
        if (!(zoom > 0.0f) || !std::isfinite(zoom) || !std::isfinite(cx) || !std::isfinite(cy))
            return fail(SPROUT_E_ARG, "draw: the zoom is a positive number of pixels per cell and the centre is finite");
        if (ew < 1u || eh < 1u || ew > kDrawMaxExtent || eh > kDrawMaxExtent)
            return fail(SPROUT_E_ARG, "draw: the extent is 1 to 16384 pixels a side");
        int rc = upload_tables(nullptr);
        if (rc != SPROUT_OK) return rc;
        if ((rc = upload_optics()) != SPROUT_OK) return rc;
        const float half_w = (float)ew * 0.5f, half_h = (float)eh * 0.5f;
        // pass 1: the sharp field, in texels of div pixels
        const float div = std::clamp(kSplatRadius * zoom / kAccumKernelTexels, 1.0f, kAccumMaxDiv);
        const uint32_t aw = std::clamp((uint32_t)std::ceil((float)ew / div), 1u, ew);
        const uint32_t ah = std::clamp((uint32_t)std::ceil((float)eh / div), 1u, eh);
        const float radius = std::max(kSplatRadius, kSplatMinTexels * div / zoom);
        const float exposure = 1.0f / 160.0f;
        DrawPass sharp{cx, cy, zoom, div, half_w, half_h, radius, (kSplatRadius / radius) * (kSplatRadius / radius), exposure,
                       (int)aw, (int)ah, 0, 1.0f / zoom, 1.0f / radius};
        // pass 1a: the tint field, TINT_DIV times coarser, where it can show something
        const bool tint_live = n_slots > 0 && shares_a_group();
        const float dt = div * (float)kTintDiv;
        const uint32_t tw = std::clamp((aw + kTintDiv - 1) / kTintDiv, 1u, (ew + kTintDiv - 1) / kTintDiv);
        const uint32_t th = std::clamp((ah + kTintDiv - 1) / kTintDiv, 1u, (eh + kTintDiv - 1) / kTintDiv);
        const float rt = std::max(kSplatRadius, kSplatMinTexels * dt / zoom);
        DrawPass tint{cx, cy, zoom, dt, half_w, half_h, rt, (kSplatRadius / rt) * (kSplatRadius / rt), exposure, (int)tw, (int)th, 1,
                      1.0f / zoom, 1.0f / rt};
        // passes 2-4: the wide field (WideLayout::new)
        const float factor = std::clamp(kWideSigma * zoom / kWideSigmaTexels, kWideMinFactor, kWideMaxFactor);
        const uint32_t iw = std::max(1u, (uint32_t)std::ceil((float)ew / kWideMinFactor));
        const uint32_t ih = std::max(1u, (uint32_t)std::ceil((float)eh / kWideMinFactor));
        const uint32_t ww = std::clamp((uint32_t)std::ceil((float)ew / factor), 1u, iw);
        const uint32_t wh = std::clamp((uint32_t)std::ceil((float)eh / factor), 1u, ih);
        DrawWide wide{(int)ww, (int)wh, (int)std::ceil(factor / div * 0.5f), factor / div, 0.5f * kWideSigma * zoom / factor};
        const size_t na = (size_t)aw * ah, nt = (size_t)tw * th, nw = (size_t)ww * wh;
        if ((rc = grow_zeroed(&drawb.acc, &cap_acc, 4 * na)) != SPROUT_OK) return rc;
        if ((rc = grow(&drawb.sharp, &cap_sharp, na)) != SPROUT_OK) return rc;
        if (tint_live) {
            if ((rc = grow_zeroed(&drawb.tacc, &cap_tacc, 8 * nt)) != SPROUT_OK) return rc;
            if ((rc = grow(&drawb.conc, &cap_conc, nt)) != SPROUT_OK) return rc;
            if ((rc = grow(&drawb.share, &cap_share, nt)) != SPROUT_OK) return rc;
        }
        if ((rc = grow(&drawb.wide0, &cap_w0, nw)) != SPROUT_OK) return rc;
        if ((rc = grow(&drawb.wide1, &cap_w1, nw)) != SPROUT_OK) return rc;
        // pass 1c: the look field (render.rs:1004-1036) of the particles the last render listed
        // (look.comp), in the sharp field's texels; without a liquid with a look it is clear
        const bool look_on = look_live() && d.plook && d_look_list && n_slots > 0;
        const float rl = std::max(kLookRadius, kSplatMinTexels * div / zoom);
        const float h0 = -0.3375f, h1 = 0.67f, h2 = 0.66f + 1.0f;   // composite.frag's key light + the view
        const float hn = std::sqrt(h0 * h0 + h1 * h1 + h2 * h2);
        DrawPass look{cx, cy, zoom, div, half_w, half_h, rl, (kLookRadius / rl) * (kLookRadius / rl), exposure, (int)aw, (int)ah, 2,
                      1.0f / zoom, 1.0f / rl, h0 / hn, h1 / hn, h2 / hn};
        if ((rc = grow(&drawb.look, &cap_look, na)) != SPROUT_OK) return rc;
        if (!look_on) CUDA_TRY(cudaMemsetAsync(drawb.look, 0, na * sizeof(ushort4), stream));
        launch_draw(d, d_optics, n_slots, sharp, tint_live ? &tint : nullptr, look_on ? &look : nullptr, d_look_list, wide,
                    drawb, stream);
        draw_dims[4][0] = aw, draw_dims[4][1] = ah;
        draw_dims[0][0] = aw, draw_dims[0][1] = ah;
        if (tint_live) draw_dims[1][0] = draw_dims[2][0] = tw, draw_dims[1][1] = draw_dims[2][1] = th;
        draw_dims[3][0] = ww, draw_dims[3][1] = wh;
        // the wet map: a new map, or a tank that started over, holds nothing wet
        const size_t nc = (size_t)W * H;
        if (!d_wet || wet_cells != nc) {
            if ((rc = grow(&d_wet, &wet_cells, nc)) != SPROUT_OK) return rc;
            wet_cells = nc;
            wet_resets = ~0ull;
        }
        if (!d_wet_clock && (rc = alloc(&d_wet_clock, 1)) != SPROUT_OK) return rc;
        if (wet_resets != resets) {
            CUDA_TRY(cudaMemsetAsync(d_wet, 0, nc * sizeof(float4), stream));
            CUDA_TRY(cudaMemsetAsync(d_wet_clock, 0, sizeof(WetClock), stream));
            wet_resets = resets;
        }
        launch_wet(d, d_wet_clock, d_wet, stream);
        CUDA_TRY(cudaGetLastError());
        return SPROUT_OK;
    }
    int download_draw(int which, void* out, size_t cap, uint32_t dims[2]) {
        if (which < 0 || which > 5)
            return fail(SPROUT_E_ARG,
                        "download_draw: which is 0 (sharp), 1 (tint), 2 (tint share), 3 (wide), 4 (wet map) or 5 (look)");
        const int k = which == 5 ? 4 : which;
        const uint32_t w = which == 4 ? (d_wet ? (uint32_t)W : 0u) : draw_dims[k][0];
        const uint32_t h = which == 4 ? (d_wet ? (uint32_t)H : 0u) : draw_dims[k][1];
        dims[0] = w, dims[1] = h;
        const size_t n = (size_t)w * h * (which == 4 ? sizeof(float4) : sizeof(ushort4));
        if (!out || n == 0) return SPROUT_OK;
        if (cap < n) return fail(SPROUT_E_ARG, "download_draw: the output holds fewer bytes than the image");
        const void* src = which == 0 ? (const void*)drawb.sharp : which == 1 ? (const void*)drawb.conc
                          : which == 2 ? (const void*)drawb.share : which == 3 ? (const void*)drawb.wide0
                          : which == 4 ? (const void*)d_wet : (const void*)drawb.look;
        CUDA_TRY(cudaStreamSynchronize(stream));
        CUDA_TRY(cudaMemcpy(out, src, n, cudaMemcpyDeviceToHost));
        d2h_bytes += n;
        return SPROUT_OK;
    }

    // spray.comp's pool (spray.cu): made, moved and listed by render calls
    SprayBufs spray{};
    int alloc_spray() {
        const size_t nc = (size_t)W * H;
        int rc;
        if ((rc = alloc(&spray.pool, (size_t)kPoolMax)) != SPROUT_OK) return rc;
        if ((rc = alloc(&spray.stack, (size_t)kDiffuseMax)) != SPROUT_OK) return rc;
        if ((rc = alloc(&spray.stack1, (size_t)kDustMax)) != SPROUT_OK) return rc;
        if ((rc = alloc(&spray.list, (size_t)kPoolMax)) != SPROUT_OK) return rc;
        if ((rc = alloc(&spray.flags, (size_t)kPoolMax)) != SPROUT_OK) return rc;
        if ((rc = alloc(&spray.dcount, 4 * nc)) != SPROUT_OK) return rc;
        if ((rc = alloc(&spray.counts, nc)) != SPROUT_OK) return rc;
        if ((rc = alloc(&spray.nspeck, (size_t)capacity + 1)) != SPROUT_OK) return rc;
        if ((rc = alloc(&spray.bsum, std::max(nc, (size_t)capacity + 1) / 1024 + 2)) != SPROUT_OK) return rc;
        if ((rc = alloc(&spray.dfield, 4 * nc)) != SPROUT_OK) return rc;
        if ((rc = alloc(&spray.ps, 1)) != SPROUT_OK) return rc;
        CUDA_TRY(cudaMemsetAsync(spray.pool, 0, (size_t)kPoolMax * sizeof(DevDiffuse), stream));
        CUDA_TRY(cudaMemsetAsync(spray.dcount, 0, 4 * nc * sizeof(uint32_t), stream));
        CUDA_TRY(cudaMemsetAsync(spray.dfield, 0, 4 * nc * sizeof(int), stream));
        CUDA_TRY(cudaMemsetAsync(spray.ps, 0, sizeof(PoolState), stream));
        return SPROUT_OK;
    }
    bool diffuse_seen = false;
    uint32_t diffuse_parity = 0;
    int download_spray(SproutDiffuse* pool, size_t pool_cap, uint32_t* stack, uint32_t* stack1, uint32_t* list, size_t cap,
                       uint32_t* foam, size_t foam_cap, uint32_t state[8]) {
        for (int k = 0; k < 8; k++) state[k] = 0;
        if (!spray.pool) return SPROUT_OK;
        CUDA_TRY(cudaStreamSynchronize(stream));
        PoolState ps;
        CUDA_TRY(cudaMemcpy(&ps, spray.ps, sizeof ps, cudaMemcpyDeviceToHost));
        state[0] = ps.hw;
        state[1] = ps.top;
        state[2] = ps.listed;
        state[3] = diffuse_parity;
        state[4] = ps.hw1;
        state[5] = ps.top1;
        const size_t nc = (size_t)W * H;
        if (pool) {
            if (pool_cap < kPoolMax) return fail(SPROUT_E_ARG, "download_spray: the pool holds 196608 entries");
            CUDA_TRY(cudaMemcpy(pool, spray.pool, (size_t)kPoolMax * sizeof(DevDiffuse), cudaMemcpyDeviceToHost));
        }
        if (stack || stack1 || list) {
            if (cap < kPoolMax) return fail(SPROUT_E_ARG, "download_spray: the stacks and list hold 196608 entries");
            if (stack) CUDA_TRY(cudaMemcpy(stack, spray.stack, (size_t)ps.top * 4, cudaMemcpyDeviceToHost));
            if (stack1) CUDA_TRY(cudaMemcpy(stack1, spray.stack1, (size_t)ps.top1 * 4, cudaMemcpyDeviceToHost));
            if (list) CUDA_TRY(cudaMemcpy(list, spray.list, (size_t)ps.listed * 4, cudaMemcpyDeviceToHost));
        }
        if (foam) {
            if (foam_cap < 4 * nc) return fail(SPROUT_E_ARG, "download_spray: the counts hold 4 x W x H");
            CUDA_TRY(cudaMemcpy(foam, spray.dcount, 4 * nc * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        }
        return SPROUT_OK;
    }
    // A liquid with platelets (cloud_shape below 2/3) or specks is in the tank (mod.rs:1718-1721).
    uint32_t* d_look_list = nullptr;   // [0] how many listed, then their slots
    bool look_live() const {
        for (int r : tank.rows) {
            const MatProps& m = params.mat[r];
            if ((m.cloud > 0.0f && m.cloud_shape < 2.0f / 3.0f) || m.dust > 0.0f) return true;
        }
        return false;
    }
    int download_look(uint32_t* state, size_t cap, uint32_t* list, size_t list_cap, uint32_t* slots, uint32_t* listed) {
        *slots = 0;
        *listed = 0;
        if (!d.plook) return SPROUT_OK;
        CUDA_TRY(cudaStreamSynchronize(stream));
        uint32_t count = 0;
        CUDA_TRY(cudaMemcpy(&count, d_look_list, sizeof count, cudaMemcpyDeviceToHost));
        *slots = n_slots;
        *listed = std::min(count, capacity);
        if (state) {
            if (cap < 4 * (size_t)n_slots) return fail(SPROUT_E_ARG, "download_look: the state holds fewer than 4 words per slot");
            CUDA_TRY(cudaMemcpy(state, d.plook, (size_t)n_slots * sizeof(uint4), cudaMemcpyDeviceToHost));
        }
        if (list) {
            if (list_cap < *listed) return fail(SPROUT_E_ARG, "download_look: the list holds fewer entries than listed");
            CUDA_TRY(cudaMemcpy(list, d_look_list + 1, (size_t)*listed * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        }
        d2h_bytes += (size_t)n_slots * sizeof(uint4) + (size_t)*listed * 4;
        return SPROUT_OK;
    }
    int flow_parity(uint32_t* parity) {
        if (!d_clock) return fail(SPROUT_E_ARG, "flow_parity before render");
        RenderClock c;
        CUDA_TRY(cudaMemcpyAsync(&c, d_clock, sizeof c, cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        *parity = c.parity;
        return SPROUT_OK;
    }

    // FluidSim::request_stats / poll_stats (mod.rs:3246-3273): the census of the slots
    // (stats.comp) into a device buffer, copied to pinned host memory behind an event.
    uint32_t* d_stats = nullptr;
    uint32_t* h_stats = nullptr;
    cudaEvent_t stats_ev = nullptr;
    bool stats_in_flight = false;
    int request_stats() {
        if (stats_in_flight) return SPROUT_OK;
        if (!d_stats) {
            int rc = alloc(&d_stats, stats_words());
            if (rc != SPROUT_OK) return rc;
            CUDA_TRY(cudaMallocHost(&h_stats, stats_words() * sizeof(uint32_t)));
            CUDA_TRY(cudaEventCreateWithFlags(&stats_ev, cudaEventDisableTiming));
        }
        launch_stats(d.part, n_slots, d_stats, stream);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaMemcpyAsync(h_stats, d_stats, stats_words() * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaEventRecord(stats_ev, stream));
        d2h_bytes += stats_words() * sizeof(uint32_t);
        stats_in_flight = true;
        return SPROUT_OK;
    }
    int poll_stats(SproutStats* out, int* ready) {
        *ready = 0;
        if (!stats_in_flight) return SPROUT_OK;
        const cudaError_t e = cudaEventQuery(stats_ev);
        if (e == cudaErrorNotReady) {
            cudaGetLastError();
            return SPROUT_OK;
        }
        CUDA_TRY(e);
        out->live = h_stats[0];
        for (int m = 0; m < SPROUT_MATERIAL_ROWS; m++) {
            out->count[m] = h_stats[1 + m];
            out->conc[m] = (float)h_stats[1 + kStatsRows + m] / 256.0f;
        }
        stats_in_flight = false;
        *ready = 1;
        return SPROUT_OK;
    }

    // FluidSim::cell_counts (mod.rs:3350-3387): live particles per cell of [lo, hi) row by
    // row after the work queued so far, the particles queued by spawn included. Blocking.
    int cell_counts(const int32_t lo[2], const int32_t hi[2], uint32_t* out, size_t cap, size_t* cells) {
        if (lo[0] < 0 || lo[1] < 0 || hi[0] > W || hi[1] > H)
            return fail(SPROUT_E_ARG, "the window of cell_counts leaves the grid");
        const int sw = std::max(hi[0] - lo[0], 0), sh = std::max(hi[1] - lo[1], 0);
        const size_t n = (size_t)sw * sh;
        if (cells) *cells = n;
        if (!out || n == 0) return SPROUT_OK;
        if (cap < n) return fail(SPROUT_E_ARG, "cell_counts: the output holds fewer cells than the window");
        if (n > window_cap) {
            if (d_window) cudaFree(d_window);
            if (h_window) cudaFreeHost(h_window);
            d_window = nullptr;
            h_window = nullptr;
            window_cap = 0;
            CUDA_TRY(cudaMalloc(&d_window, n * sizeof(uint32_t)));
            CUDA_TRY(cudaMallocHost(&h_window, n * sizeof(uint32_t)));
            window_cap = n;
        }
        launch_cell_counts(d.part, n_slots, lo[0], lo[1], sw, sh, d_window, stream);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaMemcpyAsync(h_window, d_window, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        d2h_bytes += n * sizeof(uint32_t);
        std::memcpy(out, h_window, n * sizeof(uint32_t));
        for (const SproutParticle& p : pending) {
            const int cx = (int)std::floor(p.pos[0]) - lo[0], cy = (int)std::floor(p.pos[1]) - lo[1];
            if (cx >= 0 && cy >= 0 && cx < sw && cy < sh) out[(size_t)cy * sw + cx]++;
        }
        return SPROUT_OK;
    }

    // What a step call does before its substeps run, on the sim's stream: the parameters and
    // material table (when they changed), the batch words of StepBuf.
    uint32_t frames = 0;   // FluidSim::frame: step calls so far (mod.rs:2402), wrapping
    int prepare_step(uint32_t substeps, float target, const ToolState* tool) {
        frames += 1u;
        enqueued = false;
        if (!pending.empty()) {
            int rc = take_spawns();
            if (rc != SPROUT_OK) return rc;
            enqueued = true;
        }
        if (d_emit) {   // the queue's per-step count (record clears pending_spawn)
            CUDA_TRY(cudaMemsetAsync(&d_emit->queued, 0, sizeof(uint32_t), stream));
            enqueued = true;
        }
        if (n_slots == 0 || tank.rows.empty()) return fail(SPROUT_E_ARG, "step before reset (no particles)");
        int rc = derive_viscosity();
        if (rc != SPROUT_OK) return rc;
        rc = upload_tables(tool);
        spawn_speed = 0.0f;
        if (rc != SPROUT_OK) return rc;
        if (substeps == 0) return SPROUT_OK;
        substeps_issued += substeps;
        const uint32_t fl = __builtin_bit_cast(uint32_t, std::max(target, 0.0f));
        if (!words_cached || batch_words[0] != fl || batch_words[1] != substeps) {
            batch_words[0] = fl;
            batch_words[1] = substeps;
            batch_words[2] = 0u;
            CUDA_TRY(cudaMemcpyAsync(&d.S->frame_left, &batch_words[0], 4, cudaMemcpyHostToDevice, stream));
            CUDA_TRY(cudaMemcpyAsync(&d.S->batch_steps, &batch_words[1], 8, cudaMemcpyHostToDevice, stream));
            h2d_bytes += 12;
            words_cached = cache_words;
            enqueued = true;
        }
        return SPROUT_OK;
    }
    // With cache_words, repeated step calls with the same substeps and target do not upload
    // the words again: only for a fixed dt, where k_step reads neither frame_left nor the
    // batch counters (a batch's continuous stepping of fixed-rate tanks). Off for single-sim
    // stepping, which keeps the reference's per-call upload.
    bool cache_words = false, words_cached = false;
    bool enqueued = false;   // the last prepare_step put work on the sim's stream
    uint32_t batch_words[3] = {0u, 0u, 0u};
    struct SproutBatch* batch = nullptr;   // the batch this sim steps in, if any

    int step(uint32_t substeps, float target, const ToolState* tool) {
        if (batch) return fail(SPROUT_E_ARG, "the sim belongs to a batch: step the batch (or remove it first)");
        int rc = prepare_step(substeps, target, tool);
        if (rc != SPROUT_OK || substeps == 0) return rc;
        if ((rc = ensure_graph()) != SPROUT_OK) return rc;
        for (uint32_t k = 0; k < substeps; k++) {
            if (use_graph && graph_ok) CUDA_TRY(cudaGraphLaunch(exec, stream));
            else record_substep(stream);
        }
        launch_frame_end(d, stream);   // the call is a frame: its solves adapt the recorded counts
        CUDA_TRY(cudaGetLastError());
        return end_emit_call();
    }
    // The fastest particle the device emitters queued raises the CFL limit of one step call,
    // as spawn_speed does (mod.rs:2300): cleared after the call's substeps.
    bool emitted = false;
    int end_emit_call() {
        if (!emitted) return SPROUT_OK;
        CUDA_TRY(cudaMemsetAsync(&d.S->emit_speed, 0, sizeof(float), stream));
        emitted = false;
        return SPROUT_OK;
    }

    int poll() {
        StepState S;
        CUDA_TRY(cudaMemcpyAsync(&S, d.S, sizeof S, cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        d2h_bytes += sizeof S;
        double t = (double)S.advanced - (double)__builtin_bit_cast(float, S.pad0);
        if (t > sim_time) sim_time = t;
        if (S.dt_cfl > 0.0f) dt_est = S.dt_cfl;
        return SPROUT_OK;
    }

    float dt_estimate() const { return params.fixed_hz > 0.0f ? 1.0f / params.fixed_hz : dt_est; }

    int check_device_error() {
        uint32_t err = 0;
        CUDA_TRY(cudaMemcpy(&err, &d.K->error, 4, cudaMemcpyDeviceToHost));
        if (err & ERR_DIVERGED) return fail(SPROUT_E_DIVERGED, "a solve met a non-finite right-hand side or residual and stopped");
        if (err) return fail(SPROUT_E_TIMEOUT, "a bounded device-side wait ran out (grid barrier of a persistent solve)");
        return SPROUT_OK;
    }

    // FluidSim::step_blocking (mod.rs:3315-3338).
    int step_blocking(uint32_t substeps, const ToolState* tool) {
        if (substeps == 0) {
            int rc = take_spawns();
            if (rc == SPROUT_OK) rc = upload_tables(tool);
            spawn_speed = 0.0f;
            if (rc != SPROUT_OK) return rc;
            CUDA_TRY(cudaStreamSynchronize(stream));
            return SPROUT_OK;
        }
        double seconds = (double)substeps * (double)kNominalDt;
        double start = sim_time;
        float sliver = std::max(params.min_substep_share, 1e-6f);
        for (int guard = 0; guard < 1000000; guard++) {
            double left = seconds - (sim_time - start);
            double dt = dt_estimate();
            if (left <= sliver * dt) break;
            uint32_t n = (uint32_t)std::min(std::max(std::ceil(left / dt), 1.0), 16.0);
            double target = params.fixed_hz > 0.0f ? n * dt : left;
            int rc = step(n, (float)target, tool);
            if (rc != SPROUT_OK) return rc;
            if ((rc = poll()) != SPROUT_OK) return rc;
        }
        return check_device_error();
    }

    // FluidSim::advance_blocking (mod.rs:3284-3312).
    int advance_blocking(double seconds, const ToolState* tool) {
        double goal = sim_time + seconds;
        bool first = true;
        float sliver = std::max(params.min_substep_share, 1e-6f);
        for (int guard = 0; guard < 1000000; guard++) {
            double left = goal - sim_time;
            double dt = dt_estimate();
            if (left <= sliver * dt) break;
            double nn = params.fixed_hz > 0.0f ? std::max(std::round(left / dt), 1.0) : std::ceil(left / dt);
            uint32_t n = (uint32_t)std::min(std::max(nn, 1.0), 16.0);
            double target = params.fixed_hz > 0.0f ? n * dt : left;
            ToolState t0{};
            const ToolState* use = tool;
            if (!first && tool) {
                t0 = *tool;
                t0.mode = 0;
                use = &t0;
            }
            int rc = step(n, (float)target, use);
            if (rc != SPROUT_OK) return rc;
            if ((rc = poll()) != SPROUT_OK) return rc;
            first = false;
            if (params.fixed_hz > 0.0f && (goal - sim_time) < 0.5 * dt) break;
        }
        return check_device_error();
    }
};

// ---- C ABI --------------------------------------------------------------------------------

// ---- batches: many tanks advanced by one captured graph per substep ------------------------
//
// The particle and grid stages of the batch's tanks run as concurrent branches of the graph
// (a few worker streams, tanks dealt round-robin), the pressure solves of all of them as one
// persistent kernel over their flattened tile lists (launch_pressure_batch), the viscosity
// solves one after another. A tank's results are the same as when it steps alone.
struct SproutBatch {
    static constexpr int kWorkers = 8;
    std::vector<SproutSim*> sims;
    int device = 0;
    bool mixed = false;
    cudaStream_t main = nullptr;
    cudaStream_t workers[kWorkers] = {};
    std::vector<cudaEvent_t> events;     // fork / join points of the capture
    cudaEvent_t ev_done = nullptr;
    std::vector<cudaEvent_t> ev_in;      // per tank: its uploads are on the device
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool graph_ok = false;
    // the two solves' views (the stepped tanks; those with a second solve) and their device
    // arrays, kept at a capacity and rewritten in stream order (no allocation per step)
    struct View {
        BatchView v{};
        std::vector<SproutSim*> members;
        std::vector<DevScene> scenes;   // the members' scenes as last written
        int blocks = 0;
        size_t smem = 0;
        int cap = 0;
        DevScene* ds = nullptr;
        int *doff = nullptr, *dscale = nullptr, *daoff = nullptr;
        unsigned char* dscal = nullptr;
        SolveState* dk = nullptr;
        void release() {
            for (void* p : {(void*)ds, (void*)doff, (void*)dscale, (void*)dscal, (void*)dk, (void*)daoff})
                if (p) cudaFree(p);
            ds = nullptr;
            doff = dscale = daoff = nullptr;
            dscal = nullptr;
            dk = nullptr;
            cap = 0;
            members.clear();
            scenes.clear();
            v = BatchView{};
        }
    } first, second;
    size_t h2d = 0;

    // The viscosity solves of the tanks with a second solve, batched in one persistent kernel
    // when they share a sweep count (vis_ok): the second view's scenes, level-0 prefix sums,
    // barrier word and active-tile array, with scalars of its own.
    VBatchView vis{};
    bool vis_ok = false;
    int vis_sweeps = 0, vis_blocks = 0, vis_cap = 0;
    unsigned char* dvscal = nullptr;
    int build_visc_view() {
        vis_ok = false;
        const int ns = second.v.ns;
        if (ns < 2) return SPROUT_OK;
        if (launch_req.batch_viscosity == 2u) return SPROUT_OK;   // asked for one solve per tank
        const int sw = second.members[0]->cfg.visc_sweeps;
        int max_lev = 0, tiles = 0;
        for (const SproutSim* sim : second.members) {
            if (sim->cfg.visc_sweeps != sw) return SPROUT_OK;   // mixed sweep counts: one solve per tank
            if (sim->params.viscosity_precond == 0) return SPROUT_OK;   // the Jacobi iteration: one solve per tank
            max_lev = std::max(max_lev, sim->cfg.visc_levels);
            tiles += sim->d.nwg;
        }
        // large tanks fill the device one at a time: the batched solve only adds its separate
        // reduction phases (measured: +13 to +44 % for 8-16 tanks of 128 x 72 to 256 x 144,
        // -2.5 % for 4 tanks of 1024 x 576)
        if (tiles > 1500 * ns && launch_req.batch_viscosity != 1u) return SPROUT_OK;
        if (ns > vis_cap) {
            CUDA_TRY(cudaStreamSynchronize(main));
            if (dvscal) cudaFree(dvscal);
            dvscal = nullptr;
            vis_cap = 0;
            const int cap = std::max(ns, 2 * second.cap);
            if (cudaMalloc(&dvscal, (size_t)cap * viscosity_batch_scalar_bytes()) != cudaSuccess) {
                dvscal = nullptr;
                return fail(SPROUT_E_NOMEM, "batch viscosity scalars");
            }
            vis_cap = cap;
        }
        vis = VBatchView{second.ds, ns, second.doff, dvscal, second.dk, second.daoff, max_lev};
        vis_sweeps = sw;
        const int vmx = viscosity_blocks_max(device, sw);
        vis_blocks = std::max(1, std::min(vmx, launch_req.viscosity_blocks ? (int)std::min<uint32_t>(launch_req.viscosity_blocks, (uint32_t)tiles) : tiles));
        vis_ok = true;
        return SPROUT_OK;
    }

    ~SproutBatch() {
        for (SproutSim* sim : sims) sim->batch = nullptr;
        drop_graph();
        first.release();
        second.release();
        if (dvscal) cudaFree(dvscal);
        for (cudaEvent_t e : events) cudaEventDestroy(e);
        for (cudaEvent_t e : ev_in) cudaEventDestroy(e);
        for (cudaEvent_t e : ring)
            if (e) cudaEventDestroy(e);
        if (ev_done) cudaEventDestroy(ev_done);
        for (cudaStream_t w : workers)
            if (w) cudaStreamDestroy(w);
        if (main) cudaStreamDestroy(main);
    }

    int init() {
        CUDA_TRY(cudaGetDevice(&device));
        CUDA_TRY(cudaStreamCreateWithFlags(&main, cudaStreamNonBlocking));
        for (cudaStream_t& w : workers) CUDA_TRY(cudaStreamCreateWithFlags(&w, cudaStreamNonBlocking));
        CUDA_TRY(cudaEventCreateWithFlags(&ev_done, cudaEventDisableTiming));
        return SPROUT_OK;
    }

    void drop_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        graph_ok = false;
    }

    int add(SproutSim* sim) {
        if (sim->batch == this) return SPROUT_OK;
        if (sim->batch) return fail(SPROUT_E_ARG, "the sim already belongs to another batch");
        if (sim->device != device) return fail(SPROUT_E_ARG, "the sim lives on another device than the batch");
        CUDA_TRY(cudaStreamSynchronize(sim->stream));
        sims.push_back(sim);
        sim->batch = this;
        cudaEvent_t e;
        CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ev_in.push_back(e);
        drop_graph();
        return mixed ? sim->set_precision(1) : SPROUT_OK;
    }

    int remove(SproutSim* sim) {
        auto it = std::find(sims.begin(), sims.end(), sim);
        if (it == sims.end()) return fail(SPROUT_E_ARG, "the sim is not in this batch");
        CUDA_TRY(cudaStreamSynchronize(main));
        const size_t k = (size_t)(it - sims.begin());
        sims.erase(it);
        cudaEventDestroy(ev_in[k]);
        ev_in.erase(ev_in.begin() + (long)k);
        sim->batch = nullptr;
        drop_graph();
        return SPROUT_OK;
    }

    int set_precision(int mode) {
        if (mode != 0 && mode != 1) return fail(SPROUT_E_ARG, "precision mode is 0 (plain FP32) or 1 (mixed)");
        for (SproutSim* sim : sims) {
            int rc = sim->set_precision(mode);
            if (rc != SPROUT_OK) return rc;
        }
        if (mixed != (mode == 1)) drop_graph();
        mixed = mode == 1;
        return SPROUT_OK;
    }

    // The device arrays of a batch view over `members`, written on `main`.
    int build_view(View& V, const std::vector<SproutSim*>& members) {
        const int ns = (int)members.size();
        V.members = members;
        V.scenes.assign(ns, DevScene{});
        if (ns == 0) {
            V.v = BatchView{};
            return SPROUT_OK;
        }
        if (ns > V.cap) {
            CUDA_TRY(cudaStreamSynchronize(main));
            const int cap = std::max(ns, 2 * V.cap);
            for (void* p : {(void*)V.ds, (void*)V.doff, (void*)V.dscale, (void*)V.dscal, (void*)V.dk, (void*)V.daoff})
                if (p) cudaFree(p);
            bool ok = cudaMalloc(&V.ds, cap * sizeof(DevScene)) == cudaSuccess &&
                      cudaMalloc(&V.doff, (size_t)kMaxLevels * (cap + 1) * sizeof(int)) == cudaSuccess &&
                      cudaMalloc(&V.daoff, (size_t)kMaxLevels * (cap + 1) * sizeof(int)) == cudaSuccess &&
                      cudaMalloc(&V.dscale, cap * sizeof(int)) == cudaSuccess &&
                      cudaMalloc(&V.dscal, cap * pressure_batch_scalar_bytes()) == cudaSuccess &&
                      cudaMalloc(&V.dk, sizeof(SolveState)) == cudaSuccess;
            if (!ok) return fail(SPROUT_E_NOMEM, "batch arrays");
            CUDA_TRY(cudaMemset(V.dk, 0, sizeof(SolveState)));
            CUDA_TRY(cudaMemset(V.dscal, 0, cap * pressure_batch_scalar_bytes()));
            V.cap = cap;
        }
        std::vector<int> scale(ns), off((size_t)kMaxLevels * (ns + 1), 0);
        int max_tail = 0;
        size_t smem = 0;
        for (int k = 0; k < ns; k++) {
            const SproutSim* sim = members[k];
            V.scenes[k] = sim->d;
            const LaunchCfg& c = sim->cfg;
            scale[k] = (c.visc_mode == 2 && c.twice && c.viscous_warm) ? 1 : 0;
            max_tail = std::max(max_tail, sim->d.lv.tail);
            smem = std::max(smem, pressure_batch_smem(sim->d.lv));
        }
        for (int l = 0; l < kMaxLevels; l++) {
            int* o = &off[(size_t)l * (ns + 1)];
            o[0] = 0;
            for (int k = 0; k < ns; k++) {
                const Levels& L = members[k]->d.lv;
                const int t = l <= L.tail ? ((L.w[l] + 15) / 16) * ((L.h[l] + 15) / 16) : 0;
                o[k + 1] = o[k] + t;
            }
        }
        // pageable sources: each copy is staged before the call returns, so the vectors may go
        CUDA_TRY(cudaMemcpyAsync(V.ds, V.scenes.data(), ns * sizeof(DevScene), cudaMemcpyHostToDevice, main));
        CUDA_TRY(cudaMemcpyAsync(V.doff, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, main));
        CUDA_TRY(cudaMemcpyAsync(V.dscale, scale.data(), ns * sizeof(int), cudaMemcpyHostToDevice, main));
        h2d += ns * sizeof(DevScene) + off.size() * sizeof(int) + ns * sizeof(int);
        V.v = BatchView{V.ds, ns, V.doff, V.dscal, V.dscale, V.dk, max_tail, V.daoff};
        V.smem = smem;
        const int mx = pressure_batch_blocks_max(device, smem, mixed);
        int total_tiles = 0;
        for (const SproutSim* sim : members) total_tiles += sim->d.nwg;
        const uint32_t req = mixed ? launch_req.pressure_blocks_mixed : launch_req.pressure_blocks;
        const int most = std::max(total_tiles, ns);
        V.blocks = std::max(1, std::min(mx, req ? (int)std::min<uint32_t>(req, (uint32_t)most) : most));
        return SPROUT_OK;
    }

    // The block counts of the batch's persistent solves (0: the defaults above).
    SproutLaunch launch_req{};
    int set_launch(const SproutLaunch& l) {
        CUDA_TRY(cudaStreamSynchronize(main));
        if (l.batch_viscosity > 2u) return fail(SPROUT_E_ARG, "batch_viscosity is 0 (default), 1 (batched) or 2 (one solve per tank)");
        launch_req = l;
        drop_graph();
        return SPROUT_OK;
    }

    cudaEvent_t event(size_t& k) {
        while (events.size() <= k) {
            cudaEvent_t e;
            cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
            events.push_back(e);
        }
        return events[k++];
    }
    // main -> workers
    void fork(size_t& k) {
        cudaEvent_t e = event(k);
        cudaEventRecord(e, main);
        for (cudaStream_t w : workers) cudaStreamWaitEvent(w, e, 0);
    }
    // workers -> main
    void join(size_t& k) {
        for (cudaStream_t w : workers) {
            cudaEvent_t e = event(k);
            cudaEventRecord(e, w);
            cudaStreamWaitEvent(main, e, 0);
        }
    }

    // One substep of every tank, recorded on `main` (and the workers).
    // One substep of the view's tanks. `replay`: their own stages from their small graphs
    // (the subset stepping, launched directly); else recorded kernel by kernel (into the
    // batch's graph).
    void record_substep(bool replay = false) {
        const std::vector<SproutSim*>& ms = first.members;
        size_t k = 0;
        // a tank whose implicit viscosity runs before its only pressure solve (viscous_projection
        // 0) has its cooperative viscosity kernel inside the grid stage: its stages run on the
        // main stream, never beside another tank's kernels
        auto serial = [](const SproutSim* sim) { return sim->cfg.visc_mode == 2 && !sim->cfg.twice; };
        for (SproutSim* sim : ms)
            if (serial(sim)) {
                if (replay) cudaGraphLaunch(sim->part_exec[0], main);
                else for (int st = 0; st < 4; st++) sim->record_stage(st, main);
            }
        fork(k);
        for (size_t s = 0; s < ms.size(); s++) {
            if (serial(ms[s])) continue;
            if (replay) cudaGraphLaunch(ms[s]->part_exec[0], workers[s % kWorkers]);
            else for (int st = 0; st < 4; st++) ms[s]->record_stage(st, workers[s % kWorkers]);
        }
        join(k);
        if (first.v.ns > 0) launch_pressure_batch(first.v, mixed, first.blocks, first.smem, main, 0);
        fork(k);
        for (size_t s = 0; s < ms.size(); s++) {
            if (replay) cudaGraphLaunch(ms[s]->part_exec[1], workers[s % kWorkers]);
            else ms[s]->record_stage(5, workers[s % kWorkers]);
        }
        join(k);
        if (second.v.ns > 0) {
            if (vis_ok) launch_viscosity_batch(vis, vis_sweeps, vis_blocks, main);
            else for (SproutSim* sim : second.members) launch_viscosity(sim->d, sim->cfg, main, 1);
            fork(k);
            for (size_t s = 0; s < second.members.size(); s++) launch_second_projection_rhs(second.members[s]->d, workers[s % kWorkers]);
            join(k);
            launch_pressure_batch(second.v, mixed, second.blocks, second.smem, main, 1);
            fork(k);
            for (size_t s = 0; s < second.members.size(); s++) launch_second_projection(second.members[s]->d, workers[s % kWorkers]);
            join(k);
        }
        for (SproutSim* sim : ms)
            if (sim->cfg.rigid) launch_rigid(sim->d, main);
    }

    std::vector<SproutSim*> graph_members;   // the tanks the captured graph steps

    // Launch tickets: every step call is one ticket; an event ring tells which have finished.
    static constexpr uint64_t kRing = 256;
    cudaEvent_t ring[kRing] = {};
    uint64_t issued = 0, completed = 0;
    int ticket() {
        cudaEvent_t& e = ring[issued % kRing];
        if (!e) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        if (issued - completed >= kRing) {   // the slot's previous ticket must be done first
            CUDA_TRY(cudaEventSynchronize(e));
            completed = issued - kRing + 1;
        }
        CUDA_TRY(cudaEventRecord(e, main));
        issued++;
        return SPROUT_OK;
    }
    uint64_t poll_completed() {
        while (completed < issued && cudaEventQuery(ring[completed % kRing]) == cudaSuccess) completed++;
        cudaGetLastError();   // (a not-ready query is no error)
        return completed;
    }

    // The checks a batch makes of its stepped tanks.
    int check_members(const std::vector<SproutSim*>& ms, std::vector<SproutSim*>& twice) {
        twice.clear();
        for (SproutSim* sim : ms) {
            if (sim->cfg.mixed != mixed) return fail(SPROUT_E_ARG, "a batch's tanks share its precision");
            if (sim->cfg.visc_mode == 2 && sim->cfg.twice) twice.push_back(sim);
        }
        return SPROUT_OK;
    }

    int ensure_graph() {
        bool changed = graph_members != sims;
        for (SproutSim* sim : sims) changed |= sim->refresh_cfg();
        // a tank's device arrays may have changed since the capture (its precision buffers)
        for (size_t k = 0; k < first.scenes.size() && k < sims.size() && !changed; k++)
            changed |= std::memcmp(&first.scenes[k], &sims[k]->d, sizeof(DevScene)) != 0;
        if (graph_ok && !changed) return SPROUT_OK;
        drop_graph();
        std::vector<SproutSim*> twice;
        int rc = check_members(sims, twice);
        if (rc != SPROUT_OK) return rc;
        if ((rc = build_view(first, sims)) != SPROUT_OK) return rc;
        if ((rc = build_view(second, twice)) != SPROUT_OK) return rc;
        if ((rc = build_visc_view()) != SPROUT_OK) return rc;
        CUDA_TRY(cudaStreamSynchronize(main));
        graph_members = sims;
        CUDA_TRY(cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal));
        record_substep();
        cudaError_t e = cudaStreamEndCapture(main, &graph);
        if (e != cudaSuccess) {
            graph = nullptr;
            return fail(SPROUT_E_CUDA, std::string("capturing the batch's substep: ") + cudaGetErrorString(e));
        }
        CUDA_TRY(cudaGraphInstantiate(&exec, graph, 0));
        graph_ok = true;
        return SPROUT_OK;
    }

    int step(uint32_t substeps) {
        if (sims.empty() || substeps == 0) return SPROUT_OK;
        for (size_t s = 0; s < sims.size(); s++) {
            SproutSim* sim = sims[s];
            int rc = sim->prepare_step(substeps, (float)(substeps * (double)sim->dt_estimate()), nullptr);
            if (rc != SPROUT_OK) return rc;
            CUDA_TRY(cudaEventRecord(ev_in[s], sim->stream));
            CUDA_TRY(cudaStreamWaitEvent(main, ev_in[s], 0));
        }
        int rc = ensure_graph();
        if (rc != SPROUT_OK) return rc;
        for (uint32_t k = 0; k < substeps; k++) CUDA_TRY(cudaGraphLaunch(exec, main));
        launch_frame_end_many(first.v.scenes, first.v.ns, main);   // the call is every member's frame
        CUDA_TRY(cudaEventRecord(ev_done, main));
        for (SproutSim* sim : sims) CUDA_TRY(cudaStreamWaitEvent(sim->stream, ev_done, 0));
        return ticket();
    }

    // One substep of the members at `idx` only, launched directly (no graph): the serving
    // loop's continuous batching, where the stepped set changes from launch to launch.
    int step_subset(const uint32_t* idx, uint32_t n) {
        if (n == 0) return SPROUT_OK;
        std::vector<SproutSim*> ms;
        ms.reserve(n);
        for (uint32_t k = 0; k < n; k++) {
            if (idx[k] >= sims.size()) return fail(SPROUT_E_ARG, "batch member index out of range");
            SproutSim* sim = sims[idx[k]];
            if (std::find(ms.begin(), ms.end(), sim) != ms.end()) return fail(SPROUT_E_ARG, "a member listed twice");
            // with a fixed dt the batch words are not read (k_step), so unchanged ones stay
            sim->cache_words = sim->params.fixed_hz > 0.0f;
            int rc = sim->prepare_step(1, sim->dt_estimate(), nullptr);
            if (rc != SPROUT_OK) return rc;
            sim->refresh_cfg();
            if ((rc = sim->ensure_part_graphs()) != SPROUT_OK) return rc;
            if (sim->enqueued) {
                CUDA_TRY(cudaEventRecord(ev_in[idx[k]], sim->stream));
                CUDA_TRY(cudaStreamWaitEvent(main, ev_in[idx[k]], 0));
            }
            ms.push_back(sim);
        }
        std::vector<SproutSim*> twice;
        int rc = check_members(ms, twice);
        if (rc != SPROUT_OK) return rc;
        if ((rc = build_view(first, ms)) != SPROUT_OK) return rc;
        if ((rc = build_view(second, twice)) != SPROUT_OK) return rc;
        if ((rc = build_visc_view()) != SPROUT_OK) return rc;
        graph_ok = false;   // the views no longer hold the graph's tanks
        record_substep(true);
        launch_frame_end_many(first.v.scenes, first.v.ns, main);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaEventRecord(ev_done, main));
        for (SproutSim* sim : ms) CUDA_TRY(cudaStreamWaitEvent(sim->stream, ev_done, 0));
        return ticket();
    }

    int check_error() {
        for (View* V : {&first, &second}) {
            if (V->v.ns == 0) continue;
            uint32_t err = 0;
            CUDA_TRY(cudaMemcpy(&err, &V->v.K->error, 4, cudaMemcpyDeviceToHost));
            if (err) return fail(SPROUT_E_TIMEOUT, "a bounded device-side wait ran out (grid barrier of the batched pressure solve)");
        }
        for (SproutSim* sim : sims) {
            int rc = sim->check_device_error();
            if (rc != SPROUT_OK) return rc;
        }
        return SPROUT_OK;
    }

    int profile(uint32_t substeps, float* ms) {
        cudaEvent_t a, b;
        CUDA_TRY(cudaEventCreate(&a));
        CUDA_TRY(cudaEventCreate(&b));
        int rc = step(0);
        if (rc != SPROUT_OK) return rc;
        if ((rc = ensure_graph()) != SPROUT_OK) return rc;
        CUDA_TRY(cudaEventRecord(a, main));
        for (uint32_t k = 0; k < substeps; k++) {   // each substep a frame of its own
            CUDA_TRY(cudaGraphLaunch(exec, main));
            launch_frame_end_many(first.v.scenes, first.v.ns, main);
        }
        CUDA_TRY(cudaEventRecord(b, main));
        CUDA_TRY(cudaEventSynchronize(b));
        CUDA_TRY(cudaEventElapsedTime(ms, a, b));
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return check_error();
    }
};

extern "C" {

const char* sprout_last_error(void) { return g_error.c_str(); }
const char* sprout_version(void) { return "sprout_gb300 0.1 (sm_103a)"; }

int sprout_params_new(SproutParams** out) {
    if (!out) return fail(SPROUT_E_ARG, "null out");
    *out = new (std::nothrow) SproutParams();
    return *out ? SPROUT_OK : fail(SPROUT_E_NOMEM, "host allocation failed");
}
int sprout_params_free(SproutParams* p) {
    delete p;
    return SPROUT_OK;
}
int sprout_params_copy(const SproutParams* src, SproutParams** out) {
    if (!src || !out) return fail(SPROUT_E_ARG, "null argument");
    *out = new (std::nothrow) SproutParams(*src);
    return *out ? SPROUT_OK : fail(SPROUT_E_NOMEM, "host allocation failed");
}
int sprout_params_set(SproutParams* p, const char* key, float v, int* ok) {
    if (!p || !key || !ok) return fail(SPROUT_E_ARG, "null argument");
    *ok = p->p.set(key, v) ? 1 : 0;
    return SPROUT_OK;
}
int sprout_params_set_diluent(SproutParams* p, uint32_t row, int32_t diluent, int* ok) {
    if (!p || !ok) return fail(SPROUT_E_ARG, "null argument");
    *ok = p->p.set_diluent((int)row, (int)diluent) ? 1 : 0;
    return SPROUT_OK;
}
int sprout_params_set_group(SproutParams* p, uint32_t row, uint32_t group, int* ok) {
    if (!p || !ok) return fail(SPROUT_E_ARG, "null argument");
    *ok = p->p.set_group((int)row, (int)group) ? 1 : 0;
    return SPROUT_OK;
}
int sprout_params_get(const SproutParams* p, const char* key, float* v, int* ok) {
    if (!p || !key || !v || !ok) return fail(SPROUT_E_ARG, "null argument");
    *ok = p->p.get(key, v) ? 1 : 0;
    return SPROUT_OK;
}

int sprout_scene_new(uint32_t w, uint32_t h, SproutScene** out) {
    if (!out || w < 8 || h < 8) return fail(SPROUT_E_ARG, "bad scene size");
    *out = new (std::nothrow) SproutScene();
    if (!*out) return fail(SPROUT_E_NOMEM, "host allocation failed");
    (*out)->s.w = (int)w;
    (*out)->s.h = (int)h;
    return SPROUT_OK;
}
int sprout_scene_free(SproutScene* s) {
    delete s;
    return SPROUT_OK;
}
int sprout_scene_add_box(SproutScene* s, float cx, float cy, float hx, float hy, float angle, float temp) {
    if (!s) return fail(SPROUT_E_ARG, "null scene");
    Shape sh;
    sh.kind = Shape::Box;
    sh.cx = cx; sh.cy = cy; sh.hx = hx; sh.hy = hy; sh.angle = angle;
    sh.held = !std::isnan(temp);
    sh.temp = sh.held ? temp : 0.0f;
    s->s.shapes.push_back(sh);
    return SPROUT_OK;
}
int sprout_scene_add_circle(SproutScene* s, float cx, float cy, float r, float temp) {
    if (!s) return fail(SPROUT_E_ARG, "null scene");
    Shape sh;
    sh.kind = Shape::Circle;
    sh.cx = cx; sh.cy = cy; sh.r = r;
    sh.held = !std::isnan(temp);
    sh.temp = sh.held ? temp : 0.0f;
    s->s.shapes.push_back(sh);
    return SPROUT_OK;
}
int sprout_scene_sdf(const SproutScene* s, float x, float y, float* d) {
    if (!s || !d) return fail(SPROUT_E_ARG, "null argument");
    *d = s->s.sdf(x, y);
    return SPROUT_OK;
}
int sprout_scene_rasterize(const SproutScene* s, float* sdf, float* solid4, uint32_t* region, float* temp, int* heated) {
    if (!s || !sdf || !solid4 || !region) return fail(SPROUT_E_ARG, "null argument");
    bool h = s->s.rasterize(sdf, solid4, region, temp);
    if (heated) *heated = h ? 1 : 0;
    return SPROUT_OK;
}

int sprout_scene_rasterize_device(const SproutScene* s, float* sdf, float* solid4, uint32_t* region, float* temp, int* heated) {
    if (!s || !sdf || !solid4 || !region) return fail(SPROUT_E_ARG, "null argument");
    const int w = s->s.w, h = s->s.h;
    const size_t nn = (size_t)(w + 1) * (h + 1), nc = (size_t)w * h;
    float *dsdf = nullptr, *dtemp = nullptr;
    float4* dsolid = nullptr;
    uint32_t* dregion = nullptr;
    cudaError_t e = cudaMalloc(&dsdf, nn * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&dsolid, nc * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&dregion, nc * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&dtemp, nc * sizeof(float));
    bool hot = false;
    if (e == cudaSuccess) e = rasterize_device(s->s, dsdf, dsolid, dregion, dtemp, &hot, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(sdf, dsdf, nn * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(solid4, dsolid, nc * sizeof(float4), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(region, dregion, nc * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && hot && temp) e = cudaMemcpy(temp, dtemp, nc * sizeof(float), cudaMemcpyDeviceToHost);
    for (void* p : {(void*)dsdf, (void*)dsolid, (void*)dregion, (void*)dtemp})
        if (p) cudaFree(p);
    if (e != cudaSuccess) return fail(SPROUT_E_CUDA, std::string("rasterising on the device: ") + cudaGetErrorString(e));
    if (heated) *heated = hot ? 1 : 0;
    return SPROUT_OK;
}

int sprout_sim_set_scene(SproutSim* sim, const SproutScene* s) {
    if (!sim || !s) return fail(SPROUT_E_ARG, "null argument");
    if (s->s.w != sim->W || s->s.h != sim->H) return fail(SPROUT_E_ARG, "the scene's grid is not the sim's");
    CUDA_TRY(cudaStreamSynchronize(sim->stream));
    bool hot = false;
    cudaError_t e = rasterize_device(s->s, const_cast<float*>(sim->d.sdf), const_cast<float4*>(sim->d.solid),
                                     const_cast<uint32_t*>(sim->d.region), const_cast<float*>(sim->d.solid_t), &hot,
                                     sim->stream);
    if (e != cudaSuccess) return fail(SPROUT_E_CUDA, std::string("rasterising on the device: ") + cudaGetErrorString(e));
    if (!hot) {
        std::vector<float> nt((size_t)sim->W * sim->H, NO_TEMP);
        CUDA_TRY(cudaMemcpy((void*)sim->d.solid_t, nt.data(), nt.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    sim->solids_heated = hot;
    return SPROUT_OK;
}
int sprout_fill_rect(const SproutScene* s, const float rect[4], uint32_t material, uint32_t n_before,
                     SproutParticle* out, uint32_t cap, uint32_t* n) {
    if (!s || !rect || !n) return fail(SPROUT_E_ARG, "null argument");
    if (material >= (uint32_t)kMaxMaterials) return fail(SPROUT_E_ARG, "material row out of range");
    *n = s->s.fill_rect(rect, material, n_before, reinterpret_cast<SproutParticleHost*>(out), out ? cap : 0);
    return SPROUT_OK;
}

int sprout_sim_create(uint32_t w, uint32_t h, uint32_t capacity, const SproutParams* p, SproutSim** out) {
    if (!out || !p) return fail(SPROUT_E_ARG, "null argument");
    if (w < 16 || h < 16 || w > 16384 || h > 16384) return fail(SPROUT_E_ARG, "grid must be between 16 and 16384 cells a side");
    if (capacity == 0) return fail(SPROUT_E_ARG, "capacity must be positive");
    SproutSim* s = new (std::nothrow) SproutSim();
    if (!s) return fail(SPROUT_E_NOMEM, "host allocation failed");
    int rc = s->init(w, h, capacity, p->p);
    if (rc != SPROUT_OK) {
        delete s;
        return rc;
    }
    *out = s;
    return SPROUT_OK;
}
int sprout_sim_destroy(SproutSim* sim) {
    if (sim && sim->batch) sim->batch->remove(sim);
    if (sim) cudaStreamSynchronize(sim->stream);
    delete sim;
    return SPROUT_OK;
}

int sprout_device_count(int* n) {
    if (!n) return fail(SPROUT_E_ARG, "null argument");
    CUDA_TRY(cudaGetDeviceCount(n));
    return SPROUT_OK;
}

int sprout_set_device(int device) {
    int n = 0;
    CUDA_TRY(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(SPROUT_E_ARG, "no such device");
    CUDA_TRY(cudaSetDevice(device));
    return SPROUT_OK;
}

int sprout_get_device(int* device) {
    if (!device) return fail(SPROUT_E_ARG, "null argument");
    CUDA_TRY(cudaGetDevice(device));
    return SPROUT_OK;
}

int sprout_device_memory(size_t* free_bytes, size_t* total_bytes) {
    if (!free_bytes || !total_bytes) return fail(SPROUT_E_ARG, "null argument");
    CUDA_TRY(cudaMemGetInfo(free_bytes, total_bytes));
    return SPROUT_OK;
}
int sprout_batch_create(SproutBatch** out) {
    if (!out) return fail(SPROUT_E_ARG, "null argument");
    SproutBatch* b = new SproutBatch();
    int rc = b->init();
    if (rc != SPROUT_OK) {
        delete b;
        return rc;
    }
    *out = b;
    return SPROUT_OK;
}
int sprout_batch_destroy(SproutBatch* b) {
    if (b) cudaStreamSynchronize(b->main);
    delete b;
    return SPROUT_OK;
}
int sprout_batch_add(SproutBatch* b, SproutSim* sim) {
    if (!b || !sim) return fail(SPROUT_E_ARG, "null argument");
    return b->add(sim);
}
int sprout_batch_remove(SproutBatch* b, SproutSim* sim) {
    if (!b || !sim) return fail(SPROUT_E_ARG, "null argument");
    return b->remove(sim);
}
int sprout_batch_size(SproutBatch* b, uint32_t* n) {
    if (!b || !n) return fail(SPROUT_E_ARG, "null argument");
    *n = (uint32_t)b->sims.size();
    return SPROUT_OK;
}
int sprout_batch_set_precision(SproutBatch* b, int mode) {
    if (!b) return fail(SPROUT_E_ARG, "null argument");
    return b->set_precision(mode);
}
int sprout_batch_step(SproutBatch* b, uint32_t substeps) {
    if (!b) return fail(SPROUT_E_ARG, "null argument");
    return b->step(substeps);
}
int sprout_batch_step_subset(SproutBatch* b, const uint32_t* members, uint32_t n) {
    if (!b || (!members && n > 0)) return fail(SPROUT_E_ARG, "null argument");
    return b->step_subset(members, n);
}
int sprout_batch_tickets(SproutBatch* b, uint64_t* issued, uint64_t* completed) {
    if (!b || !issued || !completed) return fail(SPROUT_E_ARG, "null argument");
    *completed = b->poll_completed();
    *issued = b->issued;
    return SPROUT_OK;
}
int sprout_batch_sync(SproutBatch* b) {
    if (!b) return fail(SPROUT_E_ARG, "null argument");
    CUDA_TRY(cudaStreamSynchronize(b->main));
    return b->check_error();
}
int sprout_batch_profile(SproutBatch* b, uint32_t substeps, float* ms) {
    if (!b || !ms) return fail(SPROUT_E_ARG, "null argument");
    return b->profile(substeps, ms);
}
int sprout_sim_trace_enable(SproutSim* sim, uint32_t rows) {
    if (!sim) return fail(SPROUT_E_ARG, "null argument");
    return sim->trace_enable(rows);
}
int sprout_sim_trace_read(SproutSim* sim, unsigned long long* out, size_t cap, size_t* words, uint32_t* cols) {
    if (!sim || !words || !cols) return fail(SPROUT_E_ARG, "null argument");
    CUDA_TRY(cudaStreamSynchronize(sim->stream));
    *words = (size_t)sim->trace_rows * sim->trace_cols;
    *cols = sim->trace_cols;
    if (out && sim->trace_buf) CUDA_TRY(cudaMemcpy(out, sim->trace_buf, std::min(*words, cap) * 8, cudaMemcpyDeviceToHost));
    return SPROUT_OK;
}
int sprout_sim_request_stats(SproutSim* sim) {
    if (!sim) return fail(SPROUT_E_ARG, "null argument");
    return sim->request_stats();
}

int sprout_sim_poll_stats(SproutSim* sim, SproutStats* out, int* ready) {
    if (!sim || !out || !ready) return fail(SPROUT_E_ARG, "null argument");
    return sim->poll_stats(out, ready);
}

int sprout_sim_set_launch(SproutSim* sim, const SproutLaunch* l) {
    if (!sim || !l) return fail(SPROUT_E_ARG, "null argument");
    return sim->set_launch(*l);
}

int sprout_sim_get_launch(SproutSim* sim, SproutLaunch* out) {
    if (!sim || !out) return fail(SPROUT_E_ARG, "null argument");
    sim->get_launch(out);
    return SPROUT_OK;
}

int sprout_sim_debug_stall(SproutSim* sim, uint32_t block, uint32_t stall_ns, uint32_t spin_limit) {
    if (!sim) return fail(SPROUT_E_ARG, "null argument");
    return sim->debug_stall(block, stall_ns, spin_limit);
}

int sprout_batch_set_launch(SproutBatch* b, const SproutLaunch* l) {
    if (!b || !l) return fail(SPROUT_E_ARG, "null argument");
    return b->set_launch(*l);
}

int sprout_sim_set_precision(SproutSim* sim, int mode) {
    if (!sim) return fail(SPROUT_E_ARG, "null argument");
    return sim->set_precision(mode);
}
int sprout_sim_set_currents(SproutSim* sim, const SproutCurrent* c, uint32_t n) {
    if (!sim || (n > 0 && !c)) return fail(SPROUT_E_ARG, "null argument");
    sim->currents.clear();
    for (uint32_t i = 0; i < n && i < (uint32_t)kMaxCurrents; i++) {
        Current q;
        std::memcpy(&q, &c[i], sizeof q);
        sim->currents.push_back(q);
    }
    return SPROUT_OK;
}
int sprout_sim_set_magnets(SproutSim* sim, const SproutMagnet* m, uint32_t n) {
    if (!sim || (n > 0 && !m)) return fail(SPROUT_E_ARG, "null argument");
    sim->magnets.clear();
    for (uint32_t i = 0; i < n && i < (uint32_t)kMaxMagnets; i++) {
        Magnet q;
        std::memcpy(&q, &m[i], sizeof q);
        sim->magnets.push_back(q);
    }
    // whether the tank needs magnet.comp changes with the magnets (mod.rs:2749-2751)
    if (!sim->tank.rows.empty()) sim->caps = sim->compute_caps();
    return SPROUT_OK;
}
int sprout_sim_set_params(SproutSim* sim, const SproutParams* p) {
    if (!sim || !p) return fail(SPROUT_E_ARG, "null argument");
    sim->params = p->p;
    return SPROUT_OK;
}
int sprout_sim_set_solids(SproutSim* sim, const float* sdf, const float* solid4, const uint32_t* region, const float* temp) {
    if (!sim || !sdf || !solid4 || !region) return fail(SPROUT_E_ARG, "null argument");
    size_t nc = (size_t)sim->W * sim->H;
    CUDA_TRY(cudaStreamSynchronize(sim->stream));
    CUDA_TRY(cudaMemcpy((void*)sim->d.sdf, sdf, (size_t)(sim->W + 1) * (sim->H + 1) * sizeof(float), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy((void*)sim->d.solid, solid4, nc * sizeof(float4), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy((void*)sim->d.region, region, nc * sizeof(uint32_t), cudaMemcpyHostToDevice));
    if (temp) {
        CUDA_TRY(cudaMemcpy((void*)sim->d.solid_t, temp, nc * sizeof(float), cudaMemcpyHostToDevice));
    } else {
        std::vector<float> nt(nc, NO_TEMP);
        CUDA_TRY(cudaMemcpy((void*)sim->d.solid_t, nt.data(), nc * sizeof(float), cudaMemcpyHostToDevice));
    }
    sim->solids_heated = temp != nullptr;
    return SPROUT_OK;
}
int sprout_sim_reset(SproutSim* sim, const SproutParticle* p, uint32_t n) {
    if (!sim || (!p && n > 0)) return fail(SPROUT_E_ARG, "null argument");
    return sim->reset(p, n);
}
int sprout_sim_spawn(SproutSim* sim, const SproutParticle* p, uint32_t n, uint32_t* accepted) {
    if (!sim || !accepted || (!p && n > 0)) return fail(SPROUT_E_ARG, "null argument");
    return sim->spawn(p, n, accepted);
}
// ---- the brush's emitters on the device ----

namespace {
constexpr float kPPCf = 4.0f;                                  // sim::PPC
constexpr float kPourSpeed[2] = {60.0f, 400.0f};               // brush.rs:5
constexpr float kJetSpeed = 320.0f;                            // brush.rs:7
constexpr float kRadsPerDeg = 3.14159265358979323846f / 180.0f;   // f32::to_radians
constexpr float kRainSpan = 3.0f;                              // brush.rs:133
constexpr uint32_t kSpawnLimit = 32768;                        // mod.rs:63
}  // namespace

int sprout_spout(int kind, float degrees, float rate, float radius, SproutSpout* out) {
    if (!out || kind < 0 || kind > 2) return fail(SPROUT_E_ARG, "sprout_spout: kind 0 (pour), 1 (jet) or 2 (faucet)");
    float dir[2] = {0.0f, -1.0f};
    if (kind != 0) {   // jet_direction (brush.rs:166-169)
        const float r = degrees * kRadsPerDeg;
        dir[0] = std::sin(r);
        dir[1] = -std::cos(r);
    }
    // Spout::pour / jet / faucet and Spout::new (brush.rs:28-47)
    const float speed = kind == 1 ? kJetSpeed : std::min(std::max(rate / (kPPCf * 2.0f * radius), kPourSpeed[0]), kPourSpeed[1]);
    out->direction[0] = dir[0];
    out->direction[1] = dir[1];
    out->speed = speed;
    out->width = std::min(rate / (kPPCf * speed), 2.0f * radius);
    return SPROUT_OK;
}

int sprout_sim_emit_stream(SproutSim* sim, const SproutSpout* spout, double* stream_time, const float from[2],
                           const float to[2], float seconds, uint32_t material) {
    if (!sim || !spout || !stream_time || !from || !to) return fail(SPROUT_E_ARG, "null argument");
    if (!(seconds > 0.0f)) return SPROUT_OK;   // World::emit: a paused brush only moves
    if (!(spout->speed > 0.0f) || !(spout->width >= 0.0f)) return fail(SPROUT_E_ARG, "a spout needs a positive speed");
    EmitArgs a{};
    a.mode = EMIT_STREAM;
    for (int c = 0; c < 2; c++) {
        a.from[c] = from[c];
        a.to[c] = to[c];
        a.dir[c] = spout->direction[c];
        a.vel[c] = spout->direction[c] * spout->speed;   // Spout::velocity
    }
    a.speed = spout->speed;
    a.width = spout->width;
    // Stream::advance (brush.rs:86-115): the frame's range of lattice indices
    a.rate = (double)(kPPCf * spout->speed * spout->width);
    a.start = *stream_time;
    a.end = a.start + (double)seconds;
    const float half = 0.5f * spout->width;
    auto index = [&](double t) { return (uint64_t)std::max(std::floor(a.rate * t - 0.5) + 1.0, 0.0); };
    uint64_t k0 = index(a.start - (double)(half / spout->speed)), k1 = index(a.end);
    if (k1 < k0) k1 = k0;
    // Only the last kSpawnLimit that appear are kept (World::stream's limit): they lie among the
    // last kSpawnLimit indices plus those that may still be crossing the arc at the frame's end.
    const uint64_t span = (uint64_t)kSpawnLimit + (uint64_t)std::ceil(a.rate * (double)(half / spout->speed)) + 2u;
    if (k1 - k0 > span) k0 = k1 - span;
    a.k0 = k0;
    a.ncand = (uint32_t)(k1 - k0);
    a.keep = kSpawnLimit;
    *stream_time = a.end;
    // World::stream (world.rs:714-727): the window reaches as far as the frame's stream
    sim->window_of(from, to, spout->speed * seconds + spout->width + 1.0f, a);
    return sim->emit(a, material, std::min<uint32_t>(a.ncand, kSpawnLimit), nullptr);
}

int sprout_sim_emit_paint(SproutSim* sim, const float from[2], const float to[2], float radius, uint32_t count,
                          int spray, uint32_t material) {
    if (!sim || !from || !to) return fail(SPROUT_E_ARG, "null argument");
    count = std::min(count, kSpawnLimit);   // World::paint (world.rs:644-648)
    if (count == 0) return SPROUT_OK;
    EmitArgs a{};
    a.mode = EMIT_PAINT;
    a.spray = spray ? 1u : 0u;
    a.count = count;
    a.radius = radius;
    a.spacing = spray ? 1.5f : 1.0f / std::sqrt(kPPCf);   // SPRAY_SPACING, brush.rs:126
    for (int c = 0; c < 2; c++) {
        a.from[c] = from[c];
        a.to[c] = to[c];
    }
    // brush::stroke's lattice bounds (brush.rs:134-141)
    const int g[2] = {sim->W, sim->H};
    for (int c = 0; c < 2; c++) {
        const float lo = std::min(std::max(std::min(from[c], to[c]) - radius, 0.0f), (float)g[c]);
        const float hi = std::min(std::max(std::max(from[c], to[c]) + radius, 0.0f), (float)g[c]);
        a.lat_lo[c] = (int)std::floor(lo / a.spacing);
        a.lat_hi[c] = (int)std::ceil(hi / a.spacing);
    }
    const int nx = std::max(a.lat_hi[0] - a.lat_lo[0], 0), ny = std::max(a.lat_hi[1] - a.lat_lo[1], 0);
    if ((uint64_t)nx * (uint64_t)ny > (1ull << 28)) return fail(SPROUT_E_ARG, "the stroke covers too many lattice points");
    a.ncand = (uint32_t)(nx * ny);
    sim->window_of(from, to, radius + 1.0f, a);
    return sim->emit(a, material, std::min(count, a.ncand), nullptr);
}

int sprout_sim_emit_rain(SproutSim* sim, const float at[2], float radius, uint32_t count, uint32_t material) {
    if (!sim || !at) return fail(SPROUT_E_ARG, "null argument");
    count = std::min(count, kSpawnLimit);
    if (count == 0) return SPROUT_OK;
    EmitArgs a{};
    a.mode = EMIT_RAIN;
    a.count = count;
    a.at[0] = at[0];
    a.at[1] = at[1];
    a.half = radius * kRainSpan;   // World::rain (world.rs:689-710)
    const float from[2] = {at[0] - a.half, at[1]}, to[2] = {at[0] + a.half, at[1]};
    for (int c = 0; c < 2; c++) {
        a.from[c] = from[c];
        a.to[c] = to[c];
    }
    sim->window_of(from, to, 3.0f, a);
    return sim->emit(a, material, count, nullptr);
}

int sprout_sim_emitter_seed(SproutSim* sim, uint32_t rng) {
    if (!sim) return fail(SPROUT_E_ARG, "null argument");
    if (!sim->d_emit) {
        int rc = sim->alloc(&sim->d_emit, 1);
        if (rc != SPROUT_OK) return rc;
    }
    CUDA_TRY(cudaMemcpyAsync(&sim->d_emit->rng, &rng, sizeof rng, cudaMemcpyHostToDevice, sim->stream));
    CUDA_TRY(cudaStreamSynchronize(sim->stream));
    return SPROUT_OK;
}

int sprout_sim_emitted(SproutSim* sim, uint64_t* total, uint32_t* last) {
    if (!sim || !total) return fail(SPROUT_E_ARG, "null argument");
    *total = 0;
    if (last) *last = 0;
    if (!sim->d_emit) return SPROUT_OK;
    EmitState e;
    CUDA_TRY(cudaMemcpyAsync(&e, sim->d_emit, sizeof e, cudaMemcpyDeviceToHost, sim->stream));
    CUDA_TRY(cudaStreamSynchronize(sim->stream));
    sim->d2h_bytes += sizeof e;
    *total = e.total;
    if (last) *last = e.count;
    return SPROUT_OK;
}

// ---- the render side's cell passes ----

int sprout_params_optics(const SproutParams* p, void* out, uint32_t rows) {
    if (!p || (!out && rows > 0)) return fail(SPROUT_E_ARG, "null argument");
    DevOptics* o = static_cast<DevOptics*>(out);
    for (uint32_t r = 0; r < rows && r < (uint32_t)kMaxMaterials; r++) optics_row(p->p, (int)r, o[r]);
    return SPROUT_OK;
}

int sprout_params_set_color(SproutParams* p, uint32_t row, const char* field, const float rgb[3], int* ok) {
    if (!p || !field || !rgb || !ok) return fail(SPROUT_E_ARG, "null argument");
    *ok = 0;
    if (row >= (uint32_t)kMaxMaterials) return SPROUT_OK;
    MatProps& m = p->p.mat[row];
    const std::string f(field);
    float* dst = f == "color" ? m.color : f == "color_solid" ? m.color_solid : f == "color_hot" ? m.color_hot
               : f == "cloud_color" ? m.cloud_color : f == "dust_color" ? m.dust_color : f == "glow_color" ? m.glow_color
               : nullptr;
    if (!dst) return SPROUT_OK;
    for (int c = 0; c < 3; c++) dst[c] = std::min(std::max(rgb[c], 0.0f), 1.0f);
    if (row >= p->p.mat_count) p->p.mat_count = row + 1;
    *ok = 1;
    return SPROUT_OK;
}

int sprout_params_get_color(const SproutParams* p, uint32_t row, const char* field, float rgb[3], int* ok) {
    if (!p || !field || !rgb || !ok) return fail(SPROUT_E_ARG, "null argument");
    *ok = 0;
    if (row >= (uint32_t)kMaxMaterials) return SPROUT_OK;
    const MatProps& m = p->p.mat[row];
    const std::string f(field);
    const float* src = f == "color" ? m.color : f == "color_solid" ? m.color_solid : f == "color_hot" ? m.color_hot
                     : f == "cloud_color" ? m.cloud_color : f == "dust_color" ? m.dust_color : f == "glow_color" ? m.glow_color
                     : nullptr;
    if (!src) return SPROUT_OK;
    for (int c = 0; c < 3; c++) rgb[c] = src[c];
    *ok = 1;
    return SPROUT_OK;
}

int sprout_params_get_row(const SproutParams* p, uint32_t row, int32_t* group, int32_t* diluent) {
    if (!p || !group || !diluent) return fail(SPROUT_E_ARG, "null argument");
    if (row >= (uint32_t)kMaxMaterials) return fail(SPROUT_E_ARG, "no such material row");
    *group = (int32_t)p->p.mat[row].group;
    *diluent = p->p.mat[row].diluent;
    return SPROUT_OK;
}

int sprout_sim_render(SproutSim* sim, float inv_speed) {
    if (!sim) return fail(SPROUT_E_ARG, "null argument");
    return sim->render(inv_speed);
}

int sprout_sim_download_render(SproutSim* sim, int which, uint16_t* out, size_t cap, size_t* words) {
    if (!sim || !words) return fail(SPROUT_E_ARG, "null argument");
    if (which < 0 || which > 3)
        return fail(SPROUT_E_ARG, "download_render: which is 0 (raw), 1 (smoothed), 2 (glow) or 3 (flow map)");
    const size_t nc = (size_t)sim->W * sim->H;
    const size_t n = 4 * (which == 0   ? SproutSim::kRenderLayers * nc
                          : which == 1 ? SproutSim::kSmoothLayers * nc
                          : which == 2 ? sim->glow_texels()
                                       : SproutSim::kFlowLayers * nc);
    *words = n;
    if (!out) return SPROUT_OK;
    if (cap < n) return fail(SPROUT_E_ARG, "download_render: the output holds fewer words than the layers");
    if (!sim->d_raw) return fail(SPROUT_E_ARG, "download_render before render");
    CUDA_TRY(cudaStreamSynchronize(sim->stream));
    const void* src = which == 0   ? (const void*)sim->d_raw
                      : which == 1 ? (const void*)sim->d_smooth
                      : which == 2 ? (const void*)(sim->d_glow + sim->glow_texels())
                                   : (const void*)sim->d_flow;
    CUDA_TRY(cudaMemcpy(out, src, n * sizeof(uint16_t), cudaMemcpyDeviceToHost));
    sim->d2h_bytes += n * sizeof(uint16_t);
    return SPROUT_OK;
}

int sprout_sim_draw(SproutSim* sim, float center_x, float center_y, float zoom, uint32_t width, uint32_t height) {
    if (!sim) return fail(SPROUT_E_ARG, "null argument");
    return sim->draw(center_x, center_y, zoom, width, height);
}

int sprout_sim_download_draw(SproutSim* sim, int which, void* out, size_t cap, uint32_t dims[2]) {
    if (!sim || !dims) return fail(SPROUT_E_ARG, "null argument");
    return sim->download_draw(which, out, cap, dims);
}

int sprout_sim_download_spray(SproutSim* sim, SproutDiffuse* pool, size_t pool_cap, uint32_t* stack, uint32_t* stack1,
                              uint32_t* list, size_t cap, uint32_t* counts, size_t counts_cap, uint32_t state[8]) {
    if (!sim || !state) return fail(SPROUT_E_ARG, "null argument");
    return sim->download_spray(pool, pool_cap, stack, stack1, list, cap, counts, counts_cap, state);
}

int sprout_sim_download_look(SproutSim* sim, uint32_t* state, size_t state_cap, uint32_t* list, size_t list_cap,
                             uint32_t* slots, uint32_t* listed) {
    if (!sim || !slots || !listed) return fail(SPROUT_E_ARG, "null argument");
    return sim->download_look(state, state_cap, list, list_cap, slots, listed);
}

int sprout_sim_recorded_iters(SproutSim* sim, uint32_t out[3]) {
    if (!sim || !out) return fail(SPROUT_E_ARG, "null argument");
    SolveState K;
    CUDA_TRY(cudaMemcpyAsync(&K, sim->d.K, sizeof K, cudaMemcpyDeviceToHost, sim->stream));
    CUDA_TRY(cudaStreamSynchronize(sim->stream));
    for (int k = 0; k < 3; k++) out[k] = K.rec[k];
    return SPROUT_OK;
}

int sprout_sim_flow_parity(SproutSim* sim, uint32_t* parity) {
    if (!sim || !parity) return fail(SPROUT_E_ARG, "null argument");
    return sim->flow_parity(parity);
}

int sprout_sim_cell_counts(SproutSim* sim, const int32_t lo[2], const int32_t hi[2], uint32_t* out, size_t cap,
                           size_t* cells) {
    if (!sim || !lo || !hi) return fail(SPROUT_E_ARG, "null argument");
    return sim->cell_counts(lo, hi, out, cap, cells);
}
int sprout_sim_step(SproutSim* sim, uint32_t substeps, float target, const SproutTool* tool) {
    if (!sim) return fail(SPROUT_E_ARG, "null sim");
    return sim->step(substeps, target, reinterpret_cast<const ToolState*>(tool));
}
int sprout_sim_frame_blocking(SproutSim* sim, uint32_t substeps, float target, const SproutTool* tool, double* advanced) {
    if (!sim || !advanced) return fail(SPROUT_E_ARG, "null argument");
    const double start = sim->sim_time;
    int rc = sim->step(substeps, target, reinterpret_cast<const ToolState*>(tool));
    if (rc == SPROUT_OK) rc = sim->poll();
    if (rc == SPROUT_OK) rc = sim->check_device_error();
    *advanced = sim->sim_time - start;
    return rc;
}
int sprout_sim_dt_estimate(SproutSim* sim, float* dt) {
    if (!sim || !dt) return fail(SPROUT_E_ARG, "null argument");
    *dt = sim->dt_estimate();
    return SPROUT_OK;
}
int sprout_sim_step_blocking(SproutSim* sim, uint32_t substeps, const SproutTool* tool) {
    if (!sim) return fail(SPROUT_E_ARG, "null sim");
    return sim->step_blocking(substeps, reinterpret_cast<const ToolState*>(tool));
}
int sprout_sim_advance_blocking(SproutSim* sim, double seconds, const SproutTool* tool) {
    if (!sim) return fail(SPROUT_E_ARG, "null sim");
    return sim->advance_blocking(seconds, reinterpret_cast<const ToolState*>(tool));
}
int sprout_sim_sync(SproutSim* sim) {
    if (!sim) return fail(SPROUT_E_ARG, "null sim");
    CUDA_TRY(cudaStreamSynchronize(sim->stream));
    return sim->check_device_error();
}
int sprout_sim_download_particles(SproutSim* sim, SproutParticle* out, uint32_t cap, uint32_t* n) {
    if (!sim || !n) return fail(SPROUT_E_ARG, "null argument");
    CUDA_TRY(cudaStreamSynchronize(sim->stream));
    *n = sim->n_slots;
    uint32_t m = std::min(cap, sim->n_slots);
    if (out && m > 0) CUDA_TRY(cudaMemcpy(out, sim->d.part, (size_t)m * sizeof(SproutParticle), cudaMemcpyDeviceToHost));
    if (out) sim->d2h_bytes += (size_t)m * sizeof(SproutParticle);
    return SPROUT_OK;
}
int sprout_sim_download_pressure(SproutSim* sim, float* out) {
    if (!sim || !out) return fail(SPROUT_E_ARG, "null argument");
    CUDA_TRY(cudaStreamSynchronize(sim->stream));
    CUDA_TRY(cudaMemcpy(out, sim->d.pres, (size_t)sim->W * sim->H * sizeof(float2), cudaMemcpyDeviceToHost));
    return SPROUT_OK;
}
int sprout_sim_download_field(SproutSim* sim, const char* name, void* out, size_t cap, size_t* bytes) {
    if (!sim || !name || !bytes) return fail(SPROUT_E_ARG, "null argument");
    const DevScene& d = sim->d;
    size_t nc = (size_t)sim->W * sim->H;
    const void* src = nullptr;
    size_t b = 0;
    std::string n(name);
    if (n == "acc") { src = d.acc; b = nc * d.stride * 4; }
    else if (n == "vel") { src = d.vel; b = nc * 16; }
    else if (n == "vel0") { src = d.vel0; b = nc * 8; }
    else if (n == "cell") { src = d.cell; b = nc * 16; }
    else if (n == "comp") { src = d.comp; b = nc * 16; }
    else if (n == "coef") { src = d.coef; b = nc * 16; }
    else if (n == "sprop") { src = d.sprop; b = nc * 16; }
    else if (n == "sdf") { src = d.sdf; b = (size_t)(sim->W + 1) * (sim->H + 1) * 4; }
    else if (n == "surf") { src = d.surf; b = nc * 16; }
    else if (n == "pjump") { src = d.pjump; b = nc * 8; }
    else if (n == "therm") { src = d.therm; b = nc * 16; }
    else if (n == "dheat") { src = d.dheat; b = nc * 16; }
    else if (n == "hcell") { src = d.hcell; b = nc * 8; }
    else if (n == "vw") { src = d.vw; b = nc * 16; }
    else if (n == "vs") { src = d.vs; b = nc * 16; }
    else if (n == "pres") { src = d.pres; b = nc * 8; }
    else if (n == "prhs") { src = d.prhs; b = nc * 16; }
    else if (n == "mga") { src = d.mga; b = (size_t)d.lv.total * 16; }
    else if (n == "mgd") { src = d.mgd; b = (size_t)d.lv.total * 4; }
    else if (n == "mgz") { src = d.mgz; b = (size_t)d.lv.total * 8; }
    else if (n == "ptile") { src = d.ptile; b = (size_t)d.lv.tiles * 4; }
    else if (n == "p2keep") { src = d.p2keep; b = nc * 4; }
    else if (n == "aux") { src = d.aux; b = nc * 16; }
    else if (n == "grho") { src = d.grho; b = nc * 16; }
    else if (n == "gbase") { src = d.gbase; b = nc * 16; }
    else if (n == "rh") { src = d.rh; b = nc * 16; }
    else if (n == "magc") { src = d.magc; b = nc * 8; }
    else if (d.estr && n == "estr") { src = d.estr; b = nc * 16; }
    else if (n == "rl") { src = d.rl; b = nc * 8; }
    else if (d.famocc && n == "famocc") { src = d.famocc; b = nc * 4 * (size_t)sim->settle_fams; }
    else if (d.dsettle && n == "dsettle") { src = d.dsettle; b = nc * 8 * (size_t)sim->settle_fams; }
    else if (n == "surf2") { src = d.surf2; b = nc * 16; }
    else if (d.mixb && n == "mixb") { src = d.mixb; b = nc * 4 * (size_t)std::max(sim->tank.families - 1, 0); }
    else if (sim->visc_alloc && n == "tiles") { src = d.tiles; b = (size_t)d.nwg * 4; }
    else if (sim->visc_alloc && n == "vtile") { src = d.vtile; b = (size_t)d.lv.tiles * 4; }
    else if (sim->visc_alloc && n == "vd") { src = d.vd; b = nc * 8; }
    else if (sim->visc_alloc && n == "vma") { src = d.vma; b = (size_t)d.lv.total * 16; }
    else if (sim->visc_alloc && n == "vmb") { src = d.vmb; b = (size_t)d.lv.total * 16; }
    else if (sim->visc_alloc && n == "vmd") { src = d.vmd; b = (size_t)d.lv.total * 8; }
    else if (n == "ledger") { src = d.ledger; b = 8 * 8; }
    else if (n == "count") { src = d.count; b = nc * 4; }
    else if (n == "start") { src = d.start; b = (nc + 1) * 4; }
    else if (n == "step") { src = d.S; b = sizeof(StepState); }
    else if (n == "solve") { src = d.K; b = sizeof(SolveState); }
    else if (n == "region_air") { src = &d.S->region_air; b = 4; }
    else return fail(SPROUT_E_ARG, "unknown field " + n);
    *bytes = b;
    if (!out) return SPROUT_OK;
    if (cap < b) return fail(SPROUT_E_ARG, "buffer too small for field " + n);
    CUDA_TRY(cudaStreamSynchronize(sim->stream));
    CUDA_TRY(cudaMemcpy(out, src, b, cudaMemcpyDeviceToHost));
    return SPROUT_OK;
}
int sprout_sim_stats(SproutSim* sim, SproutSolverStats* o) {
    if (!sim || !o) return fail(SPROUT_E_ARG, "null argument");
    StepState S;
    SolveState K;
    CUDA_TRY(cudaStreamSynchronize(sim->stream));
    CUDA_TRY(cudaMemcpy(&S, sim->d.S, sizeof S, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(&K, sim->d.K, sizeof K, cudaMemcpyDeviceToHost));
    sim->d2h_bytes += sizeof S + sizeof K;
    std::memset(o, 0, sizeof *o);
    o->substeps = S.substeps;
    o->sim_time = (double)S.advanced - (double)__builtin_bit_cast(float, S.pad0);
    o->dt = S.dt;
    o->dt_prev = S.dt_prev;
    o->pressure_iters[0] = K.p_iters[0];
    o->pressure_iters[1] = K.p_iters[1];
    o->pressure_iters_max = std::max(K.p_it_max, K.p2_it_max);
    o->pressure_unconverged = K.p_unconv;
    o->pressure2_iters_max = K.p2_it_max;
    o->pressure2_unconverged = K.p2_unconv;
    o->viscosity_iters_max = K.v_it_max;
    o->viscosity_unconverged = K.v_unconv;
    o->solves = K.solves;
    o->pressure_residual = K.p_bb[0] > 0.0f ? std::sqrt(K.p_rr[0] / K.p_bb[0]) : 0.0f;
    o->pressure_residual_max = K.p_res_max;
    o->viscosity_residual_max = K.v_res_max;
    o->umax_grid = __builtin_bit_cast(float, S.umax_grid);
    o->umax_part = __builtin_bit_cast(float, S.umax_part);
    o->n_slots = sim->n_slots;
    o->n_live = S.n_live;
    o->caps = sim->caps;
    o->acc_stride = (uint32_t)std::max(sim->tank.stride, 8);
    o->thermal = sim->thermal ? 1u : 0u;
    o->viscosity_mode = (uint32_t)sim->visc_mode;
    o->levels = (uint32_t)sim->d.lv.n;
    o->tail = (uint32_t)sim->d.lv.tail;
    o->device_error = K.error;
    o->viscosity_iters = K.v_iters;
    o->pressure2_iters = K.p2_iters;
    o->pressure_true_residual = K.p_true_res;
    o->pressure_true_residual_max = K.p_true_res_max;
    o->pressure_replacements = K.p_repl;
    o->viscosity_residual = K.v_r0 > 0.0f ? std::sqrt(K.v_rr / K.v_r0) : 0.0f;
    o->h2d_bytes = sim->h2d_bytes;
    o->d2h_bytes = sim->d2h_bytes;
    return SPROUT_OK;
}
int sprout_sim_profile(SproutSim* sim, uint32_t substeps, float* ms) {
    if (!sim || !ms) return fail(SPROUT_E_ARG, "null argument");
    if (sim->n_slots == 0) return fail(SPROUT_E_ARG, "profile before reset");
    return sim->profile(substeps, ms);
}
int sprout_sim_profile_passes(SproutSim* sim, float* ms, uint32_t n) {
    if (!sim || !ms) return fail(SPROUT_E_ARG, "null argument");
    if (n < 6) return fail(SPROUT_E_ARG, "need room for 6 stage times");
    if (sim->n_slots == 0) return fail(SPROUT_E_ARG, "profile before reset");
    float all[SproutSim::kStages];
    int rc = sim->profile_passes(all);
    if (rc != SPROUT_OK) return rc;
    uint32_t m = std::min(n, (uint32_t)SproutSim::kStages);
    for (uint32_t k = 0; k < m; k++) ms[k] = all[k];
    // with room for 6 only, the stages after the projection count with it
    for (uint32_t k = m; k < (uint32_t)SproutSim::kStages; k++) ms[5] += all[k];
    return SPROUT_OK;
}
int sprout_sim_device_bytes(SproutSim* sim, size_t* bytes) {
    if (!sim || !bytes) return fail(SPROUT_E_ARG, "null argument");
    *bytes = sim->bytes;
    return SPROUT_OK;
}

}  // extern "C"

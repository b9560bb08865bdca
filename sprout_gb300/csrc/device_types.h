// Plain structs shared by the host orchestration and the device kernels of the engine.
// DevParams / DevMat carry the per-substep constants and the material table in grid units
// (the Params uniform and Mat table of shaders/common.glsl:37-86, 224-238); StepState and
// SolveState are the device-resident step and Krylov scalars (StepBuf, SolveBuf,
// common.glsl:122-149).
#pragma once

#include <array>
#include <cstdint>

namespace std {
using array3i = std::array<int, 3>;
}

namespace sprout {

constexpr int kMaxPresent = 12;
constexpr int kMaxCurrents = 16;   // params.rs: MAX_CURRENTS
constexpr int kMaxMagnets = 8;     // params.rs: MAX_MAGNETS
constexpr int kGroups = 4;
constexpr int kMaxLevels = 24;
constexpr int kMaxDevices = 64;   // devices per process the library keeps per-device state for

constexpr uint32_t CAP_FAMILIES = 1u, CAP_THERMAL = 2u, CAP_RIGID = 4u, CAP_RHEO = 8u, CAP_MAGNET = 16u,
                   CAP_ELASTIC = 32u, CAP_SETTLE = 64u, CAP_STEAM = 128u, CAP_REACT = 256u;

struct ToolState {
    float pos[2], vel[2], radius;
    int32_t mode;
    float strength;
};

// One material row in grid units (the fields the engine's passes read).
struct DevMat {
    int ia[4];      // phase group; diluent row; channel of its weight; channel of weight x concentration
    int ib[4];      // family; rheology; temperature model; residue
    float a[4];     // relative density; ln kinematic viscosity (cells^2/s); tension vs air (cells^3/s^2); mix rate
    float b[4];     // cos, sin of the contact angle; grain (cells); relative density when frozen
    float temp[4];  // temperature law B, C (K), reference temperature (K); skin
    float th[4];    // heat capacity / water's; conductivity (grid units); solidus, liquidus (deg C)
    float th2[4];   // latent heat (degrees); emissivity; boiling point; latent heat of vaporisation
    float misc[4];  // freeze shift; load; viscosity blend exponent; thermal expansion (1/K)
    float rx[4];    // reaction rate; reaction heat; self-heating (K/s); volatility
    float rheo[4];  // yield stress / water's density (cells^2/s^2); flow index; shear time (s); viscosity ratio
    float gr[4];    // friction coefficient; fume; fizz; unused
    float el[4];    // shear modulus / water's density; relaxation time; susceptibility; residue share
};

// One row of the optics table (material.rs GpuOptics, optics.glsl struct Optics): 240 bytes.
struct DevOptics {
    float absorb[4];   // absorption (linear RGB) and mean reduced scattering, 1 / cell
    float solid[4];    // frozen colour (linear RGB); tint depth (cells)
    float opt[4];      // opacity, platelet sheen, metal, gloss
    float sty[4];      // fullness, foam, drying time of its coat (s), emissivity
    int idx[4];        // diluent row (-1 none), phase group, dried film's scatter x 1000
    float fx[4];       // volatile share, coat (FILM_UNITs), iridescence, crust
    float fx2[4];      // froth (s), fizz, specks drawn per cell, drainage time of its foam (s)
    float lum[4];      // its own light (linear RGB), the share of it that needs stirring
    float hot[4];      // absorption and scattering at thermo_hi
    float thermo[4];   // thermochromic range lo, hi; wetting; soapy aqueous
    float scat[4];     // reduced scattering red, green, blue over its mean; asymmetry g
    float opt2[4];     // refractive index; platelets' rotational diffusion; Bretherton constant; evaporation
    float dust[4];     // what one drawn speck stands for: absorption (RGB), scattering
    float dust2[4];    // speck radius (m), density, thickness over diameter, mirror reflectance
    float dcol[4];     // speck colour (linear RGB); drawn specks per cell where packed
};
static_assert(sizeof(DevOptics) == 240, "GpuOptics is 240 bytes");

// The render side's clock (FluidSim::record_cell_optics: stain_at, flow_parity), kept on the
// device so that a render call needs no read-back: the simulated time of the last call, and
// what this call's flow map uses (its step, the time after it, the copy it reads, whether it
// runs).
struct RenderClock {
    double stain;      // simulated time of the last render call, s
    float dt, now;     // this call: time since the last one (0 .. 0.25 s), and now, as f32
    uint32_t src;      // the copy (0 or 1) the flow map reads: the one that holds it now
    uint32_t parity;   // the copy that holds it after this call
    uint32_t run;      // 1: the flow map runs in this call
    uint32_t pad;
};
static_assert(sizeof(RenderClock) == 32, "RenderClock is 32 bytes");

struct DevParams {
    int grid[2];
    uint32_t n_slots;
    float dt_fixed, gravity, inv_ppc, apic_clamp;
    float pair[kGroups][kGroups];
    float misc[4];   // curvature limit; sealed vent; cell size (m); unused
    int n_present, acc_stride, n_fam;
    uint32_t group_mask, caps;
    int primary;
    uint32_t group_heat;
    int present[kMaxPresent];
    int fams[kMaxPresent][2];   // per concentration family: its row, its diluent's row (-1 none)
    uint32_t sorts;   // bit g: phase group g drifts within itself (group_sorts, common.glsl:590-602)
    float heat[4], heat2[4], heat3[4];
    float sep_tau, cfl, tool_crowd_max, density_k, dt_max, crowd_jitter, ext_speed, wall_margin;
    float tool_pos[2], tool_vel[2], tool_radius;
    int tool_mode;
    float tool_strength;
    float tol[4], ext[4], corr[4];
    uint32_t pressure_max_iters;
    int visc_mode;    // 0 none, 1 explicit, 2 implicit
    int thermal;
    // the implicit viscosity solve (params.rs:289-320)
    uint32_t viscosity_max_iters;
    int visc_levels;   // levels below the grid in its V-cycle: min(viscosity_mg_levels, tail)
    int visc_sweeps;   // Gauss-Seidel sweeps per visit of a level (1 or 2)
    int viscosity_warm, viscous_warm, viscous_projection;
    int viscosity_precond;   // 0: the Jacobi-preconditioned iteration, 1: the multigrid one
    // currents (params.rs:1113-1121): position (cells), radius, rate (1/s; negative: a drain);
    // the velocity the liquid is driven towards (cells/s). ext[3] holds how many.
    float current_zone[kMaxCurrents][4];
    float current_vel[kMaxCurrents][4];
    // magnets (params.rs:1082-1087): how many, the strongest susceptibility in the tank, its
    // saturation (T), 1 / (water density dx^2); each magnet's position (cells), radius, strength
    // (T) and the direction of its north pole
    float elastic[4];   // stress channel; the largest shear modulus / water's density (cells^2/s^2); stress cap (x G); step cap
    float mag[4];
    float magnet[kMaxMagnets][4];
    float magnet_dir[kMaxMagnets][4];
    float iters_margin;   // recorded iterations' margin over the last frame's (params.rs:284)
};

// StepBuf (common.glsl:122-135) plus the engine's own step flags.
struct StepState {
    float frame_left, advanced;
    uint32_t batch_steps, batch_done;
    float dt, dt_prev;
    uint32_t umax_grid, umax_part;
    float dt_cfl;
    uint32_t substeps;
    float umax_seen;
    uint32_t pad0;
    uint32_t gather;      // 0 on the first substep after a reset
    uint32_t region_air;  // bit per region holding a cell without liquid (grid_prep.comp)
    uint32_t n_live;      // live particles after the last sort
    float corr_gain;      // min(1 - exp(-dt / tau), density_k): rhs.comp:79
    float emit_speed;     // fastest particle the device emitters queued for the next step call
};

// SolveBuf (common.glsl:138-149): pressure scalars and statistics.
struct SolveState {
    float p_rz[2], p_alpha[2], p_beta[2], p_bb[2], p_rr[2];
    uint32_t p_done[2], p_iters[2];
    uint32_t p_it_max, p_unconv, p2_it_max, p2_unconv, solves;
    float p_res_max;
    uint32_t v_it_max, v_unconv;
    float v_res_max;
    uint32_t error;       // non-zero: a bounded wait in a persistent kernel ran out
    uint32_t bar_count, bar_gen;   // the persistent kernels' grid barrier
    uint32_t v_iters, v_done;      // the last viscosity solve
    float v_rr, v_r0;
    uint32_t p2_iters;             // iterations of the last second pressure solve
    uint32_t err_arrived;          // on a barrier timeout: blocks that had arrived, of
    uint32_t err_blocks;           // the grid's blocks (diagnostics)
    float p_true_res, p_true_res_max;   // mixed precision: |b - A x| / |b| in FP64, last / max
    // phase trace (off when null): row g % trace_rows of trace_cols words holds, per block,
    // the %globaltimer ns at which it reached the barrier of generation g; the last column
    // the time block 0 left it
    unsigned long long* trace;
    uint32_t trace_rows, trace_cols;
    uint32_t trace_base;   // barriers of the earlier launches (rows of later ones follow on)
    uint32_t p_repl;       // mixed precision: residual replacements, all solves since the reset
    // The reference's recorded iteration counts (FluidSim pressure_rec, pressure2_rec,
    // viscosity_rec; mod.rs:3093-3114) for the first pressure solve, the second and the
    // implicit viscosity solve: a solve that has not converged stops at cap, rec rounded up as
    // the reference records it (mod.rs:2569, 2603-2606). A step call is a frame: its solves'
    // most iterations (f_it) and unconverged solves (f_un) adapt rec when it ends (k_frame_end).
    uint32_t rec[3], cap[3], f_it[3], f_un[3];
    // failure injection for tests (0: off): block dbg_block arrives dbg_stall_ns late at every
    // grid barrier, and a wait gives up after dbg_spin_limit polls instead of SPIN_LIMIT
    uint32_t dbg_block, dbg_stall_ns, dbg_spin_limit, pad3;
};
// The iterations a frame records for a solve from its recorded count (mod.rs:2569, 2603-2606):
// rounded up to even, and the viscosity solve's to a multiple of 4 with the Jacobi
// preconditioner (whose iterations cost less).
#ifdef __CUDACC__
#define SP_HOST_DEVICE __host__ __device__
#else
#define SP_HOST_DEVICE
#endif
SP_HOST_DEVICE inline uint32_t recorded_limit(uint32_t rec, bool viscosity, bool mg_precond) {
    const uint32_t q = (viscosity && !mg_precond) ? 4u : 2u;
    return (rec + q - 1u) / q * q;
}

// SolveState::error bits: a bounded wait ran out; a solve's residual or right-hand side was
// not finite (the solve stopped)
constexpr uint32_t ERR_TIMEOUT = 1u, ERR_DIVERGED = 2u;

// The multigrid hierarchy (Levels, src/sim/mod.rs:714-753).
struct Levels {
    int n = 0;
    int w[kMaxLevels] = {}, h[kMaxLevels] = {};
    int off[kMaxLevels] = {};
    int toff[kMaxLevels] = {};
    int total = 0, tail = 0, tiles = 0;
    // ceil(2^32 / d) for d = the level's width and its width in 16 x 16 tiles: floor(t / d)
    // is the high word of t x that, exactly, for t < 2^20 and d < 2^11 (set_magics)
    uint32_t wm[kMaxLevels] = {}, tm[kMaxLevels] = {};
};

constexpr uint32_t div_magic(int d) { return (uint32_t)(((1ull << 32) + (unsigned long long)d - 1ull) / (unsigned long long)d); }
constexpr void set_magics(Levels& L) {
    for (int l = 0; l < L.n; l++) {
        L.wm[l] = div_magic(L.w[l]);
        L.tm[l] = div_magic((L.w[l] + 15) / 16);
    }
}

// The hierarchy of a w x h grid (Levels, src/sim/mod.rs:714-753): each level halves the one
// above, rounding up, until a level has at most 4 cells; the tail (solved by one work group)
// starts at the first level below the grid with at most 1500 cells. Level l's 16 x 16 tiles
// are numbered from toff[l], for the levels down to the tail. constexpr, so that a fixed-size
// array can be sized for the worst grid it accepts.
constexpr Levels make_levels(int w, int h) {
    Levels L;
    L.w[0] = w;
    L.h[0] = h;
    L.n = 1;
    while (L.w[L.n - 1] * L.h[L.n - 1] > 4 && L.n < kMaxLevels) {
        L.w[L.n] = (L.w[L.n - 1] + 1) / 2;
        L.h[L.n] = (L.h[L.n - 1] + 1) / 2;
        L.n++;
    }
    int total = 0;
    for (int l = 0; l < L.n; l++) {
        L.off[l] = total;
        total += L.w[l] * L.h[l];
    }
    L.total = total;
    int tail = L.n - 1;
    for (int l = 1; l < L.n; l++)
        if (L.w[l] * L.h[l] <= 1500) {
            tail = l;
            break;
        }
    L.tail = tail < 1 ? 1 : tail;
    if (L.tail > L.n - 1) L.tail = L.n - 1;
    int tiles = 0;
    for (int l = 0; l <= L.tail; l++) {
        L.toff[l] = tiles;
        tiles += ((L.w[l] + 15) / 16) * ((L.h[l] + 15) / 16);
    }
    L.tiles = tiles;
    set_magics(L);
    return L;
}

}  // namespace sprout

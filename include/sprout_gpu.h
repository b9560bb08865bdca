/*
 * sprout_gpu.h -- C ABI of the GB300 engine for Sprout's per-substep fluid solver.
 *
 * The entry points replace the Rust `FluidSim` interface of the reference
 * (src/sim/mod.rs:862-3474) and its `SimParams` parameter table (src/sim/params.rs:668-996),
 * plus the two CPU helpers the headless tools use to build a tank
 * (Scene::rasterize, src/scene.rs:215-310; maps::fill_rect, src/maps.rs:466-492).
 * Plain pointers and sizes only. Every call returns an int status (SPROUT_OK or a negative
 * SPROUT_E_* code); sprout_last_error() gives the message of the last failure on the
 * calling thread. Nothing aborts the process.
 *
 * Ownership: the library owns all device memory; host arrays passed in are copied and
 * never retained. Threading: one SproutSim = one CUDA stream; calls on one handle must be
 * serialised by the caller; distinct handles may be used from different threads.
 */
#ifndef SPROUT_GPU_H
#define SPROUT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPROUT_OK 0
#define SPROUT_E_ARG (-1)          /* a bad argument (null handle, size, unknown key) */
#define SPROUT_E_NOMEM (-2)        /* a device or host allocation failed */
#define SPROUT_E_CAPACITY (-3)     /* more particles or materials than the tank holds */
#define SPROUT_E_DIVERGED (-4)     /* a solve produced a non-finite residual */
#define SPROUT_E_TIMEOUT (-5)      /* a bounded device-side wait ran out */
#define SPROUT_E_CUDA (-6)         /* a CUDA runtime error */
#define SPROUT_E_UNSUPPORTED (-7)  /* the tank needs a capability this engine does not carry */

/* One particle, 48 bytes: Particle of src/sim/params.rs:35-54 (shaders/common.glsl:11-19). */
typedef struct SproutParticle {
    float pos[2];   /* cells */
    float vel[2];   /* cells / s */
    float c[4];     /* APIC affine matrix (du/dx, du/dy, dv/dx, dv/dy), 1 / s */
    float s;        /* concentration */
    uint32_t kind;  /* 0 dead, else material row + 1 in the low byte */
    uint32_t id;    /* permanent identity */
    float t;        /* enthalpy temperature, deg C */
} SproutParticle;

/* ToolState (src/sim/params.rs:1141-1150): the mouse tool for one step call. */
typedef struct SproutTool {
    float pos[2], vel[2], radius;
    int32_t mode;   /* 0 none, 1 grab, 2 erase, 3 push, 4 nozzle, 5 heat, 6 cool, 7 whirl, 8 hold */
    float strength;
} SproutTool;

/* Current (src/sim/params.rs:1113-1121): a zone (pos, radius, cells) that drives the liquid
 * in it towards vel (cells / s) at `rate` (1 / s), or drains it at -rate when rate < 0. */
typedef struct SproutCurrent {
    float pos[2], radius, vel[2], rate;
} SproutCurrent;
#define SPROUT_MAX_CURRENTS 16

/* Magnet (src/sim/params.rs:1082-1087): a point dipole at pos (cells), radius (cells), field
 * strength on its axis at the rim (T), north pole along dir. */
typedef struct SproutMagnet {
    float pos[2], radius, strength, dir[2];
} SproutMagnet;
#define SPROUT_MAX_MAGNETS 8

/* SolverStats (src/sim/mod.rs:334-363) plus the step scalars of StepBuf (common.glsl:122-135). */
typedef struct SproutSolverStats {
    uint64_t substeps;                 /* substeps run since the last reset */
    double sim_time;                   /* simulated seconds since the last reset */
    float dt, dt_prev;                 /* the last substep and the one before, s */
    uint32_t pressure_iters[2];        /* iterations of the last (first) pressure solve (P, psi) */
    uint32_t pressure_iters_max;       /* most iterations any pressure solve needed */
    uint32_t pressure_unconverged;     /* pressure solves that hit pressure_max_iters */
    uint32_t pressure2_iters_max, pressure2_unconverged;
    uint32_t viscosity_iters_max, viscosity_unconverged;
    uint32_t solves;
    float pressure_residual;           /* |r| / |b| of the last pressure solve */
    float pressure_residual_max;
    float viscosity_residual_max;
    float umax_grid, umax_part;        /* cells / s */
    uint32_t n_slots, n_live;
    uint32_t caps, acc_stride, thermal, viscosity_mode, levels, tail;
    uint32_t device_error;             /* non-zero: a bounded device wait ran out */
    uint64_t h2d_bytes, d2h_bytes;     /* host <-> device bytes this sim has moved (cumulative) */
    uint32_t viscosity_iters;          /* iterations of the last implicit viscosity solve */
    float viscosity_residual;          /* |r| / |r0| of the last implicit viscosity solve */
    uint32_t pressure2_iters;          /* iterations of the last second pressure solve */
    float pressure_true_residual;      /* mixed precision: |b - A x| / |b| of the last solve's
                                          pressure with about 48 significant bits (products
                                          and sums as float pairs; 0 in plain mode) */
    float pressure_true_residual_max;
    uint32_t pressure_replacements;    /* mixed precision: times the carried residual was replaced
                                          by b - A x evaluated as float pairs (cumulative) */
} SproutSolverStats;

typedef struct SproutParams SproutParams;   /* SimParams */
typedef struct SproutScene SproutScene;     /* Scene */
typedef struct SproutSim SproutSim;         /* FluidSim */

const char* sprout_last_error(void);
const char* sprout_version(void);

/* ---- parameters: SimParams (src/sim/params.rs:149-451) ------------------------------- */
/* SimParams::default() (params.rs:386-451) with the built-in material table. */
int sprout_params_new(SproutParams** out);
int sprout_params_free(SproutParams* p);
int sprout_params_copy(const SproutParams* src, SproutParams** out);
/* SimParams::set (params.rs:986-996): by name (PARAMS, ALIASES, MAT_PARAMS as
 * `<prop>_<material>` or `<material>.<prop>`, custom rows `mat<row>`), clamped to the
 * parameter's range. *ok = 1 if the name resolved and v is not NaN, else 0 and nothing
 * changes (the reference's `false`). */
int sprout_params_set(SproutParams* p, const char* key, float v, int* ok);
/* Reads a parameter by the same names; *ok = 0 for an unknown name. */
int sprout_params_get(const SproutParams* p, const char* key, float* v, int* ok);
/* The diluent of custom liquid `row` (59..95), as the library's loader resolves a liquid's
 * "diluent" reference into `MatProps::diluent` (src/library.rs:318-330): -1 for none, else
 * another row that is a built-in without a diluent of its own, or a custom liquid. The
 * liquid is then `s` parts itself and 1 - s parts the diluent (a concentration family).
 * *ok = 0 and nothing changes for a built-in row or a diluent the loader would drop. */
int sprout_params_set_diluent(SproutParams* p, uint32_t row, int32_t diluent, int* ok);
/* The phase group of custom liquid `row` (59..95), as the library's loader reads a liquid's
 * "group" (src/library.rs:283-286): 0 aqueous, 1 oil-like, 2 metal, 3 silicate. Liquids of
 * different groups are immiscible: they drift apart and meet at interfaces with the pair
 * tension of their groups. *ok = 0 and nothing changes for a built-in row or another group. */
int sprout_params_set_group(SproutParams* p, uint32_t row, uint32_t group, int* ok);

/* ---- scene: Scene (src/scene.rs) ---------------------------------------------------- */
int sprout_scene_new(uint32_t w, uint32_t h, SproutScene** out);
int sprout_scene_free(SproutScene* s);
/* Shape::Box (scene.rs:16): centre, half-extents, angle (radians); temp: the temperature
 * it is held at (deg C), or NaN for an insulating solid (Scene::temps). */
int sprout_scene_add_box(SproutScene* s, float cx, float cy, float hx, float hy, float angle, float temp);
/* Shape::Circle (scene.rs:12). */
int sprout_scene_add_circle(SproutScene* s, float cx, float cy, float r, float temp);
/* Scene::sdf (scene.rs:195-198). */
int sprout_scene_sdf(const SproutScene* s, float x, float y, float* d);
/* Scene::rasterize (scene.rs:215-310): sdf[(w+1)(h+1)], solid[4 w h] (open fraction of
 * the left face, of the bottom face, smoothed solid occupancy, open volume), region[w h],
 * temp[w h] (may be NULL; *heated = 1 if any shape is held at a temperature). */
int sprout_scene_rasterize(const SproutScene* s, float* sdf, float* solid4, uint32_t* region,
                           float* temp, int* heated);
/* Scene::rasterize computed on the current CUDA device, into the same host arrays as
 * sprout_scene_rasterize and bit-identical to it: the node distances and chamfer union depth,
 * open volumes, pocket sealing, face fractions, occupancy, regions and held temperatures as
 * device passes. Blocking. */
int sprout_scene_rasterize_device(const SproutScene* s, float* sdf, float* solid4, uint32_t* region, float* temp,
                                  int* heated);
/* maps::fill_rect (maps.rs:466-492): rest-density particles of `material` in rect
 * (x0, y0, x1, y1, cells), skipping solids. `n_before` is the number of particles already
 * placed (it seeds the jitter, as out.len() does in the reference). Writes at most `cap`
 * particles to out and sets *n to the number the rectangle holds. */
int sprout_fill_rect(const SproutScene* s, const float rect[4], uint32_t material,
                     uint32_t n_before, SproutParticle* out, uint32_t cap, uint32_t* n);

/* ---- devices ----------------------------------------------------------------------------
 * No counterpart in the reference (it opens one Vulkan device). Sims and batches are created
 * on the calling thread's current CUDA device and keep using it; these select it. One process
 * may drive several devices, one sim or batch per device at a time per thread. */
int sprout_device_count(int* n);
int sprout_set_device(int device);
int sprout_get_device(int* device);

/* ---- the simulation: FluidSim (src/sim/mod.rs:862-3474) ----------------------------- */
/* FluidSim::new (mod.rs:1034): a w x h grid for at most `capacity` particles, on the
 * current CUDA device. */
int sprout_sim_create(uint32_t w, uint32_t h, uint32_t capacity, const SproutParams* p,
                      SproutSim** out);
int sprout_sim_destroy(SproutSim* sim);
/* Replaces `params` (the pub field of FluidSim); takes effect at the next step. */
int sprout_sim_set_params(SproutSim* sim, const SproutParams* p);
/* FluidSim::set_solids (mod.rs:1976): arrays as sprout_scene_rasterize fills them. */
int sprout_sim_set_solids(SproutSim* sim, const float* sdf, const float* solid4,
                          const uint32_t* region, const float* temp);
/* FluidSim::set_solids with the scene rasterised on the device straight into the sim's
 * buffers (no host arrays, no copies): what World::new does with Scene::rasterize and
 * set_solids (world.rs), for a scene of the sim's grid size. Blocking. */
int sprout_sim_set_scene(SproutSim* sim, const SproutScene* s);
/* FluidSim::reset (mod.rs:1981-2002): replaces every particle (ids = index, spawn fields
 * settled). SPROUT_E_UNSUPPORTED if the tank needs a capability the engine lacks. */
int sprout_sim_reset(SproutSim* sim, const SproutParticle* p, uint32_t n);
/* FluidSim::set_currents (mod.rs:2008-2012): replaces the currents, keeping the first
 * SPROUT_MAX_CURRENTS; they act from the next step on and survive a reset. */
int sprout_sim_set_currents(SproutSim* sim, const SproutCurrent* c, uint32_t n);
/* FluidSim::set_magnets (mod.rs:2018-2022): replaces the magnets, keeping the first
 * SPROUT_MAX_MAGNETS; they survive a reset. With a susceptible liquid in the tank (its
 * `susceptibility`) the field's energy pulls on it (magnet.comp). */
int sprout_sim_set_magnets(SproutSim* sim, const SproutMagnet* m, uint32_t n);
/* FluidSim::spawn (mod.rs:2024-2046): queues particles for the next step call (new ids
 * follow the last given, spawn fields settled, marked fresh). *accepted = how many were
 * queued: at most SPROUT_SPAWN_MAX wait at once, particles without a material are skipped,
 * and 0 are taken (SPROUT_OK) when their materials do not fit the tank's channels. At the
 * next step they fill free slots, then recycle dead ones (claim.comp); entries beyond the
 * dead slots are dropped, as the reference drops them. SPROUT_E_ARG before a reset. */
#define SPROUT_SPAWN_MAX 32768u
int sprout_sim_spawn(SproutSim* sim, const SproutParticle* p, uint32_t n, uint32_t* accepted);
/* FluidSim::cell_counts (mod.rs:3350-3387) with count.comp: live particles per cell of the
 * window of cells [lo, hi) (inside the grid), row by row, after the work queued so far, the
 * particles queued by spawn included. *cells = the window's cell count; out may be NULL to
 * ask for it. Blocking; reads back only the window. SPROUT_E_ARG for a window outside the
 * grid (the reference asserts) or cap < *cells. */
int sprout_sim_cell_counts(SproutSim* sim, const int32_t lo[2], const int32_t hi[2], uint32_t* out,
                           size_t cap, size_t* cells);

/* ---- the brush's emitters on the device ------------------------------------------------
 * World::emit's sources (world.rs:609-727) with brush.rs's geometry, replacing the host's
 * candidates + FluidSim::cell_counts (a blocking read-back) + Admission + FluidSim::spawn:
 * the candidates are laid out, tested against the solids (World::solid_distance, from the
 * sim's own node distances) and admitted against the live particles of each cell on the
 * device, in the order World::emit takes them, and queued into particle slots with the ids
 * and the per-step cap FluidSim::spawn gives. Nothing is read back: the calls return once
 * the work is queued on the sim's stream. The material row joins the tank as a spawn of it
 * would (also when no candidate is admitted). World::rand's generator (seeded 0x12345678 as
 * World::new does) and the next particle id live on the device from the first emission on.
 * Particles queued by sprout_sim_spawn before an emission take their ids first. A sim in a
 * batch takes no emission (SPROUT_E_ARG). */
typedef struct SproutSpout {   /* brush::Spout (brush.rs:18-23) */
    float direction[2];
    float speed;               /* cells / s */
    float width;               /* cells */
} SproutSpout;
/* Spout::pour (kind 0), Spout::jet (1), Spout::faucet (2) (brush.rs:28-47); `degrees`
 * clockwise from straight down (jet and faucet), `rate` particles / s, `radius` cells. */
int sprout_spout(int kind, float degrees, float rate, float radius, SproutSpout* out);
/* World::stream (world.rs:714-727) with Stream::advance (brush.rs:86-115): the particles of
 * the spout's lattice that appear during `seconds` while the brush moves from `from` to
 * `to`, launched at the spout's velocity where no solid or full cell (1.5 x rest density)
 * holds them back. *stream_time is brush::Stream's state (simulated seconds the stream has
 * run; 0 for a new stroke), advanced by `seconds`. */
int sprout_sim_emit_stream(SproutSim* sim, const SproutSpout* spout, double* stream_time, const float from[2],
                           const float to[2], float seconds, uint32_t material);
/* World::paint (world.rs:644-685): up to `count` particles on the rest-density lattice (or,
 * with `spray`, the sparse spray lattice, jittered, launched outwards from the stroke,
 * brush::spray_velocity) inside the stroke of `radius` from `from` to `to`, in empty cells
 * only, in World::rand's shuffled order. World::stamp is from == to with count 32768. */
int sprout_sim_emit_paint(SproutSim* sim, const float from[2], const float to[2], float radius, uint32_t count,
                          int spray, uint32_t material);
/* World::rain (world.rs:689-710): `count` drops drawn in the cloud 3 radii either side of
 * `at`, falling at brush::RAIN_SPEED, where they find an empty cell. */
int sprout_sim_emit_rain(SproutSim* sim, const float at[2], float radius, uint32_t count, uint32_t material);
/* Sets World::rand's state on the device (blocking). */
int sprout_sim_emitter_seed(SproutSim* sim, uint32_t rng);
/* The particles the emitters have queued since the sim was made (and the last emission's),
 * read back (blocking): what World::emit returns, for a caller that wants it. */
int sprout_sim_emitted(SproutSim* sim, uint64_t* total, uint32_t* last);

/* ---- the render side's cell passes ----------------------------------------------------
 * FluidSim::record_cell_optics (mod.rs:1626-1660) without a window: the per-cell optics of
 * cell_optics.comp (20 layers: absorption and scattering of the aqueous and other liquids,
 * opacity / gloss, emission and speed, frozen colour and share, effects, the key light, the
 * coat, the look key, ...), the key light from above through the liquid (light.comp) and the
 * 3 x 3 smoothing with the light's sideways spread (optics_blur.comp), the light under the
 * surface (sss.comp) and the glow field (glow.comp), into device buffers of
 * RGBA16F texels as the reference's image array holds them. Not computed: the ferrofluid
 * spikes' field and phase (layers 13 xy and 14 xy stay zero), the specks' dust field (layer 18
 * zero), the film map and the smoke field.
 * material.rs optics_table: rows 0 .. rows - 1 of the optics table of a parameter set, each
 * 240 bytes laid out as GpuOptics (material.rs:551-597). */
int sprout_params_optics(const SproutParams* p, void* out, uint32_t rows);
/* A colour of a material row, as a custom liquid's library entry gives it (library.rs):
 * field one of color, color_solid, color_hot, cloud_color, dust_color, glow_color; sRGB in
 * 0 .. 1 (clamped). *ok = 0 for an unknown field or row. */
int sprout_params_set_color(SproutParams* p, uint32_t row, const char* field, const float rgb[3], int* ok);
int sprout_params_get_color(const SproutParams* p, uint32_t row, const char* field, float rgb[3], int* ok);
/* A material row's phase group and diluent row (-1 none). */
int sprout_params_get_row(const SproutParams* p, uint32_t row, int32_t* group, int32_t* diluent);
/* FluidSim::record_cell_optics (src/sim/mod.rs:1626-1712): computes the cell passes from what
 * the last substep left on the grid, on the sim's stream (no wait); `inv_speed` = 1 / the
 * speed that counts as fast, cells / s. As the reference, a call records nothing when no
 * substep, reset, table change or other inv_speed came since the last one; the flow map
 * (flow_map.comp) advances by the simulated time since the last call (at most 0.25 s, read on
 * the device) and is cleared by the first call on a new tank. */
int sprout_sim_render(SproutSim* sim, float inv_speed);
/* FluidSim::recorded_iters (mod.rs:1965-1968): the iterations the next substeps record for
 * the first pressure solve, the second and the viscosity solve (blocking). A solve that has
 * not converged stops there (rounded up to even; the Jacobi viscosity solve to a multiple of
 * 4). As in the reference, a new scene records pressure_max_iters / viscosity_max_iters, and
 * every step call (a frame; each substep of sprout_sim_profile) adapts them from its own
 * solves when it ends (mod.rs:3093-3114), where the reference adapts on the frame's read-back. */
int sprout_sim_recorded_iters(SproutSim* sim, uint32_t out[3]);
/* What the particles of a liquid with a look keep (look.comp; FluidSim's plook, mod.rs:926-929),
 * after the last sprout_sim_render that recorded (blocking): per particle slot, in the order of
 * sprout_sim_download_particles, four words (its id, 0, A_xx A_yy A_xy of its platelets at 10
 * bits each with A_xy offset by 0.5, 0), and the slots listed for the look splat (their order
 * is the device atomics'). *slots = 0 until a render found such a liquid in the tank. The
 * specks a new particle would bring into spray.comp's pool are not made (no pool). */
int sprout_sim_download_look(SproutSim* sim, uint32_t* state, size_t state_cap, uint32_t* list, size_t list_cap,
                             uint32_t* slots, uint32_t* listed);
/* spray.comp's pool (FluidSim::diffuse_buffers, mod.rs:1773-1777): the bubbles, foam, spray
 * and specks of the render calls so far (blocking). An entry is the reference's Diffuse:
 * position and velocity (cells, cells / s), life left (s; a speck: its flake's packed
 * normal), radius (cells), info (bits 0-1 state: 0 free, then bubble, foam, spray, or for a
 * speck suspended, resting, falling; bit 2 grows; bit 3 a speck; bits 8-14 the liquid's row
 * + 1; 15-31 a seed), depth or the foam's given life. pool: all 196608 entries (65536 for
 * bubbles, foam and spray, then 131072 for specks); stack, stack1: the two parts' free stacks
 * (state[1], state[5] entries); list: the live entries for the sprites (state[2]), in entry
 * order; counts: foam per cell (copies 0, 1) and resting specks per cell (2, 3), W x H each;
 * state: bubbles never handed out, their stack's height, entries listed, the copy the next
 * frame counts into, specks never handed out, their stack's height, 0, 0. Each pointer may be
 * NULL. Entries are handed out in a deterministic order: a frame's bubbles ranked by cell,
 * its specks by particle slot. */
typedef struct SproutDiffuse {
    float pos[2], vel[2], life, r;
    uint32_t info;
    float z;
} SproutDiffuse;
int sprout_sim_download_spray(SproutSim* sim, SproutDiffuse* pool, size_t pool_cap, uint32_t* stack, uint32_t* stack1,
                              uint32_t* list, size_t cap, uint32_t* counts, size_t counts_cap, uint32_t state[8]);
/* FluidSim::flow_view's parity (mod.rs:1850-1853): the copy of the flow map that holds it now
 * (blocking). */
int sprout_sim_flow_parity(SproutSim* sim, uint32_t* parity);
/* The layers (blocking), texels of four IEEE half words: which 0, raw (cell_optics.comp's 20
 * layers with light.comp's layer 10); 1, the smoothed image the composite samples
 * (optics_blur.comp's layers 0-19 with 10 left zero, and sss.comp's 20-23: the light under the
 * surface in 20, warm-started from the last call); layer-major, W x H texels each; 2, the glow
 * field (glow.comp), ceil(W / 2) x ceil(H / 2) texels; 3, the flow map (flow_map.comp), four
 * layers: copy 0 (short, long period), copy 1 (short, long), each texel the displacement of
 * two restarts half a period apart (xy, zw), cells. *words = the word count; out may be NULL
 * to ask for it. */
int sprout_sim_download_render(SproutSim* sim, int which, uint16_t* out, size_t cap, size_t* words);
/* Renderer::render's particle fields for one view (src/render.rs:886-1075) and the wet map
 * (render.rs:640-668), into headless device images on the sim's stream (no wait); replaces the
 * splat, tint, down and blur passes (shaders/splat.vert, splat.frag, tint.frag, down.frag,
 * blur.frag) and wet.frag. The view: (center_x, center_y) in cells, `zoom` pixels per cell
 * (> 0), width x height pixels (1 to 16384 each). As render.rs lays them out:
 * - the sharp field: each phase group's weight times the splat kernel, RGBA16F texels of
 *   clamp(1.5 zoom / 2.8, 1, 2) pixels, every live particle drawn stretched back along its path
 *   over 1/160 s;
 * - the tint field, twice as coarse, only when two liquids of one phase group are in the tank
 *   (else its images keep what they held): absorption (RGB) of the concentrate part and the
 *   scattering; the concentrate share, the aqueous weight, the other weight, 0;
 * - the wide field: the sharp field box-filtered down to texels of clamp(2 zoom / 3, 2, 64)
 *   pixels and blurred by a 13-tap Gaussian across, then down;
 * - the look field (render.rs:1004-1036, look.vert, look.frag), in the sharp field's texels: the
 *   particles the last sprout_sim_render listed (look.comp) as discs of radius 1 cell (at least
 *   1.5 texels), each laying down its platelets' sheen, its carried scalar, which way the
 *   platelets lie and its weight; clear without a liquid with a look;
 * - the wet map (RGBA32F, a texel per cell, kept between calls): where liquid (occupancy at least
 *   0.3) lies within 1.75 cells of a solid, its leading material row + 1, family 0's
 *   concentration and the simulated time; written once per simulated time, cleared on a new
 *   tank.
 * Each texel of a splat is the sum over the particles of kernel x weight, added as 64-bit
 * fixed point (2^-32) and rounded to half once: the same whatever order the particles land in
 * (the reference blends in the hardware's order into half floats). */
int sprout_sim_draw(SproutSim* sim, float center_x, float center_y, float zoom, uint32_t width, uint32_t height);
/* An image of the last sprout_sim_draw (blocking): which 0, the sharp field; 1, the tint field's
 * absorption image; 2, its share image; 3, the wide field; 5, the look field (RGBA16F, 8 bytes a
 * texel); 4, the wet map (RGBA32F, 16 bytes a texel, W x H). dims = its texels across and down
 * (0 x 0: not drawn);
 * out may be NULL to ask for them. */
int sprout_sim_download_draw(SproutSim* sim, int which, void* out, size_t cap, uint32_t dims[2]);
/* Stats (src/sim/mod.rs:130-136): live particles and, per material row, its particles and the
 * sum of their concentrations (in particles, a multiple of 1/256). */
#define SPROUT_MATERIAL_ROWS 96
typedef struct SproutStats {
    uint32_t live;
    uint32_t count[SPROUT_MATERIAL_ROWS];
    float conc[SPROUT_MATERIAL_ROWS];
} SproutStats;
/* FluidSim::request_stats (mod.rs:3246-3255, stats.comp): records the census of the particle
 * slots on the sim's stream, after the work queued so far; nothing while one is in flight.
 * Asynchronous. */
int sprout_sim_request_stats(SproutSim* sim);
/* FluidSim::poll_stats (mod.rs:3258-3273): *ready = 1 and *out filled when the last requested
 * census has finished on the device, else *ready = 0 (and *out untouched). Non-blocking. */
int sprout_sim_poll_stats(SproutSim* sim, SproutStats* out, int* ready);
/* FluidSim::record + submit (mod.rs:2400-2562): `substeps` substeps meant to cover
 * `target` seconds (ignored with a fixed step rate). Asynchronous on the sim's stream.
 * tool may be NULL. */
int sprout_sim_step(SproutSim* sim, uint32_t substeps, float target, const SproutTool* tool);
/* FluidSim::frame_blocking (mod.rs:3342-3349): sprout_sim_step, then waits for it; *advanced =
 * the simulated seconds it covered. */
int sprout_sim_frame_blocking(SproutSim* sim, uint32_t substeps, float target, const SproutTool* tool,
                              double* advanced);
/* FluidSim::dt_estimate (mod.rs:1960-1963): the substep length the next step will most likely
 * take, s (1 / fixed_hz with a fixed rate, else the last CFL estimate read back). */
int sprout_sim_dt_estimate(SproutSim* sim, float* dt);
/* FluidSim::step_blocking (mod.rs:3315-3338): `substeps` ticks of 1/240 s, blocking. */
int sprout_sim_step_blocking(SproutSim* sim, uint32_t substeps, const SproutTool* tool);
/* FluidSim::advance_blocking (mod.rs:3284-3312): exactly `seconds`, blocking. */
int sprout_sim_advance_blocking(SproutSim* sim, double seconds, const SproutTool* tool);
/* Waits for the sim's stream. */
int sprout_sim_sync(SproutSim* sim);
/* FluidSim::download_particles: the particle slots in the engine's order (it keeps them
 * sorted by cell, live ones first); *n = slots in use. Blocking. */
int sprout_sim_download_particles(SproutSim* sim, SproutParticle* out, uint32_t cap, uint32_t* n);
/* FluidSim::download_pressure: the two potentials per cell (p dt, psi), 2 w h floats. */
int sprout_sim_download_pressure(SproutSim* sim, float* out);
/* A named grid field (vel, cell, comp, coef, acc, pres, prhs, mga, mgd, pjump, surf, sprop,
 * therm, dheat, hcell, vw, vs, ptile, step, region_air, ledger; sdf, the solid distance at the
 * (W + 1) x (H + 1) nodes) into `out` (at most cap
 * bytes); *bytes = its size. Blocking. For tests and tools. */
int sprout_sim_download_field(SproutSim* sim, const char* name, void* out, size_t cap, size_t* bytes);
/* SolverStats and the step scalars. Blocking. */
int sprout_sim_stats(SproutSim* sim, SproutSolverStats* out);
/* Device memory the sim holds, bytes. */
int sprout_sim_device_bytes(SproutSim* sim, size_t* bytes);
/* FluidSim::substep_cost (mod.rs:2537-2558): runs `substeps` substeps of the last step
 * call's batch and returns their device time in ms, from CUDA events on the sim's stream.
 * Blocking. */
int sprout_sim_profile(SproutSim* sim, uint32_t substeps, float* ms);
/* FluidSim::profile_passes (mod.rs:3120-3160): one substep, stage by stage, each timed by
 * CUDA events: ms[0] advance (G2P, advection, collision), ms[1] sort, ms[2] P2G,
 * ms[3] grid passes (prep, coefficients, surface tension, heat, viscosity setup, rhs),
 * ms[4] pressure solve, ms[5] projection, ms[6] implicit viscosity solve, ms[7] second
 * projection (rhs_visc, second pressure solve, project_visc); the last two are zero-cost
 * unless the tank takes the implicit viscosity between two pressure solves. n >= 6; with
 * n < 8 the stages past n - 1 are added to ms[5]. Blocking. */
int sprout_sim_profile_passes(SproutSim* sim, float* ms, uint32_t n);

/* ---- tracing of the persistent solvers' phases ---------------------------------------
 * No counterpart in the reference (its profile_passes times whole dispatches). enable with
 * rows > 0 keeps the last `rows` grid-barrier generations of the sim's pressure and viscosity
 * kernels (rows == 0: off). read copies up to cap words (blocking): rows of *cols words, per
 * block the device time (ns, %globaltimer) it reached that barrier, in the last column the
 * time block 0 left it; *words = rows x cols. */
int sprout_sim_trace_enable(SproutSim* sim, uint32_t rows);
int sprout_sim_trace_read(SproutSim* sim, unsigned long long* out, size_t cap, size_t* words, uint32_t* cols);

/* ---- precision of the pressure solve -------------------------------------------------
 * No counterpart in the reference (it solves in FP32 only). mode 0: the reference's
 * arithmetic, FP32 throughout (the default). mode 1: mixed precision: the multigrid
 * hierarchy's matrices stored in BF16 (with an FP32 diagonal that keeps every row sum) and
 * computed in FP32; every vector, the CG iterate, residual and operator in FP32; the dot
 * products summed in FP32 as mode 0 sums them, their totals, the step lengths and the
 * convergence test in FP64; as refinement, each time the carried
 * residual has fallen 100x the true residual b - A x is evaluated as float pairs and replaces the
 * carried one where it exceeds it twice over and lies well above the FP32 rounding floor
 * (stats: pressure_replacements); at the end of each solve the true residual is evaluated as
 * float pairs (stats: pressure_true_residual). Both stop at the same
 * relative residual (pressure_tol) of the residual the iteration carries, as the reference
 * does. Takes effect from the next step; the first switch to mode 1 allocates the BF16
 * matrices. */
int sprout_sim_set_precision(SproutSim* sim, int mode);

/* ---- launch shape of the persistent solvers --------------------------------------------
 * No counterpart in the reference (its dispatch sizes follow from the shaders' 16 x 16 work
 * groups). The pressure and viscosity solves each run as one persistent kernel; these are
 * their block counts. 0 = the default: one block per 16 x 16 tile of the grid (a batch: of
 * its tanks), at most as many as the device holds at once; a larger count is lowered to the
 * smaller of the two. Results do not
 * depend on the counts (every block runs the same tile bodies and sums the same partials in
 * the same order; fewer blocks only take more tiles each). batch_viscosity (batches only):
 * 0 = the default (the implicit viscosity solves of a batch's tanks in one persistent kernel
 * when the tanks average at most 1,500 tiles), 1 = always in one kernel, 2 = one solve per
 * tank. The autotuner (sprout_gb300.tune) picks these per grid size from timed candidates.
 * Takes effect from the next step. */
typedef struct SproutLaunch {
    uint32_t pressure_blocks;        /* the plain FP32 pressure solve */
    uint32_t pressure_blocks_mixed;  /* the mixed-precision pressure solve */
    uint32_t viscosity_blocks;       /* the implicit viscosity solve */
    uint32_t batch_viscosity;        /* batches: 1 batched viscosity solve for small tanks, 0 one per tank */
    uint32_t reserved[4];            /* zero */
} SproutLaunch;
int sprout_sim_set_launch(SproutSim* sim, const SproutLaunch* launch);
/* The counts in effect for the tank as it is now (after the lowering to what fits). */
int sprout_sim_get_launch(SproutSim* sim, SproutLaunch* out);

/* ---- failure injection for tests ---------------------------------------------------------
 * No counterpart in the reference. Makes the persistent solvers' bounded grid-barrier wait
 * run out on purpose, to test that it ends: block `block` of every later persistent solve of
 * this sim arrives `stall_ns` nanoseconds late (its wait measured on the device's clock and
 * capped at one second), and every block gives up waiting after `spin_limit` polls instead of
 * the default (about a second). The solve then stops with every block returned, the step's
 * blocking calls report SPROUT_E_TIMEOUT, and later solves of the sim do nothing until a
 * reset, which clears the error and this setting. stall_ns = 0 and spin_limit = 0 switch it
 * off. */
int sprout_sim_debug_stall(SproutSim* sim, uint32_t block, uint32_t stall_ns, uint32_t spin_limit);

/* ---- batches: many tanks, one captured graph per substep -------------------------------
 * The batched and serving layer the reference does not have (it steps one FluidSim). A
 * batch advances its tanks (sims created, filled and reset as usual) together: their
 * particle and grid stages as concurrent branches of one CUDA graph per substep, their
 * pressure solves as one persistent kernel over all their tiles. Each tank's results are
 * the same as when it steps alone (same arithmetic, same reduction order). A sim belongs to
 * at most one batch; while it does, sprout_sim_step refuses it (step the batch); its stats,
 * downloads and parameters work as usual. The implicit viscosity is carried with
 * viscous_projection 1 (the default). Blocking: sync, profile. */
typedef struct SproutBatch SproutBatch;
/* Free and total memory of the current device (cudaMemGetInfo): a serving loop's admission. */
int sprout_device_memory(size_t* free_bytes, size_t* total_bytes);
int sprout_batch_create(SproutBatch** out);
int sprout_batch_destroy(SproutBatch* b);
int sprout_batch_add(SproutBatch* b, SproutSim* sim);
int sprout_batch_remove(SproutBatch* b, SproutSim* sim);
int sprout_batch_size(SproutBatch* b, uint32_t* n);
/* 0 plain, 1 mixed (see sprout_sim_set_precision), for every tank of the batch. */
int sprout_batch_set_precision(SproutBatch* b, int mode);
/* `substeps` substeps of every tank (each at its own dt), asynchronous. */
int sprout_batch_step(SproutBatch* b, uint32_t substeps);
/* One substep of the members at indices members[0 .. n) only (in the order they were added),
 * launched directly without a graph: for continuous batching, where the set of tanks with
 * work changes from launch to launch. Asynchronous. */
int sprout_batch_step_subset(SproutBatch* b, const uint32_t* members, uint32_t n);
/* Every sprout_batch_step / _step_subset call is one ticket, numbered from 1 in issue order.
 * Reports how many were issued and how many have finished on the device (non-blocking). */
int sprout_batch_tickets(SproutBatch* b, uint64_t* issued, uint64_t* completed);
int sprout_batch_sync(SproutBatch* b);
/* Device ms of `substeps` more substeps of the batch, from CUDA events (blocking). */
int sprout_batch_profile(SproutBatch* b, uint32_t substeps, float* ms);
/* The block counts of the batch's persistent solves (SproutLaunch; viscosity_blocks for the
 * batched viscosity solve, pressure_blocks / pressure_blocks_mixed for the batched pressure
 * solves), 0 = the default; as for a sim, results do not depend on them. */
int sprout_batch_set_launch(SproutBatch* b, const SproutLaunch* launch);

/* ---- frame pacing: Pacer (src/pacing.rs) -------------------------------------------------
 * Host-side planner of how many substeps each rendered frame records and what simulated
 * time they should cover, from the frame's length, the expected substep length, the
 * slow-motion factor, the measured device cost of a substep (sprout_sim_profile; 0 while
 * unknown) and the device time a frame may spend simulating. */
#define SPROUT_MAX_SUBSTEPS_PER_FRAME 24
typedef struct SproutPacer SproutPacer;
/* Plan (pacing.rs:43-50): substeps to record and the simulated seconds they should cover
 * (target) and are expected to cover (expected). */
typedef struct SproutPlan {
    uint32_t substeps;
    float target, expected;
} SproutPlan;
int sprout_pacer_new(SproutPacer** out);
int sprout_pacer_free(SproutPacer* p);
/* Pacer::reset (pacing.rs:58-61): forgets owed time. */
int sprout_pacer_reset(SproutPacer* p);
/* Pacer::speed (pacing.rs:63-66): simulated time delivered over asked (1: real time). */
int sprout_pacer_speed(const SproutPacer* p, float* speed);
/* Pacer::plan (pacing.rs:67-112). fixed != 0: a fixed step rate (dt exact). */
int sprout_pacer_plan(SproutPacer* p, float frame_dt, float dt, int fixed, float time_scale, float cost, float budget,
                      SproutPlan* out);

/* ---- a pressure solve that allocates nothing ------------------------------------------
 * No counterpart in the reference: an addition for callers that cannot allocate device
 * memory (a host whose allocator owns the whole device, a path that must not allocate
 * while it runs, an FFI host with a fixed memory budget). It runs the engine's pressure
 * solve (the same kernel as a substep's) on a system the caller holds on the device:
 * mga, mgd, rhs and x are device pointers, w x h cells, laid out as the engine's fields of
 * those names (mga 4 floats per cell: couplings to the left, right, bottom, top neighbour;
 * mgd the diagonal, 0 where the cell is no unknown; rhs 2 floats per cell: pressure and
 * density-correction right-hand sides; x 2 floats per cell, the starting guess on entry
 * and the solution on return, zeroed where the cell is no unknown).
 * All scratch (multigrid hierarchy, Krylov vectors, the solve's scalars) lives in one
 * fixed device array of about 17 MB inside the library, which every GPU that loads it
 * holds until the process exits. It is sized for the worst grid shape it accepts: both
 * sides at least 16 cells and at most 147,456 cells (512 x 288) in all, long thin grids
 * included; other grids are refused with SPROUT_E_CAPACITY. No cudaMalloc, cudaFree or
 * allocating routine is called.
 * The first call on each device looks up the array's device address (with that device
 * current); make that first call before any stream capture. Every call shares the array
 * and starts from cleared scratch, so calls whose work overlaps on the GPU (different
 * streams, several host threads) race: serialise them. `stream` is a cudaStream_t (NULL:
 * the default stream). iters_out (2 values) and residual_out may be NULL; if either is
 * given the call waits for the solve and reports its iterations and |r|/|b|, and returns
 * SPROUT_E_TIMEOUT if a bounded wait ran out or SPROUT_E_DIVERGED if the system was not
 * finite. With both NULL the call returns once the work is queued and reports neither:
 * pass one of them to learn how the solve ended. */
int sprout_pressure_solve_static(uint32_t w, uint32_t h, const float* mga, const float* mgd,
                                 const float* rhs, float* x, float tol_p, float tol_psi,
                                 uint32_t max_iters, void* stream, uint32_t* iters_out,
                                 float* residual_out);

#ifdef __cplusplus
}
#endif
#endif

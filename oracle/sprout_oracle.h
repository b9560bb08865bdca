/*
 * sprout_oracle.h -- C interface of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY. The oracle is a plain-C restatement of the Sprout fluid
 * substep (the reference's GLSL compute shaders under shaders/ and the Rust host code in
 * src/sim/mod.rs, src/sim/params.rs, src/scene.rs and src/maps.rs that feeds them). Only
 * tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py may load it, and
 * only as the checker. The product (sprout_gb300/, libsprout_gpu.so) never links it.
 *
 * Parity status: the scene and particle-placement code is pinned to the reference's own
 * known-answer unit tests (src/scene.rs tests, src/maps.rs tests, src/sim/params.rs
 * tests; see tests/test_oracle_golden.py). The solver arithmetic is a restatement of the
 * shaders; the reference cannot be built or run here (Rust + Vulkan), so solver-level
 * parity against the reference's own output is unpinned and rests on that restatement
 * plus the reference's physics known-answer checks (src/validate.rs).
 */
#ifndef SPROUT_ORACLE_H
#define SPROUT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One particle, 48 bytes (src/sim/params.rs:35-54; shaders/common.glsl:11-19). */
typedef struct OParticle {
    float pos[2];
    float vel[2];
    float c[4];
    float s;
    uint32_t kind;
    uint32_t id;
    float t;
} OParticle;

/* The MatProps fields the substep reads (src/sim/material.rs:160-). */
typedef struct OMat {
    uint32_t group;
    int32_t diluent;
    float density, density_solid, viscosity;
    uint32_t rheology, temp_model;
    float temp_b, temp_c, temp_ref;
    float tension, contact_angle, mix_rate, grain, load;
    float heat_capacity, conductivity, expansion;
    float melt_lo, melt_hi, latent, emissivity, boil, latent_vap;
    float freeze_shift, spawn_temp;
    float shear_modulus, susceptibility, skin, friction;
    float self_heat, volatility;
    int32_t react_with;
    float react_rate;
    float fume;
    float yield_stress, flow_index, shear_time, visc_ratio;
    float saturation;
    float relax_time;
} OMat;

#define O_MAX_MATERIALS 96
#define O_MAX_CURRENTS 16

#define O_MAX_MAGNETS 8

/* Magnet (src/sim/params.rs:1082-1087) */
typedef struct OMagnet {
    float pos[2], radius, strength, dir[2];
} OMagnet;

/* Current (src/sim/params.rs:1113-1121) */
typedef struct OCurrent {
    float pos[2], radius, vel[2], rate;
} OCurrent;
#define O_GROUPS 4

/* The SimParams fields the substep reads (src/sim/params.rs:149-375). */
typedef struct OSimParams {
    float cell_size, gravity;
    float pair_tension[O_GROUPS][O_GROUPS];
    float ambient_temp, heat_rate, air_cooling, contact_heat, eddy_heat;
    uint32_t evaporation;
    float rigid_viscosity, heat_power;
    uint32_t steam;
    float droplet_cells, cfl;
    uint32_t advection_order;
    float dt_max, fixed_hz, pressure_tol;
    uint32_t pressure_max_iters;
    float correction_tol, viscosity_tol;
    uint32_t viscosity_max_iters;
    float implicit_viscosity_min;
    uint32_t viscous_projection, viscous_warm, viscosity_warm, viscosity_precond;
    uint32_t viscosity_mg_levels, viscosity_mg_sweeps;
    float spray_cfl, speed_cap, correction_time, correction_max, correction_deadband;
    float correction_step_max, crowd_jitter, tool_crowd_max, apic_clamp, curvature_max;
    uint32_t slip_cap, sealed_vent;
    OMat mat[O_MAX_MATERIALS];
    float magnet_demag;
    float elastic_stress_max, elastic_step_max;
    uint32_t rigid_contact;
    float rigid_friction;
    float iters_margin;   /* params.rs:284: the recorded iterations' margin */
} OSimParams;

/* ToolState (src/sim/params.rs:1141-1213). */
typedef struct OTool {
    float pos[2], vel[2], radius;
    int32_t mode;
    float strength;
} OTool;

/* Shapes of a scene (src/scene.rs:10-23); kind 0 circle, 1 box. temp < -1e8: insulating. */
typedef struct OShape {
    int32_t kind;
    float c[2], half[2], r, angle;
    float temp;
} OShape;

typedef struct OStats {
    uint64_t substeps;
    float sim_time, dt, dt_prev;
    uint32_t p_iters[2], p_done[2], p2_iters, v_iters, v_done;
    uint32_t p_it_max, p_unconv, v_it_max, v_unconv, p2_it_max, p2_unconv, solves;
    float p_res_max, v_res_max;
    float p_rr[2], p_bb[2], v_rr, v_r0;
    float umax_grid, umax_part;
    uint32_t n_slots, caps, acc_stride, thermal, viscosity_mode, levels, tail;
} OStats;

typedef struct OSim OSim;

/* Defaults of SimParams::default() with the built-in rows the configs use
 * (water, honey, oil; src/sim/presets.rs:37-117); other rows hold MatProps::default(). */
void oparams_default(OSimParams* p);

/* Scene::rasterize (src/scene.rs:215-310). Outputs: sdf (w+1)(h+1); solid 4 floats per
 * cell; region per cell; temp per cell (may be NULL). Returns 1 if any shape is held at a
 * temperature (temp filled), else 0. */
int oscene_rasterize(int w, int h, int nshapes, const OShape* shapes, float* sdf,
                     float* solid4, uint32_t* region, float* temp);
/* Scene::sdf at a point (src/scene.rs:195-198). */
float oscene_sdf(int w, int h, int nshapes, const OShape* shapes, float x, float y);

/* maps::fill_rect (src/maps.rs:466-492): appends to out[n0..]; returns the new count.
 * Particles are as Particle::new makes them (s = SPAWN_S, t = SPAWN_TEMP). */
uint32_t ofill_rect(int w, int h, int nshapes, const OShape* shapes, const float rect[4],
                    uint32_t material, OParticle* out, uint32_t n0, uint32_t cap);

OSim* osim_create(int w, int h, uint32_t capacity, const OSimParams* p);
void osim_destroy(OSim* s);
int osim_set_params(OSim* s, const OSimParams* p);
int osim_set_currents(OSim* s, const OCurrent* c, uint32_t n);
int osim_set_magnets(OSim* s, const OMagnet* m, uint32_t n);
int osim_set_solids(OSim* s, const float* sdf, const float* solid4, const uint32_t* region,
                    const float* temp);
/* FluidSim::reset (src/sim/mod.rs:1981-2002): ids, settle_spawn, the tank's rows.
 * Returns 0, or a negative code if the tank needs a capability the oracle lacks. */
int osim_reset(OSim* s, const OParticle* p, uint32_t n);
/* FluidSim::spawn (src/sim/mod.rs:2024-2046): queues particles for the next osim_step (ids
 * follow the last given, settle_spawn, KIND_FRESH; at most 32768 queued). Returns how many
 * were queued: 0 when their materials do not fit the tank; a negative code as osim_reset. */
int osim_spawn(OSim* s, const OParticle* p, uint32_t n);
/* FluidSim::cell_counts (src/sim/mod.rs:3350-3387) with count.comp: live particles per cell
 * of the window [lo, hi) row by row, queued ones included. out NULL: returns the cell count
 * only. Returns -1 for a window outside the grid or cap too small. */
long osim_cell_counts(const OSim* s, const int lo[2], const int hi[2], uint32_t* out, size_t cap);
/* FluidSim::record (src/sim/mod.rs:2400-2562): `substeps` substeps covering `target`. */
int osim_step(OSim* s, uint32_t substeps, float target, const OTool* tool);
/* Reorders particles now by the stable counting sort (sort.comp, stable by slot). */
void osim_sort(OSim* s);
uint32_t osim_particles(const OSim* s, OParticle* out, uint32_t cap);
/* Copies a named field (see sprout_oracle.c: field table). Returns bytes, or -1. */
long osim_field(const OSim* s, const char* name, void* out, size_t cap);
/* cell_optics.comp, light.comp, optics_blur.comp on the current grid (mod.rs:1626-1660):
 * then sss.comp and glow.comp: optics = 96 rows of material.rs GpuOptics (240 bytes each);
 * raw 20 and smooth 24 layers of W x H RGBA16F texels (four IEEE half words), layer-major;
 * ga, gb the glow field's two half-resolution images. */
long osim_render(const OSim* s, const void* optics, float inv_speed, int sss_iters, uint16_t* raw, uint16_t* smooth,
                 uint16_t* ga, uint16_t* gb);
/* flow_map.comp over the grid from copy `src` of `flow` (4 layers) into the other copy. */
/* look.comp over the slots (the oracle keeps the state; its sort moves it), and its state. */
long osim_look(OSim* s, const void* optics, float dt, uint32_t* list, uint32_t cap);
long osim_look_state(const OSim* s, uint32_t* out, size_t cap);
/* spray.comp over the pool the oracle keeps (smooth: osim_render's smoothed layers). */
long osim_spray(OSim* s, const uint16_t* smooth, const void* optics, float dt, float amount);
long osim_spray_state(const OSim* s, void* pool, uint32_t* stack, uint32_t* stack1, uint32_t* list, uint32_t* counts,
                      uint32_t state[8]);
void osim_set_dust(OSim* s, int has_dust);
/* FluidSim::recorded_iters: the recorded iteration counts (first solve, second, viscosity). */
void osim_recorded_iters(const OSim* s, uint32_t out[3]);
long osim_flow_map(const OSim* s, const uint16_t* smooth, uint16_t* flow, float dt, float now, uint32_t src);
void osim_stats(const OSim* s, OStats* out);
/* Test hook: the implicit viscosity's assembled level-0 matrix and its matrix-free operator
 * applied to x (2 floats per cell) on the unknown faces; returns the number of unknowns. */
long osim_visc_operator(OSim* s, const float* x, float* y_mg, float* y_free);
/* Test hook: the assembled viscosity matrix of multigrid level l applied to x. */
long osim_vmg_apply(OSim* s, int l, const float* x, float* y);
/* Threads the oracle uses (OpenMP); 1 = sequential. */
void osim_set_threads(int n);

/* exp restated from the mathematics (Cody-Waite reduction, degree-7 Taylor), the same
 * arithmetic the device code uses, so both sides round identically. */
float o_expf(float x);
float o_logf(float x);
float o_powf(float x, float y);

#ifdef __cplusplus
}
#endif
#endif

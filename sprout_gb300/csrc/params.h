// Host-side parameters of the engine: SimParams / MatProps and their named table
// (src/sim/params.rs:149-996, src/sim/material.rs:160-440), the tank's accumulator layout
// (Tank::layout, src/sim/mod.rs:271-329) and the conversion to grid units
// (gpu_materials / gpu_params, src/sim/mod.rs:2179-2339).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "device_types.h"

namespace sprout {

constexpr int kMaxMaterials = 96;
constexpr int kBuiltinCount = 59;
constexpr float kWaterDensity = 998.0f;
constexpr float kWaterHeat = 998.0f * 4182.0f;
constexpr float kStefanBoltzmann = 5.670374e-8f;
constexpr float kTRef = 20.0f;

// MatProps (material.rs:160-340): every field the named table reaches.
struct MatProps {
    uint32_t group = 0;
    int32_t diluent = -1;
    float density = 998.0f, density_solid = 0.0f, viscosity = 1.0e-6f;
    uint32_t rheology = 0;
    float yield_stress = 0.0f, flow_index = 1.0f, shear_time = 1.0f, visc_ratio = 1.0f;
    uint32_t temp_model = 0;
    float temp_b = 0.0f, temp_c = 0.0f, temp_ref = kTRef;
    float tension = 0.072f, contact_angle = 90.0f;
    float mix_rate = 0.0f, grain = 0.0f, load = 1.0f;
    float heat_capacity = 4182.0f, conductivity = 0.6f, expansion = 4.0e-4f;
    float melt_lo = -1.0e9f, melt_hi = -1.0e9f, latent = 0.0f, emissivity = 0.9f;
    float boil = 1.0e9f, latent_vap = 0.0f;
    int32_t residue = -1;
    float residue_share = 0.0f, freeze_shift = 0.0f, spawn_temp = kTRef;
    float shear_modulus = 0.0f, relax_time = 0.0f, susceptibility = 0.0f, saturation = 0.05f;
    float skin = 0.0f;
    float opacity = 0.0f, metal = 0.0f, gloss = 0.3f, foam = 0.0f, solids = 0.0f;
    float cloud = 0.0f, cloud_size = 1.0e-6f, cloud_ior = 1.5f, cloud_shape = 1.0f;
    float dust = 0.0f, dust_size = 3.0e-4f, dust_density = 2650.0f, dust_shape = 1.0f, dust_reflect = 0.05f;
    float self_heat = 0.0f, volatility = 0.0f, friction = 0.0f;
    int32_t react_with = -1, react_into = -1;
    float react_rate = 0.0f, react_heat = 0.0f, froth = 0.0f, fizz = 0.0f, fume = 0.0f;
    float luminous = 0.0f, glow_shear = 0.0f, thermo_lo = 0.0f, thermo_hi = 0.0f, ior = 1.33f;
    // colours (sRGB, as material.rs holds them): dissolved, frozen, at thermo_hi, of the fine
    // particles, of the specks, of its own light (material.rs:385-416)
    float color[3] = {0.17f, 0.52f, 0.94f}, color_solid[3] = {0.8f, 0.9f, 1.0f};
    float color_hot[3] = {0.95f, 0.35f, 0.45f}, cloud_color[3] = {0.95f, 0.95f, 0.95f};
    float dust_color[3] = {0.80f, 0.75f, 0.65f}, glow_color[3] = {0.4f, 1.0f, 0.5f};

    bool freezes() const { return melt_hi > -273.0f; }
    float temp_factor_ln(float t) const;
    float viscosity_at(float t) const;
};

// SimParams (params.rs:149-375).
struct SimParams {
    float cell_size = 0.01f, gravity = 9.81f;
    MatProps mat[kMaxMaterials];
    uint32_t mat_count = kBuiltinCount;
    float pair_tension[4][4] = {};
    float ambient_temp = kTRef, heat_rate = 1.0f, air_cooling = 10.0f, contact_heat = 3000.0f;
    float eddy_heat = 0.17f;
    uint32_t evaporation = 1;
    float rigid_viscosity = 1.0f;
    uint32_t rigid_contact = 1;
    float rigid_friction = 0.6f, heat_power = 300.0f, magnet_demag = 0.0f;
    uint32_t steam = 1;
    float steam_boil = 0.02f, steam_condense = 0.005f, steam_mixing = 1.0f;
    float steam_rise = 0.4f, steam_life = 2.0f, steam_swirl = 0.1f, steam_eddy = 0.2f;
    float bubbles = 1.0f, drying = 100.0f;
    uint32_t sss_iters = 4;
    float droplet_cells = 1.0f, cfl = 4.0f;
    uint32_t advection_order = 2;
    float dt_max = 1.0f / 80.0f, fixed_hz = 0.0f, pressure_tol = 1e-4f;
    uint32_t pressure_max_iters = 60;
    float iters_margin = 0.25f, correction_tol = 1e-2f, viscosity_tol = 1e-3f;
    uint32_t viscosity_max_iters = 200;
    float implicit_viscosity_min = 1e-3f;
    uint32_t viscous_projection = 1, viscous_warm = 1, viscosity_warm = 1, viscosity_precond = 1;
    uint32_t viscosity_mg_levels = 1, viscosity_mg_sweeps = 2;
    float spray_cfl = 4.0f, speed_cap = 1.0f;
    float correction_time = (1.0f / 240.0f) / 0.693147182f;
    float correction_max = 0.5f, correction_deadband = 0.25f, correction_step_max = 0.5f;
    float crowd_jitter = 0.5f, tool_crowd_max = 2.0f, apic_clamp = 1.0f, curvature_max = 0.5f;
    uint32_t slip_cap = 1, sealed_vent = 1;
    float min_substep_share = 0.02f, elastic_stress_max = 10.0f, elastic_step_max = 0.25f;

    SimParams();
    // SimParams::set (params.rs:986-996): false for an unknown name or NaN.
    bool set(const std::string& key, float v);
    bool get(const std::string& key, float* v) const;

    float tension_cells(float sigma) const { return sigma / (kWaterDensity * cell_size * cell_size * cell_size); }
    float g_cells() const { return gravity / cell_size; }
    float speed_cap_cells(uint32_t height) const;
    float particle_heat_vol(int row) const;
    float dt_capillary(const std::vector<int>& rows) const;
    float dt_thermal(const std::vector<int>& rows) const;
    // Longest substep that keeps elastic waves within half a cell (params.rs:947-960).
    float dt_elastic(const std::vector<int>& rows) const;
    float enthalpy_temp(int row, float s, float t) const;
    // A custom liquid's diluent as the library resolves it (library.rs:318-330): -1 (none),
    // or another row that is a built-in without a diluent of its own or a custom liquid.
    // False (nothing changed) for a built-in row or a diluent the library would not take.
    bool set_diluent(int row, int diluent);
    // A custom liquid's phase group as the library reads it (library.rs:283-286): 0 aqueous,
    // 1 oil-like, 2 metal, 3 silicate. False (nothing changed) for a built-in row or another value.
    bool set_group(int row, int group);
};

// Current (params.rs:1113-1121): a zone that drives the liquid in it towards `vel` at `rate`
// (1/s), or removes it at -rate when negative (a drain).
struct Current {
    float pos[2], radius, vel[2], rate;
};

// Magnet (params.rs:1082-1087): a point dipole at pos (cells) of radius `radius`, field
// `strength` (T) on its axis at the rim, north pole along `dir`.
struct Magnet {
    float pos[2], radius, strength, dir[2];
};

// Tank (mod.rs:222-245).
struct Tank {
    std::vector<int> rows;
    std::vector<std::array3i> chan;
    int stride = 8, families = 0, primary = -1, chan_t = -1, chan_e = -1;
    uint32_t group_mask = 0;
    int chan_g[4] = {-1, -1, -1, -1};
    // Tank::layout (mod.rs:271-329). False if the rows do not fit.
    bool layout(const std::vector<int>& rows_in, const SimParams& p, bool thermal);
};

// The material table and parameters in grid units for the device.
void build_materials(const SimParams& p, const Tank& t, bool thermal, DevMat* out);
void build_params(const SimParams& p, const Tank& t, bool thermal, uint32_t caps, int W, int H,
                  uint32_t n_slots, float dt_limit, const ToolState* tool, DevParams* out,
                  const std::vector<Current>& currents = {}, const std::vector<Magnet>& magnets = {});

// The name of built-in row r (presets.rs BUILTINS keys), or "" past them.
const char* builtin_key(int r);

}  // namespace sprout

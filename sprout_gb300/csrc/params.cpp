// SimParams and its named table, the tank layout and the grid-unit tables.
// Restates src/sim/params.rs:386-996 (defaults, PARAMS, MAT_PARAMS, ALIASES, set/find,
// unit conversions, dt limits), src/sim/material.rs:343-507 (MatProps defaults, pair
// tensions) and src/sim/presets.rs:37-117 (water, honey, olive oil), and
// src/sim/mod.rs:271-329, 2179-2339 (Tank::layout, gpu_materials, gpu_params).
#include "params.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace sprout {

namespace {

const char* const kBuiltinKeys[kBuiltinCount] = {
    "water", "honey", "oil", "mud", "ink", "chocolate", "clay", "blood", "mercury", "lava",
    "glass", "milk", "slime", "ferrofluid", "brine", "wax", "oobleck", "gallium", "beer", "soap",
    "alcohol", "nitrogen", "acid", "lye", "glowfluid", "iron", "polish", "blank", "thick", "heavy",
    "light", "beady", "creeper", "putty", "paste", "thinner", "jammer", "magnetic", "glowing", "fizzy",
    "sudsy", "vanishing", "grainy", "warming", "setting", "mirror", "pearly", "glitter", "snowy", "mood",
    "dye", "silt", "parta", "partb", "ember", "sheen", "salt", "steam", "resin"};

enum class Kind { F32, U32, I32 };

// A global parameter: the field it writes (or a special writer), range, "off" value.
struct GParam {
    const char* key;
    float min, max;
    bool has_off;
    float off;
    bool integer;
    Kind kind;
    size_t offset;   // into SimParams; special < 0 handled by code
    int special;     // 0 none; 1..6 pair tensions; 7 honey mix rate
};

struct MParam {
    const char* key;
    float min, max;
    bool integer;
    Kind kind;
    size_t offset;   // into MatProps
};

#define GP(k, lo, hi, off, hasoff, integ, kind, field) {k, lo, hi, hasoff, off, integ, kind, offsetof(SimParams, field), 0}
#define GF(k, lo, hi, field) GP(k, lo, hi, 0.0f, false, false, Kind::F32, field)
#define GFO(k, lo, hi, field) GP(k, lo, hi, 0.0f, true, false, Kind::F32, field)
#define GU(k, lo, hi, field) GP(k, lo, hi, 0.0f, false, true, Kind::U32, field)
#define GUO(k, lo, hi, field) GP(k, lo, hi, 0.0f, true, true, Kind::U32, field)
#define GS(k, lo, hi, sp) {k, lo, hi, false, 0.0f, false, Kind::F32, 0, sp}

// PARAMS (params.rs:668-789), in the reference's order.
const GParam kParams[] = {
    GF("gravity", 0.0f, 30.0f, gravity),
    GF("cell_size", 5e-4f, 0.05f, cell_size),
    GF("ambient_temp", -50.0f, 200.0f, ambient_temp),
    GFO("heat_rate", 0.1f, 200.0f, heat_rate),
    GF("air_cooling", 0.0f, 500.0f, air_cooling),
    GFO("contact_heat", 10.0f, 20000.0f, contact_heat),
    GFO("eddy_heat", 0.05f, 0.4f, eddy_heat),
    GU("evaporation", 0.0f, 1.0f, evaporation),
    GF("rigid_viscosity", 0.05f, 50.0f, rigid_viscosity),
    GU("rigid_contact", 0.0f, 1.0f, rigid_contact),
    GFO("rigid_friction", 0.05f, 2.0f, rigid_friction),
    GF("heat_power", 10.0f, 5000.0f, heat_power),
    GF("magnet_demag", 0.0f, 1.0f, magnet_demag),
    GU("steam", 0.0f, 1.0f, steam),
    GF("steam_boil", 0.001f, 1.0f, steam_boil),
    GF("steam_condense", 0.0f, 1.0f, steam_condense),
    GF("steam_mixing", 0.1f, 1000.0f, steam_mixing),
    GF("steam_rise", 0.0f, 3.0f, steam_rise),
    GF("steam_life", 0.1f, 10.0f, steam_life),
    GF("steam_swirl", 0.0f, 2.0f, steam_swirl),
    GF("steam_eddy", 0.005f, 0.5f, steam_eddy),
    GFO("drying", 1.0f, 5000.0f, drying),
    GFO("bubbles", 0.1f, 4.0f, bubbles),
    GUO("sss_iters", 2.0f, 32.0f, sss_iters),
    GS("tension_oil_water", 0.0f, 0.1f, 1),
    GS("tension_metal_water", 0.0f, 0.75f, 2),
    GS("tension_metal_oil", 0.0f, 0.75f, 3),
    GS("tension_melt_water", 0.0f, 0.75f, 4),
    GS("tension_melt_oil", 0.0f, 0.75f, 5),
    GS("tension_melt_metal", 0.0f, 0.75f, 6),
    GS("mix_rate", 0.0f, 20.0f, 7),
    GF("droplet_cells", 0.1f, 4.0f, droplet_cells),
    GF("cfl", 0.5f, 6.0f, cfl),
    GU("advection_order", 1.0f, 2.0f, advection_order),
    GF("dt_max", 1e-3f, 1.0f / 60.0f, dt_max),
    GFO("fixed_hz", 30.0f, 4000.0f, fixed_hz),
    GF("pressure_tol", 1e-6f, 1e-2f, pressure_tol),
    GU("pressure_max_iters", 10.0f, 400.0f, pressure_max_iters),
    GF("iters_margin", 0.0f, 2.0f, iters_margin),
    GF("correction_tol", 1e-4f, 0.1f, correction_tol),
    GF("viscosity_tol", 1e-5f, 0.1f, viscosity_tol),
    GU("viscosity_max_iters", 20.0f, 1000.0f, viscosity_max_iters),
    GFO("implicit_viscosity_min", 1e-4f, 0.05f, implicit_viscosity_min),
    GU("viscous_projection", 0.0f, 1.0f, viscous_projection),
    GU("viscous_warm", 0.0f, 1.0f, viscous_warm),
    GU("viscosity_warm", 0.0f, 1.0f, viscosity_warm),
    GU("viscosity_precond", 0.0f, 1.0f, viscosity_precond),
    GU("viscosity_mg_levels", 1.0f, 6.0f, viscosity_mg_levels),
    GU("viscosity_mg_sweeps", 1.0f, 2.0f, viscosity_mg_sweeps),
    GFO("speed_cap", 1.0f, 4.0f, speed_cap),
    GF("spray_cfl", 1.0f, 8.0f, spray_cfl),
    GF("correction_time", 1e-3f, 0.1f, correction_time),
    GFO("correction_max", 0.05f, 1.0f, correction_max),
    GFO("correction_deadband", 0.05f, 0.5f, correction_deadband),
    GFO("correction_step_max", 0.25f, 2.0f, correction_step_max),
    GFO("crowd_jitter", 0.1f, 1.0f, crowd_jitter),
    GFO("tool_crowd_max", 1.25f, 8.0f, tool_crowd_max),
    GFO("apic_clamp", 1.0f, 4.0f, apic_clamp),
    GFO("curvature_max", 0.25f, 2.0f, curvature_max),
    GU("slip_cap", 0.0f, 1.0f, slip_cap),
    GU("sealed_vent", 0.0f, 1.0f, sealed_vent),
    GFO("elastic_stress_max", 5.0f, 500.0f, elastic_stress_max),
    GFO("elastic_step_max", 0.05f, 1.0f, elastic_step_max),
    GFO("min_substep_share", 0.005f, 0.2f, min_substep_share),
};

#define MF(k, lo, hi, field) {k, lo, hi, false, Kind::F32, offsetof(MatProps, field)}
#define MU(k, lo, hi, field) {k, lo, hi, true, Kind::U32, offsetof(MatProps, field)}

// MAT_PARAMS (params.rs:598-660).
const MParam kMatParams[] = {
    MF("density", 300.0f, 14000.0f, density),
    MF("viscosity", 1e-7f, 0.5f, viscosity),
    MF("tension", 0.0f, 0.75f, tension),
    MF("contact_angle", 0.0f, 180.0f, contact_angle),
    MF("mix_rate", 0.0f, 20.0f, mix_rate),
    MF("density_solid", 0.0f, 15000.0f, density_solid),
    MU("rheology", 0.0f, 3.0f, rheology),
    MF("yield_stress", 0.0f, 500.0f, yield_stress),
    MF("flow_index", 0.2f, 3.0f, flow_index),
    MF("shear_time", 1e-3f, 100.0f, shear_time),
    MF("visc_ratio", 1e-4f, 1e4f, visc_ratio),
    MU("temp_model", 0.0f, 2.0f, temp_model),
    MF("temp_b", 0.0f, 60000.0f, temp_b),
    MF("temp_c", 0.0f, 1500.0f, temp_c),
    MF("temp_ref", -50.0f, 1700.0f, temp_ref),
    MF("grain", 0.0f, 5e-3f, grain),
    MF("load", 0.02f, 1.0f, load),
    MF("heat_capacity", 100.0f, 6000.0f, heat_capacity),
    MF("conductivity", 0.01f, 100.0f, conductivity),
    MF("expansion", 0.0f, 0.005f, expansion),
    MF("melt_lo", -1e9f, 1700.0f, melt_lo),
    MF("melt_hi", -1e9f, 1700.0f, melt_hi),
    MF("latent", 0.0f, 1e6f, latent),
    MF("emissivity", 0.0f, 1.0f, emissivity),
    MF("boil", -270.0f, 1e9f, boil),
    MF("latent_vap", 0.0f, 1e7f, latent_vap),
    MF("residue_share", 0.0f, 1.0f, residue_share),
    MF("freeze_shift", -100.0f, 100.0f, freeze_shift),
    MF("spawn_temp", -270.0f, 1700.0f, spawn_temp),
    MF("shear_modulus", 0.0f, 2000.0f, shear_modulus),
    MF("relax_time", 0.0f, 30.0f, relax_time),
    MF("susceptibility", 0.0f, 20.0f, susceptibility),
    MF("saturation", 0.001f, 2.0f, saturation),
    MF("skin", 0.0f, 2.0f, skin),
    MF("opacity", 0.0f, 1.0f, opacity),
    MF("metal", 0.0f, 1.0f, metal),
    MF("gloss", 0.0f, 1.0f, gloss),
    MF("foam", 0.0f, 1.0f, foam),
    MF("self_heat", 0.0f, 5000.0f, self_heat),
    MF("volatility", 0.0f, 2.0f, volatility),
    MF("friction", 0.0f, 1.2f, friction),
    MF("react_rate", 0.0f, 30.0f, react_rate),
    MF("react_heat", -5e5f, 2e6f, react_heat),
    MF("froth", 0.0f, 300.0f, froth),
    MF("fizz", 0.0f, 1.0f, fizz),
    MF("fume", 0.0f, 1.0f, fume),
    MF("luminous", 0.0f, 2.0f, luminous),
    MF("glow_shear", 0.0f, 1.0f, glow_shear),
    MF("thermo_lo", -270.0f, 1700.0f, thermo_lo),
    MF("thermo_hi", -270.0f, 1700.0f, thermo_hi),
    MF("solids", 0.0f, 1.0f, solids),
    MF("cloud", 0.0f, 0.7f, cloud),
    MF("cloud_size", 5e-9f, 5e-5f, cloud_size),
    MF("cloud_ior", 1.0f, 3.0f, cloud_ior),
    MF("cloud_shape", 0.01f, 1.0f, cloud_shape),
    MF("dust", 0.0f, 0.3f, dust),
    MF("dust_size", 2e-5f, 4e-3f, dust_size),
    MF("dust_density", 10.0f, 20000.0f, dust_density),
    MF("dust_shape", 0.01f, 1.0f, dust_shape),
    MF("dust_reflect", 0.0f, 1.0f, dust_reflect),
    MF("ior", 1.0f, 2.5f, ior),
};

const std::pair<const char*, const char*> kAliases[] = {
    {"frozen_viscosity", "rigid_viscosity"}, {"diffuse", "mix_rate"}, {"droplet", "droplet_cells"},
    {"substep_hz", "fixed_hz"}, {"pressure_iters", "pressure_max_iters"},
    {"viscosity_iters", "viscosity_max_iters"}, {"density_tau", "correction_time"},
    {"density_k", "correction_max"}, {"kappa_max", "curvature_max"}};

const std::pair<const char*, const char*> kMatAliases[] = {{"nu", "viscosity"}, {"sigma", "tension"}, {"contact", "contact_angle"}};

// Rust's f32::round: half away from zero.
float round_away(float v) { return std::round(v); }

float clamp_param(float v, float lo, float hi, bool has_off, float off, bool integer) {
    if (has_off && v == off) return v;
    v = std::min(std::max(v, lo), hi);
    return integer ? round_away(v) : v;
}

void write_field(void* base, size_t offset, Kind kind, float v) {
    char* p = static_cast<char*>(base) + offset;
    if (kind == Kind::F32) std::memcpy(p, &v, 4);
    else if (kind == Kind::U32) { uint32_t u = v <= 0.0f ? 0u : (v >= 4294967295.0f ? 0xffffffffu : (uint32_t)v); std::memcpy(p, &u, 4); }
    else { int32_t i = (int32_t)v; std::memcpy(p, &i, 4); }
}

float read_field(const void* base, size_t offset, Kind kind) {
    const char* p = static_cast<const char*>(base) + offset;
    if (kind == Kind::F32) { float f; std::memcpy(&f, p, 4); return f; }
    if (kind == Kind::U32) { uint32_t u; std::memcpy(&u, p, 4); return (float)u; }
    int32_t i; std::memcpy(&i, p, 4); return (float)i;
}

int material_row(const std::string& name) {
    for (int i = 0; i < kBuiltinCount; i++)
        if (name == kBuiltinKeys[i]) return i;
    if (name.rfind("mat", 0) != 0 || name.size() <= 3) return -1;
    const std::string num = name.substr(3);
    for (char ch : num)
        if (ch < '0' || ch > '9') return -1;
    if (num.size() > 6) return -1;
    int r = std::stoi(num);
    return r < kMaxMaterials ? r : -1;
}

struct Found {
    const GParam* g = nullptr;
    const MParam* m = nullptr;
    int row = -1;
};

// Param::find (params.rs:517-536).
Found find(const std::string& key_in) {
    Found f;
    if (key_in == "sigma_oil") return f;
    std::string key = key_in;
    for (auto& a : kAliases)
        if (key == a.first) { key = a.second; break; }
    for (auto& p : kParams)
        if (key == p.key) { f.g = &p; return f; }
    std::string prop, mat;
    size_t dot = key.find('.');
    if (dot != std::string::npos) {
        mat = key.substr(0, dot);
        prop = key.substr(dot + 1);
    } else {
        const char* best = nullptr;
        size_t best_len = 0;
        auto consider = [&](const char* n) {
            size_t l = std::strlen(n);
            if (key.size() > l && key.compare(0, l, n) == 0 && key[l] == '_' && l > best_len) { best = n; best_len = l; }
        };
        for (auto& p : kMatParams) consider(p.key);
        for (auto& a : kMatAliases) consider(a.first);
        if (!best) return f;
        prop = best;
        mat = key.substr(best_len + 1);
    }
    for (auto& a : kMatAliases)
        if (prop == a.first) { prop = a.second; break; }
    int row = material_row(mat);
    if (row < 0) return f;
    for (auto& p : kMatParams)
        if (prop == p.key) { f.m = &p; f.row = row; return f; }
    return f;
}

}  // namespace

const char* builtin_key(int r) { return r >= 0 && r < kBuiltinCount ? kBuiltinKeys[r] : ""; }

float MatProps::temp_factor_ln(float t) const {
    float tk = std::max(t + 273.15f, 1.0f);
    float tref = temp_ref + 273.15f;
    float x = 0.0f;
    if (temp_model == 1) x = temp_b * (1.0f / tk - 1.0f / tref);
    else if (temp_model == 2) x = temp_b / std::max(tk - temp_c, 5.0f) - temp_b / std::max(tref - temp_c, 5.0f);
    return std::min(std::max(x, -30.0f), 30.0f);
}

float MatProps::viscosity_at(float t) const { return viscosity * std::exp(temp_factor_ln(t)); }

SimParams::SimParams() {
    auto set_pair = [&](int a, int b, float v) { pair_tension[a][b] = v; pair_tension[b][a] = v; };
    set_pair(0, 1, 0.025f);
    set_pair(0, 2, 0.375f);
    set_pair(1, 2, 0.36f);
    set_pair(0, 3, 0.2f);
    set_pair(1, 3, 0.2f);
    set_pair(2, 3, 0.4f);
    // The built-in liquids (presets.rs: BUILTINS): what differs from MatProps::default().
#define BUILTIN_P(row, field, v) mat[row].field = v;
#define BUILTIN_O(row, field, v) mat[row].field = v;
#include "builtin_rows.inc"
#undef BUILTIN_P
#undef BUILTIN_O
#define BUILTIN_C(row, field, r, g, b) do { mat[row].field[0] = r; mat[row].field[1] = g; mat[row].field[2] = b; } while (0);
#include "builtin_colors.inc"
#undef BUILTIN_C
}

bool SimParams::set_diluent(int row, int diluent) {
    if (row < kBuiltinCount || row >= kMaxMaterials) return false;
    if (diluent == -1) {
        mat[row].diluent = -1;
        return true;
    }
    if (diluent < 0 || diluent >= kMaxMaterials || diluent == row) return false;
    if (diluent < kBuiltinCount && mat[diluent].diluent >= 0) return false;
    mat[row].diluent = diluent;
    return true;
}

bool SimParams::set_group(int row, int group) {
    if (row < kBuiltinCount || row >= kMaxMaterials || group < 0 || group > 3) return false;
    mat[row].group = (uint32_t)group;
    return true;
}

bool SimParams::set(const std::string& key, float v) {
    Found f = find(key);
    if (!f.g && !f.m) return false;
    if (std::isnan(v)) return false;
    if (f.g) {
        const GParam& p = *f.g;
        float c = clamp_param(v, p.min, p.max, p.has_off, p.off, p.integer);
        static const int kPair[7][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 3}, {2, 3}};
        if (p.special >= 1 && p.special <= 6) {
            pair_tension[kPair[p.special][0]][kPair[p.special][1]] = c;
            pair_tension[kPair[p.special][1]][kPair[p.special][0]] = c;
        } else if (p.special == 7) {
            mat[1].mix_rate = c;
        } else {
            write_field(this, p.offset, p.kind, c);
        }
        return true;
    }
    const MParam& p = *f.m;
    float c = clamp_param(v, p.min, p.max, false, 0.0f, p.integer);
    write_field(&mat[f.row], p.offset, p.kind, c);
    // A custom row in use extends the live table, as loading a custom liquid does
    // (library.rs:134).
    if (f.row >= (int)mat_count) mat_count = (uint32_t)f.row + 1;
    return true;
}

bool SimParams::get(const std::string& key, float* v) const {
    Found f = find(key);
    if (f.g) {
        static const int kPair[7][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 3}, {2, 3}};
        if (f.g->special >= 1 && f.g->special <= 6) *v = pair_tension[kPair[f.g->special][0]][kPair[f.g->special][1]];
        else if (f.g->special == 7) *v = mat[1].mix_rate;
        else *v = read_field(this, f.g->offset, f.g->kind);
        return true;
    }
    if (f.m) {
        *v = read_field(&mat[f.row], f.m->offset, f.m->kind);
        return true;
    }
    return false;
}

float SimParams::speed_cap_cells(uint32_t height) const {
    float g = g_cells();
    if (speed_cap > 0.0f && g > 0.0f) return speed_cap * std::sqrt(2.0f * g * (float)height);
    return 1e30f;
}

float SimParams::particle_heat_vol(int row) const {
    int r = row == 57 ? 0 : row;
    return mat[r].density * mat[r].heat_capacity;
}

float SimParams::dt_capillary(const std::vector<int>& rows) const {
    float worst = 0.0f;
    for (int i : rows) {
        if (i == 57) continue;
        const MatProps& m = mat[i];
        worst = std::max(worst, tension_cells(m.tension) / (m.density / kWaterDensity));
        for (int j : rows) {
            if (j == 57) continue;
            const MatProps& n = mat[j];
            if (n.group != m.group) {
                float sigma = tension_cells(pair_tension[m.group][n.group]);
                worst = std::max(worst, sigma / (std::min(m.density, n.density) / kWaterDensity));
            }
        }
    }
    if (worst <= 0.0f) return INFINITY;
    return 0.5f * std::sqrt(1.0f / (2.0f * 3.14159274f * worst));
}

float SimParams::dt_elastic(const std::vector<int>& rows) const {
    const float stiff = 1.0f + (elastic_stress_max > 0.0f ? elastic_stress_max : 50.0f);
    float m = INFINITY;
    for (int i : rows)
        if (mat[i].shear_modulus > 0.0f)
            m = std::min(m, 0.5f * cell_size / std::sqrt(stiff * mat[i].shear_modulus / mat[i].density));
    return m;
}

float SimParams::dt_thermal(const std::vector<int>& rows) const {
    if (heat_rate <= 0.0f) return INFINITY;
    float dx2 = cell_size * cell_size;
    float m = INFINITY;
    for (int i : rows) m = std::min(m, 0.2f * dx2 * particle_heat_vol(i) / std::max(mat[i].conductivity, 1e-6f) / heat_rate);
    return m;
}

// enthalpy_temp / melting (params.rs:830-860).
float SimParams::enthalpy_temp(int row, float s, float t) const {
    const MatProps& own = mat[row];
    auto lat = [](const MatProps& d) { return d.freezes() ? d.latent / d.heat_capacity : 0.0f; };
    float lo, hi, l;
    if (own.diluent < 0) {
        lo = own.melt_lo;
        hi = std::max(own.melt_hi, own.melt_lo + 0.25f);
        l = lat(own);
    } else {
        const MatProps& d = mat[own.diluent];
        float shift = own.freeze_shift * s;
        float cd = d.density * d.heat_capacity, co = own.density * own.heat_capacity;
        float c = cd + (co - cd) * s;
        l = (cd * lat(d) + (co * own.latent / own.heat_capacity - cd * lat(d)) * s) / c;
        lo = d.melt_lo + shift;
        hi = std::max(d.melt_hi, d.melt_lo + 0.25f) + shift;
    }
    if (lo < -273.0f || t >= hi) return t;
    if (t <= lo) return t - l;
    float fr = (t - lo) / std::max(hi - lo, 1e-3f);
    return (lo - l) + fr * (hi - lo + l);
}

bool Tank::layout(const std::vector<int>& rows_in, const SimParams& p, bool thermal) {
    if ((int)rows_in.size() > kMaxPresent) return false;
    int next = 5;
    uint32_t gm = 0;
    int prim = -1;
    for (size_t k = 0; k < rows_in.size(); k++)
        if (p.mat[rows_in[k]].diluent == rows_in[0]) { prim = (int)k; break; }
    int fams = prim >= 0 ? 1 : 0;
    std::vector<std::array3i> ch;
    for (size_t k = 0; k < rows_in.size(); k++) {
        const MatProps& m = p.mat[rows_in[k]];
        gm |= 1u << std::min<uint32_t>(m.group, 3u);
        std::array3i c = {-1, -1, -1};
        if (k > 0 && (int)k != prim) c[0] = next++;
        if (m.diluent >= 0) {
            c[1] = next++;
            c[2] = (int)k == prim ? 0 : fams++;
        }
        ch.push_back(c);
    }
    int ct = thermal ? next : -1;
    next += thermal ? 1 : 0;
    int cg[4] = {-1, -1, -1, -1};
    if (thermal) {
        bool first = true;
        for (int g = 0; g < 4; g++)
            if (gm & (1u << g)) {
                if (!first) cg[g] = next++;
                first = false;
            }
    }
    // three stress channels after the temperature ones when an elastic material is in (mod.rs:316-317)
    bool elastic = false;
    for (int r : rows_in) elastic |= p.mat[r].shear_modulus > 0.0f;
    const int ce = elastic ? next : -1;
    next += elastic ? 3 : 0;
    if (next > 32) return false;
    rows = rows_in;
    chan = ch;
    stride = ((std::max(next, 8) + 3) / 4) * 4;
    families = fams;
    group_mask = gm;
    primary = prim >= 0 ? rows_in[prim] : -1;
    chan_t = ct;
    chan_e = ce;
    for (int g = 0; g < 4; g++) chan_g[g] = cg[g];
    return true;
}

void build_materials(const SimParams& p, const Tank& t, bool thermal, DevMat* out) {
    float dx = p.cell_size;
    for (int r = 0; r < kMaxMaterials; r++) {
        const MatProps& m = p.mat[r];
        DevMat& g = out[r];
        std::memset(&g, 0, sizeof g);
        std::array3i chan = {-1, -1, -1};
        for (size_t k = 0; k < t.rows.size(); k++)
            if (t.rows[k] == r) chan = t.chan[k];
        float ang = m.contact_angle * (3.14159274f / 180.0f);
        float sn = std::sin(ang), cs = std::cos(ang);
        float solid = m.density_solid > 0.0f ? m.density_solid : m.density;
        float cvol = p.particle_heat_vol(r);
        float ln_nu = std::log(std::max(m.viscosity / (dx * dx), 1e-8f));
        float rho = m.density;
        if (!thermal) {
            ln_nu += m.temp_factor_ln(p.ambient_temp);
            rho *= std::min(std::max(1.0f - m.expansion * (p.ambient_temp - m.temp_ref), 0.7f), 1.3f);
            if (m.freezes() && m.diluent < 0 && p.ambient_temp < m.melt_hi) {
                float fs = std::min(std::max((m.melt_hi - p.ambient_temp) / std::max(m.melt_hi - m.melt_lo, 1e-3f), 0.0f), 1.0f);
                float frozen = std::max(std::log(p.rigid_viscosity / (dx * dx)), ln_nu);
                ln_nu += (frozen - ln_nu) * fs;
                rho += (solid - rho) * fs;
            }
        }
        g.ia[0] = (int)std::min<uint32_t>(m.group, 3u);
        g.ia[1] = m.diluent;
        g.ia[2] = chan[0];
        g.ia[3] = chan[1];
        g.ib[0] = chan[2];
        g.ib[1] = (int)m.rheology;
        g.ib[2] = (int)m.temp_model;
        g.ib[3] = m.residue;
        g.a[0] = rho / kWaterDensity;
        g.a[1] = ln_nu;
        g.a[2] = p.tension_cells(m.tension);
        g.a[3] = m.mix_rate;
        g.b[0] = cs;
        g.b[1] = sn;
        g.b[2] = m.grain / dx;
        g.b[3] = solid / kWaterDensity;
        g.temp[0] = m.temp_b;
        g.temp[1] = m.temp_c;
        g.temp[2] = m.temp_ref + 273.15f;
        g.temp[3] = p.tension_cells(m.skin);
        g.th[0] = cvol / kWaterHeat;
        g.th[1] = m.conductivity / (kWaterHeat * dx * dx);
        g.th[2] = std::max(m.melt_lo, -1.0e9f);
        g.th[3] = std::max(std::max(m.melt_hi, m.melt_lo + 0.25f), -1.0e9f);
        g.th2[0] = (m.freezes() || m.diluent >= 0) ? m.latent / m.heat_capacity : 0.0f;
        g.th2[1] = m.emissivity;
        g.th2[2] = m.boil;
        g.th2[3] = m.latent_vap / m.heat_capacity;
        g.misc[0] = m.freeze_shift;
        g.misc[1] = m.load;
        g.misc[2] = 1.0f;
        g.misc[3] = m.expansion;
        g.rx[0] = m.react_rate;
        g.rx[1] = m.react_heat / m.heat_capacity;
        g.rx[2] = m.self_heat / m.heat_capacity;
        g.rx[3] = m.volatility;
        g.rheo[0] = m.yield_stress / (kWaterDensity * dx * dx);   // Pa over water's density, cells^2/s^2
        g.rheo[1] = m.flow_index;
        g.rheo[2] = m.shear_time;
        g.rheo[3] = m.visc_ratio;
        g.gr[0] = m.friction;
        g.gr[1] = m.fume;
        g.gr[2] = m.fizz;
        g.gr[3] = 0.0f;
        g.el[0] = m.shear_modulus / (kWaterDensity * dx * dx);
        g.el[1] = m.relax_time;
        g.el[2] = m.susceptibility;
        g.el[3] = m.residue_share;
    }
}

static float tool_speed(const ToolState* t) {
    if (!t) return 0.0f;
    switch (t->mode) {
    case 1: return std::hypot(t->vel[0], t->vel[1]) + 4.0f * t->radius;
    case 3:
    case 4: return std::hypot(t->vel[0], t->vel[1]);
    case 7: return std::fabs(t->vel[0]) + 2.0f * t->radius;
    default: return 0.0f;
    }
}

void build_params(const SimParams& p, const Tank& t, bool thermal, uint32_t caps, int W, int H, uint32_t n_slots,
                  float dt_limit, const ToolState* tool, DevParams* P, const std::vector<Current>& currents,
                  const std::vector<Magnet>& magnets) {
    std::memset(P, 0, sizeof *P);
    float dx = p.cell_size;
    P->grid[0] = W;
    P->grid[1] = H;
    P->n_slots = n_slots;
    P->dt_fixed = p.fixed_hz > 0.0f ? 1.0f / p.fixed_hz : 0.0f;
    P->gravity = p.g_cells();
    P->inv_ppc = 0.25f;
    P->apic_clamp = p.apic_clamp;
    for (int a = 0; a < 4; a++)
        for (int b = 0; b < 4; b++) P->pair[a][b] = p.tension_cells(p.pair_tension[a][b]);
    P->misc[0] = p.curvature_max;
    P->misc[1] = (float)p.sealed_vent;
    P->misc[2] = p.cell_size;
    P->misc[3] = p.rigid_contact != 0 ? p.rigid_friction : -1.0f;   // mod.rs:2280
    P->n_present = (int)t.rows.size();
    P->acc_stride = std::max(t.stride, 8);
    P->n_fam = t.families;
    P->group_mask = t.group_mask;
    P->caps = caps;
    P->primary = t.rows.empty() ? -1 : t.primary;
    // group_sorts (common.glsl:590-602): a group past the first with two or more plain liquids
    // and no concentrate, nor any concentrate whose diluent is in it, sorts its materials
    P->sorts = 0u;
    for (int g = 1; g < 4; g++) {
        int n = 0;
        bool no = false;
        for (int r : t.rows) {
            const MatProps& m = p.mat[r];
            const int mg = (int)std::min<uint32_t>(m.group, 3u);
            if (m.diluent >= 0 && (int)std::min<uint32_t>(p.mat[m.diluent].group, 3u) == g) { no = true; break; }
            if (mg != g) continue;
            if (m.diluent >= 0) { no = true; break; }
            n++;
        }
        if (!no && n >= 2) P->sorts |= 1u << g;
    }
    for (int j = 0; j < kMaxPresent; j++) P->fams[j][0] = P->fams[j][1] = -1;
    for (size_t k = 0; k < t.rows.size(); k++)
        if (t.chan[k][2] >= 0) {
            P->fams[t.chan[k][2]][0] = t.rows[k];
            P->fams[t.chan[k][2]][1] = p.mat[t.rows[k]].diluent;
        }
    uint32_t gh = 0;
    for (int g = 0; g < 4; g++) gh += ((uint32_t)(t.chan_g[g] + 1) & 255u) << (8 * g);
    P->group_heat = gh;
    for (size_t k = 0; k < t.rows.size(); k++) P->present[k] = t.rows[k];
    P->heat[0] = p.ambient_temp;
    P->heat[1] = p.heat_rate;
    P->heat[2] = p.air_cooling / (kWaterHeat * dx);
    P->heat[3] = kStefanBoltzmann / (kWaterHeat * dx);
    P->heat2[0] = std::log(p.rigid_viscosity / (dx * dx));
    P->heat2[1] = p.heat_power;
    P->heat2[2] = (float)t.chan_t;
    P->heat2[3] = p.contact_heat / (kWaterHeat * dx);
    P->heat3[0] = std::max(p.eddy_heat, 0.0f);
    P->heat3[1] = p.evaporation ? 2.257e6f / 1005.0f : 0.0f;
    P->heat3[3] = std::min(std::max(p.magnet_demag, 0.0f), 1.0f);
    float gmax = 0.0f;   // mod.rs:2316-2321
    for (int r : t.rows) gmax = std::max(gmax, p.mat[r].shear_modulus);
    P->elastic[0] = (float)t.chan_e;
    P->elastic[1] = std::max(gmax, 1e-3f) / (kWaterDensity * dx * dx);
    P->elastic[2] = p.elastic_stress_max;
    P->elastic[3] = p.elastic_step_max;
    // the strongest susceptibility in the tank and its saturation (mod.rs:2264)
    float chi_max = 0.0f, sat = 0.05f;
    for (int r : t.rows)
        if (p.mat[r].susceptibility > chi_max) {
            chi_max = p.mat[r].susceptibility;
            sat = p.mat[r].saturation;
        }
    P->mag[0] = (float)magnets.size();
    P->mag[1] = std::max(chi_max, 1e-6f);
    P->mag[2] = sat;
    P->mag[3] = 1.0f / (kWaterDensity * dx * dx);
    for (size_t i = 0; i < magnets.size() && i < (size_t)kMaxMagnets; i++) {   // mod.rs:2258-2263
        const Magnet& m = magnets[i];
        P->magnet[i][0] = m.pos[0];
        P->magnet[i][1] = m.pos[1];
        P->magnet[i][2] = std::max(m.radius, 0.5f);
        P->magnet[i][3] = m.strength;
        P->magnet_dir[i][0] = m.dir[0];
        P->magnet_dir[i][1] = m.dir[1];
    }
    P->sep_tau = p.droplet_cells;
    P->cfl = p.cfl;
    P->tool_crowd_max = p.tool_crowd_max;
    P->density_k = p.correction_max;
    P->dt_max = dt_limit;
    P->crowd_jitter = p.crowd_jitter;
    P->ext_speed = tool_speed(tool);
    P->wall_margin = 0.1f;
    if (tool) {
        P->tool_pos[0] = tool->pos[0];
        P->tool_pos[1] = tool->pos[1];
        P->tool_vel[0] = tool->vel[0];
        P->tool_vel[1] = tool->vel[1];
        P->tool_radius = std::max(tool->radius, 0.01f);
        P->tool_mode = tool->mode;
        P->tool_strength = tool->strength;
    } else {
        P->tool_radius = 0.01f;
    }
    P->tol[0] = p.pressure_tol;
    P->tol[1] = p.correction_tol;
    P->tol[2] = p.viscosity_tol;
    P->tol[3] = p.correction_time;
    P->ext[0] = p.speed_cap_cells((uint32_t)H);
    P->ext[1] = (float)p.advection_order;
    P->ext[2] = p.spray_cfl;
    P->ext[3] = (float)currents.size();
    for (size_t i = 0; i < currents.size() && i < (size_t)kMaxCurrents; i++) {   // mod.rs:2265-2270
        const Current& c = currents[i];
        P->current_zone[i][0] = c.pos[0];
        P->current_zone[i][1] = c.pos[1];
        P->current_zone[i][2] = std::max(c.radius, 0.01f);
        P->current_zone[i][3] = c.rate;
        P->current_vel[i][0] = c.vel[0];
        P->current_vel[i][1] = c.vel[1];
    }
    P->corr[0] = p.correction_step_max;
    P->corr[1] = p.correction_deadband;
    P->corr[2] = (float)p.slip_cap;
    P->corr[3] = p.implicit_viscosity_min;
    P->pressure_max_iters = p.pressure_max_iters;
    P->thermal = thermal ? 1 : 0;
    P->viscosity_max_iters = p.viscosity_max_iters;
    P->visc_sweeps = (int)std::min<uint32_t>(std::max<uint32_t>(p.viscosity_mg_sweeps, 1u), 2u);
    P->visc_levels = (int)std::max<uint32_t>(p.viscosity_mg_levels, 1u);   // the host clamps to the tail
    P->viscosity_warm = p.viscosity_warm != 0 ? 1 : 0;
    P->viscous_warm = p.viscous_warm != 0 ? 1 : 0;
    P->viscous_projection = p.viscous_projection != 0 ? 1 : 0;
    P->viscosity_precond = p.viscosity_precond != 0 ? 1 : 0;
    P->iters_margin = std::max(p.iters_margin, 0.0f);
}

}  // namespace sprout

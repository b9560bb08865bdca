// The optics table of the render-side passes: material.rs's `optics_table` (material.rs:
// 551-980) and the helpers it calls, in the reference's single-precision arithmetic, from the
// live material table. One row per material row: what the liquid looks like in the form the
// cell passes blend (absorption and scattering per cell from its colours and fine particles,
// opacity, gloss, films, its own light, thermochromic colour, the specks it carries).
#include <algorithm>
#include <cmath>

#include "params.h"
#include "optics.h"

namespace sprout {

namespace {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kWavelengths[3] = {610.0e-9f, 550.0e-9f, 465.0e-9f};   // material.rs:622
constexpr float kLvBody = 16.0f;
constexpr float kDustDrawMax = 4.0f;
constexpr float kDustPacking = 0.6f;
constexpr float kFoamDrainWater = 0.02f;
constexpr float kKT = 1.380649e-23f * 293.15f;
constexpr float kMaxCoefficient = 2000.0f;
constexpr float kFilmUnit = 1.0e-4f;
constexpr float kEvapWater = 1.0e-7f;
constexpr float kCoatSpeed = 0.05f;
constexpr float kTwoThirds = 2.0f / 3.0f;
constexpr float kRadsPerDeg = kPi / 180.0f;

float clampf_(float v, float lo, float hi) { return std::min(std::max(v, lo), hi); }

void linear(const float c[3], float out[3]) {   // material.rs:603-606
    for (int k = 0; k < 3; k++) {
        const float v = c[k];
        out[k] = v <= 0.04045f ? v / 12.92f : std::pow((v + 0.055f) / 1.055f, 2.4f);
    }
}

float tint_depth(const MatProps& m) {   // material.rs:616-619
    const float clear = 1.0f - clampf_(m.opacity, 0.0f, 1.0f);
    return 0.5f + 30.0f * clear * clear;
}

// mean projected area over volume, mean chord, equal-volume diameter (material.rs:640-649)
void particle_shape(float d, float r, float* area_over_vol, float* chord, float* d_eq) {
    d = std::max(d, 1e-9f);
    if (r >= kTwoThirds) {
        *area_over_vol = 1.5f / d;
        *chord = d;
        *d_eq = d;
        return;
    }
    const float t = d * std::max(r, 0.005f);
    *area_over_vol = (0.5f * d + t) / (d * t);
    *chord = 1.5f * d * t / (0.5f * d + t);
    *d_eq = d * std::cbrt(1.5f * std::max(r, 0.005f));
}

float scattering_efficiency(float x_vol, float x_path, float m) {   // material.rs:655-665
    m = std::max(m, 1e-3f);
    const float k = (m * m - 1.0f) / (m * m + 2.0f);
    const float x2 = x_vol * x_vol;
    const float qr = 8.0f / 3.0f * (x2 * x2) * k * k;
    const float rho = 2.0f * x_path * std::fabs(m - 1.0f);
    const float qa = rho < 1e-2f ? 0.5f * rho * rho
                                 : 2.0f - 4.0f / rho * std::sin(rho) + 4.0f / (rho * rho) * (1.0f - std::cos(rho));
    if (qr <= 0.0f || qa <= 0.0f) return 0.0f;
    return 1.0f / (1.0f / qr + 1.0f / qa);
}

float asymmetry(float x, float m) {   // material.rs:670-673
    const float large = clampf_(1.0f - 0.6f * std::fabs(m - 1.0f), 0.3f, 0.98f);
    return large * x * x / (x * x + 2.5f);
}

void albedo_of(const float color[3], float out[3]) {   // material.rs:677-683
    float lin[3];
    linear(color, lin);
    for (int k = 0; k < 3; k++) {
        const float r = clampf_(lin[k], 1e-3f, 0.995f);
        const float q = (1.0f - r) / (1.0f + r);
        out[k] = std::max(1.0f - q * q, 1e-4f);
    }
}

float cloud_scattering(const MatProps& m, float cell, float s[3]) {   // material.rs:687-705
    s[0] = s[1] = s[2] = 0.0f;
    if (m.cloud <= 0.0f) return 0.0f;
    float a_v, chord, d_eq;
    particle_shape(m.cloud_size, m.cloud_shape, &a_v, &chord, &d_eq);
    const float n_med = std::max(m.ior, 1.0f);
    const float rel = m.cloud_ior / n_med;
    float g_sum = 0.0f;
    for (int c = 0; c < 3; c++) {
        const float k = kPi * n_med / kWavelengths[c];
        const float q = scattering_efficiency(k * d_eq, k * chord, rel);
        const float g = asymmetry(k * d_eq, rel);
        g_sum += g;
        s[c] = clampf_(m.cloud, 0.0f, 0.74f) * a_v * q * (1.0f - g) * cell;
    }
    return g_sum / 3.0f;
}

void coefficients(const MatProps& m, const float color[3], float cell, float a[3], float sc[3]) {   // material.rs:712-734
    const float depth = tint_depth(m);
    float lin[3], s[3], w[3];
    linear(color, lin);
    for (int c = 0; c < 3; c++) lin[c] = clampf_(lin[c], 1e-3f, 0.995f);
    cloud_scattering(m, cell, s);
    albedo_of(m.cloud_color, w);
    for (int c = 0; c < 3; c++) {
        a[c] = -std::log(lin[c]) / depth + s[c] * (1.0f - w[c]) / w[c];
        sc[c] = s[c];
    }
    if (m.metal > 0.0f) {
        float wm[3];
        albedo_of(color, wm);
        const float k = clampf_(m.metal, 0.0f, 1.0f);
        for (int c = 0; c < 3; c++) {
            const float sm = 6.0f;
            a[c] += k * (sm * (1.0f - wm[c]) / wm[c] - a[c]);
            sc[c] += k * (sm - sc[c]);
        }
    }
    for (int c = 0; c < 3; c++) {
        a[c] = std::min(a[c], kMaxCoefficient);
        sc[c] = std::min(sc[c], kMaxCoefficient);
    }
}

void packed(const float a[3], const float s[3], float out[4]) {
    out[0] = a[0];
    out[1] = a[1];
    out[2] = a[2];
    out[3] = (s[0] + s[1] + s[2]) / 3.0f;
}

float fullness(const MatProps& m) {   // material.rs:761-767
    auto ss = [](float x, float lo, float hi) {
        const float t = clampf_((x - lo) / (hi - lo), 0.0f, 1.0f);
        return t * t * (3.0f - 2.0f * t);
    };
    return std::max(ss(std::log10(std::max(m.viscosity, 1e-9f)), -5.3f, -2.7f), ss(m.contact_angle, 100.0f, 145.0f));
}

float volatile_share(const MatProps& m) {   // material.rs:780-785
    if (m.boil >= 1.0e8f && m.volatility <= 0.0f) return 0.0f;
    return clampf_(1.0f - m.solids - m.cloud - m.dust, 0.0f, 1.0f);
}

float vapour_pressure(float boil, float t) {   // material.rs:789-796
    if (boil >= 1.0e8f) return 0.0f;
    const float tb = boil + 273.15f;
    const float tk = std::max(t + 273.15f, 1.0f);
    return std::exp(clampf_(10.6f * (1.0f - tb / tk), -60.0f, 5.0f));
}

float evaporation(const MatProps& m, float t, float speed) {   // material.rs:801-806
    const float rel = vapour_pressure(m.boil, t) / std::max(vapour_pressure(100.0f, kTRef), 1e-12f);
    const float vol = (m.boil >= 1.0e8f && m.volatility > 0.0f) ? m.volatility * 50.0f : rel;
    return kEvapWater * vol * speed / kFilmUnit;
}

bool freezes_on_contact(const MatProps& m) { return m.freezes() && m.melt_lo > 300.0f; }

float wetting(const MatProps& m) {   // material.rs:816-822
    if (freezes_on_contact(m)) return 0.0f;
    const float w = 0.5f * (1.0f + std::cos(m.contact_angle * kRadsPerDeg));
    return clampf_((w - 0.15f) / 0.85f, 0.0f, 1.0f);
}

float coat_thickness(const MatProps& m, float gravity) {   // material.rs:828-838
    if (freezes_on_contact(m)) return 0.0f;
    const float sigma = std::max(m.tension, 1e-3f);
    const float rho = std::max(m.density, 1.0f);
    const float lc = std::sqrt(sigma / (rho * std::max(gravity, 0.1f)));
    const float ca = std::min(m.viscosity * rho * kCoatSpeed / sigma, 1.0f);
    const float wet = 0.5f * (1.0f + std::cos(m.contact_angle * kRadsPerDeg));
    return 0.94f * lc * std::pow(ca, kTwoThirds) * wet / kFilmUnit;
}

float dry_scatter(const MatProps& m) {   // material.rs:846-857
    const bool rigid = m.cloud_ior >= 1.5f;
    const float n = std::max(m.ior, 1.0f);
    auto gain = [&](float np) {
        const float g = (np - 1.0f) / std::max(std::fabs(np - n), 0.02f);
        return clampf_(g * g, 1.0f, 6.0f);
    };
    const float wr = m.dust + (rigid ? m.cloud : 0.0f);
    const float ws = rigid ? 0.0f : m.cloud;
    if (wr + ws <= 0.0f) return 1.0f;
    return (wr * gain(m.dust > 0.0f && !rigid ? 1.55f : std::max(m.cloud_ior, 1.55f)) + ws * 0.33f) / (wr + ws);
}

float iridescence(const MatProps& m, float pair, float cell) {   // material.rs:862-870
    if (m.group == 0 || m.group == 2) return 0.0f;   // aqueous, metal
    const float spread = 0.072f - m.tension - pair;
    float a[3], s[3];
    coefficients(m, m.color, cell, a, s);
    const float murk = (a[0] + a[1] + a[2]) / 3.0f + (s[0] + s[1] + s[2]) / 3.0f;
    return clampf_(spread / 0.01f, 0.0f, 1.0f) * clampf_(std::fabs(m.ior - 1.33f) / 0.1f, 0.0f, 1.0f) *
           (1.0f - clampf_(murk / 1.5f, 0.0f, 1.0f));
}

float crust(const MatProps& m) {   // material.rs:875-880
    if (!m.freezes()) return 0.0f;
    return clampf_((m.melt_lo - 400.0f) / 400.0f, 0.0f, 1.0f);
}

float mean_area_factor(float r) {   // material.rs:915-918
    if (r >= kTwoThirds) return 0.25f * kPi;
    return 0.25f * (0.5f * kPi + kPi * std::max(r, 0.005f));
}

float dust_specks(const MatProps& m, float cell, float per_out[4]) {   // material.rs:887-913
    per_out[0] = per_out[1] = per_out[2] = per_out[3] = 0.0f;
    if (m.dust <= 0.0f) return 0.0f;
    float a_v, chord, d_eq;
    particle_shape(m.dust_size, m.dust_shape, &a_v, &chord, &d_eq);
    const float phi = clampf_(m.dust, 0.0f, 0.6f);
    const float sigma = phi * a_v * 2.0f * cell;
    const float s_red = 0.5f * sigma;
    const float area = m.dust_size * m.dust_size * mean_area_factor(m.dust_shape) / (cell * cell);
    const float tau = sigma * kLvBody;
    const float n_vis = (1.0f - std::exp(-tau)) / std::max(area, 1e-9f);
    const float n = std::min(n_vis, kDustDrawMax);
    if (n <= 1e-6f) return 0.0f;
    const float undrawn = std::max(1.0f - n / n_vis, 0.0f);
    float w[3];
    albedo_of(m.dust_color, w);
    const float r0 = clampf_(m.dust_reflect, 0.0f, 1.0f);
    const float per = undrawn / n;
    for (int c = 0; c < 3; c++) {
        const float wc = r0 + (1.0f - r0) * w[c];
        per_out[c] = s_red * (1.0f - wc) / std::max(wc, 1e-4f) * per;
    }
    per_out[3] = s_red * per;
    return n;
}

}  // namespace

void optics_row(const SimParams& p, int r, DevOptics& o) {   // material.rs:921-978
    const MatProps& m = p.mat[r];
    const float cell = p.cell_size;
    float sl[3], a[3], s[3], ah[3], sh[3];
    linear(m.color_solid, sl);
    coefficients(m, m.color, cell, a, s);
    coefficients(m, m.color_hot, cell, ah, sh);
    const float mean = (s[0] + s[1] + s[2]) / 3.0f;
    float s_unused[3];
    const float g = cloud_scattering(m, cell, s_unused);
    float ratio[3] = {1.0f, 1.0f, 1.0f};
    if (mean > 1e-9f)
        for (int c = 0; c < 3; c++) ratio[c] = s[c] / mean;
    const float plate_k = std::max(1.0f - std::min(m.cloud_shape / kTwoThirds, 1.0f), 0.0f);
    const float am = (a[0] + a[1] + a[2]) / 3.0f;
    const float plate = m.cloud > 0.0f ? plate_k * (1.0f - std::exp(-4.0f * mean)) * mean / (mean + am + 1e-6f) : 0.0f;
    const float eta = std::max(m.viscosity * m.density, 1e-6f);
    const float dsz = std::max(m.cloud_size, 1e-9f);
    const float dr = plate_k > 0.0f ? 3.0f * kKT / (4.0f * eta * dsz * dsz * dsz) : 0.0f;
    const float ar = clampf_(m.cloud_shape, 0.005f, 1.0f);
    const float bretherton = (ar * ar - 1.0f) / (ar * ar + 1.0f);
    float per[4];
    const float n_draw = dust_specks(m, cell, per);
    float dl[3];
    linear(m.dust_color, dl);
    const float pack = m.dust > 0.0f ? n_draw * kDustPacking / std::max(m.dust, 1e-6f) : 0.0f;
    const float drain = kFoamDrainWater * eta / 1.0e-3f;
    const float vshare = volatile_share(m);
    const float evap = evaporation(m, p.ambient_temp, p.drying);
    const float coat = coat_thickness(m, p.gravity);
    const float dry_time = (vshare > 0.0f && evap > 0.0f) ? clampf_(std::max(coat, 0.2f) * vshare / evap, 0.2f, 600.0f) : 600.0f;
    packed(a, s, o.absorb);
    o.solid[0] = sl[0];
    o.solid[1] = sl[1];
    o.solid[2] = sl[2];
    o.solid[3] = tint_depth(m);
    o.opt[0] = m.opacity;
    o.opt[1] = plate;
    o.opt[2] = m.metal;
    o.opt[3] = m.gloss;
    o.sty[0] = fullness(m);
    o.sty[1] = m.foam;
    o.sty[2] = dry_time;
    o.sty[3] = m.emissivity;
    o.idx[0] = m.diluent;
    o.idx[1] = (int)m.group;
    o.idx[2] = (int)std::round(dry_scatter(m) * 1000.0f);
    o.idx[3] = 0;
    o.fx[0] = vshare;
    o.fx[1] = coat;
    o.fx[2] = iridescence(m, p.pair_tension[0][std::min<uint32_t>(m.group, 3u)], cell);
    o.fx[3] = crust(m);
    o.fx2[0] = m.froth;
    o.fx2[1] = m.fizz;
    o.fx2[2] = n_draw;
    o.fx2[3] = drain;
    float gl[3];
    linear(m.glow_color, gl);
    for (int c = 0; c < 3; c++) o.lum[c] = gl[c] * m.luminous;
    o.lum[3] = m.glow_shear;
    packed(ah, sh, o.hot);
    o.thermo[0] = m.thermo_lo;
    o.thermo[1] = m.thermo_hi;
    o.thermo[2] = wetting(m);
    o.thermo[3] = (m.group == 0 && m.tension < 0.04f) ? 1.0f : 0.0f;
    o.scat[0] = ratio[0];
    o.scat[1] = ratio[1];
    o.scat[2] = ratio[2];
    o.scat[3] = g;
    o.opt2[0] = m.ior;
    o.opt2[1] = dr;
    o.opt2[2] = bretherton;
    o.opt2[3] = evap;
    for (int c = 0; c < 4; c++) o.dust[c] = per[c];
    o.dust2[0] = 0.5f * m.dust_size;
    o.dust2[1] = m.dust_density;
    o.dust2[2] = m.dust_shape;
    o.dust2[3] = m.dust_reflect;
    o.dcol[0] = dl[0];
    o.dcol[1] = dl[1];
    o.dcol[2] = dl[2];
    o.dcol[3] = pack;
}

void optics_table(const SimParams& p, DevOptics* out) {
    for (int r = 0; r < kMaxMaterials; r++) optics_row(p, r, out[r]);
}

}  // namespace sprout

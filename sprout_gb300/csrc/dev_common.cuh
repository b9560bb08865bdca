// Device-side helpers shared by the engine's kernels.
//
// All kernels are compiled with -fmad=false: every float operation rounds the way it is
// written (as the reference's shaders spell it), which makes the FP32 path reproducible
// to the bit against a CPU evaluation of the same expressions. GLSL built-ins follow the
// GLSL spec definitions: mix(x, y, a) = x (1 - a) + y a, length = sqrt(dot),
// normalize = v / length(v).
#pragma once

#include <cstdint>

#include "device_types.h"

namespace sprout {

#define DEV __device__ __forceinline__

constexpr float MASS_SCALE = 1048576.0f;   // 2^20
constexpr float MOM_SCALE = 4194304.0f;    // 2^22
constexpr int MIN_FACE_MASS = 64;
constexpr float THETA_MIN = 0.1f;
constexpr float REST_PHI = 1.0f;
constexpr float LIQUID_THR = 0.5f;
constexpr float FACE_EMPTY = 1e30f;
constexpr float FACE_CLOSED = -1e30f;
constexpr float NO_TEMP = -1e9f;
constexpr float LEDGER_SCALE = 65536.0f;
constexpr float T_SCALE = 4096.0f;
constexpr uint32_t REGION_MASK = 31u;
constexpr uint32_t REGION_VENT = 256u;
constexpr uint32_t KIND_DEAD = 0u;
constexpr uint32_t KIND_FRESH = 0x10000u;
constexpr float MG_OMEGA = 1.8f;

// Device buffers of one tank. Grid fields are W x H cells, row-major; the multigrid
// fields hold every level back to back (Levels offsets).
// Four FP64 partial sums (the mixed-precision solve's dot products).
struct alignas(16) Dbl4 {
    double x, y, z, w;
};

struct DevScene {
    int W, H, ncell, stride;
    uint32_t capacity;
    const DevParams* P;
    const DevMat* mats;
    StepState* S;
    SolveState* K;
    // particles: 3 float4 per particle (pos.xy vel.xy | c | s kind id t)
    float4* part;     // sorted by cell after every substep, live ones first
    float4* part2;    // the advanced particles in the previous order
    uint32_t* pkey;   // new cell of each advanced particle (0xffffffff: dead)
    uint32_t* prank;  // its arrival rank in that cell
    uint32_t* perm;   // sorted slot -> slot in part2
    uint32_t* crowd;  // the sort's cells of more than 16 particles: [0] how many, then the cells
    uint32_t* count;  // particles per cell (ncell + 1)
    uint32_t* start;  // first sorted slot of each cell (ncell + 1)
    uint32_t* scan_tmp;
    // grid
    int32_t* acc;
    float4 *vel, *cell, *comp, *coef, *sprop, *surf, *surf2, *aux, *grho, *therm, *dheat, *vw, *vs, *prhs;
    float2 *vel0, *pjump, *pres;
    float* p2keep;
    float* mixb;      // per cell, families 1 .. n_fam - 1: the family's concentration (-1: not here)
    float4* gbase;    // per cell: share x base density of phase groups 1 - 3 (w unused)
    float4* rh;       // per cell: its non-Newtonian liquid (share, row, concentration, stiff)
    float* famocc;    // per cell and family: the family's occupancy (settling)
    float2* dsettle;  // per cell and family: the concentration gain / loss rates settling hands the particles
    float2* magc;     // per cell: its liquid's susceptibility; the magnetic energy density of magnetic liquid there
    float4* pstress;  // per particle slot (sorted order): its viscoelastic stress (xx, yy, xy)
    float4* pstress2; // the same after the particle pass, in the pass's order
    uint4* plook;     // per particle slot: look.comp's state (its id, -, A_xx A_yy A_xy, -); null
                      // until a render finds a liquid with a look (moves with its particle)
    uint4* plook2;    // the sort's target for it
    float4* pdep;     // the stress each particle deposits this substep, in the pass's order
    float4* estr;     // per cell: the deposited stress (elastic.comp)
    int2* rl;         // per cell: rigid label (its body's root cell, -1 not rigid); at a root, its body
    unsigned long long* rbody;   // per body: 15 fixed-point sums (mass, moments, contacts), 16 apart
    uint32_t* nbodies;           // bodies labelled in the last rigid pass
    int2* hcell;
    const float4* solid;
    const float* sdf;
    const uint32_t* region;
    const float* solid_t;
    unsigned long long* ledger;
    // multigrid / Krylov
    float4* mga;
    float* mgd;
    float2 *mgx, *mgz, *mgr, *mgr2, *cgp, *cgp2, *cgq;
    uint32_t* ptile;
    uint32_t* plist;    // per level (at lv.toff), the tiles with pressure unknowns in order
    uint32_t* pcount;   // per level, how many (kMaxLevels)
    float4* partials;   // 2 x nwg
    int nwg;
    Levels lv;
    // the mixed-precision solve's copy of the hierarchy's matrices (indexed like mga / mgd)
    // and its FP64 per-tile partial sums (2 x nwg)
    uint2* hga;         // four BF16 couplings per cell
    float* hgd;         // FP32 diagonal, rebuilt so that each row keeps its exact excess over
                        // the BF16 couplings (the part of D that is no coupling: air, vent)
    float* hgi;         // 1 / hgd (0 where no unknown): the smoothers multiply by it
    Dbl4* partials64;
    // implicit viscosity (visc*.comp, vmg*.comp): Krylov vectors on the grid, the multigrid
    // hierarchy over the levels of lv, tile flags and the compact lists of active tiles
    float2 *vr, *vr2, *vp, *vq, *vq2, *vd, *vaz;
    float4 *vma, *vmb;
    float2 *vmd, *vmr, *vmx, *vmz;
    uint32_t* tiles;    // level-0 tiles that take the implicit solve (nwg)
    uint32_t* vtile;    // per level, tiles active in the last build (lv.tiles)
    uint32_t* vlist;    // per level, the active tiles in order (lv.tiles)
    uint32_t* vcount;   // per level, how many (kMaxLevels)
};

// GLSL min / max (GLSL spec 8.3): min(x, y) = y < x ? y : x, max(x, y) = x < y ? y : x.
DEV float minf(float x, float y) { return y < x ? y : x; }
DEV float maxf(float x, float y) { return x < y ? y : x; }
DEV float clampf(float x, float lo, float hi) { return minf(maxf(x, lo), hi); }
DEV int clampi(int x, int lo, int hi) { return min(max(x, lo), hi); }
DEV float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
DEV float len2(float x, float y) { return sqrtf(x * x + y * y); }
// GLSL sign(x): -1, 0 or 1.
DEV float signf(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
// The terminal velocity (cells / s) of a droplet of diameter d (cells) and density difference
// drho in a liquid of density rho_c and kinematic viscosity nu_c, drag C_d = 24 / Re + 0.44:
// the positive root of 0.44 rho_c v^2 + 24 nu_c rho_c v / d = 4/3 |drho| g d (common.glsl:370-374).
DEV float terminal(float drho, float rho_c, float nu_c, float d, float gravity) {
    const float qa = 0.44f * rho_c, qb = 24.0f * nu_c * rho_c / d, qc = 4.0f / 3.0f * fabsf(drho) * gravity * d;
    return qc > 0.0f ? 2.0f * qc / (qb + sqrtf(qb * qb + 4.0f * qa * qc)) : 0.0f;
}
DEV float smoothstepf(float e0, float e1, float x) {
    float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
DEV bool face_live(float st) { return fabsf(st) < 1e29f; }
DEV bool face_closed(float st) { return st < -1e29f; }

DEV uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// exp(x) by Cody-Waite reduction x = n ln2 + r (ln2 in two parts), e^r by its Taylor
// series to degree 7 in Horner form, times 2^n assembled from exponent bits in two factors.
// The same operations in the same order as the CPU evaluation used by the tests, so both
// round identically (relative error within 2 ulp of the true value over the range used).
DEV float sp_expf(float x) {
    if (x != x) return x;
    if (x > 88.72283f) return __int_as_float(0x7f800000);
    if (x < -103.972f) return 0.0f;
    const float LOG2E = 1.44269504f;
    const float LN2_HI = 0.693145752f;
    const float LN2_LO = 1.42860677e-06f;
    float n = floorf(x * LOG2E + 0.5f);
    float r = (x - n * LN2_HI) - n * LN2_LO;
    float p = 1.98412698e-04f;
    p = p * r + 1.38888889e-03f;
    p = p * r + 8.33333333e-03f;
    p = p * r + 4.16666667e-02f;
    p = p * r + 1.66666667e-01f;
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    int k = (int)n;
    int k1 = k / 2, k2 = k - k1;
    float s1 = __int_as_float((k1 + 127) << 23);
    float s2 = __int_as_float((k2 + 127) << 23);
    return (p * s1) * s2;
}

// ln(x) for x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)) (subnormals scaled by 2^24
// first), ln m = 2 atanh(s) with s = (m - 1) / (m + 1), |s| <= 0.172, by the atanh series
// to s^13 in Horner form in s^2, and e ln 2 added in two parts. The same operations in the
// same order as the CPU evaluation used by the tests.
DEV float sp_logf(float x) {
    if (x != x || x < 0.0f) return __int_as_float(0x7fc00000);
    if (x == 0.0f) return __int_as_float(0xff800000);
    if (x == __int_as_float(0x7f800000)) return x;
    int e = 0;
    if (x < 1.17549435e-38f) {
        x *= 16777216.0f;
        e = -24;
    }
    const uint32_t u = __float_as_uint(x);
    e += (int)((u >> 23) & 255u) - 127;
    float m = __uint_as_float((u & 0x7fffffu) | 0x3f800000u);
    if (m > 1.41421356f) {
        m *= 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float z = s * s;
    float p = 7.69230769e-02f;   // 1/13
    p = p * z + 9.09090909e-02f;  // 1/11
    p = p * z + 1.11111111e-01f;  // 1/9
    p = p * z + 1.42857143e-01f;  // 1/7
    p = p * z + 2.00000000e-01f;  // 1/5
    p = p * z + 3.33333333e-01f;  // 1/3
    p = p * z + 1.0f;
    const float lm = 2.0f * s * p;
    const float fe = (float)e;
    return fe * 0.693145752f + (fe * 1.42860677e-06f + lm);
}
// x^y as exp(y ln x) with the two functions above (x > 0; 1 for x = 1).
DEV float sp_powf(float x, float y) { return x == 1.0f ? 1.0f : sp_expf(y * sp_logf(x)); }

// The field of the magnets at x (cells), T: each a point dipole in the plane,
// B0 (R / r)^3 (3 (m.e) e - m) / 2, constant inside the rim (common.glsl:388-402).
DEV float2 magnet_field(const DevParams* P, float x, float y) {
    float bx = 0.0f, by = 0.0f;
    for (int k = 0; k < (int)P->mag[0]; k++) {
        const float* mg = P->magnet[k];
        const float mx = P->magnet_dir[k][0], my = P->magnet_dir[k][1];
        const float dx = x - mg[0], dy = y - mg[1];
        const float len = len2(dx, dy);
        const float r = maxf(len, mg[2]);
        const float ex = len > 1e-4f ? dx / len : mx, ey = len > 1e-4f ? dy / len : my;
        const float a = mg[3] * sp_powf(mg[2] / r, 3.0f) * 0.5f;
        const float me3 = 3.0f * (mx * ex + my * ey);
        bx += a * (me3 * ex - mx);
        by += a * (me3 * ey - my);
    }
    return make_float2(bx, by);
}

// look.comp look_of: the platelets' sheen weight and the specks drawn per cell of material
// `row` at concentration s, a concentrate's blended with its diluent's
DEV float2 look_of(const DevOptics* opt, uint32_t row, float s) {
    const DevOptics& o = opt[row];
    float lx = o.opt[1], ly = o.fx2[2];
    if (o.idx[0] >= 0) {
        const DevOptics& dl = opt[o.idx[0]];
        const float t = clampf(s, 0.0f, 1.0f);
        lx = mixf(dl.opt[1], lx, t);
        ly = mixf(dl.fx2[2], ly, t);
    }
    return make_float2(lx, ly);
}

// sin and cos of a float angle, each rounded once from FP64 (GLSL leaves their precision to the
// implementation): the angle reduced by the nearest multiple q of pi/2 (Cody and Waite, pi/2
// in two parts of 33 and 53 bits), the Taylor series to r^15 and r^16 on [-pi/4, pi/4], then
// the quadrant q mod 4's swap and signs. Within an ulp of the true values for |a| < 1e9.
DEV void sp_sincos(float af, float* s, float* c) {
    const double a = (double)af;
    if (!(fabs(a) < 1e9)) {
        *s = *c = af - af;
        return;
    }
    const double q = rint(a * 0.63661977236758134308);
    const double r = (a - q * 1.57079632673412561417) - q * 6.07710050650619224932e-11;
    const double x2 = r * r;
    double sn = 1.0 / 1307674368000.0;
    sn = 1.0 / 6227020800.0 - x2 * sn;
    sn = 1.0 / 39916800.0 - x2 * sn;
    sn = 1.0 / 362880.0 - x2 * sn;
    sn = 1.0 / 5040.0 - x2 * sn;
    sn = 1.0 / 120.0 - x2 * sn;
    sn = 1.0 / 6.0 - x2 * sn;
    sn = r - r * x2 * sn;
    double cs = 1.0 / 20922789888000.0;
    cs = 1.0 / 87178291200.0 - x2 * cs;
    cs = 1.0 / 479001600.0 - x2 * cs;
    cs = 1.0 / 3628800.0 - x2 * cs;
    cs = 1.0 / 40320.0 - x2 * cs;
    cs = 1.0 / 720.0 - x2 * cs;
    cs = 1.0 / 24.0 - x2 * cs;
    cs = 0.5 - x2 * cs;
    cs = 1.0 - x2 * cs;
    const int n = ((int)q) & 3;
    *s = (float)(n == 0 ? sn : n == 1 ? cs : n == 2 ? -sn : -cs);
    *c = (float)(n == 0 ? cs : n == 1 ? -sn : n == 2 ? -cs : sn);
}

// atan(y, x) rounded once from FP64 (GLSL leaves its precision to the implementation, and the
// result at x = y = 0: here 0): t = min / max of |x|, |y| in [0, 1]; atan t = 4 atan u with u
// from two halvings of the angle, u / (1 + sqrt(1 + u^2)), so |u| <= tan(pi / 16); the series
// to u^25; then the octant.
DEV float sp_atan2(float yf, float xf) {
    const double y = (double)yf, x = (double)xf, ay = fabs(y), ax = fabs(x);
    if (ax == 0.0 && ay == 0.0) return 0.0f;
    const bool swap = ay > ax;
    const double t = swap ? ax / ay : ay / ax;
    double u = t / (1.0 + sqrt(1.0 + t * t));
    u = u / (1.0 + sqrt(1.0 + u * u));
    const double u2 = u * u;
    double p = 1.0 / 25.0;
    for (int k = 11; k >= 0; k--) p = 1.0 / (double)(2 * k + 1) - u2 * p;
    double at = 4.0 * u * p;
    if (swap) at = 1.5707963267948966 - at;
    if (x < 0.0) at = 3.141592653589793 - at;
    if (y < 0.0) at = -at;
    return (float)at;
}

constexpr int kMaxBodies = 4096;   // common.glsl: MAX_BODIES
constexpr float RIGID_FIX = 65536.0f;

// A body sum as the shader reads its two words: (hi as int) 2^32 + lo, over the fixed-point scale.
DEV float get64(unsigned long long v) {
    return ((float)(int)(uint32_t)(v >> 32) * 4294967296.0f + (float)(uint32_t)v) / RIGID_FIX;
}

// Contact of a body with the solids it touches: it neither sinks into its support nor
// spins through it, and slides on it against friction mu (common.glsl:289-325).
DEV void body_contact(const unsigned long long* o, float mu, float cmx, float cmy, float& Ux, float& Uy, float& w) {
    const float nc = get64(o[7]);
    if (mu < 0.0f || nc < 0.5f) return;
    const float nsx = get64(o[8]), nsy = get64(o[9]);
    const float ln = len2(nsx, nsy);
    if (ln < 0.25f * nc) return;
    const float nx = nsx / ln, ny = nsy / ln;
    const float tx = ny, ty = -nx;
    const float ccx = get64(o[10]) / nc, ccy = get64(o[11]) / nc;
    const float sqx = get64(o[12]) / nc - ccx * ccx, sqy = get64(o[13]) / nc - ccy * ccy, sqz = get64(o[14]) / nc - ccx * ccy;
    const float ext = sqrtf(3.0f * maxf(tx * tx * sqx + ty * ty * sqy + 2.0f * tx * ty * sqz, 0.0f)) + 0.5f;
    const float rcx = ccx - cmx, rcy = ccy - cmy;
    float ucx = Ux + w * -rcy, ucy = Uy + w * rcx;
    const float vn = ucx * nx + ucy * ny;
    const float sp = (cmx - ccx) * tx + (cmy - ccy) * ty;
    float vn1 = vn, w1 = w;
    if (fabsf(sp) <= ext) {
        vn1 = maxf(vn, 0.0f);
        w1 = clampf(w, -vn1 / ext, vn1 / ext);
    } else {
        const float edge = signf(sp) * ext;
        vn1 = maxf(vn + w * edge, 0.0f) - w * edge;
    }
    if (vn1 == vn && w1 == w) return;
    const float vt = ucx * tx + ucy * ty;
    const float vt1 = signf(vt) * maxf(fabsf(vt) - mu * (vn1 - vn), 0.0f);
    ucx = ucx + ((vn1 - vn) * nx + (vt1 - vt) * tx);
    ucy = ucy + ((vn1 - vn) * ny + (vt1 - vt) * ty);
    w = w1;
    Ux = ucx - w1 * -rcy;
    Uy = ucy - w1 * rcx;
}

// The rigid motion of body b (root cell r) at x: velocity and spin (common.glsl:327-340).
DEV bool body_motion(const DevScene& d, int b, int r, float x, float y, float3& u) {
    const unsigned long long* o = d.rbody + (size_t)b * 16;
    const float M = get64(o[0]);
    if (M <= 1e-3f) return false;
    const float cmx = get64(o[1]) / M, cmy = get64(o[2]) / M;
    float Ux = get64(o[3]) / M, Uy = get64(o[4]) / M;
    const float L = get64(o[5]) - M * (cmx * Uy - cmy * Ux);
    const float I = get64(o[6]) - M * (cmx * cmx + cmy * cmy);
    float w = I > 1e-3f ? L / I : 0.0f;
    body_contact(o, d.P->misc[3], cmx, cmy, Ux, Uy, w);
    const float dx = x - ((float)(r % d.W) + 0.5f) - cmx, dy = y - ((float)(r / d.W) + 0.5f) - cmy;
    u = make_float3(Ux + w * -dy, Uy + w * dx, w);
    return true;
}

// Quadratic B-spline weights (common.glsl:639-643) of a point at offset f from its base node.
DEV void bspline(float fx, float fy, float wx[3], float wy[3]) {
    wx[0] = 0.5f * (1.5f - fx) * (1.5f - fx);
    wy[0] = 0.5f * (1.5f - fy) * (1.5f - fy);
    wx[1] = 0.75f - (fx - 1.0f) * (fx - 1.0f);
    wy[1] = 0.75f - (fy - 1.0f) * (fy - 1.0f);
    wx[2] = 0.5f * (fx - 0.5f) * (fx - 0.5f);
    wy[2] = 0.5f * (fy - 0.5f) * (fy - 0.5f);
}

DEV float row_density(const DevMat* mats, uint32_t row, float s) {
    int d = mats[row].ia[1];
    float rho = mats[row].a[0];
    return d >= 0 ? mixf(mats[d].a[0], rho, s) : rho;
}

DEV float expansion_of(const DevMat* mats, uint32_t row, float s, float T) {
    const DevMat& m = mats[row];
    int d = m.ia[1];
    float b = m.misc[3], tr = m.temp[2] - 273.15f, tb = m.th2[2];
    if (d >= 0) {
        b = mixf(mats[d].misc[3], b, s);
        tr = mixf(mats[d].temp[2] - 273.15f, tr, s);
        tb = mixf(mats[d].th2[2], tb, s);
    }
    return clampf(1.0f - b * (minf(T, tb) - tr), 0.7f, 1.3f);
}

// Solidus, liquidus, latent heat (degrees), heat capacity of `row` at concentration s.
DEV float4 thermal_of(const DevMat* mats, uint32_t row, float s) {
    const DevMat& m = mats[row];
    float ld = m.th2[0];
    int d = m.ia[1];
    if (d < 0) return make_float4(m.th[2], m.th[3], ld, m.th[0]);
    const DevMat& dm = mats[d];
    float shift = m.misc[0] * s;
    float C = mixf(dm.th[0], m.th[0], s);
    return make_float4(dm.th[2] + shift, dm.th[3] + shift, mixf(dm.th[0] * dm.th2[0], m.th[0] * ld, s) / C, C);
}

// The enthalpy temperature that keeps a particle's heat when its heat capacity changes from
// c0 to c1 (particles.comp:78-80).
DEV float keep_heat(float t, float c0, float c1) { return c0 == c1 ? t : (t + 273.15f) * c0 / c1 - 273.15f; }

// Temperature and frozen share from the enthalpy temperature.
DEV float2 phase_of(float te, float4 m) {
    if (te >= m.y) return make_float2(te, 0.0f);
    float lo = m.x - m.z;
    if (te <= lo) return make_float2(te + m.z, 1.0f);
    float fr = (te - lo) / (m.y - lo);
    return make_float2(m.x + fr * (m.y - m.x), 1.0f - fr);
}

DEV float temp_law(const DevMat* mats, int r, float T) {
    int model = mats[r].ib[2];
    if (model == 0) return 0.0f;
    const float* tp = mats[r].temp;
    float Tk = maxf(T + 273.15f, 1.0f);
    float x = model == 1 ? tp[0] * (1.0f / Tk - 1.0f / tp[2]) : tp[0] / maxf(Tk - tp[1], 5.0f) - tp[0] / maxf(tp[2] - tp[1], 5.0f);
    return clampf(x, -30.0f, 30.0f);
}

DEV int group_heat_chan(const DevParams* P, int g) { return (int)((P->group_heat >> (8u * (uint32_t)g)) & 255u) - 1; }

// ln nu of `row` at concentration s and temperature T (common.glsl:631-636; every concentrate
// here blends with exponent 1).
DEV float row_lnu(const DevMat* mats, uint32_t row, float s, float T, bool thermal) {
    float l = mats[row].a[1] + (thermal ? temp_law(mats, (int)row, T) : 0.0f);
    const int dl = mats[row].ia[1];
    if (dl >= 0) l = mixf(mats[dl].a[1] + (thermal ? temp_law(mats, dl, T) : 0.0f), l, s);
    return l;
}

DEV int2 heat_quanta(float C, float T) {
    int ci = (int)floorf(C * MASS_SCALE + 0.5f);
    return make_int2(ci, (int)floorf((float)ci * (T + 273.15f) / T_SCALE + 0.5f));
}

DEV void ledger_add(unsigned long long* ledger, int entry, float v) {
    uint32_t x = (uint32_t)(v * LEDGER_SCALE + 0.5f);
    if (x == 0u) return;
    atomicAdd(&ledger[entry], (unsigned long long)x);
}

// Warp max of a non-negative float, then one atomicMax of its bits per warp.
DEV void report_max(uint32_t* slot, float m) {
    uint32_t b = __float_as_uint(m);
    b = __reduce_max_sync(0xffffffffu, b);
    if ((threadIdx.x & 31) == 0) atomicMax(slot, b);
}

}  // namespace sprout

/*
 * sprout_oracle.c -- CPU oracle of the Sprout fluid substep.
 *
 * TEST INFRASTRUCTURE ONLY (see sprout_oracle.h). A plain-C restatement, one function per
 * reference shader, of the per-substep 2D APIC/PIC solver of Testro-lol/Sprout:
 *   step.comp, sort.comp, particles.comp (core branches), grid_prep.comp, grid_coef.comp,
 *   surf_smooth.comp, surf_curv.comp, surf_apply.comp, heat.comp, visc_setup.comp +
 *   visc_apply.comp (explicit viscosity), rhs.comp, mg_build.comp, mg_tail.comp,
 *   mg_down.comp, mg_up.comp, cg_scale.comp, cg_init.comp, cg_apply.comp, cg_update.comp,
 *   reduce.glsl + reduce_tail.glsl, project.comp,
 * plus the Rust host code that sets them up: Scene::rasterize (src/scene.rs:215-470),
 * maps::fill_rect (src/maps.rs:455-492), Tank::layout (src/sim/mod.rs:271-329),
 * Levels::new (src/sim/mod.rs:714-753), gpu_materials / gpu_params
 * (src/sim/mod.rs:2179-2339), record / record_substep / record_pressure
 * (src/sim/mod.rs:2400-2708, 2929-3010).
 *
 * Build: -O2 -ffp-contract=off (no fused multiply-add: every float operation rounds the
 * way the shader source writes it). GLSL built-ins are spelled out per the GLSL spec:
 * mix(x, y, a) = x * (1 - a) + y * a, length(v) = sqrt(dot(v, v)), normalize(v) =
 * v / length(v), smoothstep per its definition. Work-group reductions keep the shaders'
 * order (256-invocation trees per 16 x 16 tile, then the strided totals of
 * reduce_tail.glsl:28-41).
 */
#include "sprout_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------------------ */
/* Small vector algebra (GLSL semantics)                                                 */
/* ------------------------------------------------------------------------------------ */

typedef struct { float x, y; } V2;
typedef struct { float x, y, z, w; } V4;
typedef struct { int x, y; } I2;

static inline V2 v2(float x, float y) { V2 r = {x, y}; return r; }
static inline V4 v4(float x, float y, float z, float w) { V4 r = {x, y, z, w}; return r; }
/* GLSL min / max (GLSL spec 8.3): min(x, y) = y < x ? y : x, max(x, y) = x < y ? y : x */
static inline float minf(float x, float y) { return y < x ? y : x; }
static inline float maxf(float x, float y) { return x < y ? y : x; }
static inline float clampf(float x, float lo, float hi) { return minf(maxf(x, lo), hi); }
static inline int mini(int a, int b) { return a < b ? a : b; }
static inline int maxi(int a, int b) { return a > b ? a : b; }
static inline int clampi(int x, int lo, int hi) { return mini(maxi(x, lo), hi); }
static inline float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
static inline float signf(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
static inline float len2(V2 v) { return sqrtf(v.x * v.x + v.y * v.y); }
static inline float smoothstepf(float e0, float e1, float x) {
    float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
static inline uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float bitsf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* air.glsl:4-11 */
static inline uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

/* exp(x): Cody & Waite argument reduction x = n ln2 + r with ln2 split in two parts,
 * |r| <= ln2 / 2, e^r by its Taylor series to degree 7 (Horner), times 2^n assembled from
 * the exponent bits (two factors, so subnormal results stay exact). */
float o_expf(float x) {
    if (x != x) return x;
    if (x > 88.72283f) return bitsf(0x7f800000u);
    if (x < -103.972f) return 0.0f;
    const float LOG2E = 1.44269504f;
    const float LN2_HI = 0.693145752f;   /* 0x3f317200: 16 significant bits */
    const float LN2_LO = 1.42860677e-06f;
    float n = floorf(x * LOG2E + 0.5f);
    float r = (x - n * LN2_HI) - n * LN2_LO;
    float p = 1.98412698e-04f;           /* 1/5040 */
    p = p * r + 1.38888889e-03f;         /* 1/720 */
    p = p * r + 8.33333333e-03f;         /* 1/120 */
    p = p * r + 4.16666667e-02f;         /* 1/24 */
    p = p * r + 1.66666667e-01f;         /* 1/6 */
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    int k = (int)n;
    int k1 = k / 2, k2 = k - k1;
    float s1 = bitsf((uint32_t)(k1 + 127) << 23);
    float s2 = bitsf((uint32_t)(k2 + 127) << 23);
    return (p * s1) * s2;
}

/* ln(x), x > 0: x = m 2^e, m in [sqrt(1/2), sqrt(2)) (subnormals scaled by 2^24 first);
 * ln m = 2 atanh(s), s = (m - 1) / (m + 1), by the atanh series to s^13 (Horner in s^2);
 * e ln 2 added in two parts. */
float o_logf(float x) {
    if (x != x || x < 0.0f) return bitsf(0x7fc00000u);
    if (x == 0.0f) return bitsf(0xff800000u);
    if (x == bitsf(0x7f800000u)) return x;
    int e = 0;
    if (x < 1.17549435e-38f) {
        x *= 16777216.0f;
        e = -24;
    }
    uint32_t u;
    memcpy(&u, &x, 4);
    e += (int)((u >> 23) & 255u) - 127;
    float m = bitsf((u & 0x7fffffu) | 0x3f800000u);
    if (m > 1.41421356f) {
        m *= 0.5f;
        e += 1;
    }
    float sv = (m - 1.0f) / (m + 1.0f);
    float z = sv * sv;
    float q = 7.69230769e-02f;   /* 1/13 */
    q = q * z + 9.09090909e-02f;
    q = q * z + 1.11111111e-01f;
    q = q * z + 1.42857143e-01f;
    q = q * z + 2.00000000e-01f;
    q = q * z + 3.33333333e-01f;
    q = q * z + 1.0f;
    float lm = 2.0f * sv * q;
    float fe = (float)e;
    return fe * 0.693145752f + (fe * 1.42860677e-06f + lm);
}

/* x^y = exp(y ln x) with the two functions above (x > 0; 1 for x = 1) */
float o_powf(float x, float y) { return x == 1.0f ? 1.0f : o_expf(y * o_logf(x)); }

/* ------------------------------------------------------------------------------------ */
/* Constants (shaders/common.glsl, src/sim/ sources)                                       */
/* ------------------------------------------------------------------------------------ */

#define KIND_DEAD 0u
#define KIND_FRESH 0x10000u
#define KIND_REAL_T 0x20000u
#define SPAWN_TEMP (-1.0e4f)
#define SPAWN_S (-1.0f)
#define MAX_PRESENT 12
#define SPAWN_MAX 32768u     /* mod.rs:63 */
#define GROUPS 4
#define MASS_SCALE 1048576.0f
#define MOM_SCALE 4194304.0f
#define MIN_FACE_MASS 64
#define THETA_MIN 0.1f
#define REST_PHI 1.0f
#define LIQUID_THR 0.5f
#define FACE_EMPTY 1e30f
#define FACE_CLOSED (-1e30f)
#define NO_TEMP (-1e9f)
#define LEDGER_SCALE 65536.0f
#define T_SCALE 4096.0f
#define REGION_MASK 31u
#define REGION_VENT 256u
#define CAP_FAMILIES 1u
#define CAP_THERMAL 2u
#define CAP_RIGID 4u
#define CAP_RHEO 8u
#define CAP_MAGNET 16u
#define CAP_ELASTIC 32u
#define CAP_SETTLE 64u
#define CAP_STEAM 128u
#define CAP_REACT 256u
#define WATER_DENSITY 998.0f
#define WATER_HEAT (998.0f * 4182.0f)
#define STEFAN_BOLTZMANN 5.670374e-8f
#define T_REF 20.0f
#define NO_MELT (-1.0e9f)
#define ACC_MIN 8
#define ACC_MAX 32
#define ACC_FIRST 5
#define COARSEST_CELLS 4
#define TAIL_CELLS 1500
#define MG_OMEGA 1.8f
#define GRID_GROUP 16
#define WALL 3.0f
#define PPC 4

static int is_inside_f(float d) { return d < 0.0f; }

/* ------------------------------------------------------------------------------------ */
/* Parameters: SimParams::default and the built-ins the configs use                      */
/* ------------------------------------------------------------------------------------ */

static void mat_default(OMat* m) {
    memset(m, 0, sizeof *m);
    m->group = 0;
    m->diluent = -1;
    m->density = 998.0f;
    m->density_solid = 0.0f;
    m->viscosity = 1.0e-6f;
    m->rheology = 0;
    m->temp_model = 0;
    m->temp_b = 0.0f;
    m->temp_c = 0.0f;
    m->temp_ref = T_REF;
    m->tension = 0.072f;
    m->contact_angle = 90.0f;
    m->mix_rate = 0.0f;
    m->grain = 0.0f;
    m->load = 1.0f;
    m->heat_capacity = 4182.0f;
    m->conductivity = 0.6f;
    m->expansion = 4.0e-4f;
    m->melt_lo = -1.0e9f;
    m->melt_hi = -1.0e9f;
    m->latent = 0.0f;
    m->emissivity = 0.9f;
    m->boil = 1.0e9f;
    m->latent_vap = 0.0f;
    m->freeze_shift = 0.0f;
    m->spawn_temp = T_REF;
    m->react_with = -1;
    m->yield_stress = 0.0f;
    m->flow_index = 1.0f;
    m->shear_time = 1.0f;
    m->visc_ratio = 1.0f;
    m->saturation = 0.05f;
}

void oparams_default(OSimParams* p) {
    memset(p, 0, sizeof *p);
    p->cell_size = 0.01f;
    p->gravity = 9.81f;
    /* material.rs:489-507 */
    float t[GROUPS][GROUPS] = {{0}};
#define SETPT(a, b, v) (t[a][b] = (v), t[b][a] = (v))
    SETPT(0, 1, 0.025f);
    SETPT(0, 2, 0.375f);
    SETPT(1, 2, 0.36f);
    SETPT(0, 3, 0.2f);
    SETPT(1, 3, 0.2f);
    SETPT(2, 3, 0.4f);
#undef SETPT
    memcpy(p->pair_tension, t, sizeof t);
    p->ambient_temp = T_REF;
    p->heat_rate = 1.0f;
    p->air_cooling = 10.0f;
    p->contact_heat = 3000.0f;
    p->eddy_heat = 0.17f;
    p->evaporation = 1;
    p->rigid_viscosity = 1.0f;
    p->heat_power = 300.0f;
    p->steam = 1;
    p->droplet_cells = 1.0f;
    p->cfl = 4.0f;
    p->advection_order = 2;
    p->dt_max = 1.0f / 80.0f;
    p->fixed_hz = 0.0f;
    p->pressure_tol = 1e-4f;
    p->pressure_max_iters = 60;
    p->iters_margin = 0.25f;
    p->correction_tol = 1e-2f;
    p->viscosity_tol = 1e-3f;
    p->viscosity_max_iters = 200;
    p->implicit_viscosity_min = 1e-3f;
    p->viscous_projection = 1;
    p->viscous_warm = 1;
    p->viscosity_warm = 1;
    p->viscosity_precond = 1;
    p->viscosity_mg_levels = 1;
    p->viscosity_mg_sweeps = 2;
    p->spray_cfl = 4.0f;
    p->speed_cap = 1.0f;
    p->correction_time = (1.0f / 240.0f) / 0.693147182f;
    p->correction_max = 0.5f;
    p->correction_deadband = 0.25f;
    p->correction_step_max = 0.5f;
    p->crowd_jitter = 0.5f;
    p->tool_crowd_max = 2.0f;
    p->apic_clamp = 1.0f;
    p->curvature_max = 0.5f;
    p->slip_cap = 1;
    p->sealed_vent = 1;
    p->elastic_stress_max = 10.0f;   /* params.rs:447-448 */
    p->elastic_step_max = 0.25f;
    p->rigid_contact = 1;   /* params.rs: rigid_contact, rigid_friction */
    p->rigid_friction = 0.6f;
    for (int r = 0; r < O_MAX_MATERIALS; r++) mat_default(&p->mat[r]);
    /* the built-in liquids (presets.rs: BUILTINS): the fields the oracle carries */
#define BUILTIN_P(row, field, v) p->mat[row].field = v;
#define BUILTIN_O(row, field, v)
#include "../sprout_gb300/csrc/builtin_rows.inc"
#undef BUILTIN_P
#undef BUILTIN_O
}

/* ------------------------------------------------------------------------------------ */
/* Scene (src/scene.rs)                                                                  */
/* ------------------------------------------------------------------------------------ */

static void rotate2(float px, float py, float angle, float* ox, float* oy) {
    float s = sinf(angle), c = cosf(angle);
    *ox = c * px + s * py;
    *oy = -s * px + c * py;
}

/* Shape::sdf (scene.rs:68-93): circle and box. */
static float shape_sdf(const OShape* s, float px, float py) {
    if (s->kind == 0) return hypotf(px - s->c[0], py - s->c[1]) - s->r;
    float qx, qy;
    rotate2(px - s->c[0], py - s->c[1], s->angle, &qx, &qy);
    float dx = fabsf(qx) - s->half[0], dy = fabsf(qy) - s->half[1];
    return hypotf(maxf(dx, 0.0f), maxf(dy, 0.0f)) + minf(maxf(dx, dy), 0.0f);
}

static void shape_bound(const OShape* s, float* c, float* r) {
    c[0] = s->c[0];
    c[1] = s->c[1];
    *r = s->kind == 0 ? s->r : hypotf(s->half[0], s->half[1]);
}

static float wall_sdf(int w, int h, float x, float y) {
    float W = (float)w, H = (float)h;
    return fminf(fminf(fminf(x - WALL, W - WALL - x), y - WALL), H - WALL - y);
}

float oscene_sdf(int w, int h, int nshapes, const OShape* shapes, float x, float y) {
    float d = wall_sdf(w, h, x, y);
    for (int k = 0; k < nshapes; k++) d = fminf(d, shape_sdf(&shapes[k], x, y));
    return d;
}

/* open_fraction (scene.rs:177-189) */
static float open_fraction(float d0, float d1) {
    float f;
    if (d0 > 0.0f && d1 > 0.0f) f = 1.0f;
    else if (d0 <= 0.0f && d1 <= 0.0f) f = 0.0f;
    else f = fmaxf(d0, d1) / (fmaxf(d0, d1) - fminf(d0, d1));
    return f < 0.05f ? 0.0f : f;
}

/* Scene::union_depth (scene.rs:318-381) */
static void union_depth(float* sdf, int nw, int nh) {
    const float FAR = 1e9f;
    float* depth = (float*)calloc((size_t)nw * nh, sizeof(float));
    static const int NB8[8][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
    for (int j = 0; j < nh; j++)
        for (int i = 0; i < nw; i++) {
            int k = j * nw + i;
            if (!is_inside_f(sdf[k])) continue;
            int edge = 0;
            for (int q = 0; q < 8; q++) {
                int a = i + NB8[q][0], b = j + NB8[q][1];
                if (a >= 0 && b >= 0 && a < nw && b < nh && !is_inside_f(sdf[b * nw + a])) { edge = 1; break; }
            }
            depth[k] = edge ? -sdf[k] : FAR;
        }
    const float D = 1.41421354f;
#define RELAX(k, n, st) do { if (depth[n] + (st) < depth[k]) depth[k] = depth[n] + (st); } while (0)
    for (int j = 0; j < nh; j++)
        for (int i = 0; i < nw; i++) {
            int k = j * nw + i;
            if (depth[k] == 0.0f) continue;
            if (i > 0) RELAX(k, k - 1, 1.0f);
            if (j > 0) {
                RELAX(k, k - nw, 1.0f);
                if (i > 0) RELAX(k, k - nw - 1, D);
                if (i + 1 < nw) RELAX(k, k - nw + 1, D);
            }
        }
    for (int j = nh - 1; j >= 0; j--)
        for (int i = nw - 1; i >= 0; i--) {
            int k = j * nw + i;
            if (depth[k] == 0.0f) continue;
            if (i + 1 < nw) RELAX(k, k + 1, 1.0f);
            if (j + 1 < nh) {
                RELAX(k, k + nw, 1.0f);
                if (i + 1 < nw) RELAX(k, k + nw + 1, D);
                if (i > 0) RELAX(k, k + nw - 1, D);
            }
        }
#undef RELAX
    for (int k = 0; k < nw * nh; k++)
        if (is_inside_f(sdf[k]) && depth[k] < FAR) sdf[k] = fminf(sdf[k], -depth[k]);
    free(depth);
}

static void faces_of(const float* open, const float* sdf, int w, int i, int j, float out[2]) {
    int nw = w + 1;
    int here = open[j * w + i] > 0.0f;
    int left = here && i > 0 && open[j * w + i - 1] > 0.0f;
    int below = here && j > 0 && open[(j - 1) * w + i] > 0.0f;
    out[0] = left ? open_fraction(sdf[j * nw + i], sdf[(j + 1) * nw + i]) : 0.0f;
    out[1] = below ? open_fraction(sdf[j * nw + i], sdf[j * nw + i + 1]) : 0.0f;
}

/* Scene::seal_pockets (scene.rs:431-470) */
static void seal_pockets(float* open, float* sdf, int w, int h) {
    int nw = w + 1;
    size_t n = (size_t)w * h;
    uint32_t* label = (uint32_t*)malloc(n * sizeof(uint32_t));
    int* stack = (int*)malloc(n * sizeof(int));
    int* members = (int*)malloc(n * sizeof(int));
    for (size_t k = 0; k < n; k++) label[k] = 0xffffffffu;
    for (int start = 0; start < (int)n; start++) {
        if (open[start] == 0.0f || label[start] != 0xffffffffu) continue;
        int nm = 0, sp = 0;
        label[start] = (uint32_t)start;
        stack[sp++] = start;
        while (sp > 0) {
            int k = stack[--sp];
            members[nm++] = k;
            int i = k % w, j = k / w;
            float lb[2], rr[2], ab[2];
            faces_of(open, sdf, w, i, j, lb);
            float right = 0.0f, above = 0.0f;
            if (i + 1 < w) { faces_of(open, sdf, w, i + 1, j, rr); right = rr[0]; }
            if (j + 1 < h) { faces_of(open, sdf, w, i, j + 1, ab); above = ab[1]; }
            int nb[4] = {k - 1, k + 1, k - w, k + w};
            float a[4] = {lb[0], right, lb[1], above};
            for (int q = 0; q < 4; q++)
                if (a[q] > 0.0f && label[nb[q]] == 0xffffffffu) {
                    label[nb[q]] = (uint32_t)start;
                    stack[sp++] = nb[q];
                }
        }
        if (nm < 16) {
            for (int m = 0; m < nm; m++) {
                int k = members[m];
                open[k] = 0.0f;
                int i = k % w, j = k / w;
                int nodes[4] = {j * nw + i, j * nw + i + 1, (j + 1) * nw + i, (j + 1) * nw + i + 1};
                for (int q = 0; q < 4; q++) sdf[nodes[q]] = fminf(sdf[nodes[q]], -0.5f);
            }
        }
    }
    free(label);
    free(stack);
    free(members);
}

/* Scene::regions (scene.rs:385-425) */
static void regions_of(const float* solid4, int w, int h, uint32_t* region) {
    size_t n = (size_t)w * h;
    int* stack = (int*)malloc(n * sizeof(int));
    for (size_t k = 0; k < n; k++) region[k] = 0xffffffffu;
    uint32_t count = 0;
    for (int start = 0; start < (int)n; start++) {
        if (solid4[4 * start + 3] == 0.0f || region[start] != 0xffffffffu) continue;
        uint32_t id = count < 31u ? count : 31u;
        count++;
        int vent = start, sp = 0;
        region[start] = id;
        stack[sp++] = start;
        while (sp > 0) {
            int k = stack[--sp];
            if (k / w > vent / w || (k / w == vent / w && k < vent)) vent = k;
            int i = k % w, j = k / w;
            int okl = i > 0, okr = i + 1 < w, okb = j > 0, okt = j + 1 < h;
            float al = solid4[4 * k + 0];
            float ar = okr ? solid4[4 * (k + 1) + 0] : 0.0f;
            float ab = solid4[4 * k + 1];
            float at = okt ? solid4[4 * (k + w) + 1] : 0.0f;
            int nb[4] = {k - 1, k + 1, k - w, k + w};
            int ok[4] = {okl, okr, okb, okt};
            float a[4] = {al, ar, ab, at};
            for (int q = 0; q < 4; q++)
                if (ok[q] && a[q] > 0.0f && region[nb[q]] == 0xffffffffu) {
                    region[nb[q]] = id;
                    stack[sp++] = nb[q];
                }
        }
        region[vent] |= REGION_VENT;
    }
    for (size_t k = 0; k < n; k++)
        if (region[k] == 0xffffffffu) region[k] = 0;
    free(stack);
}

int oscene_rasterize(int w, int h, int nshapes, const OShape* shapes, float* sdf,
                     float* solid4, uint32_t* region, float* temp) {
    int nw = w + 1, nh = h + 1;
    for (int j = 0; j < nh; j++)
        for (int i = 0; i < nw; i++) sdf[j * nw + i] = wall_sdf(w, h, (float)i, (float)j);
    const float REACH = 6.0f;
    for (int s = 0; s < nshapes; s++) {
        float c[2], r;
        shape_bound(&shapes[s], c, &r);
        r = r + REACH;
        int i0 = (int)fmaxf(floorf(c[0] - r), 0.0f);
        int i1 = clampi((int)ceilf(c[0] + r), 0, nw - 1);
        int j0 = (int)fmaxf(floorf(c[1] - r), 0.0f);
        int j1 = clampi((int)ceilf(c[1] + r), 0, nh - 1);
        int jend = mini(maxi(j1, j0), nh - 1), iend = mini(maxi(i1, i0), nw - 1);
        for (int j = j0; j <= jend; j++)
            for (int i = i0; i <= iend; i++) {
                float* d = &sdf[j * nw + i];
                *d = fminf(*d, shape_sdf(&shapes[s], (float)i, (float)j));
            }
    }
    union_depth(sdf, nw, nh);
    float* open = (float*)malloc((size_t)w * h * sizeof(float));
    static const float FX[4][2] = {{0.25f, 0.25f}, {0.75f, 0.25f}, {0.25f, 0.75f}, {0.75f, 0.75f}};
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            float d[4] = {sdf[j * nw + i], sdf[j * nw + i + 1], sdf[(j + 1) * nw + i], sdf[(j + 1) * nw + i + 1]};
            float acc = 0.0f;
            for (int q = 0; q < 4; q++) {
                float fx = FX[q][0], fy = FX[q][1];
                float v = (d[0] * (1.0f - fx) + d[1] * fx) * (1.0f - fy) + (d[2] * (1.0f - fx) + d[3] * fx) * fy;
                acc += clampf(v / 0.5f + 0.5f, 0.0f, 1.0f);
            }
            open[j * w + i] = acc * 0.25f < 0.1f ? 0.0f : acc * 0.25f;
        }
    seal_pockets(open, sdf, w, h);
    static const float K[3] = {1.0f / 6.0f, 2.0f / 3.0f, 1.0f / 6.0f};
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            float occ = 0.0f;
            for (int b = 0; b < 3; b++)
                for (int a = 0; a < 3; a++) {
                    int ii = i + a - 1, jj = j + b - 1;
                    float sv = (ii < 0 || jj < 0 || ii >= w || jj >= h) ? 1.0f : 1.0f - open[jj * w + ii];
                    occ += K[a] * K[b] * sv;
                }
            float f[2];
            faces_of(open, sdf, w, i, j, f);
            float* o = &solid4[4 * (j * w + i)];
            o[0] = f[0];
            o[1] = f[1];
            o[2] = occ;
            o[3] = open[j * w + i];
        }
    regions_of(solid4, w, h, region);
    int any = 0;
    for (int s = 0; s < nshapes; s++) any |= shapes[s].temp > -1e8f;
    if (any && temp) {
        for (int k = 0; k < w * h; k++) temp[k] = NO_TEMP;
        for (int s = 0; s < nshapes; s++) {
            if (!(shapes[s].temp > -1e8f)) continue;
            float c[2], r;
            shape_bound(&shapes[s], c, &r);
            r = r + 2.0f;
            int i0 = (int)fmaxf(floorf(c[0] - r), 0.0f);
            int i1 = mini((int)fmaxf(ceilf(c[0] + r), 0.0f), w);
            int j0 = (int)fmaxf(floorf(c[1] - r), 0.0f);
            int j1 = mini((int)fmaxf(ceilf(c[1] + r), 0.0f), h);
            for (int j = j0; j < j1; j++)
                for (int i = i0; i < i1; i++)
                    if (shape_sdf(&shapes[s], (float)i + 0.5f, (float)j + 0.5f) < 0.75f) temp[j * w + i] = shapes[s].temp;
        }
    }
    free(open);
    return any;
}

/* maps.rs:455-492. Rust's f32::round rounds half away from zero, as C's roundf. */
static float rng_next(uint32_t* s) {
    *s ^= *s << 13;
    *s ^= *s >> 17;
    *s ^= *s << 5;
    return (float)(*s >> 8) / (float)(1u << 24);
}

uint32_t ofill_rect(int w, int h, int nshapes, const OShape* shapes, const float rect[4],
                    uint32_t material, OParticle* out, uint32_t n0, uint32_t cap) {
    const int sub = 2;
    const float step = 1.0f / (float)sub;
    float W = (float)w, H = (float)h;
    int x0 = (int)roundf(fmaxf(rect[0], WALL) / step);
    int x1 = (int)roundf(fminf(rect[2], W - WALL) / step);
    int y0 = (int)roundf(fmaxf(rect[1], WALL) / step);
    int y1 = (int)roundf(fminf(rect[3], H - WALL) / step);
    uint32_t rng = 0x9E3779B9u ^ (n0 * 747796405u + 1u);
    uint32_t n = n0;
    for (int j = y0; j < y1; j++)
        for (int i = x0; i < x1; i++) {
            float px = ((float)i + 0.5f + (rng_next(&rng) - 0.5f) * 0.5f) * step;
            float py = ((float)j + 0.5f + (rng_next(&rng) - 0.5f) * 0.5f) * step;
            if (oscene_sdf(w, h, nshapes, shapes, px, py) > 0.1f) {
                if (n < cap) {
                    OParticle* p = &out[n];
                    memset(p, 0, sizeof *p);
                    p->pos[0] = px;
                    p->pos[1] = py;
                    p->s = SPAWN_S;
                    p->kind = material + 1u;
                    p->t = SPAWN_TEMP;
                }
                n++;
            }
        }
    return n;
}

/* ------------------------------------------------------------------------------------ */
/* GPU-side tables: materials and parameters in grid units                                */
/* ------------------------------------------------------------------------------------ */

typedef struct GMat {   /* common.glsl:224-238 (the fields the restated passes read) */
    int ia[4], ib[4];
    float a[4], b[4], temp[4], th[4], th2[4], el[4], misc[4], rx[4];
    float rheo[4];   /* yield stress / water's density (cells^2/s^2); flow index; shear time; ratio */
    float gr[4];     /* friction; fume; fizz; unused */
} GMat;

typedef struct GParams {   /* common.glsl:37-86 (subset) */
    int grid[2];
    uint32_t n_slots;
    float dt_fixed, gravity, inv_ppc, apic_clamp;
    float pair[GROUPS][GROUPS];
    float misc[4];
    int n_present, acc_stride, n_fam;
    uint32_t group_mask, caps;
    int primary;
    uint32_t group_heat;
    int present[MAX_PRESENT];
    int fams[MAX_PRESENT][2];   /* per family: its row, its diluent's row (mod.rs:2250-2255) */
    float heat[4], heat2[4];
    float sep_tau, cfl, tool_crowd_max, density_k, dt_max, crowd_jitter, ext_speed, wall_margin;
    float tool_pos[2], tool_vel[2], tool_radius;
    int tool_mode;
    float tool_strength;
    float tol[4], ext[4], corr[4], heat3[4];
    float elastic[4];   /* stress channel, largest modulus / rho_w (cells^2/s^2), stress cap, step cap */
    float mag[4];   /* magnets, strongest susceptibility, its saturation, 1 / (rho_w dx^2) */
    float magnet[O_MAX_MAGNETS][4], magnet_dir[O_MAX_MAGNETS][4];
    float current_zone[O_MAX_CURRENTS][4];   /* common.glsl:76-77 */
    float current_vel[O_MAX_CURRENTS][4];
    float corr_gain;   /* min(1 - exp(-dt / tol.w), density_k) is per substep: see rhs */
} GParams;

typedef struct Tank {   /* mod.rs:222-245 */
    int nrows;
    int rows[MAX_PRESENT];
    int chan[MAX_PRESENT][3];
    int stride, families, primary, chan_t, chan_e;
    uint32_t group_mask;
    int chan_g[GROUPS];
} Tank;

typedef struct StepBuf {   /* common.glsl:122-135 */
    float frame_left, advanced;
    uint32_t batch_steps, batch_done;
    float dt, dt_prev;
    uint32_t umax_grid, umax_part;
    float dt_cfl;
    uint32_t substeps;
    float umax_seen;
    uint32_t pad0;
} StepBuf;

typedef struct SolveBuf {   /* common.glsl:138-149 */
    float p_rz[2], p_alpha[2], p_beta[2], p_bb[2], p_rr[2];
    uint32_t p_done[2], p_iters[2];
    uint32_t p_it_max, p_unconv, p2_it_max, p2_unconv, solves;
    float p_res_max;
    float v_rz, v_alpha, v_beta, v_r0, v_rr, v_pq;
    uint32_t v_done, v_iters, v_it_max, v_unconv;
    float v_res_max;
    uint32_t p1_iters[2], p2_last;   /* bookkeeping: the last first and second solves' iterations */
    /* the recorded iteration counts (pressure_rec, pressure2_rec, viscosity_rec), the limits a
     * frame's solves stop at, and the frame's most iterations and unconverged solves */
    uint32_t rec[3], cap[3], f_it[3], f_un[3];
} SolveBuf;

typedef struct Levels {   /* mod.rs:714-753 */
    int n;
    int dims[24][2];
    int offs[24];
    int total, tail;
    int tile_offs[24];
    int tiles;
} Levels;

struct OSim {
    int W, H;
    uint32_t capacity, n_slots;
    OSimParams prm;
    Tank tank;
    int thermal, solids_heated, cleared, grid_valid;
    uint32_t caps;
    int visc_mode;   /* 0 none, 1 explicit, 2 implicit */
    uint32_t since_sort;
    uint64_t substeps_done;
    GMat mats[O_MAX_MATERIALS];
    GParams P;
    StepBuf S;
    SolveBuf K;
    Levels lv;
    int nwg;
    double sim_time;
    /* particles */
    OParticle* particles;
    OParticle* sorted;
    /* grid */
    int32_t* acc;
    V4 *vel, *cell, *comp, *coef, *sprop, *surf, *surf2, *aux, *grho, *therm, *dheat, *vw, *vs, *prhs;
    V4* gbase;   /* per cell: share x base density of phase groups 1 - 3 (grid_prep.comp:53, 172, 247) */
    V4* rh;      /* per cell: its non-Newtonian liquid: share, row, concentration, stiff */
    float* famocc;   /* per cell and family: its occupancy (settling) */
    V2* dsettle;     /* per cell and family: the concentration gain / loss rates of settling */
    int settle_fams; /* families the settling buffers hold */
    OCurrent currents[O_MAX_CURRENTS];   /* set_currents, kept across resets */
    OMagnet magnets[O_MAX_MAGNETS];      /* set_magnets, likewise */
    int n_magnets;
    V2* magc;   /* per cell: susceptibility; magnetic energy density (magnet.comp) */
    V4* pstress;   /* per particle slot: viscoelastic stress (xx, yy, xy), in place */
    uint32_t* plook;   /* per particle slot: look.comp's four words (null until a look pass runs) */
    uint32_t frame;    /* FluidSim::frame: step calls so far (mod.rs:2402) */
    /* spray.comp's pool: entries, free stack, listed entries, foam per cell (two copies),
     * the counters (never handed out, stack height, listed), the copy counted next */
    struct ODiffuse* dpool;   /* 65536 bubbles' entries, then 131072 specks' */
    uint32_t *dstack, *dstack1, *dlist, *dcount;   /* counts: foam x 2, resting specks x 2 */
    int32_t* dfield;          /* the dust field, 4 ints a cell */
    uint32_t d_hw, d_top, d_listed, d_parity, d_hw1, d_top1;
    int d_seen;       /* a liquid that foams, fizzes or carries specks has been in the tank */
    int has_dust;     /* a liquid with specks is in the tank (set before a render) */
    V4* estr;      /* per cell: the deposited stress (elastic.comp) */
    I2* rl;        /* per cell: rigid label (root cell, -1 not rigid); its body at the root */
    int64_t* rbody;   /* per body: 15 fixed-point sums (rigid.comp) */
    uint32_t nbodies;
    int elastic_on;
    int n_currents;
    V2 *vel0, *pjump, *pres;
    float* p2keep;
    float* mixb;   /* per cell, families 1 .. n_fam - 1: the concentration (-1: not here) */
    I2* hcell;
    V4* solid;
    float* sdf;
    uint32_t* region;
    uint32_t region_air;
    float* solid_t;
    uint64_t ledger[8];
    /* multigrid / Krylov */
    V4* mga;
    float* mgd;
    V2 *mgx, *mgz, *mgr, *cgp, *cgp2, *cgq;
    uint32_t* ptile;
    V4* part;
    /* implicit viscosity (visc*.comp, vmg*.comp) */
    V2 *vr, *vr2, *vp, *vq, *vq2, *vd, *vaz;
    V4 *vma, *vmb;
    V2 *vmd, *vmr, *vmx, *vmz;
    uint32_t *tiles, *vtile;
    /* scratch for the particle pass */
    struct Scat* scat;
    /* spawn queue (mod.rs:1026, 2024-2046): taken into the buffer by the next step */
    OParticle* pending;
    uint32_t n_pending, next_id;
    float spawn_speed;
};

static int g_threads = 1;
void osim_set_threads(int n) { g_threads = n > 0 ? n : 1; }

static float tension_cells(const OSimParams* p, float sigma) {
    float dx = p->cell_size;
    return sigma / (WATER_DENSITY * dx * dx * dx);
}

static int freezes(const OMat* m) { return m->melt_hi > -273.0f; }

static float temp_factor_ln(const OMat* m, float t) {   /* material.rs:429-440 */
    float tk = maxf(t + 273.15f, 1.0f);
    float tref = m->temp_ref + 273.15f;
    float x = 0.0f;
    if (m->temp_model == 1) x = m->temp_b * (1.0f / tk - 1.0f / tref);
    else if (m->temp_model == 2) x = m->temp_b / maxf(tk - m->temp_c, 5.0f) - m->temp_b / maxf(tref - m->temp_c, 5.0f);
    return clampf(x, -30.0f, 30.0f);
}

static float viscosity_at(const OMat* m, float t) { return m->viscosity * expf(temp_factor_ln(m, t)); }

/* Tank::layout (mod.rs:271-329). rows ascending. Returns 0 if they do not fit. */
static int tank_layout(Tank* t, const int* rows, int nrows, const OSimParams* p, int thermal) {
    memset(t, 0, sizeof *t);
    if (nrows > MAX_PRESENT) return 0;
    int next = ACC_FIRST;
    uint32_t gm = 0;
    int primary = -1;
    for (int k = 0; k < nrows; k++)
        if (p->mat[rows[k]].diluent == rows[0]) { primary = k; break; }
    int families = primary >= 0 ? 1 : 0;
    for (int k = 0; k < nrows; k++) {
        const OMat* m = &p->mat[rows[k]];
        gm |= 1u << (m->group < GROUPS - 1 ? m->group : GROUPS - 1);
        int c[3] = {-1, -1, -1};
        if (k > 0 && k != primary) c[0] = next++;
        if (m->diluent >= 0) {
            c[1] = next++;
            if (k == primary) c[2] = 0;
            else c[2] = families++;
        }
        memcpy(t->chan[k], c, sizeof c);
        t->rows[k] = rows[k];
    }
    t->nrows = nrows;
    t->chan_t = thermal ? next : -1;
    next += thermal ? 1 : 0;
    for (int g = 0; g < GROUPS; g++) t->chan_g[g] = -1;
    if (thermal) {
        int first = 1;
        for (int g = 0; g < GROUPS; g++)
            if (gm & (1u << g)) {
                if (!first) t->chan_g[g] = next++;
                first = 0;
            }
    }
    int elastic = 0;   /* three stress channels when an elastic material is in (mod.rs:316-317) */
    for (int k = 0; k < nrows; k++) elastic |= p->mat[rows[k]].shear_modulus > 0.0f;
    t->chan_e = elastic ? next : -1;
    next += elastic ? 3 : 0;
    if (next > ACC_MAX) return 0;
    int stride = next > ACC_MIN ? next : ACC_MIN;
    stride = (stride + 3) / 4 * 4;
    t->stride = stride;
    t->families = families;
    t->group_mask = gm;
    t->primary = primary >= 0 ? rows[primary] : -1;
    return 1;
}

static float dt_capillary(const OSimParams* p, const Tank* t) {   /* params.rs:962-982 */
    float worst = 0.0f;
    for (int a = 0; a < t->nrows; a++) {
        if (t->rows[a] == 57) continue;
        const OMat* m = &p->mat[t->rows[a]];
        worst = maxf(worst, tension_cells(p, m->tension) / (m->density / WATER_DENSITY));
        for (int b = 0; b < t->nrows; b++) {
            if (t->rows[b] == 57) continue;
            const OMat* n = &p->mat[t->rows[b]];
            if (n->group != m->group) {
                float sigma = tension_cells(p, p->pair_tension[m->group][n->group]);
                worst = maxf(worst, sigma / (minf(m->density, n->density) / WATER_DENSITY));
            }
        }
    }
    if (worst <= 0.0f) return INFINITY;
    return 0.5f * sqrtf(1.0f / (2.0f * 3.14159274f * worst));
}

static float particle_heat_vol(const OSimParams* p, int row) {
    int r = row == 57 ? 0 : row;
    return p->mat[r].density * p->mat[r].heat_capacity;
}

static float dt_thermal(const OSimParams* p, const Tank* t) {   /* params.rs:907-914 */
    if (p->heat_rate <= 0.0f) return INFINITY;
    float dx2 = p->cell_size * p->cell_size;
    float m = INFINITY;
    for (int k = 0; k < t->nrows; k++) {
        int i = t->rows[k];
        float v = 0.2f * dx2 * particle_heat_vol(p, i) / maxf(p->mat[i].conductivity, 1e-6f) / p->heat_rate;
        m = minf(m, v);
    }
    return m;
}

/* params.rs:947-960: the longest substep that keeps elastic waves within half a cell */
static float dt_elastic(const OSimParams* p, const Tank* t) {
    float stiff = 1.0f + (p->elastic_stress_max > 0.0f ? p->elastic_stress_max : 50.0f);
    float m = INFINITY;
    for (int k = 0; k < t->nrows; k++) {
        const OMat* q = &p->mat[t->rows[k]];
        if (q->shear_modulus > 0.0f) m = minf(m, 0.5f * p->cell_size / sqrtf(stiff * q->shear_modulus / q->density));
    }
    return m;
}

static float dt_limit(const OSim* s) {   /* mod.rs:2332-2339 */
    const OSimParams* p = &s->prm;
    float dt = minf(p->dt_max, dt_capillary(p, &s->tank));
    if (s->thermal) dt = minf(dt, dt_thermal(p, &s->tank));
    return minf(dt, dt_elastic(p, &s->tank));
}

static int viscosity_mode(const OSim* s) {   /* mod.rs:2768-2792 */
    float dt = dt_limit(s);
    const OSimParams* p = &s->prm;
    float d = 0.0f;
    for (int k = 0; k < s->tank.nrows; k++) {
        const OMat* m = &p->mat[s->tank.rows[k]];
        float cells = 1.0f / (p->cell_size * p->cell_size);
        float nu;
        if (!s->thermal) nu = viscosity_at(m, p->ambient_temp) * cells;
        else if (freezes(m) || m->temp_model != 0) nu = INFINITY;
        else nu = m->viscosity * cells;
        d = maxf(d, nu * dt);
    }
    if (d <= 0.0f) return 0;
    if (d <= 0.05f) return 1;
    return 2;
}

/* mod.rs:2139-2143: a family in the tank settles (a concentrate with grains, under gravity) */
static int settles(const OSim* s) {
    if (!(s->prm.gravity > 0.0f)) return 0;
    for (int k = 0; k < s->tank.nrows; k++) {
        const OMat* m = &s->prm.mat[s->tank.rows[k]];
        if (m->diluent >= 0 && m->grain > 0.0f) return 1;
    }
    return 0;
}

/* mod.rs:2114-2136: the settling buffers for fams families; new zeroed ones when the count
 * grows or drops to none, the present ones otherwise */
static int set_settling(OSim* s, int fams) {
    if (fams == s->settle_fams || (fams > 0 && fams < s->settle_fams)) return 0;
    size_t n = (size_t)s->W * s->H * (size_t)fams;
    if (n < 1) n = 1;
    free(s->famocc);
    free(s->dsettle);
    s->famocc = calloc(n, sizeof(float));
    s->dsettle = calloc(n, sizeof(V2));
    if (!s->famocc || !s->dsettle) return -2;
    s->settle_fams = fams;
    return 0;
}

/* mod.rs:2084-2110: the particles' stress buffer while an elastic material is in the tank,
 * zero-filled each time it is taken up again */
static int set_elastic(OSim* s, int on) {
    if (on == s->elastic_on) return 0;
    if (on) {
        free(s->pstress);
        free(s->estr);
        s->pstress = calloc((size_t)s->capacity, sizeof(V4));
        s->estr = calloc((size_t)s->W * s->H, sizeof(V4));
        if (!s->pstress || !s->estr) return -2;
    }
    s->elastic_on = on;
    return 0;
}

static uint32_t compute_caps(const OSim* s) {   /* mod.rs:2717-2761 (the bits that apply) */
    const OSimParams* p = &s->prm;
    uint32_t caps = 0;
    if (s->tank.families > 0) caps |= CAP_FAMILIES;
    if (s->settle_fams >= s->tank.families && s->tank.families > 0 && settles(s)) caps |= CAP_SETTLE;
    if (s->tank.chan_e >= 0 && s->elastic_on) caps |= CAP_ELASTIC;   /* mod.rs:2746-2748 */
    if (s->thermal) caps |= CAP_THERMAL;
    int rigid = 0;
    for (int k = 0; k < s->tank.nrows; k++) {
        const OMat* m = &p->mat[s->tank.rows[k]];
        const OMat* dil = m->diluent >= 0 ? &p->mat[m->diluent] : NULL;
        if (m->rheology != 0 || m->skin > 0.0f || m->friction > 0.0f) {
            caps |= CAP_RHEO;
            rigid |= m->rheology == 2 || m->rheology == 3 || m->skin > 0.0f || m->friction > 0.0f;
        }
        if (s->thermal)
            rigid |= freezes(m) || (dil && freezes(dil)) || m->temp_model != 0 || (dil && dil->temp_model != 0);
        rigid |= viscosity_at(m, p->ambient_temp) >= p->rigid_viscosity || (!s->thermal && freezes(m) && p->ambient_temp < m->melt_hi);
    }
    if (rigid) caps |= CAP_RIGID;
    for (int k = 0; k < s->tank.nrows; k++)
        if (s->tank.rows[k] == 57 && s->thermal) caps |= CAP_STEAM;
    for (int k = 0; k < s->tank.nrows; k++)   /* mod.rs:2749-2751 */
        if (s->n_magnets > 0 && p->mat[s->tank.rows[k]].susceptibility > 0.0f) caps |= CAP_MAGNET;
    for (int k = 0; k < s->tank.nrows; k++) {   /* mod.rs:2755-2757 */
        const OMat* m = &p->mat[s->tank.rows[k]];
        if (m->react_with >= 0 && m->react_rate > 0.0f)
            for (int j = 0; j < s->tank.nrows; j++)
                if (s->tank.rows[j] == m->react_with) caps |= CAP_REACT;
    }
    return caps;
}

/* gpu_materials (mod.rs:2179-2236) */
static void build_mats(OSim* s) {
    const OSimParams* p = &s->prm;
    float dx = p->cell_size;
    for (int r = 0; r < O_MAX_MATERIALS; r++) {
        const OMat* m = &p->mat[r];
        GMat* g = &s->mats[r];
        memset(g, 0, sizeof *g);
        int chan[3] = {-1, -1, -1};
        for (int k = 0; k < s->tank.nrows; k++)
            if (s->tank.rows[k] == r) memcpy(chan, s->tank.chan[k], sizeof chan);
        float ang = m->contact_angle * (3.14159274f / 180.0f);
        float sn = sinf(ang), cs = cosf(ang);
        float solid = m->density_solid > 0.0f ? m->density_solid : m->density;
        float cvol = particle_heat_vol(p, r);
        float ln_nu = logf(maxf(m->viscosity / (dx * dx), 1e-8f));
        float rho = m->density;
        if (!s->thermal) {
            ln_nu += temp_factor_ln(m, p->ambient_temp);
            rho *= clampf(1.0f - m->expansion * (p->ambient_temp - m->temp_ref), 0.7f, 1.3f);
            if (freezes(m) && m->diluent < 0 && p->ambient_temp < m->melt_hi) {
                float fs = clampf((m->melt_hi - p->ambient_temp) / maxf(m->melt_hi - m->melt_lo, 1e-3f), 0.0f, 1.0f);
                float frozen = maxf(logf(p->rigid_viscosity / (dx * dx)), ln_nu);
                ln_nu += (frozen - ln_nu) * fs;
                rho += (solid - rho) * fs;
            }
        }
        g->ia[0] = (int)(m->group < GROUPS - 1 ? m->group : GROUPS - 1);
        g->ia[1] = m->diluent;
        g->ia[2] = chan[0];
        g->ia[3] = chan[1];
        g->ib[0] = chan[2];
        g->ib[1] = (int)m->rheology;
        g->ib[2] = (int)m->temp_model;
        g->ib[3] = -1;
        g->a[0] = rho / WATER_DENSITY;
        g->a[1] = ln_nu;
        g->a[2] = tension_cells(p, m->tension);
        g->a[3] = m->mix_rate;
        g->b[0] = cs;
        g->b[1] = sn;
        g->b[2] = m->grain / dx;
        g->b[3] = solid / WATER_DENSITY;
        g->temp[0] = m->temp_b;
        g->temp[1] = m->temp_c;
        g->temp[2] = m->temp_ref + 273.15f;
        g->temp[3] = tension_cells(p, m->skin);
        g->th[0] = cvol / WATER_HEAT;
        g->th[1] = m->conductivity / (WATER_HEAT * dx * dx);
        g->th[2] = maxf(m->melt_lo, NO_MELT);
        g->th[3] = maxf(maxf(m->melt_hi, m->melt_lo + 0.25f), NO_MELT);
        g->th2[0] = (freezes(m) || m->diluent >= 0) ? m->latent / m->heat_capacity : 0.0f;
        g->th2[1] = m->emissivity;
        g->th2[2] = m->boil;
        g->th2[3] = m->latent_vap / m->heat_capacity;
        g->el[0] = m->shear_modulus / (WATER_DENSITY * dx * dx);   /* mod.rs:2184 stress() */
        g->el[1] = m->relax_time;
        g->el[2] = m->susceptibility;
        g->misc[0] = m->freeze_shift;
        g->misc[1] = m->load;
        g->misc[2] = 1.0f;
        g->misc[3] = m->expansion;
        g->rx[2] = m->self_heat / m->heat_capacity;
        g->rx[3] = m->volatility;
        g->rheo[0] = m->yield_stress / (WATER_DENSITY * dx * dx);   /* mod.rs:2184 stress() */
        g->rheo[1] = m->flow_index;
        g->rheo[2] = m->shear_time;
        g->rheo[3] = m->visc_ratio;
        g->gr[0] = m->friction;
        g->gr[1] = m->fume;
    }
}

static float speed_cap_cells(const OSimParams* p, int height) {
    float g = p->gravity / p->cell_size;
    if (p->speed_cap > 0.0f && g > 0.0f) return p->speed_cap * sqrtf(2.0f * g * (float)height);
    return 1e30f;
}

static float tool_speed(const OTool* t) {   /* params.rs:1201-1208 */
    switch (t->mode) {
    case 1: return hypotf(t->vel[0], t->vel[1]) + 4.0f * t->radius;
    case 3:
    case 4: return hypotf(t->vel[0], t->vel[1]);
    case 7: return fabsf(t->vel[0]) + 2.0f * t->radius;
    default: return 0.0f;
    }
}

/* gpu_params (mod.rs:2238-2328) */
static void build_params(OSim* s, const OTool* tool) {
    const OSimParams* p = &s->prm;
    GParams* P = &s->P;
    memset(P, 0, sizeof *P);
    float dx = p->cell_size;
    P->grid[0] = s->W;
    P->grid[1] = s->H;
    P->n_slots = s->n_slots;
    P->dt_fixed = p->fixed_hz > 0.0f ? 1.0f / p->fixed_hz : 0.0f;
    P->gravity = p->gravity / p->cell_size;
    P->inv_ppc = 1.0f / (float)PPC;
    P->apic_clamp = p->apic_clamp;
    for (int a = 0; a < GROUPS; a++)
        for (int b = 0; b < GROUPS; b++) P->pair[a][b] = tension_cells(p, p->pair_tension[a][b]);
    P->misc[0] = p->curvature_max;
    P->misc[1] = (float)p->sealed_vent;
    P->misc[2] = p->cell_size;
    P->misc[3] = p->rigid_contact != 0 ? p->rigid_friction : -1.0f;   /* mod.rs:2280 */
    P->n_present = s->tank.nrows;
    P->acc_stride = s->tank.stride > ACC_MIN ? s->tank.stride : ACC_MIN;
    P->n_fam = s->tank.families;
    P->group_mask = s->tank.group_mask;
    P->caps = s->caps;
    P->primary = s->tank.nrows == 0 ? -1 : s->tank.primary;
    uint32_t gh = 0;
    for (int g = 0; g < GROUPS; g++) gh += ((uint32_t)(s->tank.chan_g[g] + 1) & 255u) << (8 * g);
    P->group_heat = gh;
    for (int k = 0; k < s->tank.nrows; k++) P->present[k] = s->tank.rows[k];
    for (int j = 0; j < MAX_PRESENT; j++) P->fams[j][0] = P->fams[j][1] = -1;
    for (int k = 0; k < s->tank.nrows; k++)
        if (s->tank.chan[k][2] >= 0) {
            P->fams[s->tank.chan[k][2]][0] = s->tank.rows[k];
            P->fams[s->tank.chan[k][2]][1] = p->mat[s->tank.rows[k]].diluent;
        }
    P->heat[0] = p->ambient_temp;
    P->heat[1] = p->heat_rate;
    P->heat[2] = p->air_cooling / (WATER_HEAT * dx);
    P->heat[3] = STEFAN_BOLTZMANN / (WATER_HEAT * dx);
    P->heat2[0] = logf(p->rigid_viscosity / (dx * dx));
    P->heat2[1] = p->heat_power;
    P->heat2[2] = (float)s->tank.chan_t;
    P->heat2[3] = p->contact_heat / (WATER_HEAT * dx);
    P->sep_tau = p->droplet_cells;
    P->cfl = p->cfl;
    P->tool_crowd_max = p->tool_crowd_max;
    P->density_k = p->correction_max;
    P->dt_max = dt_limit(s);
    P->crowd_jitter = p->crowd_jitter;
    P->ext_speed = maxf(tool ? tool_speed(tool) : 0.0f, s->spawn_speed);   /* mod.rs:2300 */
    P->wall_margin = 0.1f;
    if (tool) {
        P->tool_pos[0] = tool->pos[0];
        P->tool_pos[1] = tool->pos[1];
        P->tool_vel[0] = tool->vel[0];
        P->tool_vel[1] = tool->vel[1];
        P->tool_radius = maxf(tool->radius, 0.01f);
        P->tool_mode = tool->mode;
        P->tool_strength = tool->strength;
    } else {
        P->tool_radius = 0.01f;
    }
    P->tol[0] = p->pressure_tol;
    P->tol[1] = p->correction_tol;
    P->tol[2] = p->viscosity_tol;
    P->tol[3] = p->correction_time;
    P->ext[0] = speed_cap_cells(p, s->H);
    P->ext[1] = (float)p->advection_order;
    P->ext[2] = p->spray_cfl;
    P->ext[3] = (float)s->n_currents;
    for (int i = 0; i < s->n_currents; i++) {   /* mod.rs:2265-2270 */
        const OCurrent* c = &s->currents[i];
        P->current_zone[i][0] = c->pos[0];
        P->current_zone[i][1] = c->pos[1];
        P->current_zone[i][2] = maxf(c->radius, 0.01f);
        P->current_zone[i][3] = c->rate;
        P->current_vel[i][0] = c->vel[0];
        P->current_vel[i][1] = c->vel[1];
    }
    P->corr[0] = p->correction_step_max;
    P->corr[1] = p->correction_deadband;
    P->corr[2] = (float)p->slip_cap;
    P->corr[3] = p->implicit_viscosity_min;
    P->heat3[0] = maxf(p->eddy_heat, 0.0f);
    P->heat3[1] = p->evaporation ? 2.257e6f / 1005.0f : 0.0f;
    P->heat3[2] = 0.0f;
    P->heat3[3] = clampf(p->magnet_demag, 0.0f, 1.0f);
    float gmax = 0.0f;   /* mod.rs:2316-2321 */
    for (int k = 0; k < s->tank.nrows; k++) gmax = maxf(gmax, p->mat[s->tank.rows[k]].shear_modulus);
    P->elastic[0] = (float)s->tank.chan_e;
    P->elastic[1] = maxf(gmax, 1e-3f) / (WATER_DENSITY * p->cell_size * p->cell_size);
    P->elastic[2] = p->elastic_stress_max;
    P->elastic[3] = p->elastic_step_max;
    float chi_max = 0.0f, sat = 0.05f;   /* mod.rs:2264 */
    for (int k = 0; k < s->tank.nrows; k++) {
        const OMat* m = &p->mat[s->tank.rows[k]];
        if (m->susceptibility > chi_max) {
            chi_max = m->susceptibility;
            sat = m->saturation;
        }
    }
    P->mag[0] = (float)s->n_magnets;
    P->mag[1] = maxf(chi_max, 1e-6f);
    P->mag[2] = sat;
    P->mag[3] = 1.0f / (WATER_DENSITY * p->cell_size * p->cell_size);
    for (int i = 0; i < s->n_magnets; i++) {   /* mod.rs:2258-2263 */
        const OMagnet* m = &s->magnets[i];
        P->magnet[i][0] = m->pos[0];
        P->magnet[i][1] = m->pos[1];
        P->magnet[i][2] = maxf(m->radius, 0.5f);
        P->magnet[i][3] = m->strength;
        P->magnet_dir[i][0] = m->dir[0];
        P->magnet_dir[i][1] = m->dir[1];
    }
}

/* Levels::new (mod.rs:734-753) */
static void levels_new(Levels* L, int w, int h) {
    memset(L, 0, sizeof *L);
    L->dims[0][0] = w;
    L->dims[0][1] = h;
    L->n = 1;
    while (L->dims[L->n - 1][0] * L->dims[L->n - 1][1] > COARSEST_CELLS) {
        int pw = L->dims[L->n - 1][0], ph = L->dims[L->n - 1][1];
        L->dims[L->n][0] = (pw + 1) / 2;
        L->dims[L->n][1] = (ph + 1) / 2;
        L->n++;
    }
    int total = 0;
    for (int l = 0; l < L->n; l++) {
        L->offs[l] = total;
        total += L->dims[l][0] * L->dims[l][1];
    }
    L->total = total;
    int tail = L->n - 1;
    for (int l = 1; l < L->n; l++)
        if (L->dims[l][0] * L->dims[l][1] <= TAIL_CELLS) { tail = l; break; }
    if (tail < 1) tail = 1;
    if (tail > L->n - 1) tail = L->n - 1;
    L->tail = tail;
    int tiles = 0;
    for (int l = 0; l <= tail; l++) {
        L->tile_offs[l] = tiles;
        tiles += ((L->dims[l][0] + 15) / 16) * ((L->dims[l][1] + 15) / 16);
    }
    L->tiles = tiles;
}

/* ------------------------------------------------------------------------------------ */
/* Helpers over the tables (common.glsl)                                                 */
/* ------------------------------------------------------------------------------------ */

#define P_ (s->P)
static inline int cidx(const OSim* s, int x, int y) { return y * s->W + x; }
static inline int face_live(float st) { return fabsf(st) < 1e29f; }
static inline int face_closed(float st) { return st < -1e29f; }
static inline int has_cap(const OSim* s, uint32_t c) { return (s->caps & c) != 0u; }

static float row_density(const OSim* s, uint32_t row, float sc) {   /* common.glsl:475-479 */
    int d = s->mats[row].ia[1];
    float rho = s->mats[row].a[0];
    return d >= 0 ? mixf(s->mats[d].a[0], rho, sc) : rho;
}

/* common.glsl:590-602: whether phase group g drifts within itself (two or more plain liquids
 * of the group in the tank, and no concentrate in or of it) */
static int group_sorts(const OSim* s, int g) {
    if (g <= 0) return 0;
    int n = 0;
    for (int j = 0; j < P_.n_present; j++) {
        const int* ia = s->mats[P_.present[j]].ia;
        if (ia[1] >= 0 && s->mats[ia[1]].ia[0] == g) return 0;
        if (ia[0] != g) continue;
        if (ia[1] >= 0) return 0;
        n++;
    }
    return n >= 2;
}

/* common.glsl:370-374: terminal velocity of a droplet, drag 24 / Re + 0.44 */
static float terminal(const OSim* s, float drho, float rho_c, float nu_c, float d) {
    float qa = 0.44f * rho_c, qb = 24.0f * nu_c * rho_c / d, qc = 4.0f / 3.0f * fabsf(drho) * P_.gravity * d;
    return qc > 0.0f ? 2.0f * qc / (qb + sqrtf(qb * qb + 4.0f * qa * qc)) : 0.0f;
}

static float v4c(V4 v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }
static int lead4(V4 f) { return f.x >= maxf(f.y, maxf(f.z, f.w)) ? 0 : f.y >= maxf(f.z, f.w) ? 1 : f.z >= f.w ? 2 : 3; }

static float expansion_of(const OSim* s, uint32_t row, float sc, float T) {   /* common.glsl:485-494 */
    const GMat* m = &s->mats[row];
    int d = m->ia[1];
    float b = m->misc[3], tr = m->temp[2] - 273.15f, tb = m->th2[2];
    if (d >= 0) {
        b = mixf(s->mats[d].misc[3], b, sc);
        tr = mixf(s->mats[d].temp[2] - 273.15f, tr, sc);
        tb = mixf(s->mats[d].th2[2], tb, sc);
    }
    return clampf(1.0f - b * (minf(T, tb) - tr), 0.7f, 1.3f);
}

static V4 thermal_of(const OSim* s, uint32_t row, float sc) {   /* common.glsl:500-509 */
    const GMat* m = &s->mats[row];
    float ld = m->th2[0];
    int d = m->ia[1];
    if (d < 0) return v4(m->th[2], m->th[3], ld, m->th[0]);
    const float* dth = s->mats[d].th;
    float shift = m->misc[0] * sc;
    float C = mixf(dth[0], m->th[0], sc);
    return v4(dth[2] + shift, dth[3] + shift, mixf(dth[0] * s->mats[d].th2[0], m->th[0] * ld, sc) / C, C);
}

/* particles.comp:78-80: the enthalpy temperature that keeps the heat when the heat capacity
 * changes from c0 to c1 */
static float keep_heat(float t, float c0, float c1) { return c0 == c1 ? t : (t + 273.15f) * c0 / c1 - 273.15f; }

static V2 phase_of(float te, V4 m) {   /* common.glsl:515-521 */
    if (te >= m.y) return v2(te, 0.0f);
    float lo = m.x - m.z;
    if (te <= lo) return v2(te + m.z, 1.0f);
    float fr = (te - lo) / (m.y - lo);
    return v2(m.x + fr * (m.y - m.x), 1.0f - fr);
}

static float temp_law(const OSim* s, int r, float T) {   /* common.glsl:410-417 */
    int model = s->mats[r].ib[2];
    if (model == 0) return 0.0f;
    const float* tp = s->mats[r].temp;
    float Tk = maxf(T + 273.15f, 1.0f);
    float x = model == 1 ? tp[0] * (1.0f / Tk - 1.0f / tp[2])
                         : tp[0] / maxf(Tk - tp[1], 5.0f) - tp[0] / maxf(tp[2] - tp[1], 5.0f);
    return clampf(x, -30.0f, 30.0f);
}

static int group_heat_chan(const OSim* s, int g) { return (int)((P_.group_heat >> (8u * (uint32_t)g)) & 255u) - 1; }

static void bspline(float fx, float fy, V2 w[3]) {   /* common.glsl:639-643 */
    w[0] = v2(0.5f * (1.5f - fx) * (1.5f - fx), 0.5f * (1.5f - fy) * (1.5f - fy));
    w[1] = v2(0.75f - (fx - 1.0f) * (fx - 1.0f), 0.75f - (fy - 1.0f) * (fy - 1.0f));
    w[2] = v2(0.5f * (fx - 0.5f) * (fx - 0.5f), 0.5f * (fy - 0.5f) * (fy - 0.5f));
}

static void ledger_add(OSim* s, int entry, float v) {   /* common.glsl:448-453 */
    uint32_t x = (uint32_t)(v * LEDGER_SCALE + 0.5f);
    if (x == 0u) return;
#pragma omp atomic
    s->ledger[entry] += x;
}

/* air.glsl:13-22 */
static float sample_sdf(const OSim* s, V2 x, V2* grad) {
    float gx = clampf(x.x, 0.0f, (float)s->W - 0.001f), gy = clampf(x.y, 0.0f, (float)s->H - 0.001f);
    int ix = (int)gx, iy = (int)gy;
    float fx = gx - (float)ix, fy = gy - (float)iy;
    int w1 = s->W + 1;
    int k = iy * w1 + ix;
    float d00 = s->sdf[k], d10 = s->sdf[k + 1], d01 = s->sdf[k + w1], d11 = s->sdf[k + w1 + 1];
    grad->x = mixf(d10 - d00, d11 - d01, fy);
    grad->y = mixf(d01 - d00, d11 - d10, fx);
    return mixf(mixf(d00, d10, fx), mixf(d01, d11, fx), fy);
}

/* air.glsl:31-37 */
static V2 tool_target(const OSim* s, V2 d) {
    float l = len2(d);
    if (P_.tool_mode == 3) { float q = maxf(l, 0.15f * P_.tool_radius); return v2(-d.x / q * P_.tool_vel[0], -d.y / q * P_.tool_vel[0]); }
    if (P_.tool_mode == 4) return v2(P_.tool_vel[0], P_.tool_vel[1]);
    if (P_.tool_mode == 7) {
        float q = maxf(l, 0.4f * P_.tool_radius);
        return v2(d.y / q * P_.tool_vel[0] + d.x * 2.0f, -d.x / q * P_.tool_vel[0] + d.y * 2.0f);
    }
    if (P_.tool_mode == 8) return v2(0.0f, 0.0f);
    return v2(P_.tool_vel[0] + d.x * 4.0f, P_.tool_vel[1] + d.y * 4.0f);
}

/* air.glsl:41-78 */
static V2 sample_vel(const OSim* s, V2 x, V2 fallback) {
    V2 o = fallback;
    {
        float gx = x.x, gy = x.y - 0.5f;
        int bx = (int)floorf(gx), by = (int)floorf(gy);
        float fx = gx - (float)bx, fy = gy - (float)by;
        float sw = 0.0f, su = 0.0f;
        for (int b = 0; b < 2; b++)
            for (int a = 0; a < 2; a++) {
                V4 q = s->vel[cidx(s, bx + a, by + b)];
                if (face_live(q.z)) {
                    float wt = (a == 0 ? 1.0f - fx : fx) * (b == 0 ? 1.0f - fy : fy);
                    sw += wt;
                    su += wt * q.x;
                }
            }
        if (sw > 1e-3f) o.x = su / sw;
    }
    {
        float gx = x.x - 0.5f, gy = x.y;
        int bx = (int)floorf(gx), by = (int)floorf(gy);
        float fx = gx - (float)bx, fy = gy - (float)by;
        float sw = 0.0f, su = 0.0f;
        for (int b = 0; b < 2; b++)
            for (int a = 0; a < 2; a++) {
                V4 q = s->vel[cidx(s, bx + a, by + b)];
                if (face_live(q.w)) {
                    float wt = (a == 0 ? 1.0f - fx : fx) * (b == 0 ? 1.0f - fy : fy);
                    sw += wt;
                    su += wt * q.y;
                }
            }
        if (sw > 1e-3f) o.y = su / sw;
    }
    return o;
}

/* particles.comp:51-65 */
static int collide(const OSim* s, V2* x, V2* v, int beyond) {
    V2 n;
    float d = sample_sdf(s, *x, &n);
    if (d < P_.wall_margin) {
        float l = len2(n);
        if (l > 1e-5f) {
            n.x /= l;
            n.y /= l;
            float push = P_.wall_margin - d + (beyond ? maxf(-d, 0.0f) : 0.0f);
            x->x += n.x * push;
            x->y += n.y * push;
            float vn = v->x * n.x + v->y * n.y;
            if (vn < 0.0f) {
                v->x -= vn * n.x;
                v->y -= vn * n.y;
            }
            return 1;
        }
    }
    return 0;
}

/* particles.comp:70-73 */
static I2 heat_quanta(float C, float T) {
    int ci = (int)floorf(C * MASS_SCALE + 0.5f);
    I2 r = {ci, (int)floorf((float)ci * (T + 273.15f) / T_SCALE + 0.5f)};
    return r;
}

/* ------------------------------------------------------------------------------------ */
/* step.comp                                                                             */
/* ------------------------------------------------------------------------------------ */

static void k_step(OSim* s) {
    StepBuf* S = &s->S;
    float u = maxf(minf(bitsf(S->umax_grid), P_.ext[0]), bitsf(S->umax_part));
    u = maxf(u, P_.ext_speed);
    float dt_cfl = P_.cfl / (u + sqrtf(5.0f * maxf(P_.gravity, 0.0f)) + 1e-6f);
    float dt;
    if (P_.dt_fixed > 0.0f) {
        dt = P_.dt_fixed;
    } else {
        uint32_t left = S->batch_steps > S->batch_done ? S->batch_steps - S->batch_done : 1u;
        dt = minf(minf(dt_cfl, P_.dt_max), maxf(S->frame_left, 0.0f) / (float)left);
    }
    dt = maxf(dt, 1e-6f);
    S->dt_prev = S->dt > 0.0f ? S->dt : dt;
    S->dt = dt;
    S->dt_cfl = minf(dt_cfl, P_.dt_max);
    S->umax_seen = u;
    S->frame_left -= dt;
    float lo = bitsf(S->pad0);
    float y = dt - lo;
    float t = S->advanced + y;
    S->pad0 = fbits((t - S->advanced) - y);
    S->advanced = t;
    S->batch_done += 1u;
    S->substeps += 1u;
    S->umax_grid = 0u;
    S->umax_part = 0u;
    s->region_air = 0u;
}

/* ------------------------------------------------------------------------------------ */
/* particles.comp                                                                        */
/* ------------------------------------------------------------------------------------ */

typedef struct Scat {
    int live;
    V2 pos, vs;
    V4 Cs;
    float rho, sc, CT;
    int cw, cs, ct, cg;
    int ce;     /* stress channel, -1: nothing to deposit */
    V4 te;      /* stress / the largest modulus x STRESS_FIX */
} Scat;

static void report_umax(uint32_t* slot, float m) {
    uint32_t b = fbits(m);
#pragma omp critical(umax)
    {
        if (m > bitsf(*slot)) *slot = b;
    }
}

/* advance() (particles.comp:98-985) restricted to the capabilities the oracle carries:
 * single phase group or several without drift, no families, no rigid bodies, elasticity,
 * settling, steam, reactions or evaporation; thermal conduction and exchange supported. */
#define O_MAX_BODIES 4096   /* common.glsl: MAX_BODIES */
typedef struct { float x, y, z; } V3f;
static float row_lnu(const OSim* s, uint32_t row, float sc, float T, int thermal);
static int body_motion(const OSim* s, int b, int r, V2 x, V3f* u);

static void advance(OSim* s, uint32_t id, int gather, Scat* g) {
    g->live = 0;
    if (id >= P_.n_slots) return;
    OParticle p = s->particles[id];
    if (p.kind == KIND_DEAD) return;
    if ((p.kind & 255u) == 0u) return;   /* puffs are not made by the supported tanks */
    float dt = s->S.dt;
    uint32_t row = (p.kind & 255u) - 1u;
    const int* Mia = s->mats[row].ia;
    int fam = s->mats[row].ib[0];   /* particles.comp:143 */
    int thermal = has_cap(s, CAP_THERMAL);
    V2 pos = v2(p.pos[0], p.pos[1]);
    /* particles.comp:144-151: frozen, or too viscous to flow: part of a rigid body */
    int rigid_cap = has_cap(s, CAP_RIGID);
    int frozen = 0;
    if (rigid_cap) {
        V2 ph = thermal ? phase_of(p.t, thermal_of(s, row, p.s)) : v2(P_.heat[0], 0.0f);
        frozen = ph.y > 0.5f || row_lnu(s, row, p.s, ph.x, thermal) >= P_.heat2[0];
    }
    int held = 0;
    /* viscoelastic stress (particles.comp:152-156) */
    int elastic = has_cap(s, CAP_ELASTIC);
    V4 tau = v4(0.0f, 0.0f, 0.0f, 0.0f);
    if (elastic && (p.kind & KIND_FRESH) == 0u && s->mats[row].el[0] > 0.0f) tau = s->pstress[id];
    if (gather) {
        V2 v = v2(p.vel[0], p.vel[1]);
        V4 C = v4(p.c[0], p.c[1], p.c[2], p.c[3]);
        V2 corr = v2(0.0f, 0.0f);
        float slip = 0.0f, crowd = 0.0f;
        V2 w[3];
        /* u faces */
        {
            V2 gp = v2(pos.x - 0.0f, pos.y - 0.5f);
            int bx = (int)floorf(gp.x - 0.5f), by = (int)floorf(gp.y - 0.5f);
            float fx = gp.x - (float)bx, fy = gp.y - (float)by;
            bspline(fx, fy, w);
            float sw = 0.0f, su = 0.0f, sc = 0.0f;
            V2 sd = v2(0, 0), sud = v2(0, 0);
            for (int b = 0; b < 3; b++)
                for (int a = 0; a < 3; a++) {
                    V4 q = s->vel[cidx(s, bx + a, by + b)];
                    if (face_live(q.z)) {
                        float wt = w[a].x * w[b].y;
                        V2 d = v2((float)a - fx, (float)b - fy);
                        sw += wt;
                        su += wt * q.x;
                        sc += wt * q.z;
                        sd.x += wt * d.x;
                        sd.y += wt * d.y;
                        sud.x += wt * q.x * d.x;
                        sud.y += wt * q.x * d.y;
                    }
                }
            if (sw > 1e-4f) {
                float u = su / sw;
                v.x = u;
                corr.x = sc / sw;
                C.x = 4.0f * (sud.x - u * sd.x) / sw;
                C.y = 4.0f * (sud.y - u * sd.y) / sw;
            }
        }
        /* v faces */
        {
            V2 gp = v2(pos.x - 0.5f, pos.y - 0.0f);
            int bx = (int)floorf(gp.x - 0.5f), by = (int)floorf(gp.y - 0.5f);
            float fx = gp.x - (float)bx, fy = gp.y - (float)by;
            bspline(fx, fy, w);
            float sw = 0.0f, su = 0.0f, sc = 0.0f;
            V2 sd = v2(0, 0), sud = v2(0, 0);
            for (int b = 0; b < 3; b++)
                for (int a = 0; a < 3; a++) {
                    V4 q = s->vel[cidx(s, bx + a, by + b)];
                    if (face_live(q.w)) {
                        float wt = w[a].x * w[b].y;
                        V2 d = v2((float)a - fx, (float)b - fy);
                        sw += wt;
                        su += wt * q.y;
                        sc += wt * q.w;
                        sd.x += wt * d.x;
                        sd.y += wt * d.y;
                        sud.x += wt * q.y * d.x;
                        sud.y += wt * q.y * d.y;
                    }
                }
            if (sw > 1e-4f) {
                float u = su / sw;
                v.y = u;
                corr.y = sc / sw;
                C.z = 4.0f * (sud.x - u * sd.x) / sw;
                C.w = 4.0f * (sud.y - u * sd.y) / sw;
            }
        }
        /* particles.comp:222-248: a frozen particle, a yield-stress plug's particle in a sparse
         * cell, or any particle in a rigid cell moves exactly with the body around it */
        if (rigid_cap) {
            int pcx = clampi((int)pos.x, 0, s->W - 1), pcy = clampi((int)pos.y, 0, s->H - 1);
            int plug = (s->mats[row].rheo[0] > 0.0f || s->mats[row].temp[3] > 0.0f) && s->cell[cidx(s, pcx, pcy)].w <= 0.0f;
            int c0x = clampi((int)pos.x, 1, s->W - 2), c0y = clampi((int)pos.y, 1, s->H - 2);
            int in_body = row != 57u && s->rl[cidx(s, c0x, c0y)].x >= 0;
            if (frozen || plug || in_body) {
                static const int ox[9] = {0, -1, 1, 0, 0, -1, 1, -1, 1}, oy[9] = {0, 0, 0, -1, 1, -1, -1, 1, 1};
                for (int k = 0; k < 9 && !held; k++) {
                    int root = s->rl[cidx(s, c0x + ox[k], c0y + oy[k])].x;
                    if (root < 0 || s->rl[root].y < 0) continue;
                    V3f u;
                    if (body_motion(s, s->rl[root].y, root, pos, &u)) {
                        v = v2(u.x, u.y);
                        C = v4(0.0f, -u.z, u.z, 0.0f);
                        held = 1;
                    }
                }
            }
        }
        /* the upper-convected Maxwell update (particles.comp:250-279) */
        if (elastic) {
            float G = s->mats[row].el[0];
            if (G > 0.0f) {
                float l00 = C.x, l01 = C.y, l10 = C.z, l11 = C.w;   /* L = [[du/dx, du/dy], [dv/dx, dv/dy]] */
                float lnorm = sqrtf(C.x * C.x + C.y * C.y + C.z * C.z + C.w * C.w) * dt;
                if (P_.elastic[3] > 0.0f && lnorm > P_.elastic[3]) {
                    float k = P_.elastic[3] / lnorm;
                    l00 *= k; l01 *= k; l10 *= k; l11 *= k;
                }
                float t00 = tau.x, t01 = tau.z, t10 = tau.z, t11 = tau.y;
                /* D = L T + T L^T + G (L + L^T) */
                float d00 = ((l00 * t00 + l01 * t10) + (t00 * l00 + t01 * l01)) + G * (l00 + l00);
                float d01 = ((l00 * t01 + l01 * t11) + (t00 * l10 + t01 * l11)) + G * (l01 + l10);
                float d10 = ((l10 * t00 + l11 * t10) + (t10 * l00 + t11 * l01)) + G * (l10 + l01);
                float d11 = ((l10 * t01 + l11 * t11) + (t10 * l10 + t11 * l11)) + G * (l11 + l11);
                float lam = maxf(s->mats[row].el[1], 1e-4f);
                float den = 1.0f + dt / lam;
                float n00 = (t00 + dt * d00) / den, n01 = (t01 + dt * d01) / den;
                float n10 = (t10 + dt * d10) / den, n11 = (t11 + dt * d11) / den;
                tau = v4(n00, n11, 0.5f * (n01 + n10), 0.0f);
                float tn = sqrtf(tau.x * tau.x + tau.y * tau.y + tau.z * tau.z);
                if (P_.elastic[2] > 0.0f && tn > P_.elastic[2] * G) {
                    float k = P_.elastic[2] * G / tn;
                    tau = v4(tau.x * k, tau.y * k, tau.z * k, tau.w * k);
                }
                int c1x = clampi((int)pos.x, 1, s->W - 2), c1y = clampi((int)pos.y, 1, s->H - 2);
                float around = 0.0f;
                for (int b = -1; b <= 1; b++)
                    for (int a = -1; a <= 1; a++) around += minf(s->cell[cidx(s, c1x + a, c1y + b)].x, 1.0f);
                if (around < 1.0f) tau = v4(0.0f, 0.0f, 0.0f, 0.0f);
            }
            s->pstress[id] = tau;
        }
        if (P_.apic_clamp > 0.0f) {
            float lim = P_.apic_clamp / dt;
            C.x = clampf(C.x, -lim, lim);
            C.y = clampf(C.y, -lim, lim);
            C.z = clampf(C.z, -lim, lim);
            C.w = clampf(C.w, -lim, lim);
        }
        if (P_.corr[0] > 0.0f) {
            float cl = len2(corr), cmax = P_.corr[0] / dt;
            if (cl > cmax) {
                corr.x *= cmax / cl;
                corr.y *= cmax / cl;
            }
        }
        /* composition (particles.comp:288-571) */
        {
            V2 gp = v2(pos.x - 0.5f, pos.y - 0.5f);
            int bx = (int)floorf(gp.x - 0.5f), by = (int)floorf(gp.y - 0.5f);
            float fx = gp.x - (float)bx, fy = gp.y - (float)by;
            bspline(fx, fy, w);
            /* sw: weight of the cells holding liquid; sfw, sfs: weight and concentration of
             * those holding the particle's own family (a diluent's: family 0) */
            float sw = 0.0f, sfw = 0.0f, sfs = 0.0f;
            const int nmix = P_.n_fam - 1;
            /* sg: shares of groups 1 - 3; sbg: share x base density of the particle's group */
            float sg[3] = {0.0f, 0.0f, 0.0f}, sbg = 0.0f;
            const int more = (P_.group_mask & 12u) != 0u;
            const int groups = (P_.group_mask & (P_.group_mask - 1u)) != 0u;
            const int sorts = group_sorts(s, Mia[0]);
            for (int b = 0; b < 3; b++)
                for (int a = 0; a < 3; a++) {
                    int ci = cidx(s, bx + a, by + b);
                    V4 q = s->comp[ci];
                    float wt = w[a].x * w[b].y;
                    crowd += wt * q.w;
                    if (q.x > 0.0f) {
                        sw += wt;
                        sg[0] += wt * q.y;
                        if (more) {
                            sg[1] += wt * s->aux[ci].z;
                            sg[2] += wt * s->aux[ci].w;
                        }
                        if (sorts) sbg += wt * v4c(s->gbase[ci], Mia[0] - 1);
                        float sb = fam > 0 ? s->mixb[(size_t)ci * nmix + fam - 1] : q.z;
                        if (sb >= 0.0f) {
                            sfw += wt;
                            sfs += wt * sb;
                        }
                    }
                }
            /* settling: each cell's change of its family's concentration (particles.comp:331-352) */
            {
                int dil0 = fam < 0 && P_.primary >= 0 && P_.fams[0][1] == (int)row;
                int sf = dil0 ? 0 : fam;
                if ((s->caps & CAP_SETTLE) && sf >= 0 && (p.kind & KIND_FRESH) == 0u && s->mats[dil0 ? (uint32_t)P_.primary : row].b[2] > 0.0f) {
                    V2 ds = v2(0.0f, 0.0f);
                    for (int b = 0; b < 3; b++)
                        for (int a = 0; a < 3; a++) {
                            V2 v = s->dsettle[(size_t)cidx(s, bx + a, by + b) * P_.n_fam + sf];
                            float wt = w[a].x * w[b].y;
                            ds.x += wt * v.x;
                            ds.y += wt * v.y;
                        }
                    float s0 = dil0 ? 0.0f : p.s;
                    float s1 = clampf(s0 + (1.0f - s0) * ds.x - s0 * ds.y, 0.0f, 1.0f);
                    float c0 = thermal ? thermal_of(s, row, p.s).w : 0.0f;
                    if (dil0 && s1 > 0.0f) {
                        row = (uint32_t)P_.primary;
                        Mia = s->mats[row].ia;
                        fam = 0;
                        p.kind = (p.kind & ~255u) | (row + 1u);
                    }
                    if (!dil0 || s1 > 0.0f) p.s = s1;
                    if (thermal) p.t = keep_heat(p.t, c0, thermal_of(s, row, p.s).w);
                }
            }
            if (thermal && (p.kind & KIND_FRESH) == 0u) {
                float dT = 0.0f;
                for (int b = 0; b < 3; b++)
                    for (int a = 0; a < 3; a++) dT += w[a].x * w[b].y * s->dheat[cidx(s, bx + a, by + b)].x;
                int ox = clampi((int)floorf(pos.x), 0, s->W - 1), oy = clampi((int)floorf(pos.y), 0, s->H - 1);
                V4 own = s->dheat[cidx(s, ox, oy)];
                if (own.y > 0.0f) {
                    V4 th = thermal_of(s, row, p.s);
                    float tb = Mia[1] >= 0 ? mixf(s->mats[Mia[1]].th2[2], s->mats[row].th2[2], p.s) : s->mats[row].th2[2];
                    I2 q = heat_quanta(th.w, minf(phase_of(p.t, th).x, tb));
                    dT += own.y * (own.z - (float)q.y / (float)q.x) * T_SCALE;
                }
                p.t += dT;
            }
            if (sw > 1e-4f) {
                /* drift between immiscible phase groups (particles.comp:374-476) */
                for (int q = 0; q < 3; q++) sg[q] /= sw;
                int g = Mia[0];
                float fg = g == 0 ? 1.0f - sg[0] - sg[1] - sg[2] : sg[g - 1];
                float others = 1.0f - fg;
                if (others > 1e-4f && groups && !held) {
                    V4 sgr = v4(0.0f, 0.0f, 0.0f, 0.0f), snu = sgr, snw = sgr;
                    for (int b = 0; b < 3; b++)
                        for (int a = 0; a < 3; a++) {
                            int ci = cidx(s, bx + a, by + b);
                            V4 q = s->comp[ci];
                            if (q.x <= 0.0f) continue;
                            float wt = w[a].x * w[b].y;
                            V4 gr = s->grho[ci];
                            sgr.x += wt * gr.x; sgr.y += wt * gr.y; sgr.z += wt * gr.z; sgr.w += wt * gr.w;
                            V4 ax = s->aux[ci];
                            V4 fc = v4(1.0f - q.y - ax.z - ax.w, q.y, ax.z, ax.w);
                            float top = maxf(maxf(fc.x, fc.y), maxf(fc.z, fc.w));
                            V4 oh = v4(fc.x == top ? 1.0f : 0.0f, fc.y == top ? 1.0f : 0.0f, fc.z == top ? 1.0f : 0.0f, fc.w == top ? 1.0f : 0.0f);
                            float on = maxf(oh.x + oh.y + oh.z + oh.w, 1.0f);
                            oh = v4(oh.x / on, oh.y / on, oh.z / on, oh.w / on);
                            float wn = wt * ax.x;
                            snu.x += wn * oh.x; snu.y += wn * oh.y; snu.z += wn * oh.z; snu.w += wn * oh.w;
                            snw.x += wt * oh.x; snw.y += wt * oh.y; snw.z += wt * oh.z; snw.w += wt * oh.w;
                        }
                    sgr = v4(sgr.x / sw, sgr.y / sw, sgr.z / sw, sgr.w / sw);
                    float rho_g = fg > 1e-4f ? v4c(sgr, g) / fg : row_density(s, row, p.s);
                    float rho_o = (sgr.x + sgr.y + sgr.z + sgr.w - v4c(sgr, g)) / others;
                    float drho = rho_g - rho_o;
                    int W = s->W;
                    int k = clampi((int)pos.y, 1, s->H - 2) * W + clampi((int)pos.x, 1, W - 2);
                    V4 fsv = v4(1.0f - sg[0] - sg[1] - sg[2], sg[0], sg[1], sg[2]);
                    int G = lead4(fsv);
                    float rho_c = v4c(sgr, G) / maxf(v4c(fsv, G), 1e-4f);
                    float nu_c = v4c(snw, G) > 1e-6f ? v4c(snu, G) / v4c(snw, G) : s->aux[k].x;
                    float vt = terminal(s, drho, rho_c, nu_c, P_.sep_tau);
                    float sep_max = P_.corr[2] > 0.0f ? P_.cfl / dt : 1e30f;
                    slip = -minf(vt, sep_max) * signf(drho) * others;
                    V4 fs = fsv;
                    if (g == 0) fs.x = -1.0f; else if (g == 1) fs.y = -1.0f; else if (g == 2) fs.z = -1.0f; else fs.w = -1.0f;
                    int h = lead4(fs);
                    float bond = fabsf(drho) * P_.gravity / maxf(P_.pair[g][h], 1e-9f);
                    float hold = clampf(1.0f - bond, 0.0f, 1.0f);
                    if (slip != 0.0f && hold > 0.0f) {
                        int hi = g > h ? g : h;
                        float gx, gy;
                        if (hi == 1) {
                            gx = 0.5f * (s->surf[k + 1].y - s->surf[k - 1].y);
                            gy = 0.5f * (s->surf[k + W].y - s->surf[k - W].y);
                        } else if (hi == 2) {
                            gx = 0.5f * (s->surf2[k + 1].x - s->surf2[k - 1].x);
                            gy = 0.5f * (s->surf2[k + W].x - s->surf2[k - W].x);
                        } else {
                            gx = 0.5f * (s->surf2[k + 1].y - s->surf2[k - 1].y);
                            gy = 0.5f * (s->surf2[k + W].y - s->surf2[k - W].y);
                        }
                        float resolved = 1.0f - clampf((0.12f - len2(v2(gx, gy))) / (0.12f - 0.04f), 0.0f, 1.0f);
                        slip *= 1.0f - hold * resolved;
                    }
                }
                /* drift within a phase group (particles.comp:478-502) */
                if (sorts && !held) {
                    float fgi = groups ? sg[Mia[0] - 1] : 1.0f;
                    if (fgi > 1e-4f) {
                        float rmean = sbg / sw / fgi;
                        float drho = s->mats[row].a[0] - rmean;
                        int pcx = clampi((int)pos.x, 0, s->W - 1), pcy = clampi((int)pos.y, 0, s->H - 1);
                        V4 cq = s->cell[cidx(s, pcx, pcy)];
                        float nu_c = cq.y > 0.0f ? cq.z / cq.y : s->aux[cidx(s, pcx, pcy)].x;
                        float vt = terminal(s, drho, rmean, nu_c, P_.sep_tau);
                        float sep_max = P_.corr[2] > 0.0f ? P_.cfl / dt : 1e30f;
                        slip -= minf(vt, sep_max) * signf(drho);
                    }
                }
                /* miscible exchange within a family (particles.comp:519-543) */
                int diluent0 = fam < 0 && P_.primary >= 0 && P_.fams[0][1] == (int)row;
                if (fam >= 0 || diluent0) {
                    if (sfw > 1e-4f) {
                        float s0 = diluent0 ? 0.0f : p.s;
                        float rate = s->mats[diluent0 ? (uint32_t)P_.primary : row].a[3];
                        float s1 = clampf(s0 + (sfs / sfw - s0) * (1.0f - o_expf(-rate * dt)), 0.0f, 1.0f);
                        float c0 = thermal ? thermal_of(s, row, p.s).w : 0.0f;
                        if (!diluent0) {
                            p.s = s1;
                        } else if (s1 > 0.0f) {
                            row = (uint32_t)P_.primary;
                            Mia = s->mats[row].ia;
                            p.kind = (p.kind & ~255u) | (row + 1u);
                            p.s = s1;
                        }
                        if (thermal) p.t = keep_heat(p.t, c0, thermal_of(s, row, p.s).w);
                    }
                }
                /* a pure diluent next to another of its concentrates joins that family
                 * (particles.comp:544-569) */
                if (fam < 0 && has_cap(s, CAP_FAMILIES) && (p.kind & 255u) - 1u == row && s->mats[row].ib[0] < 0) {
                    for (int j = P_.primary >= 0 ? 1 : 0; j < P_.n_fam; j++) {
                        if (P_.fams[j][1] != (int)row) continue;
                        float found = 0.0f;
                        if (j == 0) {
                            found = sfw;
                        } else {
                            for (int b = 0; b < 3; b++)
                                for (int a = 0; a < 3; a++)
                                    if (s->mixb[(size_t)cidx(s, bx + a, by + b) * nmix + j - 1] >= 0.0f) found += w[a].x * w[b].y;
                        }
                        if (found > 1e-4f) {
                            row = (uint32_t)P_.fams[j][0];
                            Mia = s->mats[row].ia;
                            p.kind = (p.kind & ~255u) | (row + 1u);
                            p.s = 0.0f;
                            break;
                        }
                    }
                }
            }
        }
        if (held && crowd <= REST_PHI + maxf(P_.corr[1], 0.05f)) corr = v2(0.0f, 0.0f);   /* particles.comp:576 */
        /* drains (particles.comp:577-594) */
        for (int c = 0; c < (int)P_.ext[3]; c++) {
            const float* z = P_.current_zone[c];
            if (z[3] >= 0.0f) continue;
            V2 dz = v2(pos.x - z[0], pos.y - z[1]);
            float r2 = (dz.x * dz.x + dz.y * dz.y) / (z[2] * z[2]);
            if (r2 < 1.0f) {
                float u = (float)(hash32(p.id * 2246822519u + s->S.substeps * 3266489917u + (uint32_t)c) >> 8) / 16777216.0f;
                if (u < -z[3] * (1.0f - 0.75f * r2) * dt) {
                    s->particles[id].kind = KIND_DEAD;
                    return;
                }
            }
        }
        /* mouse tool (particles.comp:596-631) */
        int pushed = 0;
        if (P_.tool_mode != 0) {
            V2 d = v2(P_.tool_pos[0] - pos.x, P_.tool_pos[1] - pos.y);
            float r2 = (d.x * d.x + d.y * d.y) / (P_.tool_radius * P_.tool_radius);
            if (r2 < 1.0f) {
                if (P_.tool_mode == 2) {
                    s->particles[id].kind = KIND_DEAD;
                    return;
                }
                float fall = 1.0f - r2;
                if (P_.tool_mode == 5 || P_.tool_mode == 6) {
                    if (thermal) {
                        float e = P_.heat2[1] * fall * dt;
                        float Cc = thermal_of(s, row, p.s).w;
                        if (P_.tool_mode == 6) e = minf(e, maxf(phase_of(p.t, thermal_of(s, row, p.s)).x + 150.0f, 0.0f) * Cc);
                        p.t += (P_.tool_mode == 5 ? e : -e) / Cc;
                        ledger_add(s, P_.tool_mode == 5 ? 4 : 5, e * P_.inv_ppc);
                    }
                } else {
                    float k = clampf(P_.tool_strength * fall * dt, 0.0f, 1.0f);
                    if (P_.tool_crowd_max > 0.0f && P_.tool_mode != 4)
                        k *= clampf((P_.tool_crowd_max - crowd) / (0.25f * P_.tool_crowd_max), 0.0f, 1.0f);
                    V2 tt = tool_target(s, d);
                    v = v2(mixf(v.x, tt.x, k), mixf(v.y, tt.y, k));
                    pushed = 1;
                }
            }
        }
        /* self-heating (particles.comp:735-739) */
        if (thermal && s->mats[row].rx[2] > 0.0f) {
            float e = s->mats[row].rx[2] * s->mats[row].th[0] * (Mia[1] >= 0 ? p.s : 1.0f) * dt * P_.heat[1];
            p.t += e / thermal_of(s, row, p.s).w;
            ledger_add(s, 7, e * P_.inv_ppc);
        }
        /* currents (particles.comp:809-835) */
        {
            float drive = P_.tool_crowd_max > 0.0f ? clampf((P_.tool_crowd_max - crowd) / (0.25f * P_.tool_crowd_max), 0.0f, 1.0f) : 1.0f;
            for (int c = 0; c < (int)P_.ext[3] && drive > 0.0f; c++) {
                const float* z = P_.current_zone[c];
                if (z[3] <= 0.0f) continue;
                V2 dz = v2(pos.x - z[0], pos.y - z[1]);
                float r2 = (dz.x * dz.x + dz.y * dz.y) / (z[2] * z[2]);
                if (r2 < 1.0f) {
                    V2 target = v2(P_.current_vel[c][0], P_.current_vel[c][1]);
                    float speed = len2(target);
                    V2 dir = v2(target.x / maxf(speed, 1e-6f), target.y / maxf(speed, 1e-6f));
                    float fall = (1.0f - r2) * (1.0f - r2);
                    float gap = maxf(speed - (v.x * dir.x + v.y * dir.y), 0.0f);
                    float e = 1.0f - o_expf(-z[3] * fall * dt);
                    v.x += dir.x * gap * e * drive;
                    v.y += dir.y * gap * e * drive;
                }
            }
        }
        /* speed cap */
        float vcap = P_.ext[0];
        {
            float sp = len2(v);
            if (sp > vcap) {
                v.x *= vcap / sp;
                v.y *= vcap / sp;
            }
        }
        /* advect (particles.comp:847-865) */
        V2 va = v;
        if (P_.ext[1] >= 2.0f && !pushed && !held) {
            V2 xm = v2(clampf(pos.x + 0.5f * dt * (v.x + corr.x + 0.0f), 2.01f, (float)s->W - 2.01f),
                       clampf(pos.y + 0.5f * dt * (v.y + corr.y + slip), 2.01f, (float)s->H - 2.01f));
            V2 here = sample_vel(s, pos, v);
            V2 there = sample_vel(s, xm, here);
            va = v2(v.x + there.x - here.x, v.y + there.y - here.y);
            float sp = len2(va);
            if (sp > vcap) {
                va.x *= vcap / sp;
                va.y *= vcap / sp;
            }
            if (crowd < LIQUID_THR && (va.x * va.x + va.y * va.y) < 0.01f * (v.x * v.x + v.y * v.y)) v = va;
        }
        V2 disp = v2(va.x + corr.x + 0.0f, va.y + corr.y + slip);
        {
            float mine = len2(disp);
            if (crowd < LIQUID_THR) mine /= P_.ext[2];
            report_umax(&s->S.umax_part, mine);
        }
        V2 step_d = v2(dt * disp.x, dt * disp.y);
        int pieces = clampi((int)ceilf(len2(step_d)), 1, 32);
        step_d.x /= (float)pieces;
        step_d.y /= (float)pieces;
        V2 x = pos;
        for (int k = 1; k < pieces; k++) {
            x.x += step_d.x;
            x.y += step_d.y;
            collide(s, &x, &v, 1);
        }
        x.x += step_d.x;
        x.y += step_d.y;
        float excess = clampf(crowd - 1.5f, 0.0f, 1.0f);
        if (excess > 0.0f && P_.crowd_jitter > 0.0f) {
            uint32_t hh = hash32(p.id ^ hash32(fbits(pos.x) ^ s->S.substeps));
            x.x += ((float)(hh & 0xffffu) / 65535.0f - 0.5f) * P_.crowd_jitter * excess;
            x.y += ((float)(hh >> 16) / 65535.0f - 0.5f) * P_.crowd_jitter * excess;
        }
        collide(s, &x, &v, 1);
        int again = collide(s, &x, &v, 1);
        if (again) {
            V2 gg;
            if (sample_sdf(s, x, &gg) < -1.0f) collide(s, &x, &v, 0);
        }
        x.x = clampf(x.x, 2.01f, (float)s->W - 2.01f);
        x.y = clampf(x.y, 2.01f, (float)s->H - 2.01f);
        p.pos[0] = x.x;
        p.pos[1] = x.y;
        p.vel[0] = v.x;
        p.vel[1] = v.y;
        p.c[0] = C.x;
        p.c[1] = C.y;
        p.c[2] = C.z;
        p.c[3] = C.w;
        p.kind &= ~KIND_FRESH;
        s->particles[id] = p;
    }
    float rho_p = row_density(s, row, p.s);
    float CT = 0.0f;
    if (thermal) {
        V4 th = thermal_of(s, row, p.s);
        V2 ph = phase_of(p.t, th);
        float tb = Mia[1] >= 0 ? mixf(s->mats[Mia[1]].th2[2], s->mats[row].th2[2], p.s) : s->mats[row].th2[2];
        rho_p *= expansion_of(s, row, p.s, ph.x);
        if (ph.y > 0.0f) {
            float rs = Mia[1] >= 0 ? mixf(s->mats[Mia[1]].b[3], s->mats[row].b[3], p.s) : s->mats[row].b[3];
            rho_p = mixf(rho_p, rs, ph.y);
        }
        CT = th.w * (minf(ph.x, tb) + 273.15f) / T_SCALE;
        int hx = clampi((int)floorf(p.pos[0]), 0, s->W - 1), hy = clampi((int)floorf(p.pos[1]), 0, s->H - 1);
        int hc = cidx(s, hx, hy);
        I2 q = heat_quanta(th.w, minf(ph.x, tb));
#pragma omp atomic
        s->hcell[hc].x += q.x;
#pragma omp atomic
        s->hcell[hc].y += q.y;
    }
    g->live = 1;
    g->pos = v2(p.pos[0], p.pos[1]);
    g->vs = v2(p.vel[0] * s->S.dt, p.vel[1] * s->S.dt);
    g->Cs = v4(p.c[0] * s->S.dt, p.c[1] * s->S.dt, p.c[2] * s->S.dt, p.c[3] * s->S.dt);
    g->rho = rho_p;
    g->sc = p.s;
    g->CT = CT;
    g->cw = Mia[2];
    g->cs = Mia[3];
    g->ct = thermal ? (int)P_.heat2[2] : -1;
    g->cg = thermal ? group_heat_chan(s, Mia[0]) : -1;
    /* particles.comp:983-984 */
    g->ce = elastic && (tau.x != 0.0f || tau.y != 0.0f || tau.z != 0.0f || tau.w != 0.0f) ? (int)P_.elastic[0] : -1;
    g->te = v4(tau.x / P_.elastic[1] * 65536.0f, tau.y / P_.elastic[1] * 65536.0f, tau.z / P_.elastic[1] * 65536.0f, 0.0f);
}

static inline void acc_add(OSim* s, int x, int y, int ch, int v) {
#pragma omp atomic
    s->acc[cidx(s, x, y) * P_.acc_stride + ch] += v;
}

/* deposit() (particles.comp:1006-1062) */
static void deposit(OSim* s, const Scat* g) {
    V2 w[3];
    {
        V2 gp = v2(g->pos.x - 0.0f, g->pos.y - 0.5f);
        int bx = (int)floorf(gp.x - 0.5f), by = (int)floorf(gp.y - 0.5f);
        float fx = gp.x - (float)bx, fy = gp.y - (float)by;
        bspline(fx, fy, w);
        for (int b = 0; b < 3; b++)
            for (int a = 0; a < 3; a++) {
                float m = w[a].x * w[b].y * g->rho;
                V2 d = v2((float)a - fx, (float)b - fy);
                acc_add(s, bx + a, by + b, 0, (int)floorf(m * MASS_SCALE + 0.5f));
                acc_add(s, bx + a, by + b, 1, (int)floorf(m * (g->vs.x + (g->Cs.x * d.x + g->Cs.y * d.y)) * MOM_SCALE + 0.5f));
            }
    }
    {
        V2 gp = v2(g->pos.x - 0.5f, g->pos.y - 0.0f);
        int bx = (int)floorf(gp.x - 0.5f), by = (int)floorf(gp.y - 0.5f);
        float fx = gp.x - (float)bx, fy = gp.y - (float)by;
        bspline(fx, fy, w);
        for (int b = 0; b < 3; b++)
            for (int a = 0; a < 3; a++) {
                float m = w[a].x * w[b].y * g->rho;
                V2 d = v2((float)a - fx, (float)b - fy);
                acc_add(s, bx + a, by + b, 2, (int)floorf(m * MASS_SCALE + 0.5f));
                acc_add(s, bx + a, by + b, 3, (int)floorf(m * (g->vs.y + (g->Cs.z * d.x + g->Cs.w * d.y)) * MOM_SCALE + 0.5f));
            }
    }
    {
        V2 gp = v2(g->pos.x - 0.5f, g->pos.y - 0.5f);
        int bx = (int)floorf(gp.x - 0.5f), by = (int)floorf(gp.y - 0.5f);
        float fx = gp.x - (float)bx, fy = gp.y - (float)by;
        bspline(fx, fy, w);
        for (int b = 0; b < 3; b++)
            for (int a = 0; a < 3; a++) {
                int nx = bx + a, ny = by + b;
                int wi = (int)floorf(w[a].x * w[b].y * MASS_SCALE + 0.5f);
                acc_add(s, nx, ny, 4, wi);
                if (g->cw >= 0) acc_add(s, nx, ny, g->cw, wi);
                if (g->cs >= 0 && g->sc > 0.0f) acc_add(s, nx, ny, g->cs, (int)floorf(w[a].x * w[b].y * g->sc * MASS_SCALE + 0.5f));
                if (g->ce >= 0) {   /* particles.comp:1053-1058 */
                    float wab = w[a].x * w[b].y;
                    acc_add(s, nx, ny, g->ce, (int)floorf(wab * g->te.x + 0.5f));
                    acc_add(s, nx, ny, g->ce + 1, (int)floorf(wab * g->te.y + 0.5f));
                    acc_add(s, nx, ny, g->ce + 2, (int)floorf(wab * g->te.z + 0.5f));
                }
                if (g->ct >= 0) {
                    int hq = (int)floorf(w[a].x * w[b].y * g->CT * MASS_SCALE + 0.5f);
                    acc_add(s, nx, ny, g->ct, hq);
                    if (g->cg >= 0) acc_add(s, nx, ny, g->cg, hq);
                }
            }
    }
}

static void k_particles(OSim* s, int gather) {
    int n = (int)P_.n_slots;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int i = 0; i < n; i++) {
        Scat g;
        advance(s, (uint32_t)i, gather, &g);
        if (g.live) deposit(s, &g);
    }
}

/* ------------------------------------------------------------------------------------ */
/* sort.comp: stable counting sort by cell, dead slots last                              */
/* ------------------------------------------------------------------------------------ */

void osim_sort(OSim* s) {
    int ncell = s->W * s->H;
    uint32_t* count = (uint32_t*)calloc((size_t)ncell + 1, sizeof(uint32_t));
    uint32_t n = s->n_slots;
    for (uint32_t i = 0; i < n; i++) {
        const OParticle* p = &s->particles[i];
        if (p->kind == KIND_DEAD) continue;
        int cx = clampi((int)p->pos[0], 0, s->W - 1), cy = clampi((int)p->pos[1], 0, s->H - 1);
        count[cidx(s, cx, cy)]++;
    }
    uint32_t run = 0;
    for (int c = 0; c < ncell; c++) {
        uint32_t k = count[c];
        count[c] = run;
        run += k;
    }
    memset(s->sorted, 0, (size_t)n * sizeof(OParticle));
    /* the look's state and the viscoelastic stress move with their particle (sort.comp's
     * plook, pstress: sort.comp:66); dead slots end zeroed */
    uint32_t* look2 = s->plook ? (uint32_t*)calloc((size_t)n * 4 + 4, sizeof(uint32_t)) : NULL;
    V4* stress2 = s->pstress ? (V4*)calloc((size_t)n + 1, sizeof(V4)) : NULL;
    for (uint32_t i = 0; i < n; i++) {
        const OParticle* p = &s->particles[i];
        if (p->kind == KIND_DEAD) continue;
        int cx = clampi((int)p->pos[0], 0, s->W - 1), cy = clampi((int)p->pos[1], 0, s->H - 1);
        uint32_t dst = count[cidx(s, cx, cy)]++;
        s->sorted[dst] = *p;
        if (look2) memcpy(look2 + 4 * (size_t)dst, s->plook + 4 * (size_t)i, 4 * sizeof(uint32_t));
        if (stress2) stress2[dst] = s->pstress[i];
    }
    memcpy(s->particles, s->sorted, (size_t)n * sizeof(OParticle));
    if (look2) {
        memcpy(s->plook, look2, (size_t)n * 4 * sizeof(uint32_t));
        free(look2);
    }
    if (stress2) {
        memcpy(s->pstress, stress2, (size_t)n * sizeof(V4));
        free(stress2);
    }
    free(count);
}

/* ------------------------------------------------------------------------------------ */
/* grid_prep.comp                                                                        */
/* ------------------------------------------------------------------------------------ */

static int packed(const OSim* s, int i) {
    V4 sol = s->solid[i];
    float phi_f = (float)s->acc[i * P_.acc_stride + 4] / MASS_SCALE * P_.inv_ppc;
    return sol.w > 0.02f && phi_f > 0.04f && phi_f + sol.z > LIQUID_THR;
}

static void group_temperatures(const OSim* s, int k, int cw, float Csh, const float Cg[GROUPS], float* T, float Tg[GROUPS]) {
    for (int g = 0; g < GROUPS; g++) Tg[g] = *T;
    if (Csh <= 0.0f) return;
    int Htot = s->acc[k + (int)P_.heat2[2]];
    *T = (float)Htot * T_SCALE / (Csh * (float)cw) - 273.15f;
    for (int g = 0; g < GROUPS; g++) Tg[g] = *T;
    int rest = Htot;
    int first = -1;
    for (int g = 0; g < GROUPS; g++) {
        int ch = group_heat_chan(s, g);
        if (ch >= 0) {
            int hh = s->acc[k + ch];
            rest -= hh;
            if (Cg[g] > 0.0f) Tg[g] = (float)hh * T_SCALE / (Cg[g] * (float)cw) - 273.15f;
        } else if (first < 0 && (P_.group_mask & (1u << (uint32_t)g)) != 0u) {
            first = g;
        }
    }
    if (first >= 0 && Cg[first] > 0.0f) Tg[first] = (float)rest * T_SCALE / (Cg[first] * (float)cw) - 273.15f;
}

static void k_grid_prep(OSim* s) {
    int W = s->W, H = s->H;
    uint32_t region_air = 0;
#pragma omp parallel for schedule(static) num_threads(g_threads) reduction(| : region_air)
    for (int cy = 0; cy < H; cy++)
        for (int cx = 0; cx < W; cx++) {
            int i = cidx(s, cx, cy);
            int k = i * P_.acc_stride;
            int um = s->acc[k], umom = s->acc[k + 1], vm = s->acc[k + 2], vmom = s->acc[k + 3];
            int cw = s->acc[k + 4];
            V4 sol = s->solid[i];
            float dt = s->S.dt;
            V4 o = v4(0.0f, 0.0f, FACE_EMPTY, FACE_EMPTY);
            if (sol.x <= 0.0f) o.z = FACE_CLOSED;
            else if (um >= MIN_FACE_MASS) {
                o.x = ((float)umom / MOM_SCALE) / ((float)um / MASS_SCALE) / dt;
                o.z = 0.0f;
            }
            if (sol.y <= 0.0f) o.w = FACE_CLOSED;
            else if (vm >= MIN_FACE_MASS) {
                o.y = ((float)vmom / MOM_SCALE) / ((float)vm / MASS_SCALE) / dt - P_.gravity * dt;
                o.w = 0.0f;
            }
            s->vel[i] = o;
            s->vel0[i] = v2(o.x, o.y);
            float phi_f = (float)cw / MASS_SCALE * P_.inv_ppc;
            float f[GROUPS] = {0}, rg[GROUPS] = {0}, lg[GROUPS] = {0};
            float sigma = 0.0f;
            V2 contact = v2(0.0f, 0.0f);
            float fam0 = -1.0f;
            V4 nn = v4(0.0f, -1.0f, 1.0f, 0.0f);   /* grid_prep.comp:62: the cell's non-Newtonian liquid */
            float chi = 0.0f;   /* grid_prep.comp:63 */
            float rho = 0.0f, mu = 0.0f, rho_c = 0.0f, nu_c = 0.0f;
            int thermal = has_cap(s, CAP_THERMAL);
            const int nmix = P_.n_fam - 1;   /* grid_prep.comp:67-68 */
            for (int q = 0; q < nmix; q++) s->mixb[(size_t)i * nmix + q] = -1.0f;
            float bg[3] = {0.0f, 0.0f, 0.0f};   /* share x base density of groups 1 - 3 */
            const int settle = (s->caps & CAP_SETTLE) != 0u;   /* grid_prep.comp:69-70, 147 */
            if (settle)
                for (int q = 0; q < P_.n_fam; q++) s->famocc[(size_t)i * P_.n_fam + q] = 0.0f;
            float T = P_.heat[0], kappa = 0.0f, emis = 0.0f, frozen = 0.0f, Craw = 0.0f;
            int major = 0, top_row = -1;
            float top_share = 0.0f;
            if (cw > 0) {
                int others = 0;
                for (int j = 0; j < P_.n_present; j++) {
                    int ch = s->mats[P_.present[j]].ia[2];
                    if (ch >= 0) others += s->acc[k + ch];
                }
                float sh[MAX_PRESENT], scn[MAX_PRESENT];
                float Csh = 0.0f;
                float Cg[GROUPS] = {0};
                for (int j = 0; j < P_.n_present; j++) {
                    sh[j] = 0.0f;
                    scn[j] = 1.0f;
                    int r = P_.present[j];
                    const int* ia = s->mats[r].ia;
                    if (ia[2] < 0 && P_.primary >= 0 && r != P_.primary) continue;
                    int wgt = ia[2] >= 0 ? s->acc[k + ia[2]] : maxi(cw - others, 0);
                    if (wgt <= 0) continue;
                    sh[j] = wgt >= cw ? 1.0f : clampf((float)wgt / (float)cw, 0.0f, 1.0f);
                    if (ia[1] >= 0 && ia[3] >= 0) scn[j] = clampf((float)s->acc[k + ia[3]] / (float)wgt, 0.0f, 1.0f);
                    if (thermal) {
                        float cr = sh[j] * thermal_of(s, (uint32_t)r, scn[j]).w;
                        Csh += cr;
                        Cg[ia[0]] += cr;
                        float kp = s->mats[r].th[1];
                        kappa += sh[j] * (ia[1] >= 0 ? mixf(s->mats[ia[1]].th[1], kp, scn[j]) : kp);
                        float em = s->mats[r].th2[1];
                        emis += sh[j] * (ia[1] >= 0 ? mixf(s->mats[ia[1]].th2[1], em, scn[j]) : em);
                    }
                }
                float Tg[GROUPS];
                group_temperatures(s, k, cw, thermal ? Csh : 0.0f, Cg, &T, Tg);
                for (int j = 0; j < P_.n_present; j++) {
                    float share = sh[j];
                    if (share <= 0.0f) continue;
                    int r = P_.present[j];
                    const int* ia = s->mats[r].ia;
                    float sc = scn[j];
                    const float* ma = s->mats[r].a;
                    float rho_m = ma[0], lnu = ma[1], sig = ma[2];
                    float Tm = Tg[ia[0]];
                    if (thermal) lnu += temp_law(s, r, Tm);
                    float xp = thermal ? expansion_of(s, (uint32_t)r, sc, Tm) : 1.0f;
                    V2 csv = v2(s->mats[r].b[0], s->mats[r].b[1]);
                    if (ia[1] >= 0) {
                        const float* da = s->mats[ia[1]].a;
                        rho_m = mixf(da[0], rho_m, sc);
                        /* blend_share(s, e) = s: every concentrate here blends with exponent 1 */
                        lnu = mixf(thermal ? da[1] + temp_law(s, ia[1], Tm) : da[1], lnu, sc);
                        sig = mixf(da[2], sig, sc);
                        csv = v2(mixf(s->mats[ia[1]].b[0], csv.x, sc), mixf(s->mats[ia[1]].b[1], csv.y, sc));
                        /* grid_prep.comp:144-146 */
                        const int fam = s->mats[r].ib[0];
                        if (fam == 0) fam0 = sc;
                        else if (fam > 0) s->mixb[(size_t)i * nmix + fam - 1] = sc;
                        if (settle && fam >= 0) s->famocc[(size_t)i * P_.n_fam + fam] = share * phi_f;
                    }
                    rho_m *= xp;
                    if (thermal) {
                        V4 th = thermal_of(s, (uint32_t)r, sc);
                        float fs = th.y > -1e8f ? clampf((th.y - Tm) / maxf(th.y - th.x, 1e-3f), 0.0f, 1.0f) : 0.0f;
                        if (fs > 0.0f) {
                            lnu = mixf(lnu, maxf(lnu, P_.heat2[0]), fs);
                            float rs = s->mats[r].b[3];
                            rho_m = mixf(rho_m, ia[1] >= 0 ? mixf(s->mats[ia[1]].b[3], rs, sc) : rs, fs);
                            frozen += share * fs;
                        }
                    }
                    if ((s->mats[r].ib[1] != 0 || s->mats[r].temp[3] > 0.0f || s->mats[r].gr[0] > 0.0f) && share > nn.x)
                        nn = v4(share, (float)r, sc, 0.0f);   /* grid_prep.comp:162 */
                    if (r != 57 && share > top_share) {
                        top_share = share;
                        top_row = r;
                    }
                    chi += share * s->mats[r].el[2];   /* grid_prep.comp:168 */
                    int g = ia[0];
                    if (g > 0) bg[g - 1] += share * ma[0];   /* grid_prep.comp:172 */
                    f[g] += share;
                    rg[g] += share * rho_m;
                    lg[g] += share * lnu;
                    sigma += share * sig;
                    contact.x += share * csv.x;
                    contact.y += share * csv.y;
                }
                for (int g = 0; g < GROUPS; g++) {
                    if (f[g] <= 0.0f) continue;
                    rho += rg[g];
                    mu += rg[g] * o_expf(lg[g] / f[g]);
                    if (f[g] > f[major]) major = g;
                }
                if (f[major] > 0.0f) {
                    rho_c = rg[major] / f[major];
                    nu_c = o_expf(lg[major] / f[major]);
                }
                Craw = Csh * (float)cw / MASS_SCALE;
            }
            float phi_t = phi_f + sol.z;
            int has = phi_f > 0.04f && sol.w > 0.02f;
            float level = has ? phi_t - LIQUID_THR : -LIQUID_THR;
            if (has && level <= 0.0f && cx > 0 && cy > 0 && cx < W - 1 && cy < H - 1) {
                if ((packed(s, i - 1) && packed(s, i + 1)) || (packed(s, i - W) && packed(s, i + W))) level = 0.05f;
                else if (P_.gravity > 0.0f && nn.x <= 0.0f && phi_t > 0.25f && packed(s, i - W)) level = 0.05f;
                else if ((s->caps & CAP_MAGNET) && nn.x <= 0.0f && phi_t > 0.25f && chi > 0.0f) {   /* grid_prep.comp:216-220 */
                    float km = chi / P_.mag[1] / maxf(rho, 0.05f);
                    float pk = -km * 0.5f;
                    V2 pull = v2(pk * (s->magc[i + 1].y - s->magc[i - 1].y) - 0.0f, pk * (s->magc[i + W].y - s->magc[i - W].y) - P_.gravity);
                    int toward = fabsf(pull.x) > fabsf(pull.y) ? (pull.x > 0.0f ? i + 1 : i - 1) : (pull.y > 0.0f ? i + W : i - W);
                    if (packed(s, toward)) level = 0.05f;
                }
            }
            if (sol.w > 0.0f && level <= 0.0f) region_air |= 1u << (s->region[i] & REGION_MASK);
            if (s->caps & CAP_MAGNET) s->magc[i].x = chi;   /* grid_prep.comp:240 */
            if (s->caps & CAP_ELASTIC) {   /* grid_prep.comp:241-244 */
                int ce = (int)P_.elastic[0];
                float sc = P_.elastic[1] * P_.inv_ppc / 65536.0f;
                s->estr[i] = v4((float)s->acc[k + ce] * sc, (float)s->acc[k + ce + 1] * sc, (float)s->acc[k + ce + 2] * sc, 0.0f * sc);
            }
            if (s->caps & (CAP_RIGID | CAP_RHEO)) {   /* grid_prep.comp:232-237 */
                float cap = rho * o_expf(P_.heat2[0]);
                if (mu >= cap && level > 0.0f) nn.w = 1.0f;
                mu = minf(mu, cap);
                s->rh[i] = nn;
            }
            s->cell[i] = v4(phi_f, rho, mu, level);
            s->comp[i] = v4(rho, f[1], fam0, phi_t);
            if (group_sorts(s, 1) || group_sorts(s, 2) || group_sorts(s, 3)) s->gbase[i] = v4(bg[0], bg[1], bg[2], 0.0f);
            if ((P_.group_mask & (P_.group_mask - 1u)) != 0u) {
                s->aux[i] = v4(nu_c, rho_c, f[2], f[3]);
                s->grho[i] = v4(rg[0], rg[1], rg[2], rg[3]);
            }
            s->sprop[i] = v4(sigma, contact.x, contact.y, (float)major + (float)(top_row + 1) / 128.0f);
            if (thermal) {
                s->therm[i] = v4(T, Craw, kappa, frozen);
                s->dheat[i] = v4(P_.heat[1] > 0.0f ? emis : 0.0f, 0.0f, 0.0f, 0.0f);
            }
            if (level <= 0.0f) s->pres[i] = v2(0.0f, 0.0f);
        }
    s->region_air |= region_air;
}

/* ------------------------------------------------------------------------------------ */
/* grid_coef.comp, surf_smooth.comp, surf_curv.comp, surf_apply.comp                      */
/* ------------------------------------------------------------------------------------ */

/* common.glsl:527-540: the shear rate of cell i from its faces (gravity's last increment taken
 * back out when pre) */
static float shear_rate(const OSim* s, int i, int pre) {
    int W = s->W;
    float gv = pre ? P_.gravity * s->S.dt : 0.0f;
#define UF(k) (face_live(s->vel[k].z) ? s->vel[k].x : 0.0f)
#define VF(k) (face_live(s->vel[k].w) ? s->vel[k].y + gv : 0.0f)
    float dxx = UF(i + 1) - UF(i);
    float dyy = VF(i + W) - VF(i);
    float duy = 0.25f * (UF(i + W) + UF(i + 1 + W) - UF(i - W) - UF(i + 1 - W));
    float dvx = 0.25f * (VF(i + 1) + VF(i + 1 + W) - VF(i - 1) - VF(i - 1 + W));
#undef UF
#undef VF
    float dxy = 0.5f * (duy + dvx);
    return sqrtf(2.0f * (dxx * dxx + dyy * dyy + 2.0f * dxy * dxy));
}

/* common.glsl:546-571: the non-Newtonian factor F and yield stress tau of the cell's liquid */
static void nn_eval(const OSim* s, int i, V4 q, float g, float* Fo, float* tauo) {
    const GMat* m = &s->mats[(int)q.y];
    const float* rp = m->rheo;
    int model = m->ib[1];
    float F = 1.0f, tau = 0.0f;
    if (model == 1) {
        F = rp[3] + (1.0f - rp[3]) * o_powf(1.0f + (rp[2] * g) * (rp[2] * g), 0.5f * (rp[1] - 1.0f));
    } else if (model == 2) {
        F = o_powf(maxf(g, 1e-6f), rp[1] - 1.0f);
        tau = rp[0] * q.z;
    } else if (model == 3) {
        F = minf(o_powf(1.0f + (rp[2] * g) * (rp[2] * g), 0.5f * (rp[1] - 1.0f)), rp[3]);
    }
    float fr = m->gr[0];
    if (fr > 0.0f) tau += fr * q.z * q.z * q.z * maxf(s->pres[i].x, 0.0f) / maxf(s->S.dt, 1e-6f);
    int W = s->W;
    float skin = m->temp[3];
    if (skin > 0.0f && (s->cell[i - 1].w <= 0.0f || s->cell[i + 1].w <= 0.0f || s->cell[i - W].w <= 0.0f || s->cell[i + W].w <= 0.0f))
        tau += skin;
    *Fo = 1.0f + q.x * (F - 1.0f);
    *tauo = tau * q.x;
}

/* elastic.comp: the divergence of the deposited stress accelerates the faces */
static float txy_node(const OSim* s, int i) {
    int W = s->W;
    return 0.25f * (s->estr[i].z + s->estr[i - 1].z + s->estr[i - W].z + s->estr[i - W - 1].z);
}

static void k_elastic(OSim* s) {
    int W = s->W, H = s->H;
    float dt = s->S.dt;
#pragma omp parallel for schedule(static)
    for (int cy = 2; cy < H - 1; cy++)
        for (int cx = 2; cx < W - 1; cx++) {
            int i = cy * W + cx;
            V4 q = s->vel[i];
            V4 a = s->cell[i], l = s->cell[i - 1], b = s->cell[i - W];
            if (face_live(q.z)) {
                float rho = (a.x * a.y + l.x * l.y) / maxf(a.x + l.x, 1e-6f);
                float f = (s->estr[i].x - s->estr[i - 1].x) + (txy_node(s, i + W) - txy_node(s, i));
                q.x += dt * f / maxf(rho, 0.05f);
            }
            if (face_live(q.w)) {
                float rho = (a.x * a.y + b.x * b.y) / maxf(a.x + b.x, 1e-6f);
                float f = (s->estr[i].y - s->estr[i - W].y) + (txy_node(s, i + 1) - txy_node(s, i));
                q.y += dt * f / maxf(rho, 0.05f);
            }
            s->vel[i] = q;
        }
}

/* ---- rigid bodies (rigid.comp; common.glsl:265-340) ------------------------------- */
#define O_FIX 65536.0f

/* common.glsl:275-277: a body sum, as the shader reads its two words */
static float get64(int64_t v) {
    uint64_t u = (uint64_t)v;
    return ((float)(int32_t)(uint32_t)(u >> 32) * 4294967296.0f + (float)(uint32_t)u) / O_FIX;
}

/* rigid.comp add64: x rounded to an integer, added in 64 bits */
static void add64(int64_t* w, float x) {
    x = floorf(x + 0.5f);
    *w += (int64_t)x;
}

/* common.glsl:631-636 */
static float row_lnu(const OSim* s, uint32_t row, float sc, float T, int thermal) {
    float l = s->mats[row].a[1] + (thermal ? temp_law(s, (int)row, T) : 0.0f);
    int d = s->mats[row].ia[1];
    if (d >= 0) l = mixf(s->mats[d].a[1] + (thermal ? temp_law(s, d, T) : 0.0f), l, sc);
    return l;
}

/* common.glsl:289-325: contact of a body with the solids it touches */
static void body_contact(const int64_t* o, float mu, V2 cm, V2* U, float* w) {
    float nc = get64(o[7]);
    if (mu < 0.0f || nc < 0.5f) return;
    V2 ns = v2(get64(o[8]), get64(o[9]));
    if (len2(ns) < 0.25f * nc) return;
    float ln = len2(ns);
    V2 n = v2(ns.x / ln, ns.y / ln);
    V2 t = v2(n.y, -n.x);
    V2 cc = v2(get64(o[10]) / nc, get64(o[11]) / nc);
    float sqx = get64(o[12]) / nc - cc.x * cc.x, sqy = get64(o[13]) / nc - cc.y * cc.y, sqz = get64(o[14]) / nc - cc.x * cc.y;
    float ext = sqrtf(3.0f * maxf(t.x * t.x * sqx + t.y * t.y * sqy + 2.0f * t.x * t.y * sqz, 0.0f)) + 0.5f;
    V2 rc = v2(cc.x - cm.x, cc.y - cm.y);
    V2 uc = v2(U->x + *w * -rc.y, U->y + *w * rc.x);
    float vn = uc.x * n.x + uc.y * n.y;
    float sp = (cm.x - cc.x) * t.x + (cm.y - cc.y) * t.y;
    float vn1 = vn, w1 = *w;
    if (fabsf(sp) <= ext) {
        vn1 = maxf(vn, 0.0f);
        w1 = clampf(*w, -vn1 / ext, vn1 / ext);
    } else {
        float edge = signf(sp) * ext;
        vn1 = maxf(vn + *w * edge, 0.0f) - *w * edge;
    }
    if (vn1 == vn && w1 == *w) return;
    float vt = uc.x * t.x + uc.y * t.y;
    float vt1 = signf(vt) * maxf(fabsf(vt) - mu * (vn1 - vn), 0.0f);
    uc = v2(uc.x + ((vn1 - vn) * n.x + (vt1 - vt) * t.x), uc.y + ((vn1 - vn) * n.y + (vt1 - vt) * t.y));
    *w = w1;
    *U = v2(uc.x - w1 * -rc.y, uc.y - w1 * rc.x);
}

/* common.glsl:327-340: the rigid motion of body b (root cell r) at x: velocity, spin */
static int body_motion(const OSim* s, int b, int r, V2 x, V3f* u) {
    const int64_t* o = s->rbody + (size_t)b * 16;
    float M = get64(o[0]);
    if (M <= 1e-3f) return 0;
    V2 cm = v2(get64(o[1]) / M, get64(o[2]) / M);
    V2 U = v2(get64(o[3]) / M, get64(o[4]) / M);
    float L = get64(o[5]) - M * (cm.x * U.y - cm.y * U.x);
    float I = get64(o[6]) - M * (cm.x * cm.x + cm.y * cm.y);
    float w = I > 1e-3f ? L / I : 0.0f;
    body_contact(o, P_.misc[3], cm, &U, &w);
    V2 d = v2(x.x - ((float)(r % s->W) + 0.5f) - cm.x, x.y - ((float)(r / s->W) + 0.5f) - cm.y);
    u->x = U.x + w * -d.y;
    u->y = U.y + w * d.x;
    u->z = w;
    return 1;
}

/* rigid.comp:10-25: whether liquid cell i moves rigidly */
static int cell_rigid(const OSim* s, int cx, int cy, int i) {
    V4 me = s->cell[i];
    if (me.w <= 0.0f) return 0;
    if ((s->caps & CAP_THERMAL) && s->therm[i].w > 0.5f) return 1;
    V4 q = s->rh[i];
    if (q.w > 0.5f) return 1;
    if (!(s->caps & CAP_RHEO) || q.x <= 0.0f || cx < 1 || cy < 1 || cx >= s->W - 1 || cy >= s->H - 1) return 0;
    float g = shear_rate(s, i, 0);
    float F, tau;
    nn_eval(s, i, q, g, &F, &tau);
    if (tau > 0.0f && me.z * g < tau) return 1;
    return s->mats[(int)q.y].ib[1] == 3 && me.z * F >= me.y * o_expf(P_.heat2[0]);
}

/* rigid.comp:27-36: the node SDF bilinearly, and its gradient */
static float rigid_sdf(const OSim* s, float x, float y, V2* grad) {
    float gx = clampf(x, 0.0f, (float)s->W - 0.001f), gy = clampf(y, 0.0f, (float)s->H - 0.001f);
    int ix = (int)gx, iy = (int)gy;
    float fx = gx - (float)ix, fy = gy - (float)iy;
    int w1 = s->W + 1, k = iy * w1 + ix;
    float d00 = s->sdf[k], d10 = s->sdf[k + 1], d01 = s->sdf[k + w1], d11 = s->sdf[k + w1 + 1];
    *grad = v2(mixf(d10 - d00, d11 - d01, fy), mixf(d01 - d00, d11 - d10, fx));
    return mixf(mixf(d00, d10, fx), mixf(d01, d11, fx), fy);
}

static int rl_find(const OSim* s, int i) {
    while (s->rl[i].x != i) i = s->rl[i].x;
    return i;
}

/* rigid.comp modes 0-4: label the rigid cells, join them into bodies (each body's root is
 * its smallest cell), sum each body's mass, moments and contacts, and move the faces inside
 * a body with it */
static void k_rigid(OSim* s) {
    int W = s->W, H = s->H;
    size_t nc = (size_t)W * H;
    for (int cy = 0; cy < H; cy++)
        for (int cx = 0; cx < W; cx++) {
            int i = cy * W + cx;
            s->rl[i] = (I2){cell_rigid(s, cx, cy, i) ? i : -1, -1};
        }
    s->nbodies = 0;
    for (int cy = 0; cy < H; cy++)
        for (int cx = 0; cx < W; cx++) {
            int i = cy * W + cx;
            if (s->rl[i].x < 0) continue;
            int nb[4] = {cx > 0 ? i - 1 : -1, cy > 0 ? i - W : -1, (cy > 0 && cx > 0) ? i - W - 1 : -1,
                         (cy > 0 && cx < W - 1) ? i - W + 1 : -1};
            for (int q = 0; q < 4; q++) {
                if (nb[q] < 0 || s->rl[nb[q]].x < 0) continue;
                int a = rl_find(s, i), b = rl_find(s, nb[q]);
                if (a < b) s->rl[b].x = a;
                else if (b < a) s->rl[a].x = b;
            }
        }
    for (size_t i = 0; i < nc; i++) {
        if (s->rl[i].x < 0) continue;
        int r = rl_find(s, (int)i);
        s->rl[i].x = r;
        if (r == (int)i && s->nbodies < O_MAX_BODIES) {
            uint32_t b = s->nbodies++;
            memset(s->rbody + (size_t)b * 16, 0, 16 * sizeof(int64_t));
            s->rl[i].y = (int)b;
        }
    }
    for (int cy = 0; cy < H; cy++)
        for (int cx = 0; cx < W; cx++) {
            int i = cy * W + cx;
            int l = s->rl[i].x;
            if (l < 0) continue;
            int b = s->rl[l].y;
            if (b < 0) continue;
            int64_t* o = s->rbody + (size_t)b * 16;
            float m = s->cell[i].y * minf(s->cell[i].x, 1.0f) * O_FIX;
            V2 d = v2((float)(cx - l % W), (float)(cy - l / W));
            V4 q = s->vel[i];
            float ur = cx < W - 1 ? s->vel[i + 1].x : 0.0f, ut = cy < H - 1 ? s->vel[i + W].y : 0.0f;
            V2 u = v2(0.5f * (q.x + ur), 0.5f * (q.y + ut));
            add64(&o[0], m);
            add64(&o[1], m * d.x);
            add64(&o[2], m * d.y);
            add64(&o[3], m * u.x);
            add64(&o[4], m * u.y);
            add64(&o[5], m * (d.x * u.y - d.y * u.x));
            add64(&o[6], m * ((d.x * d.x + d.y * d.y) + 1.0f / 6.0f));
            if (P_.misc[3] >= 0.0f) {
                V2 g;
                float dist = rigid_sdf(s, (float)cx + 0.5f, (float)cy + 0.5f, &g);
                if (dist < 1.0f && g.x * g.x + g.y * g.y > 1e-8f) {
                    float gl = len2(g);
                    V2 nrm = v2(g.x / gl, g.y / gl);
                    add64(&o[7], O_FIX);
                    add64(&o[8], O_FIX * nrm.x);
                    add64(&o[9], O_FIX * nrm.y);
                    add64(&o[10], O_FIX * d.x);
                    add64(&o[11], O_FIX * d.y);
                    add64(&o[12], O_FIX * d.x * d.x);
                    add64(&o[13], O_FIX * d.y * d.y);
                    add64(&o[14], O_FIX * d.x * d.y);
                }
            }
        }
    float clump = REST_PHI + maxf(P_.corr[1], 0.05f);
#pragma omp parallel for schedule(static)
    for (int cy = 0; cy < H; cy++)
        for (int cx = 0; cx < W; cx++) {
            int i = cy * W + cx;
            int l = s->rl[i].x;
            V4 q = s->vel[i];
            int changed = 0, cl = s->cell[i].x > clump;
            V3f u;
            if (l >= 0 && cx > 0 && s->rl[i - 1].x == l && face_live(q.z) && s->rl[l].y >= 0 &&
                body_motion(s, s->rl[l].y, l, v2((float)cx, (float)cy + 0.5f), &u)) {
                q.x = u.x;
                if (!cl && s->cell[i - 1].x <= clump) q.z = 0.0f;
                changed = 1;
            }
            if (l >= 0 && cy > 0 && s->rl[i - W].x == l && face_live(q.w) && s->rl[l].y >= 0 &&
                body_motion(s, s->rl[l].y, l, v2((float)cx + 0.5f, (float)cy), &u)) {
                q.y = u.y;
                if (!cl && s->cell[i - W].x <= clump) q.w = 0.0f;
                changed = 1;
            }
            if (changed) s->vel[i] = q;
        }
}

/* common.glsl:388-402: the magnets' field at (x, y), T */
static V2 magnet_field(const OSim* s, float x, float y) {
    V2 B = v2(0.0f, 0.0f);
    for (int k = 0; k < (int)P_.mag[0]; k++) {
        const float* mg = P_.magnet[k];
        V2 m = v2(P_.magnet_dir[k][0], P_.magnet_dir[k][1]);
        V2 d = v2(x - mg[0], y - mg[1]);
        float len = len2(d);
        float r = maxf(len, mg[2]);
        V2 e = len > 1e-4f ? v2(d.x / len, d.y / len) : m;
        float a = mg[3] * o_powf(mg[2] / r, 3.0f) * 0.5f;
        float me3 = 3.0f * (m.x * e.x + m.y * e.y);
        B.x += a * (me3 * e.x - m.x);
        B.y += a * (me3 * e.y - m.y);
    }
    return B;
}

/* magnet.comp mode 0: the magnetic energy density of pure magnetic liquid per cell */
static void k_magnet_energy(OSim* s) {
    int W = s->W, H = s->H;
    const float MU0 = 1.25663706e-6f;
#pragma omp parallel for schedule(static)
    for (int cy = 0; cy < H; cy++)
        for (int cx = 0; cx < W; cx++) {
            int i = cy * W + cx;
            V2 B = magnet_field(s, (float)cx + 0.5f, (float)cy + 0.5f);
            float Bl = len2(B);
            float Hf = Bl / MU0;
            float psi = 0.0f;
            float chi = P_.mag[1];
            if (Hf > 0.0f && chi > 0.0f) {
                float N = 1.0f / 3.0f;
                if (P_.heat3[3] > 0.0f) {
                    V2 g = v2(0.0f, 0.0f);
                    if (cx > 0 && cy > 0 && cx < W - 1 && cy < H - 1)
                        g = v2(0.5f * (s->surf[i + 1].x - s->surf[i - 1].x), 0.5f * (s->surf[i + W].x - s->surf[i - W].x));
                    float gl = len2(g);
                    float nh = gl > 1e-6f ? (g.x / gl) * (B.x / Bl) + (g.y / gl) * (B.y / Bl) : 0.0f;
                    N = mixf(1.0f / 3.0f, nh * nh, clampf(gl / 0.25f, 0.0f, 1.0f) * P_.heat3[3]);
                }
                float ce = chi / (1.0f + N * chi);
                float Ms = P_.mag[2] / MU0;
                float xs = ce * Hf / Ms;
                float f = xs < 0.02f ? xs * xs * (0.5f - xs * (1.0f / 3.0f - 0.25f * xs)) : xs - o_logf(1.0f + xs);
                psi = -MU0 * Ms * Ms / ce * f * P_.mag[3];
            }
            s->magc[i].y = psi;
        }
}

/* magnet.comp mode 1: the energy gradient's force on the liquid's faces */
static float magnet_face_force(const OSim* s, int i, int n, float rho) {
    int li = s->cell[i].w > 0.0f, ln = s->cell[n].w > 0.0f;
    float sc = (li == ln ? 0.5f * (s->magc[i].x + s->magc[n].x) : li ? s->magc[i].x : s->magc[n].x) / P_.mag[1];
    return -s->S.dt * sc * (s->magc[i].y - s->magc[n].y) / maxf(rho, 0.05f);
}

static void k_magnet_force(OSim* s) {
    int W = s->W, H = s->H;
#pragma omp parallel for schedule(static)
    for (int cy = 1; cy < H; cy++)
        for (int cx = 1; cx < W; cx++) {
            int i = cy * W + cx;
            V4 me = s->vel[i];
            V4 cf = s->coef[i];
            if (face_live(me.z) && cf.x != 0.0f) me.x += magnet_face_force(s, i, i - 1, cf.z);
            if (face_live(me.w) && cf.y != 0.0f) me.y += magnet_face_force(s, i, i - W, cf.w);
            s->vel[i] = me;
        }
}

/* settle.comp:8-16: family f's settling flux from an upper cell into a lower one */
static float settle_flux(const OSim* s, int up, int dn, int f, float vt) {
    int nf = P_.n_fam;
    float ou = s->famocc[(size_t)up * nf + f], od = s->famocc[(size_t)dn * nf + f];
    if (ou <= 1e-3f || od <= 1e-3f) return 0.0f;
    float su = f == 0 ? s->comp[up].z : s->mixb[(size_t)up * (nf - 1) + f - 1];
    float sd = f == 0 ? s->comp[dn].z : s->mixb[(size_t)dn * (nf - 1) + f - 1];
    if (su <= 0.0f || sd < 0.0f) return 0.0f;
    float F = vt * su * (1.0f - sd) * minf(ou, od);
    return minf(F, minf(su * ou, (1.0f - sd) * od) / s->S.dt);
}

/* settle.comp:18-52: per cell and family with grains, the concentration gain / loss rates */
static void k_settle(OSim* s) {
    int W = s->W, H = s->H, nf = P_.n_fam;
    int thermal = has_cap(s, CAP_THERMAL);
#pragma omp parallel for schedule(static)
    for (int cy = 0; cy < H; cy++)
        for (int cx = 0; cx < W; cx++) {
            int i = cy * W + cx;
            for (int f = 0; f < nf; f++) {
                int row = P_.fams[f][0], dl = P_.fams[f][1];
                float gd = s->mats[row].b[2];
                float occ = s->famocc[(size_t)i * nf + f];
                V2 ds = v2(0.0f, 0.0f);
                if (gd > 0.0f && occ > 1e-3f && cy > 0 && cy < H - 1) {
                    float drho = s->mats[row].a[0] - s->mats[dl].a[0];
                    float T = thermal ? s->therm[i].x : P_.heat[0];
                    float lnu = s->mats[dl].a[1] + (thermal ? temp_law(s, dl, T) : 0.0f);   /* row_lnu(dl, 1) */
                    float vt = terminal(s, drho, s->mats[dl].a[0], o_expf(lnu), gd);
                    float gain = drho > 0.0f ? settle_flux(s, i + W, i, f, vt) : settle_flux(s, i - W, i, f, vt);
                    float loss = drho > 0.0f ? settle_flux(s, i, i - W, f, vt) : settle_flux(s, i, i + W, f, vt);
                    float sv = f == 0 ? s->comp[i].z : s->mixb[(size_t)i * (nf - 1) + f - 1];
                    float dt = s->S.dt;
                    ds = v2(dt * (gain / maxf(occ * (1.0f - sv), 1e-6f)), dt * (loss / maxf(occ * sv, 1e-6f)));
                }
                s->dsettle[(size_t)i * nf + f] = ds;
            }
        }
}

/* rheo.comp: a non-Newtonian cell's viscosity at its shear rate, capped at rigid_viscosity */
static void k_rheo(OSim* s) {
    int W = s->W, H = s->H;
#pragma omp parallel for schedule(static)
    for (int cy = 1; cy < H - 1; cy++)
        for (int cx = 1; cx < W - 1; cx++) {
            int i = cy * W + cx;
            V4 me = s->cell[i];
            V4 q = s->rh[i];
            if (me.w <= 0.0f || q.x <= 0.0f) continue;
            float g = shear_rate(s, i, 1);
            float F, tau;
            nn_eval(s, i, q, g, &F, &tau);
            float eff = me.z * F + tau / maxf(g, 1e-6f);
            float cap = me.y * o_expf(P_.heat2[0]);
            float skin = q.x * s->mats[(int)q.y].temp[3];
            if (skin > 0.0f && me.y * g * g < skin &&
                (s->cell[i - 1].w <= 0.0f || s->cell[i + 1].w <= 0.0f || s->cell[i - W].w <= 0.0f || s->cell[i + W].w <= 0.0f)) {
                q.w = 1.0f;
                s->rh[i] = q;
            }
            me.z = minf(eff, cap);
            s->cell[i] = me;
        }
}

static void coef_face(V4 a, V4 b, float open, float* g, float* rho) {
    float wsum = a.x + b.x;
    *rho = wsum > 1e-6f ? (a.x * a.y + b.x * b.y) / wsum : 1.0f;
    *g = 0.0f;
    int fa = a.w > 0.0f, fb = b.w > 0.0f;
    if (open <= 0.0f || !(fa || fb)) return;
    float theta = 1.0f;
    if (fa != fb) {
        float lf = fa ? a.w : b.w;
        float la = fa ? b.w : a.w;
        theta = clampf(lf / (lf - la), THETA_MIN, 1.0f);
    }
    *g = 1.0f / (maxf(*rho, 0.05f) * theta);
}

static void k_grid_coef(OSim* s) {
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int cy = 0; cy < s->H; cy++)
        for (int cx = 0; cx < s->W; cx++) {
            int i = cidx(s, cx, cy);
            V4 o = v4(0.0f, 0.0f, 1.0f, 1.0f);
            if (cx > 0 && cy > 0) {
                V4 me = s->cell[i];
                V4 sol = s->solid[i];
                coef_face(me, s->cell[i - 1], sol.x, &o.x, &o.z);
                coef_face(me, s->cell[i - s->W], sol.y, &o.y, &o.w);
            }
            s->coef[i] = o;
        }
}

static void k_surf_smooth(OSim* s) {
    static const float B5[5] = {1.0f, 4.0f, 6.0f, 4.0f, 1.0f};
    int more = (P_.group_mask & 12u) != 0u;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int cy = 0; cy < s->H; cy++)
        for (int cx = 0; cx < s->W; cx++) {
            V2 sum = v2(0, 0), sum2 = v2(0, 0);
            float wsum = 0.0f;
            for (int b = -2; b <= 2; b++)
                for (int a = -2; a <= 2; a++) {
                    int nx = cx + a, ny = cy + b;
                    if (nx < 0 || ny < 0 || nx >= s->W || ny >= s->H) continue;
                    int j = cidx(s, nx, ny);
                    float open = s->solid[j].w;
                    if (open <= 0.02f) continue;
                    float phi = clampf(s->cell[j].x / (REST_PHI * open), 0.0f, 1.0f);
                    float w = B5[a + 2] * B5[b + 2];
                    sum.x += w * phi;
                    sum.y += w * (phi * s->comp[j].y);
                    if (more) {
                        sum2.x += w * phi * s->aux[j].z;
                        sum2.y += w * phi * s->aux[j].w;
                    }
                    wsum += w;
                }
            int i = cidx(s, cx, cy);
            s->surf[i].x = wsum > 0.0f ? sum.x / wsum : 0.0f;
            s->surf[i].y = wsum > 0.0f ? sum.y / wsum : 0.0f;
            if (more) {
                s->surf2[i].x = wsum > 0.0f ? sum2.x / wsum : 0.0f;
                s->surf2[i].y = wsum > 0.0f ? sum2.y / wsum : 0.0f;
            }
        }
}

static float surf_field(const OSim* s, int x, int y, int k) {
    x = clampi(x, 0, s->W - 1);
    y = clampi(y, 0, s->H - 1);
    int i = cidx(s, x, y);
    if (k < 2) return k == 0 ? s->surf[i].x : s->surf[i].y;
    return k == 2 ? s->surf2[i].x : s->surf2[i].y;
}

static V2 grad_node(const OSim* s, int nx, int ny, int k) {
    float a = surf_field(s, nx, ny, k), b = surf_field(s, nx - 1, ny, k), d = surf_field(s, nx, ny - 1, k), e = surf_field(s, nx - 1, ny - 1, k);
    return v2(0.5f * (a + d - b - e), 0.5f * (a + b - d - e));
}

static float node_sdf(const OSim* s, int x, int y) {
    x = clampi(x, 0, s->W);
    y = clampi(y, 0, s->H);
    return s->sdf[y * (s->W + 1) + x];
}

static V2 contact_at(const OSim* s, int nx, int ny) {
    int i0 = cidx(s, clampi(nx, 0, s->W - 1), clampi(ny, 0, s->H - 1));
    V2 cs = v2(s->sprop[i0].y, s->sprop[i0].z);
    if (cs.x * cs.x + cs.y * cs.y > 1e-12f) {
        float l = len2(cs);
        return v2(cs.x / l, cs.y / l);
    }
    for (int b = -3; b <= 2; b++)
        for (int a = -3; a <= 2; a++) {
            int j = cidx(s, clampi(nx + a, 0, s->W - 1), clampi(ny + b, 0, s->H - 1));
            cs.x += s->sprop[j].y * s->cell[j].x;
            cs.y += s->sprop[j].z * s->cell[j].x;
        }
    if (cs.x * cs.x + cs.y * cs.y > 1e-12f) {
        float l = len2(cs);
        return v2(cs.x / l, cs.y / l);
    }
    return v2(0.0f, 1.0f);
}

static V2 normal_node(const OSim* s, int nx, int ny, int k, float* mag) {
    const float G_MIN = 0.05f, WALL_BAND = 0.5f;
    V2 g = grad_node(s, nx, ny, k);
    *mag = len2(g);
    if (*mag < G_MIN) return v2(0.0f, 0.0f);
    V2 nn = v2(-g.x / *mag, -g.y / *mag);
    if (k == 0) {
        float d = node_sdf(s, nx, ny);
        if (d < WALL_BAND) {
            V2 gw = v2(node_sdf(s, nx + 1, ny) - node_sdf(s, nx - 1, ny), node_sdf(s, nx, ny + 1) - node_sdf(s, nx, ny - 1));
            if (len2(gw) > 1e-4f) {
                float lw = len2(gw);
                V2 nw = v2(gw.x / lw, gw.y / lw);
                float gd = g.x * nw.x + g.y * nw.y;
                V2 gt = v2(g.x - gd * nw.x, g.y - gd * nw.y);
                float along = len2(gt);
                if (along > 0.5f * G_MIN) {
                    V2 t = v2(-gt.x / along, -gt.y / along);
                    V2 cs = contact_at(s, nx, ny);
                    V2 nc = v2(cs.x * nw.x + cs.y * t.x, cs.x * nw.y + cs.y * t.y);
                    float sm = smoothstepf(0.5f * G_MIN, G_MIN, along);
                    V2 m = v2(mixf(nn.x, nc.x, sm), mixf(nn.y, nc.y, sm));
                    float lm = len2(m);
                    nn = lm > 1e-4f ? v2(m.x / lm, m.y / lm) : nc;
                }
            }
        }
    }
    return nn;
}

static float curvature_at(const OSim* s, int cx, int cy, int k, float kmax) {
    float m00, m10, m01, m11;
    V2 n00 = normal_node(s, cx, cy, k, &m00);
    V2 n10 = normal_node(s, cx + 1, cy, k, &m10);
    V2 n01 = normal_node(s, cx, cy + 1, k, &m01);
    V2 n11 = normal_node(s, cx + 1, cy + 1, k, &m11);
    if (0.25f * (m00 + m10 + m01 + m11) < 0.05f) return 0.0f;
    float kap = 0.5f * (n10.x + n11.x - n00.x - n01.x) + 0.5f * (n01.y + n11.y - n00.y - n10.y);
    return kmax > 0.0f ? clampf(kap, -kmax, kmax) : kap;
}

static void k_surf_curv(OSim* s) {
    float kmax = P_.misc[0];
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int cy = 0; cy < s->H; cy++)
        for (int cx = 0; cx < s->W; cx++) {
            int i = cidx(s, cx, cy);
            float k0 = curvature_at(s, cx, cy, 0, kmax);
            float k1 = curvature_at(s, cx, cy, 1, kmax);
            s->surf[i].z = k0;
            s->surf[i].w = k1;
            if ((P_.group_mask & 12u) != 0u) {
                s->surf2[i].z = (P_.group_mask & 4u) != 0u ? curvature_at(s, cx, cy, 2, kmax) : 0.0f;
                s->surf2[i].w = (P_.group_mask & 8u) != 0u ? curvature_at(s, cx, cy, 3, kmax) : 0.0f;
            }
        }
}

static float air_jump(const OSim* s, int a, int b) {
    int la = s->cell[a].w > 0.0f;
    int liq = la ? a : b, air = la ? b : a;
    float lf = s->cell[liq].w, lgv = s->cell[air].w;
    float theta = clampf(lf / (lf - lgv), THETA_MIN, 1.0f);
    float kl = s->surf[liq].z, kg = s->surf[air].z;
    float kap = kg != 0.0f ? mixf(kl, kg, theta) : kl;
    return s->S.dt * s->sprop[liq].x * kap;
}

static float share_of(const OSim* s, int i, int g) {
    if (g == 1) return s->comp[i].y;
    if (g == 2) return s->aux[i].z;
    if (g == 3) return s->aux[i].w;
    return 1.0f - s->comp[i].y - s->aux[i].z - s->aux[i].w;
}

static float curv_of(const OSim* s, int i, int g) { return g == 1 ? s->surf[i].w : g == 2 ? s->surf2[i].z : s->surf2[i].w; }

static float pair_jump(const OSim* s, int c, int n) {
    int gc = (int)s->sprop[c].w, gn = (int)s->sprop[n].w;
    if (gc == gn) return 0.0f;
    int hi = maxi(gc, gn), lo = mini(gc, gn);
    float dc = share_of(s, c, hi) - share_of(s, c, lo), dn = share_of(s, n, hi) - share_of(s, n, lo);
    if (dc * dn >= 0.0f) return 0.0f;
    float theta = -dn / (dc - dn);
    float kc = curv_of(s, c, hi), kn = curv_of(s, n, hi);
    float kap = kc == 0.0f ? kn : kn == 0.0f ? kc : mixf(kn, kc, theta);
    float j = s->S.dt * P_.pair[hi][lo] * kap;
    return gc == hi ? j : -j;
}

static float face_jump(const OSim* s, int c, int n, float open) {
    if (open <= 0.0f) return 0.0f;
    int lc = s->cell[c].w > 0.0f, ln = s->cell[n].w > 0.0f;
    if (lc != ln) return air_jump(s, c, n);
    if (lc && ln) return pair_jump(s, c, n);
    return 0.0f;
}

static void k_surf_apply(OSim* s) {
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int cy = 0; cy < s->H; cy++)
        for (int cx = 0; cx < s->W; cx++) {
            int i = cidx(s, cx, cy);
            V2 pj = v2(0.0f, 0.0f);
            if (cx > 0 && cy > 0) {
                V4 sol = s->solid[i];
                pj.x = face_jump(s, i, i - 1, sol.x);
                pj.y = face_jump(s, i, i - s->W, sol.y);
            }
            s->pjump[i] = pj;
        }
}

/* ------------------------------------------------------------------------------------ */
/* heat.comp                                                                             */
/* ------------------------------------------------------------------------------------ */

static float y_sat(float T) {
    T = clampf(T, -40.0f, 99.0f);
    float p = 0.61078f * o_expf(17.27f * T / (T + 237.3f));
    return 0.622f * p / (101.325f - 0.378f * p);
}

static V2 centre_vel(const OSim* s, int i) {
    int last = s->W * s->H - 1;
    V4 v = s->vel[i], vr = s->vel[mini(i + 1, last)], vt = s->vel[mini(i + s->W, last)];
    V2 a = v2(face_live(v.z) ? v.x : 0.0f, face_live(v.w) ? v.y : 0.0f);
    V2 b = v2(face_live(vr.z) ? vr.x : 0.0f, face_live(vt.w) ? vt.y : 0.0f);
    return v2(0.5f * (a.x + b.x), 0.5f * (a.y + b.y));
}

static int lead_of(float w) { float f = w - floorf(w); return (int)(f * 128.0f + 0.5f); }

static void k_heat(OSim* s) {
    /* dheat is rewritten in place (dheat.x holds the emissivity on entry), so read it first */
    int W = s->W, H = s->H;
    V4* out = (V4*)malloc((size_t)W * H * sizeof(V4));
    float air_tot_pos = 0, air_tot_neg = 0;
    (void)air_tot_pos; (void)air_tot_neg;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int cy = 0; cy < H; cy++)
        for (int cx = 0; cx < W; cx++) {
            int i = cidx(s, cx, cy);
            V4 me = s->therm[i];
            float emis = s->dheat[i].x;
            float phi = s->cell[i].x;
            float k = s->S.dt * P_.heat[1];
            I2 hsum = s->hcell[i];
            V2 own = v2(0.0f, 0.0f);
            if (hsum.x > 0 && me.y > 0.0f && phi > 0.0f) {
                float rate = 5.78f * me.z * 3.14159265f / (P_.inv_ppc * me.y * P_.inv_ppc / phi);
                own = v2(1.0f - o_expf(-k * rate), (float)hsum.y / (float)hsum.x);
            }
            if (phi <= 0.04f || me.y <= 0.0f || cx < 1 || cy < 1 || cx >= W - 1 || cy >= H - 1) {
                out[i] = v4(0.0f, own.x, own.y, 0.0f);
                continue;
            }
            phi = minf(phi, 1.0f);
            int nb[4] = {i - 1, i + 1, i - W, i + W};
            float open[4] = {s->solid[i].x, s->solid[i + 1].x, s->solid[i].y, s->solid[i + W].y};
            float Tk = me.x + 273.15f, Ta = P_.heat[0] + 273.15f;
            float cond = 0.0f, air = 0.0f, wall = 0.0f, contact = 0.0f;
            float cpc = me.y * P_.inv_ppc;
            float hc = P_.heat2[3];
            int lead = lead_of(s->sprop[i].w);
            float eddy_l2 = P_.heat3[0] * P_.heat3[0] / 0.85f;
            int eddy = eddy_l2 > 0.0f && me.w < 0.5f;
            V2 u_me = eddy ? centre_vel(s, i) : v2(0.0f, 0.0f);
            float eddy_max = 0.2f / maxf(k, 1e-9f);
            float per_rate = 1.0f / maxf(P_.heat[1], 1e-6f);
            float evap = 0.0f;
            for (int q = 0; q < 4; q++) {
                int n = nb[q];
                float a = open[q];
                float pn = s->cell[n].x;
                V4 o = s->therm[n];
                if (a > 0.0f) {
                    float pl = (pn > 0.04f && o.y > 0.0f) ? minf(pn, 1.0f) : 0.0f;
                    if (pl > 0.0f) {
                        float gc = 2.0f * me.z * o.z / maxf(me.z + o.z, 1e-12f);
                        if (eddy && o.w < 0.5f && lead_of(s->sprop[n].w) == lead) {
                            V2 cn = centre_vel(s, n);
                            float strain = 1.4142f * len2(v2(cn.x - u_me.x, cn.y - u_me.y));
                            float alpha = minf(eddy_l2 * strain * per_rate, eddy_max);
                            float c1 = cpc / phi, c2 = o.y * P_.inv_ppc / pl;
                            gc += alpha * 2.0f * c1 * c2 / maxf(c1 + c2, 1e-12f);
                        }
                        cond += a * minf(phi, pl) * gc * (o.x - me.x);
                        if (hc > 0.0f && lead_of(s->sprop[n].w) != lead) {
                            float g1 = maxf(2.0f * me.z, hc), g2 = maxf(2.0f * o.z, hc);
                            float gx = maxf(g1 * g2 / (g1 + g2) - gc, 0.0f) * a * minf(phi, pl);
                            float cn = o.y * P_.inv_ppc;
                            float x = gx * k * (1.0f / cpc + 1.0f / cn);
                            contact += 0.25f * (1.0f - o_expf(-4.0f * x)) * cpc * cn / (cpc + cn) * (o.x - me.x);
                        }
                    }
                    float exposed = maxf(phi - pl, 0.0f);
                    if (exposed > 0.0f && s->solid[n].w > 0.02f) {
                        float hh = P_.heat[2] + emis * P_.heat[3] * (Ta * Ta + Tk * Tk) * (Ta + Tk);
                        air += a * exposed * hh * (P_.heat[0] - me.x);
                        if (P_.heat3[1] > 0.0f && lead > 0 && s->mats[lead - 1].ia[0] == 0 && s->mats[lead - 1].th2[2] < 150.0f && me.w < 0.5f)
                            evap += a * exposed * P_.heat[2] * P_.heat3[1] * maxf(y_sat(me.x) - y_sat(P_.heat[0]), 0.0f);
                    }
                }
                if (a < 1.0f) {
                    float ts = maxf(s->solid_t[n], s->solid_t[i]);
                    if (ts > 0.5f * NO_TEMP) wall += (1.0f - a) * phi * 2.0f * me.z * (ts - me.x);
                }
            }
            if (evap > 0.0f) air -= evap;
            air *= k;
            wall *= k;
            float lim = cpc * fabsf(P_.heat[0] - me.x);
            air = clampf(air, -lim, lim);
            float e = k * cond + contact + air + wall;
            out[i] = v4(e / cpc, own.x, own.y, 0.0f);
            if (air > 0.0f) ledger_add(s, 0, air); else ledger_add(s, 1, -air);
            if (wall > 0.0f) ledger_add(s, 2, wall); else ledger_add(s, 3, -wall);
        }
    memcpy(s->dheat, out, (size_t)W * H * sizeof(V4));
    free(out);
}

/* ------------------------------------------------------------------------------------ */
/* Explicit viscosity: visc.glsl, visc_setup.comp, visc_apply.comp mode 2                 */
/* ------------------------------------------------------------------------------------ */

static inline int live_u(const OSim* s, int i) { return face_live(s->vel[i].z); }
static inline int live_v(const OSim* s, int i) { return face_live(s->vel[i].w); }
static inline int closed_u(const OSim* s, int i) { return face_closed(s->vel[i].z); }
static inline int closed_v(const OSim* s, int i) { return face_closed(s->vel[i].w); }
static inline float vel_u(const OSim* s, int i) { return live_u(s, i) ? s->vel[i].x : 0.0f; }
static inline float vel_v(const OSim* s, int i) { return live_v(s, i) ? s->vel[i].y : 0.0f; }

static V4 strain_of_vel(const OSim* s, int i, V2 w) {
    int W = s->W;
    V4 o = v4(0, 0, 0, 0);
    if (w.x > 0.0f) {
        o.x = w.x * (vel_u(s, i + 1) - vel_u(s, i));
        o.y = w.x * (vel_v(s, i + W) - vel_v(s, i));
    }
    if (w.y > 0.0f) {
        float ua = vel_u(s, i), ub = vel_u(s, i - W), va = vel_v(s, i), vb = vel_v(s, i - 1);
        if (closed_u(s, i) && live_u(s, i - W)) ua = -ub;
        if (closed_u(s, i - W) && live_u(s, i)) ub = -ua;
        if (closed_v(s, i) && live_v(s, i - 1)) va = -vb;
        if (closed_v(s, i - 1) && live_v(s, i)) vb = -va;
        o.z = w.y * 0.5f * ((ua - ub) + (va - vb));
    }
    return o;
}

static inline int ok_u(const OSim* s, int i) { return live_u(s, i) || closed_u(s, i); }
static inline int ok_v(const OSim* s, int i) { return live_v(s, i) || closed_v(s, i); }

static void k_visc_setup(OSim* s) {
    int W = s->W, H = s->H;
    float dt = s->S.dt;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int cy = 0; cy < H; cy++)
        for (int cx = 0; cx < W; cx++) {
            int i = cidx(s, cx, cy);
            float wc = 0.0f, wn = 0.0f;
            if (cx >= 1 && cy >= 1 && cx < W - 1 && cy < H - 1) {
                V4 me = s->cell[i];
                if (me.w > 0.0f && ok_u(s, i) && ok_u(s, i + 1) && ok_v(s, i) && ok_v(s, i + W)) wc = 2.0f * dt * me.z;
                int cs[4] = {i - W - 1, i - W, i - 1, i};
                int nliq = 0, any_air = 0;
                float mu = 0.0f;
                for (int k = 0; k < 4; k++) {
                    V4 q = s->cell[cs[k]];
                    if (q.w > 0.0f) {
                        nliq++;
                        mu += q.z;
                    } else if (s->solid[cs[k]].w > 0.02f) {
                        any_air = 1;
                    }
                }
                if (nliq > 0 && !any_air && ok_u(s, i) && ok_u(s, i - W) && ok_v(s, i) && ok_v(s, i - 1))
                    wn = 4.0f * dt * (mu / (float)nliq) * ((float)nliq / 4.0f);
            }
            s->vw[i].x = wc;
            s->vw[i].y = wn;
            /* the tiles that need the implicit solve (visc_setup.comp:111-120) */
            V4 me = s->cell[i];
            if (s->visc_mode == 2 && me.w > 0.0f && dt * me.z / maxf(me.y, 0.05f) >= P_.corr[3]) {
                int tw = (W + 15) >> 4;
                for (int b = -1; b <= 1; b++)
                    for (int a = -1; a <= 1; a++) {
                        int nx = clampi(cx + a, 0, W - 1), ny = clampi(cy + b, 0, H - 1);
                        s->tiles[(ny >> 4) * tw + (nx >> 4)] = 1u;
                    }
            }
        }
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int i = 0; i < W * H; i++) s->vs[i] = strain_of_vel(s, i, v2(s->vw[i].x, s->vw[i].y));
}

static V2 gts(const OSim* s, int i) {
    int W = s->W;
    V2 g = v2(0.0f, 0.0f);
    if (live_u(s, i)) {
        float c1 = closed_u(s, i - W) ? 1.0f : 0.5f, c2 = closed_u(s, i + W) ? -1.0f : -0.5f;
        g.x = s->vs[i - 1].x - s->vs[i].x + s->vs[i].z * c1 + s->vs[i + W].z * c2;
    }
    if (live_v(s, i)) {
        float d1 = closed_v(s, i - 1) ? 1.0f : 0.5f, d2 = closed_v(s, i + 1) ? -1.0f : -0.5f;
        g.y = s->vs[i - W].y - s->vs[i].y + s->vs[i].z * d1 + s->vs[i + 1].z * d2;
    }
    return g;
}

static void k_visc_apply_explicit(OSim* s) {
    int W = s->W, H = s->H;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int cy = 1; cy < H - 1; cy++)
        for (int cx = 1; cx < W - 1; cx++) {
            int i = cidx(s, cx, cy);
            V2 g = gts(s, i);
            int lu = live_u(s, i), lv = live_v(s, i);
            V4 cf = s->coef[i];
            V4 v = s->vel[i];
            if (lu) v.x -= g.x / cf.z;
            if (lv) v.y -= g.y / cf.w;
            s->vel[i].x = v.x;
            s->vel[i].y = v.y;
        }
}

/* ------------------------------------------------------------------------------------ */
/* rhs.comp                                                                              */
/* ------------------------------------------------------------------------------------ */

static void k_rhs(OSim* s) {
    int W = s->W, H = s->H;
    int tw = (W + 15) / 16;
    float dt = s->S.dt;
    float gain = P_.corr_gain;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int cy = 0; cy < H; cy++)
        for (int cx = 0; cx < W; cx++) {
            int i = cidx(s, cx, cy);
            V4 me = s->cell[i];
            if (me.w <= 0.0f || cx == 0 || cy == 0 || cx == W - 1 || cy == H - 1) {
                s->mga[i] = v4(0, 0, 0, 0);
                s->mgd[i] = 0.0f;
                s->prhs[i] = v4(0, 0, 0, 0);
                continue;
            }
            V4 sol = s->solid[i];
            V4 cf = s->coef[i];
            float aL = sol.x, aB = sol.y, aR = s->solid[i + 1].x, aT = s->solid[i + W].y;
            V4 w = v4(aL * cf.x, aR * s->coef[i + 1].x, aB * cf.y, aT * s->coef[i + W].y);
            float diag = w.x + w.y + w.z + w.w;
            {
                uint32_t rg = s->region[i];
                if ((rg & REGION_VENT) != 0u && (s->region_air & (1u << (rg & REGION_MASK))) == 0u && P_.misc[1] > 0.0f)
                    diag += 1.0f / maxf(me.y, 0.05f);
            }
            V4 vme = s->vel[i];
            float div = aR * s->vel[i + 1].x - aL * vme.x + aT * s->vel[i + W].y - aB * vme.y;
            int lL = s->cell[i - 1].w > 0.0f, lR = s->cell[i + 1].w > 0.0f, lB = s->cell[i - W].w > 0.0f, lT = s->cell[i + W].w > 0.0f;
            (void)lL; (void)lB;
            float jump = w.x * s->pjump[i].x + w.y * (lR ? -s->pjump[i + 1].x : s->pjump[i + 1].x)
                       + w.z * s->pjump[i].y + w.w * (lT ? -s->pjump[i + W].y : s->pjump[i + W].y);
            float err = clampf(s->comp[i].w - REST_PHI, -0.5f, 0.5f);
            {
                int interior = (aL <= 0.0f || s->cell[i - 1].w > 0.0f) && (aR <= 0.0f || s->cell[i + 1].w > 0.0f)
                            && (aB <= 0.0f || s->cell[i - W].w > 0.0f) && (aT <= 0.0f || s->cell[i + W].w > 0.0f);
                int pressed = s->pres[i].x * (dt / s->S.dt_prev) > 0.5f * me.y * P_.gravity * dt;
                if (interior && !pressed) err = maxf(err - P_.corr[1], 0.0f);
                else if (!interior && err < 0.0f) err = 0.0f;
            }
            float sv = gain * err;
            if ((s->region_air & (1u << (s->region[i] & REGION_MASK))) == 0u && P_.misc[1] > 0.0f) sv = 0.0f;
            if (diag > 1e-9f) {
                int t = (cy >> 4) * tw + (cx >> 4);
                s->ptile[t] = 1u;
            }
            s->mga[i] = diag > 1e-9f ? w : v4(0, 0, 0, 0);
            s->mgd[i] = diag > 1e-9f ? diag : 0.0f;
            s->prhs[i] = v4(-div + jump, sv / dt, 0.0f, 0.0f);
        }
}

/* ------------------------------------------------------------------------------------ */
/* Pressure MGPCG: mg_build, mg_tail, mg_down, mg_up, cg_*, reduce_tail                   */
/* ------------------------------------------------------------------------------------ */

static inline float wcomp(V4 w, int k) { return k == 0 ? w.x : k == 1 ? w.y : k == 2 ? w.z : w.w; }
static const int NBX[4] = {-1, 1, 0, 0}, NBY[4] = {0, 0, -1, 1};

typedef struct Lv { int off, w, h, toff; } Lv;
static Lv lev(const OSim* s, int l) { Lv r = {s->lv.offs[l], s->lv.dims[l][0], s->lv.dims[l][1], s->lv.tile_offs[l]}; return r; }
static inline int l_inside(Lv L, int x, int y) { return x >= 0 && y >= 0 && x < L.w && y < L.h; }
static inline int l_at(Lv L, int x, int y) { return L.off + y * L.w + x; }
static inline int l_unknown(const OSim* s, Lv L, int x, int y) { return l_inside(L, x, y) && s->mgd[l_at(L, x, y)] > 0.0f; }

/* mg_build.comp: level l+1 from level l, tile by tile of level l+1 */
static void k_mg_build(OSim* s, int l) {
    Lv F = lev(s, l), C = lev(s, l + 1);
    int tfx = (F.w + 15) >> 4, tfy = (F.h + 15) >> 4;
    int tcx = (C.w + 15) >> 4, tcy = (C.h + 15) >> 4;
    for (int ty = 0; ty < tcy; ty++)
        for (int tx = 0; tx < tcx; tx++) {
            uint32_t on = 0;
            for (int k = 0; k < 4; k++) {
                int fx = 2 * tx + (k & 1), fy = 2 * ty + (k >> 1);
                if (fx < tfx && fy < tfy) on |= s->ptile[F.toff + fy * tfx + fx];
            }
            uint32_t slot = (uint32_t)C.toff + (uint32_t)(ty * tcx + tx);
            uint32_t was = s->ptile[slot];
            s->ptile[slot] = on != 0u ? 1u : 0u;
            uint32_t state = (on != 0u ? 1u : 0u) | (was != 0u ? 2u : 0u);
            if (state == 0u) continue;
            for (int ly = 0; ly < 16; ly++)
                for (int lx = 0; lx < 16; lx++) {
                    int Cx = tx * 16 + lx, Cy = ty * 16 + ly;
                    if (Cx >= C.w || Cy >= C.h) continue;
                    int o = l_at(C, Cx, Cy);
                    if ((state & 1u) == 0u) {
                        s->mgd[o] = 0.0f;
                        s->mga[o] = v4(0, 0, 0, 0);
                        continue;
                    }
                    float D = 0.0f;
                    V4 A = v4(0, 0, 0, 0);
                    for (int k = 0; k < 4; k++) {
                        int cx = 2 * Cx + (k & 1), cy = 2 * Cy + (k >> 1);
                        if (!l_unknown(s, F, cx, cy)) continue;
                        int i = l_at(F, cx, cy);
                        D += s->mgd[i];
                        V4 w = s->mga[i];
                        for (int d = 0; d < 4; d++) {
                            int nx = cx + NBX[d], ny = cy + NBY[d];
                            if (!l_unknown(s, F, nx, ny)) continue;
                            float wd = wcomp(w, d);
                            if ((nx >> 1) == Cx && (ny >> 1) == Cy) D -= wd;
                            else if (d == 0) A.x += wd;
                            else if (d == 1) A.y += wd;
                            else if (d == 2) A.z += wd;
                            else A.w += wd;
                        }
                    }
                    s->mgd[o] = D > 1e-7f ? D : 0.0f;
                    s->mga[o] = D > 1e-7f ? A : v4(0, 0, 0, 0);
                }
        }
}

/* mg_tail.comp mode 1: Galerkin matrices of the tail levels */
static void k_tail_build(OSim* s) {
    for (int l = s->lv.tail; l < s->lv.n - 1; l++) {
        Lv F = lev(s, l), C = lev(s, l + 1);
        for (int t = 0; t < C.w * C.h; t++) {
            int ccx = t % C.w, ccy = t / C.w;
            float D = 0.0f;
            V4 A = v4(0, 0, 0, 0);
            for (int k = 0; k < 4; k++) {
                int cx = 2 * ccx + (k & 1), cy = 2 * ccy + (k >> 1);
                if (!l_unknown(s, F, cx, cy)) continue;
                int i = l_at(F, cx, cy);
                D += s->mgd[i];
                V4 w = s->mga[i];
                for (int d = 0; d < 4; d++) {
                    int nx = cx + NBX[d], ny = cy + NBY[d];
                    if (!l_unknown(s, F, nx, ny)) continue;
                    float wd = wcomp(w, d);
                    if ((nx >> 1) == ccx && (ny >> 1) == ccy) D -= wd;
                    else if (d == 0) A.x += wd;
                    else if (d == 1) A.y += wd;
                    else if (d == 2) A.z += wd;
                    else A.w += wd;
                }
            }
            int o = C.off + t;
            s->mgd[o] = D > 1e-7f ? D : 0.0f;
            s->mga[o] = D > 1e-7f ? A : v4(0, 0, 0, 0);
        }
    }
}

static inline int tile_on(const OSim* s, Lv L, int tx, int ty) {
    int tw = (L.w + 15) >> 4;
    return s->ptile[L.toff + ty * tw + tx] != 0u;
}

/* mg_down.comp black(): value of black cell n after the half-sweep from zero */
static V2 down_black(const OSim* s, Lv L, int nx, int ny) {
    int i = l_at(L, nx, ny);
    V4 w = s->mga[i];
    V2 sum = s->mgr[i];
    for (int d = 0; d < 4; d++) {
        int mx = nx + NBX[d], my = ny + NBY[d];
        if (!l_unknown(s, L, mx, my)) continue;
        int j = l_at(L, mx, my);
        float wd = wcomp(w, d);
        sum.x += wd * s->mgr[j].x / s->mgd[j];
        sum.y += wd * s->mgr[j].y / s->mgd[j];
    }
    return v2(sum.x / s->mgd[i], sum.y / s->mgd[i]);
}

static void k_mg_down(OSim* s, int l) {
    Lv F = lev(s, l), C = lev(s, l + 1);
    int tw = (F.w + 15) >> 4, th = (F.h + 15) >> 4;
    for (int ty = 0; ty < th; ty++)
        for (int tx = 0; tx < tw; tx++) {
            if (!tile_on(s, F, tx, ty)) continue;
            V2 sz[256];
            for (int ly = 0; ly < 16; ly++)
                for (int lx = 0; lx < 16; lx++) {
                    int cx = tx * 16 + lx, cy = ty * 16 + ly;
                    int red = ((cx + cy) & 1) == 0;
                    int unk = l_unknown(s, F, cx, cy);
                    V2 z = v2(0, 0);
                    if (l_inside(F, cx, cy)) {
                        int i = l_at(F, cx, cy);
                        if (unk) z = red ? v2(s->mgr[i].x / s->mgd[i], s->mgr[i].y / s->mgd[i]) : down_black(s, F, cx, cy);
                        s->mgx[i] = z;
                    }
                    sz[ly * 16 + lx] = z;
                }
            for (int ly = 0; ly < 16; ly += 2)
                for (int lx = 0; lx < 16; lx += 2) {
                    int cx = tx * 16 + lx, cy = ty * 16 + ly;
                    int Cx = cx >> 1, Cy = cy >> 1;
                    if (Cx >= C.w || Cy >= C.h) continue;
                    V2 sum = v2(0, 0);
                    for (int k = 0; k < 2; k++) {
                        int qx = cx + k, qy = cy + k;
                        if (!l_unknown(s, F, qx, qy)) continue;
                        V4 w = s->mga[l_at(F, qx, qy)];
                        int lqx = lx + k, lqy = ly + k;
                        for (int d = 0; d < 4; d++) {
                            int nx = qx + NBX[d], ny = qy + NBY[d];
                            if (!l_unknown(s, F, nx, ny)) continue;
                            int lnx = lqx + NBX[d], lny = lqy + NBY[d];
                            int here = lnx >= 0 && lny >= 0 && lnx < 16 && lny < 16;
                            V2 zb = here ? sz[lny * 16 + lnx] : down_black(s, F, nx, ny);
                            float wd = wcomp(w, d);
                            sum.x += wd * zb.x;
                            sum.y += wd * zb.y;
                        }
                    }
                    s->mgr[l_at(C, Cx, Cy)] = sum;
                }
        }
}

/* mg_up.comp black(): new value of black cell n after the coarse correction */
static V2 up_black(const OSim* s, Lv L, Lv C, int nx, int ny) {
    int i = l_at(L, nx, ny);
    V4 w = s->mga[i];
    V2 sum = s->mgr[i];
    for (int d = 0; d < 4; d++) {
        int mx = nx + NBX[d], my = ny + NBY[d];
        if (!l_unknown(s, L, mx, my)) continue;
        V2 xm = s->mgx[l_at(L, mx, my)];
        V2 zc = s->mgz[l_at(C, mx >> 1, my >> 1)];
        float wd = wcomp(w, d);
        sum.x += wd * (xm.x + MG_OMEGA * zc.x);
        sum.y += wd * (xm.y + MG_OMEGA * zc.y);
    }
    return v2(sum.x / s->mgd[i], sum.y / s->mgd[i]);
}

/* work-group sum of reduce.glsl:5-14: the tree over 256 invocations */
static V4 group_tree(V4 buf[256]) {
    for (int st = 128; st > 0; st >>= 1)
        for (int t = 0; t < st; t++) {
            buf[t].x += buf[t + st].x;
            buf[t].y += buf[t + st].y;
            buf[t].z += buf[t + st].z;
            buf[t].w += buf[t + st].w;
        }
    return buf[0];
}

/* mg_up on level l; on level 0 (flag) writes part[slot] = (r.z, r.r) sums */
static void k_mg_up(OSim* s, int l, int flag) {
    Lv F = lev(s, l), C = lev(s, l + 1);
    int tw = (F.w + 15) >> 4, th = (F.h + 15) >> 4;
    for (int ty = 0; ty < th; ty++)
        for (int tx = 0; tx < tw; tx++) {
            int slot = ty * tw + tx;
            if (!tile_on(s, F, tx, ty)) {
                if (flag) s->part[slot] = v4(0, 0, 0, 0);
                continue;
            }
            V2 sz[256];
            V4 accb[256];
            for (int ly = 0; ly < 16; ly++)
                for (int lx = 0; lx < 16; lx++) {
                    int cx = tx * 16 + lx, cy = ty * 16 + ly;
                    int red = ((cx + cy) & 1) == 0;
                    V2 z = v2(0, 0);
                    if (l_unknown(s, F, cx, cy) && !red) z = up_black(s, F, C, cx, cy);
                    sz[ly * 16 + lx] = z;
                }
            for (int ly = 0; ly < 16; ly++)
                for (int lx = 0; lx < 16; lx++) {
                    int cx = tx * 16 + lx, cy = ty * 16 + ly;
                    int red = ((cx + cy) & 1) == 0;
                    V2 z = sz[ly * 16 + lx];
                    V4 a4 = v4(0, 0, 0, 0);
                    if (l_inside(F, cx, cy)) {
                        int i = l_at(F, cx, cy);
                        if (l_unknown(s, F, cx, cy)) {
                            V2 r = s->mgr[i];
                            if (red) {
                                V4 w = s->mga[i];
                                V2 sum = r;
                                for (int d = 0; d < 4; d++) {
                                    int nx = cx + NBX[d], ny = cy + NBY[d];
                                    if (!l_unknown(s, F, nx, ny)) continue;
                                    int lnx = lx + NBX[d], lny = ly + NBY[d];
                                    int here = lnx >= 0 && lny >= 0 && lnx < 16 && lny < 16;
                                    V2 zb = here ? sz[lny * 16 + lnx] : up_black(s, F, C, nx, ny);
                                    float wd = wcomp(w, d);
                                    sum.x += wd * zb.x;
                                    sum.y += wd * zb.y;
                                }
                                z = v2(sum.x / s->mgd[i], sum.y / s->mgd[i]);
                            }
                            a4 = v4(r.x * z.x, r.y * z.y, r.x * r.x, r.y * r.y);
                        }
                        s->mgz[i] = z;
                    }
                    accb[ly * 16 + lx] = a4;
                }
            if (flag) s->part[slot] = group_tree(accb);
        }
}

/* mg_tail.comp mode 0: the V-cycle on the tail levels, rhs in mgr[first], result in mgz[first] */
static void k_tail_vcycle(OSim* s) {
    int first = s->lv.tail, last = s->lv.n - 1;
    Lv Fst = lev(s, first);
    int base = Fst.off;
    Lv E = lev(s, last);
    int total = E.off + E.w * E.h - base;
    int nf = Fst.w * Fst.h;
    V2* sx = (V2*)calloc((size_t)total, sizeof(V2));
    float* sd = (float*)malloc((size_t)total * sizeof(float));
    V2* sr = (V2*)calloc((size_t)(total > nf ? total - nf : 1), sizeof(V2));
    for (int t = 0; t < total; t++) sd[t] = s->mgd[base + t];
#define RHS_AT(sl) ((sl) < nf ? s->mgr[base + (sl)] : sr[(sl) - nf])
#define SAT(L, x, y) ((L).off - base + (y) * (L).w + (x))
#define SUNK(L, x, y) (l_inside((L), (x), (y)) && sd[SAT((L), (x), (y))] > 0.0f)
    /* A half-sweep reads only cells of the other colour (5-point stencil), so the loop
     * order within it does not change the result. */
#define SWEEP(L, colour, zero)                                                                 \
    do {                                                                                      \
        for (int t = 0; t < (L).w * (L).h; t++) {                                             \
            int x = t % (L).w, y = t / (L).w;                                                 \
            int sl = (L).off - base + t;                                                      \
            float D = sd[sl];                                                                 \
            if (D <= 0.0f) { if (zero) sx[sl] = v2(0, 0); continue; }                         \
            if (((x + y) & 1) != (colour)) { if (zero) sx[sl] = v2(0, 0); continue; }         \
            V2 sum = RHS_AT(sl);                                                              \
            if (!(zero)) {                                                                    \
                V4 w = s->mga[base + sl];                                                     \
                for (int d = 0; d < 4; d++) {                                                 \
                    int nx = x + NBX[d], ny = y + NBY[d];                                     \
                    if (SUNK(L, nx, ny)) {                                                    \
                        float wd = wcomp(w, d);                                               \
                        V2 xn = sx[SAT(L, nx, ny)];                                           \
                        sum.x += wd * xn.x;                                                   \
                        sum.y += wd * xn.y;                                                   \
                    }                                                                         \
                }                                                                             \
            }                                                                                 \
            sx[sl] = v2(sum.x / D, sum.y / D);                                                \
        }                                                                                     \
    } while (0)
    for (int l = first; l < last; l++) {
        Lv L = lev(s, l), C = lev(s, l + 1);
        SWEEP(L, 0, 1);
        SWEEP(L, 1, 0);
        for (int t = 0; t < C.w * C.h; t++) {
            int ccx = t % C.w, ccy = t / C.w;
            V2 sum = v2(0, 0);
            for (int k = 0; k < 4; k++) {
                int cx = 2 * ccx + (k & 1), cy = 2 * ccy + (k >> 1);
                if (!SUNK(L, cx, cy)) continue;
                int sl = SAT(L, cx, cy);
                V4 w = s->mga[base + sl];
                V2 az = v2(sd[sl] * sx[sl].x, sd[sl] * sx[sl].y);
                for (int d = 0; d < 4; d++) {
                    int nx = cx + NBX[d], ny = cy + NBY[d];
                    if (SUNK(L, nx, ny)) {
                        float wd = wcomp(w, d);
                        V2 xn = sx[SAT(L, nx, ny)];
                        az.x -= wd * xn.x;
                        az.y -= wd * xn.y;
                    }
                }
                V2 rh = RHS_AT(sl);
                sum.x += rh.x - az.x;
                sum.y += rh.y - az.y;
            }
            sr[C.off - base + t - nf] = sum;
        }
    }
    {
        Lv L = lev(s, last);
        SWEEP(L, 0, 1);
        for (int st = 1; st < 9; st++) SWEEP(L, st & 1, 0);
    }
    for (int l = last - 1; l >= first; l--) {
        Lv F = lev(s, l), C = lev(s, l + 1);
        for (int t = 0; t < F.w * F.h; t++) {
            int x = t % F.w, y = t / F.w;
            if (((x + y) & 1) == 0) continue;
            int sl = F.off - base + t;
            float D = sd[sl];
            if (D <= 0.0f) continue;
            V4 w = s->mga[base + sl];
            V2 sum = RHS_AT(sl);
            for (int d = 0; d < 4; d++) {
                int nx = x + NBX[d], ny = y + NBY[d];
                if (!SUNK(F, nx, ny)) continue;
                float wd = wcomp(w, d);
                V2 xn = sx[SAT(F, nx, ny)];
                V2 xc = sx[SAT(C, nx >> 1, ny >> 1)];
                sum.x += wd * (xn.x + MG_OMEGA * xc.x);
                sum.y += wd * (xn.y + MG_OMEGA * xc.y);
            }
            sx[sl] = v2(sum.x / D, sum.y / D);
        }
        SWEEP(F, 0, 0);
    }
    for (int t = 0; t < nf; t++) s->mgz[base + t] = sx[t];
#undef SWEEP
#undef SUNK
#undef SAT
#undef RHS_AT
    free(sx);
    free(sd);
    free(sr);
}

static void vcycle(OSim* s) {
    for (int l = 0; l < s->lv.tail; l++) k_mg_down(s, l);
    k_tail_vcycle(s);
    for (int l = s->lv.tail - 1; l >= 0; l--) k_mg_up(s, l, l == 0);
}

/* reduce_tail.glsl:28-41: sum of n partials starting at base, in the shader's order */
static V4 total(const OSim* s, int base, int n) {
    V4 buf[256];
    for (int t = 0; t < 256; t++) {
        V4 a = v4(0, 0, 0, 0);
        for (int k = t; k < n; k += 256) {
            a.x += s->part[base + k].x;
            a.y += s->part[base + k].y;
            a.z += s->part[base + k].z;
            a.w += s->part[base + k].w;
        }
        buf[t] = a;
    }
    return group_tree(buf);
}

static void k_cg_scale(OSim* s, int mode) {
    Lv F = lev(s, 0);
    float ratio = s->S.dt / s->S.dt_prev;
    for (int cy = 0; cy < F.h; cy++)
        for (int cx = 0; cx < F.w; cx++) {
            if (!tile_on(s, F, cx >> 4, cy >> 4)) continue;
            int i = l_at(F, cx, cy);
            if (s->mgd[i] > 0.0f) {
                float p = s->pres[i].x;
                if (mode == 1) p -= s->p2keep[i];
                else s->p2keep[i] = 0.0f;
                s->pres[i].x = p * ratio;
            } else {
                s->pres[i] = v2(0, 0);
            }
        }
}

static void k_cg_init(OSim* s) {
    Lv F = lev(s, 0);
    int tw = (F.w + 15) >> 4, th = (F.h + 15) >> 4;
    int n = s->nwg;
    for (int ty = 0; ty < th; ty++)
        for (int tx = 0; tx < tw; tx++) {
            int slot = ty * tw + tx;
            if (!tile_on(s, F, tx, ty)) {
                s->part[n + slot] = v4(0, 0, 0, 0);
                continue;
            }
            V4 accb[256];
            for (int ly = 0; ly < 16; ly++)
                for (int lx = 0; lx < 16; lx++) {
                    int cx = tx * 16 + lx, cy = ty * 16 + ly;
                    V4 a4 = v4(0, 0, 0, 0);
                    if (l_inside(F, cx, cy)) {
                        int i = l_at(F, cx, cy);
                        float D = s->mgd[i];
                        if (D > 0.0f) {
                            V2 x = s->pres[i];
                            V4 w = s->mga[i];
                            V2 ax = v2(D * x.x, D * x.y);
                            for (int d = 0; d < 4; d++) {
                                int nx = cx + NBX[d], ny = cy + NBY[d];
                                if (l_unknown(s, F, nx, ny)) {
                                    float wd = wcomp(w, d);
                                    V2 pn = s->pres[l_at(F, nx, ny)];
                                    ax.x -= wd * pn.x;
                                    ax.y -= wd * pn.y;
                                }
                            }
                            V2 b = v2(s->prhs[i].x, s->prhs[i].y);
                            s->mgr[i] = v2(b.x - ax.x, b.y - ax.y);
                            a4 = v4(b.x * b.x, b.y * b.y, 0.0f, 0.0f);
                        } else {
                            s->mgr[i] = v2(0, 0);
                        }
                    }
                    accb[ly * 16 + lx] = a4;
                }
            s->part[n + slot] = group_tree(accb);
        }
}

static V2 cg_direction(const OSim* s, const V2* cgp, int i) {
    V2 z = s->mgz[i];
    const float* b = s->K.p_beta;
    if (b[0] == 0.0f && b[1] == 0.0f) return z;
    V2 po = cgp[i];
    return v2(b[0] != 0.0f ? z.x + b[0] * po.x : z.x, b[1] != 0.0f ? z.y + b[1] * po.y : z.y);
}

static void k_cg_apply(OSim* s, const V2* cgp, V2* cgp2) {
    Lv F = lev(s, 0);
    int tw = (F.w + 15) >> 4, th = (F.h + 15) >> 4;
    int n = s->nwg;
    for (int ty = 0; ty < th; ty++)
        for (int tx = 0; tx < tw; tx++) {
            int slot = ty * tw + tx;
            if (!tile_on(s, F, tx, ty)) {
                s->part[n + slot] = v4(0, 0, 0, 0);
                continue;
            }
            V4 accb[256];
            for (int ly = 0; ly < 16; ly++)
                for (int lx = 0; lx < 16; lx++) {
                    int cx = tx * 16 + lx, cy = ty * 16 + ly;
                    V4 a4 = v4(0, 0, 0, 0);
                    if (l_inside(F, cx, cy)) {
                        int i = l_at(F, cx, cy);
                        float D = s->mgd[i];
                        if (D > 0.0f) {
                            V2 p = cg_direction(s, cgp, i);
                            V4 w = s->mga[i];
                            V2 q = v2(D * p.x, D * p.y);
                            for (int d = 0; d < 4; d++) {
                                int nx = cx + NBX[d], ny = cy + NBY[d];
                                if (l_unknown(s, F, nx, ny)) {
                                    V2 pn = cg_direction(s, cgp, l_at(F, nx, ny));
                                    float wd = wcomp(w, d);
                                    q.x -= wd * pn.x;
                                    q.y -= wd * pn.y;
                                }
                            }
                            cgp2[i] = p;
                            s->cgq[i] = q;
                            a4 = v4(0.0f, 0.0f, p.x * q.x, p.y * q.y);
                        } else {
                            cgp2[i] = v2(0, 0);
                        }
                    }
                    accb[ly * 16 + lx] = a4;
                }
            s->part[n + slot] = group_tree(accb);
        }
}

static void k_cg_update(OSim* s, const V2* cgp2) {
    Lv F = lev(s, 0);
    const float* a = s->K.p_alpha;
    for (int cy = 0; cy < F.h; cy++)
        for (int cx = 0; cx < F.w; cx++) {
            if (!tile_on(s, F, cx >> 4, cy >> 4)) continue;
            int i = l_at(F, cx, cy);
            if (s->mgd[i] <= 0.0f) continue;
            s->pres[i].x += a[0] * cgp2[i].x;
            s->pres[i].y += a[1] * cgp2[i].y;
            s->mgr[i].x -= a[0] * s->cgq[i].x;
            s->mgr[i].y -= a[1] * s->cgq[i].y;
        }
}

/* reduce_tail.glsl:61-116, the pressure modes */
static void reduce_start(OSim* s, int mode) {
    int n = s->nwg;
    V4 a = total(s, 0, n), b = total(s, n, n);
    SolveBuf* K = &s->K;
    K->p_bb[0] = b.x;
    K->p_bb[1] = b.y;
    K->p_rz[0] = a.x;
    K->p_rz[1] = a.y;
    K->p_rr[0] = a.z;
    K->p_rr[1] = a.w;
    K->p_beta[0] = K->p_beta[1] = 0.0f;
    K->p_alpha[0] = K->p_alpha[1] = 0.0f;
    K->p_iters[0] = K->p_iters[1] = 0u;
    float tx = P_.tol[0], ty = P_.tol[1];
    K->p_done[0] = a.z <= tx * tx * b.x;
    K->p_done[1] = a.w <= ty * ty * b.y;
    if (mode == 8) K->p_done[1] = 1u;
    K->solves += 1u;
}

static void reduce_alpha(OSim* s) {
    int n = s->nwg;
    V4 b = total(s, n, n);
    SolveBuf* K = &s->K;
    float ax = 0.0f, ay = 0.0f;
    if (K->p_done[0] == 0u && b.z > 0.0f) ax = K->p_rz[0] / b.z;
    if (K->p_done[1] == 0u && b.w > 0.0f) ay = K->p_rz[1] / b.w;
    K->p_alpha[0] = ax;
    K->p_alpha[1] = ay;
}

static void reduce_beta(OSim* s) {
    int n = s->nwg;
    V4 a = total(s, 0, n);
    SolveBuf* K = &s->K;
    uint32_t was0 = K->p_done[0], was1 = K->p_done[1];
    K->p_iters[0] += 1u - was0;
    K->p_iters[1] += 1u - was1;
    float tx = P_.tol[0], ty = P_.tol[1];
    uint32_t now0 = a.z <= tx * tx * K->p_bb[0], now1 = a.w <= ty * ty * K->p_bb[1];
    uint32_t d0 = was0 > now0 ? was0 : now0, d1 = was1 > now1 ? was1 : now1;
    float bx = 0.0f, by = 0.0f;
    if (d0 == 0u && K->p_rz[0] > 0.0f) bx = a.x / K->p_rz[0];
    if (d1 == 0u && K->p_rz[1] > 0.0f) by = a.y / K->p_rz[1];
    K->p_beta[0] = bx;
    K->p_beta[1] = by;
    K->p_rz[0] = a.x;
    K->p_rz[1] = a.y;
    K->p_rr[0] = mixf(a.z, K->p_rr[0], (float)was0);
    K->p_rr[1] = mixf(a.w, K->p_rr[1], (float)was1);
    K->p_done[0] = d0;
    K->p_done[1] = d1;
}

static void reduce_end(OSim* s, int mode) {
    SolveBuf* K = &s->K;
    if (mode == 3) {
        uint32_t m = K->p_iters[0] > K->p_iters[1] ? K->p_iters[0] : K->p_iters[1];
        if (m > K->p_it_max) K->p_it_max = m;
        if (K->p_done[0] == 0u) K->p_unconv += 1u;
        if (m > K->f_it[0]) K->f_it[0] = m;
        if (K->p_done[0] == 0u) K->f_un[0] += 1u;
    } else {
        if (K->p_iters[0] > K->p2_it_max) K->p2_it_max = K->p_iters[0];
        if (K->p_done[0] == 0u) K->p2_unconv += 1u;
        if (K->p_iters[0] > K->f_it[1]) K->f_it[1] = K->p_iters[0];
        if (K->p_done[0] == 0u) K->f_un[1] += 1u;
    }
    float rel = K->p_bb[0] > 0.0f ? sqrtf(K->p_rr[0] / K->p_bb[0]) : 0.0f;
    K->p_res_max = maxf(K->p_res_max, rel);
}

/* record_pressure + record_cg (mod.rs:2956-3010): the iterations run until both potentials
 * are done or the frame's recorded iterations (K.cap) have run. */
static void pressure_solve(OSim* s, int second) {
    if (!second) {
        for (int l = 1; l <= s->lv.tail; l++) k_mg_build(s, l - 1);
        if (s->lv.tail < s->lv.n - 1) k_tail_build(s);
        int warm = s->visc_mode == 2 && s->prm.viscous_projection != 0 && s->prm.viscous_warm != 0;
        k_cg_scale(s, warm ? 1 : 0);
    }
    k_cg_init(s);
    vcycle(s);
    reduce_start(s, second ? 8 : 0);
    V2* pa = s->cgp;
    V2* pb = s->cgp2;
    const uint32_t cap = s->K.cap[second ? 1 : 0];
    for (uint32_t k = 0; k < cap; k++) {
        if (s->K.p_done[0] && s->K.p_done[1]) break;
        k_cg_apply(s, pa, pb);
        reduce_alpha(s);
        k_cg_update(s, pb);
        vcycle(s);
        reduce_beta(s);
        V2* t = pa;
        pa = pb;
        pb = t;
    }
    reduce_end(s, second ? 9 : 3);
    if (!second) {
        s->K.p1_iters[0] = s->K.p_iters[0];
        s->K.p1_iters[1] = s->K.p_iters[1];
    } else {
        s->K.p2_last = s->K.p_iters[0];
    }
}

/* ------------------------------------------------------------------------------------ */
/* project.comp                                                                          */
/* ------------------------------------------------------------------------------------ */

static float p_difference(int lc, int ln, float pc, float pn, float j) {
    if (lc && ln) return pc - pn - j;
    return (lc ? pc : j) - (ln ? pn : j);
}

static void k_project(OSim* s) {
    int W = s->W;
    float m_all = 0.0f;
    for (int cy = 1; cy < s->H; cy++)
        for (int cx = 1; cx < W; cx++) {
            int i = cidx(s, cx, cy);
            V4 cf = s->coef[i];
            V4 me = s->vel[i];
            if (s->mgd[i] > 0.0f) s->prhs[i].z = s->pres[i].x;
            if (cf.x != 0.0f || cf.y != 0.0f) {
                V2 p = s->pres[i];
                int liq = s->cell[i].w > 0.0f;
                if (face_live(me.z) && cf.x != 0.0f) {
                    int n = i - 1;
                    me.x -= cf.x * p_difference(liq, s->cell[n].w > 0.0f, p.x, s->pres[n].x, s->pjump[i].x);
                    me.z = -cf.x * (p.y - s->pres[n].y);
                }
                if (face_live(me.w) && cf.y != 0.0f) {
                    int n = i - W;
                    me.y -= cf.y * p_difference(liq, s->cell[n].w > 0.0f, p.x, s->pres[n].x, s->pjump[i].y);
                    me.w = -cf.y * (p.y - s->pres[n].y);
                }
                s->vel[i] = me;
            }
            float m = 0.0f;
            if (face_live(me.z) && cf.x != 0.0f) m = fabsf(me.x);
            if (face_live(me.w) && cf.y != 0.0f) m = maxf(m, fabsf(me.y));
            if (m > m_all) m_all = m;
        }
    if (m_all > bitsf(s->S.umax_grid)) s->S.umax_grid = fbits(m_all);
}

/* ------------------------------------------------------------------------------------ */
/* Implicit viscosity: visc_split, visc_diag, vmg_build, visc_strain, visc_apply mode 0,  */
/* visc_iter WARM, vmg_down / vmg_up / visc_mgu / visc_mgz, reduce_tail modes 4-13        */
/* ------------------------------------------------------------------------------------ */
/* The reference works in 16 x 16 tiles with a shrinking halo recomputed in shared memory
 * (vmg.glsl:142-147): after h half-sweeps the values in ring >= h of a tile's region are
 * exactly those of red-black half-sweeps over the whole level. The restatement below
 * therefore sweeps whole levels; cells of inactive tiles carry zero matrices (visc_diag,
 * vmg_build clear them) and so stay zero, as they do in the reference. */

static inline int in_grid_c(const OSim* s, int x, int y) { return x >= 0 && y >= 0 && x < s->W && y < s->H; }
static inline int interior_c(const OSim* s, int x, int y) { return x >= 1 && y >= 1 && x < s->W - 1 && y < s->H - 1; }
static inline uint32_t tile_of_c(const OSim* s, int x, int y) { return (uint32_t)((y >> 4) * ((s->W + 15) >> 4) + (x >> 4)); }
static inline int tile_active_c(const OSim* s, int x, int y) { return s->tiles[tile_of_c(s, x, y)] != 0u; }

/* visc_split.comp: explicit step in the inactive tiles */
static void k_visc_split(OSim* s) {
    int W = s->W, H = s->H;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int cy = 1; cy < H - 1; cy++)
        for (int cx = 1; cx < W - 1; cx++) {
            if (tile_active_c(s, cx, cy)) continue;
            int i = cidx(s, cx, cy);
            V2 g = gts(s, i);
            V4 cf = s->coef[i];
            if (live_u(s, i)) s->vel[i].x -= g.x / cf.z;
            if (live_v(s, i)) s->vel[i].y -= g.y / cf.w;
        }
}

static inline V2 wts(const OSim* s, int x, int y, int i) {
    return s->tiles[tile_of_c(s, x, y)] != 0u ? v2(s->vw[i].x, s->vw[i].y) : v2(0.0f, 0.0f);
}
static inline int unk_u(const OSim* s, int x, int y) { return interior_c(s, x, y) && s->tiles[tile_of_c(s, x, y)] != 0u && live_u(s, cidx(s, x, y)); }
static inline int unk_v(const OSim* s, int x, int y) { return interior_c(s, x, y) && s->tiles[tile_of_c(s, x, y)] != 0u && live_v(s, cidx(s, x, y)); }

/* visc_diag.comp:23-52 */
static void couplings(const OSim* s, int cx, int cy, int i, V4* a, V4* b) {
    int W = s->W;
    int u = unk_u(s, cx, cy), v = unk_v(s, cx, cy);
    *a = v4(0, 0, 0, 0);
    *b = v4(0, 0, 0, 0);
    if (u && unk_u(s, cx - 1, cy)) a->x = -wts(s, cx - 1, cy, i - 1).x;
    if (v && unk_v(s, cx, cy - 1)) a->w = -wts(s, cx, cy - 1, i - W).x;
    float wn = wts(s, cx, cy, i).y;
    if (wn > 0.0f) {
        float ua = u ? (closed_u(s, i - W) ? 1.0f : 0.5f) : 0.0f;
        float ub = unk_u(s, cx, cy - 1) ? -(closed_u(s, i) ? 1.0f : 0.5f) : 0.0f;
        float va = v ? (closed_v(s, i - 1) ? 1.0f : 0.5f) : 0.0f;
        float vb = unk_v(s, cx - 1, cy) ? -(closed_v(s, i) ? 1.0f : 0.5f) : 0.0f;
        a->y = wn * ua * ub;
        a->z = wn * va * vb;
        b->x = wn * ua * va;
        b->y = wn * ua * vb;
    }
    float wu = wts(s, cx, cy + 1, i + W).y;
    if (wu > 0.0f && u) {
        float ub = -(closed_u(s, i + W) ? 1.0f : 0.5f);
        float va = unk_v(s, cx, cy + 1) ? (closed_v(s, i + W - 1) ? 1.0f : 0.5f) : 0.0f;
        float vb = unk_v(s, cx - 1, cy + 1) ? -(closed_v(s, i + W) ? 1.0f : 0.5f) : 0.0f;
        b->z = wu * ub * va;
        b->w = wu * ub * vb;
    }
}

/* visc_diag.comp:56-119 */
static void k_visc_diag(OSim* s, int warm, int mg) {
    int W = s->W, H = s->H;
    int tw = (W + 15) >> 4, th = (H + 15) >> 4;
    float ratio = s->S.dt / s->S.dt_prev;
    /* vw.zw and the warm start first: the couplings read vw.xy only */
    uint32_t* was = (uint32_t*)malloc((size_t)tw * th * sizeof(uint32_t));
    for (int t = 0; t < tw * th; t++) {
        was[t] = s->vtile[t];
        if (mg) s->vtile[t] = s->tiles[t];
    }
    V4* outw = (V4*)malloc((size_t)W * H * sizeof(V4));
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int cy = 0; cy < H; cy++)
        for (int cx = 0; cx < W; cx++) {
            int i = cidx(s, cx, cy);
            int on = tile_active_c(s, cx, cy);
            V2 d = v2(1.0f, 1.0f);
            if (interior_c(s, cx, cy)) {
                V4 cf = s->coef[i];
                V2 me = wts(s, cx, cy, i);
                if (live_u(s, i)) {
                    float c1 = closed_u(s, i - W) ? 1.0f : 0.5f, c2 = closed_u(s, i + W) ? 1.0f : 0.5f;
                    d.x = cf.z + wts(s, cx - 1, cy, i - 1).x + me.x + me.y * c1 * c1 + wts(s, cx, cy + 1, i + W).y * c2 * c2;
                }
                if (live_v(s, i)) {
                    float d1 = closed_v(s, i - 1) ? 1.0f : 0.5f, d2 = closed_v(s, i + 1) ? 1.0f : 0.5f;
                    d.y = cf.w + wts(s, cx, cy - 1, i - W).x + me.x + me.y * d1 * d1 + wts(s, cx + 1, cy, i + 1).y * d2 * d2;
                }
            }
            V4 o = s->vw[i];
            o.z = d.x;
            o.w = d.y;
            V2 dv = v2(0.0f, 0.0f);
            if (warm && on && interior_c(s, cx, cy)) {
                dv = v2(s->vd[i].x * ratio * (live_u(s, i) ? 1.0f : 0.0f), s->vd[i].y * ratio * (live_v(s, i) ? 1.0f : 0.0f));
            }
            s->vd[i] = dv;
            if (!on) {
                o.x = 0.0f;
                o.y = 0.0f;
            }
            outw[i] = o;
        }
    /* the level-0 matrix (reads vw.xy through wts, which is zero in inactive tiles already) */
    if (mg) {
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int cy = 0; cy < H; cy++)
            for (int cx = 0; cx < W; cx++) {
                int i = cidx(s, cx, cy);
                int on = tile_active_c(s, cx, cy);
                if (!(on || was[tile_of_c(s, cx, cy)] != 0u)) continue;
                V4 a = v4(0, 0, 0, 0), b = v4(0, 0, 0, 0);
                V2 dm = v2(0.0f, 0.0f);
                if (on && interior_c(s, cx, cy)) {
                    couplings(s, cx, cy, i, &a, &b);
                    dm = v2(outw[i].z * (live_u(s, i) ? 1.0f : 0.0f), outw[i].w * (live_v(s, i) ? 1.0f : 0.0f));
                }
                if (!on) {
                    s->vmz[i] = v2(0, 0);
                    s->vaz[i] = v2(0, 0);
                    s->vr2[i] = v2(0, 0);
                    s->vq2[i] = v2(0, 0);
                }
                s->vma[i] = a;
                s->vmb[i] = b;
                s->vmd[i] = dm;
            }
    }
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int i = 0; i < W * H; i++) {
        int cx = i % W, cy = i / W;
        s->vw[i] = outw[i];
        if (!tile_active_c(s, cx, cy)) {
            s->vs[i] = v4(0, 0, 0, 0);
            s->vr[i] = v2(0, 0);
            s->vp[i] = v2(0, 0);
            s->vq[i] = v2(0, 0);
        }
    }
    free(outw);
    free(was);
}

/* vmg_build.comp: viscosity level l from level l - 1 */
static void k_vmg_build(OSim* s, int l) {
    Lv F = lev(s, l - 1), C = lev(s, l);
    int tfx = (F.w + 15) >> 4, tfy = (F.h + 15) >> 4;
    int tcx = (C.w + 15) >> 4, tcy = (C.h + 15) >> 4;
    static const int UVX[4] = {0, -1, 0, -1}, UVY[4] = {0, 0, 1, 1};
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int ty = 0; ty < tcy; ty++)
        for (int tx = 0; tx < tcx; tx++) {
            uint32_t on = 0u;
            for (int k = 0; k < 4; k++) {
                int fx = 2 * tx + (k & 1), fy = 2 * ty + (k >> 1);
                if (fx < tfx && fy < tfy) on |= (l - 1 == 0) ? s->tiles[fy * tfx + fx] : s->vtile[F.toff + fy * tfx + fx];
            }
            uint32_t slot = (uint32_t)C.toff + (uint32_t)(ty * tcx + tx);
            uint32_t was = s->vtile[slot];
            s->vtile[slot] = on != 0u ? 1u : 0u;
            uint32_t state = (on != 0u ? 1u : 0u) | (was != 0u ? 2u : 0u);
            if (state == 0u) continue;
            for (int ly = 0; ly < 16; ly++)
                for (int lx = 0; lx < 16; lx++) {
                    int ccx = tx * 16 + lx, ccy = ty * 16 + ly;
                    if (!l_inside(C, ccx, ccy)) continue;
                    int o = l_at(C, ccx, ccy);
                    if ((state & 1u) == 0u) {
                        s->vma[o] = v4(0, 0, 0, 0);
                        s->vmb[o] = v4(0, 0, 0, 0);
                        s->vmd[o] = v2(0, 0);
                        continue;
                    }
                    V2 D = v2(0, 0);
                    V4 A = v4(0, 0, 0, 0), B = v4(0, 0, 0, 0);
                    for (int k = 0; k < 4; k++) {
                        int abx = k & 1, aby = k >> 1;
                        int fx = 2 * ccx + abx, fy = 2 * ccy + aby;
                        if (!l_inside(F, fx, fy)) continue;
                        int i = l_at(F, fx, fy);
                        V4 a = s->vma[i], b = s->vmb[i];
                        D.x += s->vmd[i].x;
                        D.y += s->vmd[i].y;
                        if (abx == 1) { D.x += 2.0f * a.x; D.y += 2.0f * a.z; }
                        else { A.x += a.x; A.z += a.z; }
                        if (aby == 1) { D.x += 2.0f * a.y; D.y += 2.0f * a.w; }
                        else { A.y += a.y; A.w += a.w; }
                        for (int m = 0; m < 4; m++) {
                            int rx = ((fx + UVX[m]) >> 1) - ccx, ry = ((fy + UVY[m]) >> 1) - ccy;
                            int sl = (rx == 0 ? 0 : 1) + (ry == 0 ? 0 : 2);
                            float bm = m == 0 ? b.x : m == 1 ? b.y : m == 2 ? b.z : b.w;
                            if (sl == 0) B.x += bm; else if (sl == 1) B.y += bm; else if (sl == 2) B.z += bm; else B.w += bm;
                        }
                    }
                    s->vma[o] = A;
                    s->vmb[o] = B;
                    s->vmd[o] = v2(maxf(D.x, 0.0f), maxf(D.y, 0.0f));
                }
        }
}

/* visc_strain.comp: strain of the current velocity in the active tiles */
static void k_visc_strain(OSim* s) {
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int cy = 0; cy < s->H; cy++)
        for (int cx = 0; cx < s->W; cx++) {
            if (!tile_active_c(s, cx, cy)) continue;
            int i = cidx(s, cx, cy);
            s->vs[i] = strain_of_vel(s, i, v2(s->vw[i].x, s->vw[i].y));
        }
}

/* per-tile partial sums over level-0 tiles (group_sum, reduce.glsl), inactive tiles zero */
typedef V4 (*CellDot)(OSim* s, int cx, int cy, void* ctx);
static void tile_partials(OSim* s, V4* part, CellDot f, void* ctx) {
    int tw = (s->W + 15) >> 4, th = (s->H + 15) >> 4;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int ty = 0; ty < th; ty++)
        for (int tx = 0; tx < tw; tx++) {
            int slot = ty * tw + tx;
            if (s->tiles[slot] == 0u) {
                part[slot] = v4(0, 0, 0, 0);
                continue;
            }
            V4 buf[256];
            for (int ly = 0; ly < 16; ly++)
                for (int lx = 0; lx < 16; lx++) buf[ly * 16 + lx] = f(s, tx * 16 + lx, ty * 16 + ly, ctx);
            part[slot] = group_tree(buf);
        }
}

static inline float dot2(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }

/* visc_apply.comp mode 0 at one cell: r = -G^T W G u*, z = r / diag */
static V4 cell_visc_start(OSim* s, int cx, int cy, void* ctx) {
    (void)ctx;
    if (!in_grid_c(s, cx, cy)) return v4(0, 0, 0, 0);
    int i = cidx(s, cx, cy);
    if (interior_c(s, cx, cy)) {
        V2 g = gts(s, i);
        V2 live = v2(live_u(s, i) ? 1.0f : 0.0f, live_v(s, i) ? 1.0f : 0.0f);
        V2 diag = v2(s->vw[i].z, s->vw[i].w);
        V2 r = v2(-g.x * live.x, -g.y * live.y);
        V2 z = v2(r.x / diag.x, r.y / diag.y);
        s->vr[i] = r;
        s->vp[i] = z;
        return v4(dot2(r, z), dot2(r, r), 0.0f, 0.0f);
    }
    s->vr[i] = v2(0, 0);
    s->vp[i] = v2(0, 0);
    return v4(0, 0, 0, 0);
}

/* visc_iter.comp WARM: step to u* + d and r -= A d; p and its strain from vd */
static inline V2 warm_dir(const OSim* s, int x, int y) {
    if (!in_grid_c(s, x, y) || !interior_c(s, x, y)) return v2(0, 0);
    return s->vd[cidx(s, x, y)];
}
static inline float pU(const OSim* s, int x, int y, int i) { return live_u(s, i) ? warm_dir(s, x, y).x : 0.0f; }
static inline float pV(const OSim* s, int x, int y, int i) { return live_v(s, i) ? warm_dir(s, x, y).y : 0.0f; }
static V4 strain_of_dir(const OSim* s, int cx, int cy) {
    if (!in_grid_c(s, cx, cy)) return v4(0, 0, 0, 0);
    int i = cidx(s, cx, cy), W = s->W;
    V4 o = v4(0, 0, 0, 0);
    V4 w = s->vw[i];
    if (w.x > 0.0f) {
        o.x = w.x * (pU(s, cx + 1, cy, i + 1) - pU(s, cx, cy, i));
        o.y = w.x * (pV(s, cx, cy + 1, i + W) - pV(s, cx, cy, i));
    }
    if (w.y > 0.0f) {
        float ua = pU(s, cx, cy, i), ub = pU(s, cx, cy - 1, i - W), va = pV(s, cx, cy, i), vb = pV(s, cx - 1, cy, i - 1);
        if (closed_u(s, i) && live_u(s, i - W)) ua = -ub;
        if (closed_u(s, i - W) && live_u(s, i)) ub = -ua;
        if (closed_v(s, i) && live_v(s, i - 1)) va = -vb;
        if (closed_v(s, i - 1) && live_v(s, i)) vb = -va;
        o.z = w.y * 0.5f * ((ua - ub) + (va - vb));
    }
    return o;
}
static V4 cell_visc_warm(OSim* s, int cx, int cy, void* ctx) {
    (void)ctx;
    if (!in_grid_c(s, cx, cy) || !interior_c(s, cx, cy)) return v4(0, 0, 0, 0);
    int i = cidx(s, cx, cy), W = s->W;
    V2 g = v2(0, 0);
    if (live_u(s, i)) {
        float c1 = closed_u(s, i - W) ? 1.0f : 0.5f, c2 = closed_u(s, i + W) ? -1.0f : -0.5f;
        V4 sl = strain_of_dir(s, cx - 1, cy), sc = strain_of_dir(s, cx, cy), su = strain_of_dir(s, cx, cy + 1);
        g.x = sl.x - sc.x + sc.z * c1 + su.z * c2;
    }
    if (live_v(s, i)) {
        float d1 = closed_v(s, i - 1) ? 1.0f : 0.5f, d2 = closed_v(s, i + 1) ? -1.0f : -0.5f;
        V4 sd = strain_of_dir(s, cx, cy - 1), sc = strain_of_dir(s, cx, cy), sr = strain_of_dir(s, cx + 1, cy);
        g.y = sd.y - sc.y + sc.z * d1 + sr.z * d2;
    }
    V2 live = v2(live_u(s, i) ? 1.0f : 0.0f, live_v(s, i) ? 1.0f : 0.0f);
    V4 cf = s->coef[i];
    V2 dd = warm_dir(s, cx, cy);
    V2 d = v2(dd.x * live.x, dd.y * live.y);
    V2 q = v2((cf.z * d.x + g.x) * live.x, (cf.w * d.y + g.y) * live.y);
    /* results are written after every cell's inputs were read (the kernel reads vd, vw and
     * the velocity flags, which the update does not change) */
    V2* outr = (V2*)ctx;
    s->vel[i].x += d.x;
    s->vel[i].y += d.y;
    V2 r = v2(s->vr[i].x - q.x, s->vr[i].y - q.y);
    outr[i] = r;
    V2 z = v2(r.x / s->vw[i].z, r.y / s->vw[i].w);
    return v4(dot2(r, z), dot2(r, r), 0.0f, 0.0f);
}

/* vmg.glsl: the viscosity multigrid on one level, as whole-level sweeps */
static inline V4 vma_at(const OSim* s, Lv L, int x, int y) { return l_inside(L, x, y) ? s->vma[l_at(L, x, y)] : v4(0, 0, 0, 0); }
static inline V4 vmb_at(const OSim* s, Lv L, int x, int y) { return l_inside(L, x, y) ? s->vmb[l_at(L, x, y)] : v4(0, 0, 0, 0); }
static inline V2 vx_at(const V2* X, Lv L, int x, int y) { return l_inside(L, x, y) ? X[y * L.w + x] : v2(0, 0); }

/* offd (vmg.glsl:189-197) of X (level-local array) at (x, y) */
static V2 voffd(const OSim* s, Lv L, const V2* X, int x, int y) {
    V4 a = vma_at(s, L, x, y), b = vmb_at(s, L, x, y);
    V2 xl = vx_at(X, L, x - 1, y), xr = vx_at(X, L, x + 1, y), xd = vx_at(X, L, x, y - 1), xu = vx_at(X, L, x, y + 1);
    V2 xc = vx_at(X, L, x, y);
    float u = a.x * xl.x + vma_at(s, L, x + 1, y).x * xr.x + a.y * xd.x + vma_at(s, L, x, y + 1).y * xu.x
            + b.x * xc.y + b.y * xl.y + b.z * xu.y + b.w * vx_at(X, L, x - 1, y + 1).y;
    float v = a.z * xl.y + vma_at(s, L, x + 1, y).z * xr.y + a.w * xd.y + vma_at(s, L, x, y + 1).w * xu.y
            + b.x * xc.x + vmb_at(s, L, x + 1, y).y * xr.x + vmb_at(s, L, x, y - 1).z * xd.x
            + vmb_at(s, L, x + 1, y - 1).w * vx_at(X, L, x + 1, y - 1).x;
    return v2(u, v);
}

/* one half-sweep of one colour over the level: every update reads the values before it */
static void vhalf_sweep(const OSim* s, Lv L, V2* X, const V2* R, int red) {
    int n = L.w * L.h;
    V2* nv = (V2*)malloc((size_t)n * sizeof(V2));
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int t = 0; t < n; t++) {
        int x = t % L.w, y = t / L.w;
        if ((((x + y) & 1) == 0) != red) continue;
        V2 d = s->vmd[L.off + t];
        V2 o = voffd(s, L, X, x, y);
        V2 sv = v2(R[t].x - o.x, R[t].y - o.y);
        nv[t] = v2(d.x > 0.0f ? sv.x / d.x : 0.0f, d.y > 0.0f ? sv.y / d.y : 0.0f);
    }
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int t = 0; t < n; t++) {
        int x = t % L.w, y = t / L.w;
        if ((((x + y) & 1) == 0) == red) X[t] = nv[t];
    }
    free(nv);
}

/* way_down (vmg.glsl:264-287) on level l with right-hand side R: pre-smoothing from zero,
 * the result to vmx, the residual summed over 2 x 2 aggregates into vmr of level l + 1 */
static void vmg_down(OSim* s, int l, const V2* R, int coarsest, int halo) {
    Lv L = lev(s, l);
    int n = L.w * L.h;
    V2* X = (V2*)calloc((size_t)n, sizeof(V2));
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int t = 0; t < n; t++) {
        int x = t % L.w, y = t / L.w;
        V2 d = s->vmd[L.off + t];
        V2 xr = v2(d.x > 0.0f ? R[t].x / d.x : 0.0f, d.y > 0.0f ? R[t].y / d.y : 0.0f);
        X[t] = ((x + y) & 1) == 0 ? xr : v2(0, 0);
    }
    for (int h = 1; h < halo; h++) vhalf_sweep(s, L, X, R, (h & 1) == 0);
    for (int t = 0; t < n; t++) s->vmx[L.off + t] = X[t];
    if (!coarsest) {
        Lv C = lev(s, l + 1);
        V2* res = (V2*)calloc((size_t)n, sizeof(V2));
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int t = 0; t < n; t++) {
            int x = t % L.w, y = t / L.w;
            V2 d = s->vmd[L.off + t];
            V2 o = voffd(s, L, X, x, y);
            V2 rr = v2(R[t].x - d.x * X[t].x - o.x, R[t].y - d.y * X[t].y - o.y);
            res[t] = v2(rr.x * (d.x > 0.0f ? 1.0f : 0.0f), rr.y * (d.y > 0.0f ? 1.0f : 0.0f));
        }
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int cy = 0; cy < C.h; cy++)
            for (int cx = 0; cx < C.w; cx++) {
                V2 a = vx_at(res, L, 2 * cx, 2 * cy), b = vx_at(res, L, 2 * cx + 1, 2 * cy);
                V2 c = vx_at(res, L, 2 * cx, 2 * cy + 1), e = vx_at(res, L, 2 * cx + 1, 2 * cy + 1);
                s->vmr[l_at(C, cx, cy)] = v2(a.x + b.x + c.x + e.x, a.y + b.y + c.y + e.y);
            }
        free(res);
    }
    free(X);
}

/* the way up (vmg_up.comp / visc_mgz.comp): x = vmx + the coarse values, post-smoothing
 * black then red; result in X (level-local) */
static void vmg_up_into(OSim* s, int l, const V2* R, int coarse_corr, int halo, V2* X) {
    Lv L = lev(s, l);
    int n = L.w * L.h;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int t = 0; t < n; t++) {
        int x = t % L.w, y = t / L.w;
        V2 xv = s->vmx[L.off + t];
        if (coarse_corr) {
            Lv C = lev(s, l + 1);
            V2 zc = s->vmz[l_at(C, x >> 1, y >> 1)];
            xv = v2(xv.x + zc.x, xv.y + zc.y);
        }
        V2 d = s->vmd[L.off + t];
        X[t] = v2(xv.x * (d.x > 0.0f ? 1.0f : 0.0f), xv.y * (d.y > 0.0f ? 1.0f : 0.0f));
    }
    for (int h = 1; h <= halo; h++) vhalf_sweep(s, L, X, R, (h & 1) == 0);
}

/* the coarse levels of one viscosity V-cycle (record_visc_coarse, mod.rs:2835-2853) */
static void vmg_coarse(OSim* s, int nlev, int halo) {
    for (int l = 1; l <= nlev; l++) {
        Lv L = lev(s, l);
        vmg_down(s, l, s->vmr + L.off, l == nlev, halo);
    }
    for (int l = nlev; l >= 1; l--) {
        Lv L = lev(s, l);
        int n = L.w * L.h;
        V2* X = (V2*)malloc((size_t)n * sizeof(V2));
        vmg_up_into(s, l, s->vmr + L.off, l != nlev, halo, X);
        memcpy(s->vmz + L.off, X, (size_t)n * sizeof(V2));
        free(X);
    }
}

/* visc_mgz.comp: the way up on level 0 with A z and the dot products of the solve */
typedef struct MgzCtx { V2* Z; V2* AZ; const V2* R; const V2* Q; } MgzCtx;
static V4 cell_mgz(OSim* s, int cx, int cy, void* ctx) {
    MgzCtx* c = (MgzCtx*)ctx;
    if (!in_grid_c(s, cx, cy)) return v4(0, 0, 0, 0);
    int i = cidx(s, cx, cy);
    V2 z = c->Z[i], az = c->AZ[i];
    s->vmz[i] = z;
    s->vaz[i] = az;
    return v4(dot2(c->R[i], z), dot2(z, az), dot2(z, c->Q[i]), 0.0f);
}
static void visc_mgz(OSim* s, const V2* R, const V2* Q, int halo) {
    int n = s->W * s->H;
    Lv L0 = lev(s, 0);
    V2* Z = (V2*)malloc((size_t)n * sizeof(V2));
    V2* AZ = (V2*)malloc((size_t)n * sizeof(V2));
    vmg_up_into(s, 0, R, 1, halo, Z);
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int t = 0; t < n; t++) {
        int x = t % s->W, y = t / s->W;
        V2 d = s->vmd[t];
        V2 o = voffd(s, L0, Z, x, y);
        AZ[t] = v2(d.x * Z[t].x + o.x, d.y * Z[t].y + o.y);
    }
    MgzCtx c = {Z, AZ, R, Q};
    tile_partials(s, s->part, cell_mgz, &c);
    free(Z);
    free(AZ);
}

/* visc_mgu.comp at one cell: p, q, x, r of the iteration, before the way down */
typedef struct MguCtx { const V2* Rold; const V2* Qold; V2* Rnew; V2* Qnew; } MguCtx;
static V4 cell_mgu(OSim* s, int cx, int cy, void* ctx) {
    MguCtx* c = (MguCtx*)ctx;
    if (!in_grid_c(s, cx, cy)) return v4(0, 0, 0, 0);
    int i = cidx(s, cx, cy);
    float a = s->K.v_alpha, b = s->K.v_beta;
    V2 z = s->vmz[i];
    V2 p = b == 0.0f ? z : v2(z.x + b * s->vp[i].x, z.y + b * s->vp[i].y);
    V2 sq = s->vaz[i];
    V2 q = b == 0.0f ? sq : v2(sq.x + b * c->Qold[i].x, sq.y + b * c->Qold[i].y);
    V2 r = v2(c->Rold[i].x - a * q.x, c->Rold[i].y - a * q.y);
    if (interior_c(s, cx, cy)) {
        if (face_live(s->vel[i].z)) s->vel[i].x += a * p.x;
        if (face_live(s->vel[i].w)) s->vel[i].y += a * p.y;
        s->vd[i].x += a * p.x;
        s->vd[i].y += a * p.y;
    }
    s->vp[i] = p;
    c->Qnew[i] = q;
    c->Rnew[i] = r;
    return v4(0.0f, dot2(r, r), dot2(p, q), 0.0f);
}

/* new_r of visc_mgu.comp at every cell of the level: the residual the way down reads */
static void mgu_new_r(OSim* s, const V2* Rold, const V2* Qold, V2* out) {
    float a = s->K.v_alpha, b = s->K.v_beta;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int i = 0; i < s->W * s->H; i++) {
        V2 sq = s->vaz[i];
        V2 q = b == 0.0f ? sq : v2(sq.x + b * Qold[i].x, sq.y + b * Qold[i].y);
        out[i] = v2(Rold[i].x - a * q.x, Rold[i].y - a * q.y);
    }
}

/* visc_iter.comp (not WARM), the Jacobi-preconditioned iteration (viscosity_precond 0): the
 * direction p = z + beta p_old (z = r / diag) at every interior cell, its weighted strain, and
 * per cell of an active tile q = M p + G^T s into vq, p into Pnew; partial sums of p.q */
typedef struct JacCtx {
    const V2* P;   /* the new direction at every cell */
    const V4* S;   /* its weighted strain at every cell */
    V2* Pnew;
} JacCtx;
static inline float jU(const JacCtx* c, const OSim* s, int x, int y, int i) {
    return live_u(s, i) ? c->P[cidx(s, x, y)].x : 0.0f;
}
static inline float jV(const JacCtx* c, const OSim* s, int x, int y, int i) {
    return live_v(s, i) ? c->P[cidx(s, x, y)].y : 0.0f;
}
static V4 jac_strain(const JacCtx* c, const OSim* s, int cx, int cy) {
    if (!in_grid_c(s, cx, cy)) return v4(0, 0, 0, 0);
    int i = cidx(s, cx, cy), W = s->W;
    V4 o = v4(0, 0, 0, 0);
    V4 w = s->vw[i];
    if (w.x > 0.0f) {
        o.x = w.x * (jU(c, s, cx + 1, cy, i + 1) - jU(c, s, cx, cy, i));
        o.y = w.x * (jV(c, s, cx, cy + 1, i + W) - jV(c, s, cx, cy, i));
    }
    if (w.y > 0.0f) {
        float ua = jU(c, s, cx, cy, i), ub = jU(c, s, cx, cy - 1, i - W), va = jV(c, s, cx, cy, i), vb = jV(c, s, cx - 1, cy, i - 1);
        if (closed_u(s, i) && live_u(s, i - W)) ua = -ub;
        if (closed_u(s, i - W) && live_u(s, i)) ub = -ua;
        if (closed_v(s, i) && live_v(s, i - 1)) va = -vb;
        if (closed_v(s, i - 1) && live_v(s, i)) vb = -va;
        o.z = w.y * 0.5f * ((ua - ub) + (va - vb));
    }
    return o;
}
static V4 cell_jac_iter(OSim* s, int cx, int cy, void* ctx) {
    JacCtx* c = (JacCtx*)ctx;
    if (!in_grid_c(s, cx, cy)) return v4(0, 0, 0, 0);
    int i = cidx(s, cx, cy), W = s->W;
    V2 pn = c->P[i];
    c->Pnew[i] = pn;
    if (!interior_c(s, cx, cy)) {
        s->vq[i] = v2(0, 0);
        return v4(0, 0, 0, 0);
    }
    V2 g = v2(0, 0);
    if (live_u(s, i)) {
        float c1 = closed_u(s, i - W) ? 1.0f : 0.5f, c2 = closed_u(s, i + W) ? -1.0f : -0.5f;
        V4 sl = c->S[i - 1], sc = c->S[i], su = c->S[i + W];
        g.x = sl.x - sc.x + sc.z * c1 + su.z * c2;
    }
    if (live_v(s, i)) {
        float d1 = closed_v(s, i - 1) ? 1.0f : 0.5f, d2 = closed_v(s, i + 1) ? -1.0f : -0.5f;
        V4 sd = c->S[i - W], sc = c->S[i], sr = c->S[i + 1];
        g.y = sd.y - sc.y + sc.z * d1 + sr.z * d2;
    }
    V2 live = v2(live_u(s, i) ? 1.0f : 0.0f, live_v(s, i) ? 1.0f : 0.0f);
    V4 cf = s->coef[i];
    V2 p = v2(pn.x * live.x, pn.y * live.y);
    V2 q = v2((cf.z * p.x + g.x) * live.x, (cf.w * p.y + g.y) * live.y);
    s->vq[i] = q;
    return v4(0.0f, 0.0f, dot2(p, q), 0.0f);
}
/* visc_update.comp: u += alpha p, the warm-start step, r -= alpha q; partial sums of r.z, r.r */
static V4 cell_jac_update(OSim* s, int cx, int cy, void* ctx) {
    const V2* Pcur = (const V2*)ctx;
    if (!in_grid_c(s, cx, cy) || !interior_c(s, cx, cy)) return v4(0, 0, 0, 0);
    int i = cidx(s, cx, cy);
    float a = s->K.v_alpha;
    V2 p = Pcur[i];
    if (live_u(s, i)) s->vel[i].x += a * p.x;
    if (live_v(s, i)) s->vel[i].y += a * p.y;
    s->vd[i].x += a * (live_u(s, i) ? p.x : 0.0f);
    s->vd[i].y += a * (live_v(s, i) ? p.y : 0.0f);
    V2 r = v2(s->vr[i].x - a * s->vq[i].x, s->vr[i].y - a * s->vq[i].y);
    s->vr[i] = r;
    V2 z = v2(r.x / s->vw[i].z, r.y / s->vw[i].w);
    return v4(dot2(r, z), dot2(r, r), 0.0f, 0.0f);
}
/* the Jacobi-preconditioned conjugate gradients (record_viscosity_solve, mod.rs:2909-2921):
 * per iteration visc_iter + cg_reduce mode 5, visc_update + mode 6. The directions alternate
 * between vp and vr2 (free without the multigrid) as vp / vp2 swap in the reference. */
static void viscosity_jacobi(OSim* s) {
    SolveBuf* K = &s->K;
    const float tz = P_.tol[2];
    int n = s->W * s->H;
    V2* P = (V2*)malloc((size_t)n * sizeof(V2));
    V4* S = (V4*)malloc((size_t)n * sizeof(V4));
    V2 *pa = s->vp, *pb = s->vr2;
    for (uint32_t k = 0; k < K->cap[2] && !K->v_done; k++) {
        float b = K->v_beta;
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < n; i++) {
            int cx = i % s->W, cy = i / s->W;
            V2 p = v2(0, 0);
            if (interior_c(s, cx, cy)) {
                V2 z = v2(s->vr[i].x / s->vw[i].z, s->vr[i].y / s->vw[i].w);
                p = b == 0.0f ? z : v2(z.x + b * pa[i].x, z.y + b * pa[i].y);
            }
            P[i] = p;
        }
        JacCtx c = {P, S, pb};
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < n; i++) S[i] = jac_strain(&c, s, i % s->W, i / s->W);
        tile_partials(s, s->part, cell_jac_iter, &c);
        {   /* mode 5 */
            V4 t = total(s, 0, s->nwg);
            K->v_alpha = (K->v_done == 0u && t.z > 0.0f) ? K->v_rz / t.z : 0.0f;
        }
        tile_partials(s, s->part, cell_jac_update, pb);
        {   /* mode 6 */
            V4 t = total(s, 0, s->nwg);
            uint32_t was = K->v_done;
            K->v_iters += 1u - was;
            uint32_t now = t.y <= tz * tz * K->v_r0;
            uint32_t done = was > now ? was : now;
            K->v_beta = (done == 0u && K->v_rz > 0.0f) ? t.x / K->v_rz : 0.0f;
            K->v_rz = t.x;
            if (was == 0u) K->v_rr = t.y;
            K->v_done = done;
        }
        V2* tmp = pa;
        pa = pb;
        pb = tmp;
    }
    free(P);
    free(S);
}

/* record_viscosity_solve (mod.rs:2867-2923) with the device-decided loop */
static void viscosity_solve(OSim* s, int restrain) {
    const int nlev = (int)mini(maxi((int)s->prm.viscosity_mg_levels, 1), s->lv.tail);
    const int halo = 2 * (int)mini(maxi((int)s->prm.viscosity_mg_sweeps, 1), 2);
    const float tz = P_.tol[2];
    SolveBuf* K = &s->K;
    int n = s->W * s->H;
    if (restrain) k_visc_strain(s);
    /* visc_apply mode 0 + cg_reduce mode 4 */
    tile_partials(s, s->part, cell_visc_start, NULL);
    {
        V4 a = total(s, 0, s->nwg);
        K->v_rz = a.x;
        K->v_r0 = a.y;
        K->v_rr = a.y;
        K->v_beta = 0.0f;
        K->v_alpha = 0.0f;
        K->v_iters = 0u;
        K->v_done = (a.y <= 1e-30f || a.x <= 0.0f) ? 1u : 0u;
    }
    if (s->prm.viscosity_warm != 0 && !K->v_done) {
        V2* outr = (V2*)malloc((size_t)n * sizeof(V2));
        memcpy(outr, s->vr, (size_t)n * sizeof(V2));
        tile_partials(s, s->part, cell_visc_warm, outr);
        memcpy(s->vr, outr, (size_t)n * sizeof(V2));
        free(outr);
        V4 a = total(s, 0, s->nwg);
        K->v_rz = a.x;
        K->v_rr = a.y;
        K->v_beta = 0.0f;
        K->v_done = (a.y <= tz * tz * K->v_r0 || a.x <= 0.0f) ? 1u : 0u;
    }
    if (s->prm.viscosity_precond == 0) {
        viscosity_jacobi(s);
        goto stats;
    }
    /* the buffers of the two parities: the current residual alternates between vr and vr2 */
    V2 *RA = s->vr, *RB = s->vr2, *QA = s->vq, *QB = s->vq2;
    if (!K->v_done) {
        vmg_down(s, 0, RA, 0, halo);
        vmg_coarse(s, nlev, halo);
        visc_mgz(s, RA, QA, halo);
        V4 a = total(s, 0, s->nwg);
        K->v_rz = a.x;
        K->v_beta = 0.0f;
        K->v_pq = a.y;
        K->v_alpha = a.y > 0.0f ? a.x / a.y : 0.0f;
        if (a.x <= 0.0f || a.y <= 0.0f) K->v_done = 1u;
    }
    V2* newr = (V2*)malloc((size_t)n * sizeof(V2));
    for (uint32_t k = 0; k < K->cap[2] && !K->v_done; k++) {
        V2 *Rold = (k % 2 == 0) ? RA : RB, *Qold = (k % 2 == 0) ? QA : QB;
        V2 *Rnew = (k % 2 == 0) ? RB : RA, *Qnew = (k % 2 == 0) ? QB : QA;
        mgu_new_r(s, Rold, Qold, newr);
        MguCtx c = {Rold, Qold, Rnew, Qnew};
        tile_partials(s, s->part, cell_mgu, &c);
        vmg_down(s, 0, newr, 0, halo);
        {
            V4 a = total(s, 0, s->nwg);
            uint32_t was = K->v_done;
            K->v_iters += 1u - was;
            uint32_t now = a.y <= tz * tz * K->v_r0;
            if (was == 0u) K->v_rr = a.y;
            K->v_pq = a.z;
            K->v_done = was > now ? was : now;
        }
        if (K->v_done) break;
        vmg_coarse(s, nlev, halo);
        visc_mgz(s, Rnew, Qnew, halo);
        {
            V4 a = total(s, 0, s->nwg);
            float beta = (K->v_done == 0u && K->v_rz > 0.0f) ? a.x / K->v_rz : 0.0f;
            float pq = a.y + 2.0f * beta * a.z + beta * beta * K->v_pq;
            K->v_beta = beta;
            K->v_alpha = (K->v_done == 0u && pq > 0.0f) ? a.x / pq : 0.0f;
            K->v_rz = a.x;
        }
    }
    free(newr);
stats:
    /* mode 7 */
    if (K->v_iters > K->v_it_max) K->v_it_max = K->v_iters;
    if (K->v_done == 0u) K->v_unconv += 1u;
    if (K->v_iters > K->f_it[2]) K->f_it[2] = K->v_iters;
    if (K->v_done == 0u) K->f_un[2] += 1u;
    float rel = K->v_r0 > 0.0f ? sqrtf(K->v_rr / K->v_r0) : 0.0f;
    K->v_res_max = maxf(K->v_res_max, rel);
}

/* rhs_visc.comp */
static void k_rhs_visc(OSim* s, int warm) {
    int W = s->W, H = s->H;
    float ratio = s->S.dt / s->S.dt_prev;
    V4* out = (V4*)malloc((size_t)W * H * sizeof(V4));
    memcpy(out, s->prhs, (size_t)W * H * sizeof(V4));
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int cy = 0; cy < H; cy++)
        for (int cx = 0; cx < W; cx++) {
            int i = cidx(s, cx, cy);
            float D = s->mgd[i];
            if (D <= 0.0f) {
                out[i].z = 0.0f;
                continue;
            }
            V4 w = s->mga[i];
            float p1 = s->prhs[i].z;
            float ap = D * p1;
            if (s->mgd[i - 1] > 0.0f) ap -= w.x * s->prhs[i - 1].z;
            if (s->mgd[i + 1] > 0.0f) ap -= w.y * s->prhs[i + 1].z;
            if (s->mgd[i - W] > 0.0f) ap -= w.z * s->prhs[i - W].z;
            if (s->mgd[i + W] > 0.0f) ap -= w.w * s->prhs[i + W].z;
            float aL = s->solid[i].x, aB = s->solid[i].y, aR = s->solid[i + 1].x, aT = s->solid[i + W].y;
            V4 vme = s->vel[i];
            float div = aR * s->vel[i + 1].x - aL * vme.x + aT * s->vel[i + W].y - aB * vme.y;
            V4 r = s->prhs[i];
            out[i] = v4(ap - div, r.y, p1, 0.0f);
            if (warm) s->pres[i].x = p1 + s->p2keep[i] * ratio;
        }
    memcpy(s->prhs, out, (size_t)W * H * sizeof(V4));
    free(out);
}

/* project_visc.comp */
static float p2_of(const OSim* s, int i) { return s->mgd[i] > 0.0f ? s->pres[i].x - s->prhs[i].z : 0.0f; }
static void k_project_visc(OSim* s) {
    int W = s->W;
    float m_all = 0.0f;
    float* keep = (float*)malloc((size_t)W * s->H * sizeof(float));
    memcpy(keep, s->p2keep, (size_t)W * s->H * sizeof(float));
#pragma omp parallel for schedule(static) num_threads(g_threads) reduction(max : m_all)
    for (int cy = 1; cy < s->H; cy++)
        for (int cx = 1; cx < W; cx++) {
            int i = cidx(s, cx, cy);
            keep[i] = p2_of(s, i);
            V4 cf = s->coef[i];
            V4 me = s->vel[i];
            int lu = face_live(me.z) && cf.x != 0.0f, lv = face_live(me.w) && cf.y != 0.0f;
            if (lu || lv) {
                float pc = p2_of(s, i);
                if (lu) me.x -= cf.x * (pc - p2_of(s, i - 1));
                if (lv) me.y -= cf.y * (pc - p2_of(s, i - W));
                s->vel[i] = me;
            }
            float m = 0.0f;
            if (lu) m = fabsf(me.x);
            if (lv) m = maxf(m, fabsf(me.y));
            if (m > m_all) m_all = m;
        }
    memcpy(s->p2keep, keep, (size_t)W * s->H * sizeof(float));
    free(keep);
    if (m_all > bitsf(s->S.umax_grid)) s->S.umax_grid = fbits(m_all);
}

/* ------------------------------------------------------------------------------------ */
/* The substep (record_substep, mod.rs:2615-2708)                                         */
/* ------------------------------------------------------------------------------------ */

static void substep(OSim* s, int gather) {
    k_step(s);
    /* The per-substep gain of the density correction (rhs.comp:79) depends only on dt. */
    P_.corr_gain = minf(1.0f - o_expf(-s->S.dt / P_.tol[3]), P_.density_k);
    memset(s->acc, 0, (size_t)s->W * s->H * P_.acc_stride * sizeof(int32_t));
    if (s->thermal) memset(s->hcell, 0, (size_t)s->W * s->H * sizeof(I2));
    k_particles(s, gather);
    k_grid_prep(s);
    if (s->caps & CAP_RHEO) k_rheo(s);
    if (s->caps & CAP_ELASTIC) k_elastic(s);
    if (s->caps & CAP_SETTLE) k_settle(s);
    k_grid_coef(s);
    k_surf_smooth(s);
    k_surf_curv(s);
    k_surf_apply(s);
    if (s->caps & CAP_MAGNET) {
        k_magnet_energy(s);
        k_magnet_force(s);
    }
    if (s->thermal && s->prm.heat_rate > 0.0f) k_heat(s);
    if (s->visc_mode == 1) {
        k_visc_setup(s);
        k_visc_apply_explicit(s);
    }
    /* implicit viscosity between two pressure solves (viscous_projection) or before one */
    const int twice = s->visc_mode == 2 && s->prm.viscous_projection != 0;
    if (s->visc_mode == 2) {
        /* record_viscosity_split (mod.rs:2812-2836) */
        memset(s->tiles, 0, (size_t)s->nwg * sizeof(uint32_t));
        k_visc_setup(s);
        k_visc_split(s);
        k_visc_diag(s, s->prm.viscosity_warm != 0, 1);
        const int nlev = mini(maxi((int)s->prm.viscosity_mg_levels, 1), s->lv.tail);
        for (int l = 1; l <= nlev; l++) k_vmg_build(s, l);
        if (!twice) viscosity_solve(s, 0);
    }
    memset(s->ptile, 0, (size_t)s->nwg * sizeof(uint32_t));
    k_rhs(s);
    pressure_solve(s, 0);
    k_project(s);
    if (twice) {
        viscosity_solve(s, 1);
        k_rhs_visc(s, s->prm.viscous_warm != 0);
        pressure_solve(s, 1);
        k_project_visc(s);
    }
    if (s->caps & CAP_RIGID) k_rigid(s);   /* mod.rs:2701-2707 */
}

/* ------------------------------------------------------------------------------------ */
/* API                                                                                   */
/* ------------------------------------------------------------------------------------ */

#define ALLOC(ptr, n) do { (ptr) = calloc((size_t)(n), sizeof(*(ptr))); } while (0)

OSim* osim_create(int w, int h, uint32_t capacity, const OSimParams* p) {
    if (w < 16 || h < 16) return NULL;
    OSim* s = (OSim*)calloc(1, sizeof(OSim));
    s->W = w;
    s->H = h;
    s->capacity = capacity;
    s->prm = *p;
    levels_new(&s->lv, w, h);
    s->nwg = ((w + 15) / 16) * ((h + 15) / 16);
    size_t nc = (size_t)w * h;
    ALLOC(s->particles, capacity);
    ALLOC(s->sorted, capacity);
    ALLOC(s->acc, nc * ACC_MAX);
    ALLOC(s->vel, nc); ALLOC(s->cell, nc); ALLOC(s->comp, nc); ALLOC(s->coef, nc);
    ALLOC(s->sprop, nc); ALLOC(s->surf, nc); ALLOC(s->surf2, nc); ALLOC(s->aux, nc);
    ALLOC(s->grho, nc); ALLOC(s->therm, nc); ALLOC(s->dheat, nc); ALLOC(s->vw, nc);
    ALLOC(s->vs, nc); ALLOC(s->prhs, nc); ALLOC(s->vel0, nc); ALLOC(s->pjump, nc);
    ALLOC(s->mixb, nc * (MAX_PRESENT - 1));
    ALLOC(s->gbase, nc);
    ALLOC(s->rh, nc);
    ALLOC(s->magc, nc);
    ALLOC(s->rl, nc);
    ALLOC(s->rbody, (size_t)O_MAX_BODIES * 16);
    for (size_t k = 0; k < nc; k++) s->rl[k] = (I2){-1, -1};
    ALLOC(s->pres, nc); ALLOC(s->p2keep, nc); ALLOC(s->hcell, nc); ALLOC(s->solid, nc);
    ALLOC(s->sdf, (size_t)(w + 1) * (h + 1)); ALLOC(s->region, nc); ALLOC(s->solid_t, nc);
    ALLOC(s->mga, s->lv.total); ALLOC(s->mgd, s->lv.total); ALLOC(s->mgx, s->lv.total);
    ALLOC(s->mgz, s->lv.total); ALLOC(s->mgr, s->lv.total);
    ALLOC(s->cgp, nc); ALLOC(s->cgp2, nc); ALLOC(s->cgq, nc);
    ALLOC(s->vr, nc); ALLOC(s->vr2, nc); ALLOC(s->vp, nc); ALLOC(s->vq, nc); ALLOC(s->vq2, nc);
    ALLOC(s->vd, nc); ALLOC(s->vaz, nc);
    ALLOC(s->vma, s->lv.total); ALLOC(s->vmb, s->lv.total); ALLOC(s->vmd, s->lv.total);
    ALLOC(s->vmr, s->lv.total); ALLOC(s->vmx, s->lv.total); ALLOC(s->vmz, s->lv.total);
    ALLOC(s->tiles, s->nwg); ALLOC(s->vtile, s->lv.tiles);
    ALLOC(s->ptile, s->lv.tiles);
    ALLOC(s->part, 2 * s->nwg);
    ALLOC(s->pending, SPAWN_MAX);
    for (size_t k = 0; k < nc; k++) s->solid_t[k] = NO_TEMP;
    return s;
}

void osim_destroy(OSim* s) {
    if (!s) return;
    free(s->plook);
    free(s->dpool);
    free(s->dstack1);
    free(s->dfield);
    free(s->dstack);
    free(s->dlist);
    free(s->dcount);
    void* ptrs[] = {s->particles, s->sorted, s->acc, s->vel, s->cell, s->comp, s->coef, s->sprop,
                    s->surf, s->surf2, s->aux, s->grho, s->therm, s->dheat, s->vw, s->vs, s->prhs,
                    s->vel0, s->pjump, s->pres, s->p2keep, s->hcell, s->solid, s->sdf, s->region,
                    s->solid_t, s->mga, s->mgd, s->mgx, s->mgz, s->mgr, s->cgp, s->cgp2, s->cgq,
                    s->ptile, s->part, s->vr, s->vr2, s->vp, s->vq, s->vq2, s->vd, s->vaz, s->vma,
                    s->vmb, s->vmd, s->vmr, s->vmx, s->vmz, s->tiles, s->vtile, s->pending, s->mixb, s->gbase, s->rh, s->famocc, s->dsettle, s->magc, s->pstress, s->estr, s->rl, s->rbody};
    for (size_t k = 0; k < sizeof ptrs / sizeof ptrs[0]; k++) free(ptrs[k]);
    free(s);
}

int osim_set_magnets(OSim* s, const OMagnet* m, uint32_t n) {   /* mod.rs:2018-2022 */
    s->n_magnets = 0;
    for (uint32_t i = 0; i < n && i < O_MAX_MAGNETS; i++) s->magnets[s->n_magnets++] = m[i];
    if (s->tank.nrows > 0) s->caps = compute_caps(s);
    return 0;
}

int osim_set_currents(OSim* s, const OCurrent* c, uint32_t n) {   /* mod.rs:2008-2012 */
    s->n_currents = 0;
    for (uint32_t i = 0; i < n && i < O_MAX_CURRENTS; i++) s->currents[s->n_currents++] = c[i];
    return 0;
}

int osim_set_params(OSim* s, const OSimParams* p) {
    s->prm = *p;
    return 0;
}

int osim_set_solids(OSim* s, const float* sdf, const float* solid4, const uint32_t* region, const float* temp) {
    size_t nc = (size_t)s->W * s->H;
    memcpy(s->sdf, sdf, (size_t)(s->W + 1) * (s->H + 1) * sizeof(float));
    memcpy(s->solid, solid4, nc * sizeof(V4));
    memcpy(s->region, region, nc * sizeof(uint32_t));
    s->solids_heated = temp != NULL;
    for (size_t k = 0; k < nc; k++) s->solid_t[k] = temp ? temp[k] : NO_TEMP;
    return 0;
}

static float melting_lat(const OMat* d) { return freezes(d) ? d->latent / d->heat_capacity : 0.0f; }

/* SimParams::enthalpy_temp (params.rs:848-860) with melting (params.rs:830-845) */
static float enthalpy_temp(const OSimParams* p, int row, float sc, float t) {
    const OMat* own = &p->mat[row];
    float lo, hi, l;
    if (own->diluent < 0) {
        lo = own->melt_lo;
        hi = maxf(own->melt_hi, own->melt_lo + 0.25f);
        l = melting_lat(own);
    } else {
        const OMat* d = &p->mat[own->diluent];
        float shift = own->freeze_shift * sc;
        float cd = d->density * d->heat_capacity, co = own->density * own->heat_capacity;
        float c = cd + (co - cd) * sc;
        l = (cd * melting_lat(d) + (co * own->latent / own->heat_capacity - cd * melting_lat(d)) * sc) / c;
        lo = d->melt_lo + shift;
        hi = maxf(d->melt_hi, d->melt_lo + 0.25f) + shift;
    }
    if (lo < -273.0f || t >= hi) return t;
    if (t <= lo) return t - l;
    float fr = (t - lo) / maxf(hi - lo, 1e-3f);
    return (lo - l) + fr * (hi - lo + l);
}

/* Particle::settle_spawn (params.rs:70-85) and the position range every substep leaves a
 * particle in (particles.comp:912), so that the first gather's 3 x 3 stencils stay on the
 * grid. Returns 0, or -1 for a non-finite position. */
static int settle(const OSim* s, OParticle* q) {
    const OSimParams* p = &s->prm;
    if (!isfinite(q->pos[0]) || !isfinite(q->pos[1])) return -1;
    q->pos[0] = minf(maxf(q->pos[0], 2.01f), (float)s->W - 2.01f);
    q->pos[1] = minf(maxf(q->pos[1], 2.01f), (float)s->H - 2.01f);
    uint32_t mat = (q->kind & 255u);
    if (mat != 0u && q->kind != KIND_DEAD) {
        const OMat* def = &p->mat[mat - 1u];
        if (q->t == SPAWN_TEMP) {
            q->t = def->spawn_temp;
            q->kind |= KIND_REAL_T;
        }
        if (q->s == SPAWN_S) q->s = def->diluent >= 0 ? clampf(def->load, 0.0f, 1.0f) : 1.0f;
        if (q->kind & KIND_REAL_T) {
            q->kind &= ~KIND_REAL_T;
            q->t = enthalpy_temp(p, (int)mat - 1, q->s, q->t);
        }
    }
    return 0;
}

/* Marks the materials of particles in present[] and widens *thermal by their temperatures
 * (note_materials, mod.rs:2050-2060). */
static void mark_materials(const OSim* s, const OParticle* q, uint32_t n, int* present, int* thermal) {
    const OSimParams* p = &s->prm;
    for (uint32_t k = 0; k < n; k++) {
        uint32_t m = q[k].kind & 255u;
        if (m == 0u || q[k].kind == KIND_DEAD) continue;
        present[m - 1u] = 1;
        *thermal |= fabsf(q[k].t - p->ambient_temp) > 0.05f || p->mat[m - 1u].self_heat > 0.0f;
    }
}

/* The tank for the rows marked in present[] (ascending) and the thermal flag: Tank::layout
 * (mod.rs:271-329), the capabilities and viscosity mode that follow. A concentrate brings
 * its diluent into the tank's rows (mod.rs:223: the materials "with their diluents"). Changes
 * s only when every check passes; returns -2 (the rows do not fit) or -4 (a capability the
 * oracle does not carry) otherwise. */
static int set_tank(OSim* s, const int* present_in, int thermal) {
    const OSimParams* p = &s->prm;
    int present[O_MAX_MATERIALS];
    for (int r = 0; r < O_MAX_MATERIALS; r++) present[r] = present_in[r];
    for (int r = 0; r < O_MAX_MATERIALS; r++)
        if (present_in[r] && p->mat[r].diluent >= 0) present[p->mat[r].diluent] = 1;
    int rows[MAX_PRESENT], nrows = 0;
    for (int r = 0; r < O_MAX_MATERIALS; r++)
        if (present[r]) {
            if (nrows == MAX_PRESENT) return -2;
            rows[nrows++] = r;
        }
    Tank t;
    if (!tank_layout(&t, rows, nrows, p, thermal)) return -2;
    const Tank old_tank = s->tank;
    const int old_thermal = s->thermal, old_visc = s->visc_mode;
    const uint32_t old_caps = s->caps;
    s->tank = t;
    s->thermal = thermal;
    s->caps = compute_caps(s);
    int rc = 0;
    if (s->caps & (CAP_STEAM | CAP_REACT)) rc = -4;
    for (int k = 0; k < nrows; k++) {
        const OMat* m = &p->mat[rows[k]];
        if (m->volatility > 0.0f || (thermal && m->boil < 1e8f)) rc = -4;
    }
    if (rc == 0) rc = set_settling(s, settles(s) ? s->tank.families : 0);
    if (rc == 0) rc = set_elastic(s, s->tank.chan_e >= 0);
    if (rc == 0) s->caps = compute_caps(s);   /* with the settling buffers in place */
    if (rc == 0) {
        s->visc_mode = viscosity_mode(s);
        /* the multigrid-preconditioned implicit solve needs at least one coarse level */
        if (s->visc_mode == 2 && s->prm.viscosity_precond != 0 && s->lv.tail < 1) rc = -4;
    }
    if (rc != 0) {
        s->tank = old_tank;
        s->thermal = old_thermal;
        s->caps = old_caps;
        s->visc_mode = old_visc;
        return rc;
    }
    build_mats(s);
    return 0;
}

static uint32_t recorded_limit(uint32_t rec, int viscosity, int mg_precond);

int osim_reset(OSim* s, const OParticle* in, uint32_t n) {
    if (n > s->capacity) n = s->capacity;
    const OSimParams* p = &s->prm;
    /* reset: ids, settle_spawn (mod.rs:1981-2002) */
    for (uint32_t k = 0; k < n; k++) {
        OParticle q = in[k];
        q.id = k;
        if (settle(s, &q) != 0) return -1;
        s->particles[k] = q;
    }
    s->n_slots = n;
    s->next_id = n;
    s->n_pending = 0;
    s->spawn_speed = 0.0f;
    /* the tank: rows present (note_materials), thermal from heated solids or temperatures */
    int present[O_MAX_MATERIALS] = {0};
    int thermal = s->solids_heated;
    mark_materials(s, s->particles, n, present, &thermal);
    if (fabsf(p->ambient_temp - T_REF) > 0.05f) thermal = 1;
    int rc = set_tank(s, present, thermal);
    if (rc != 0) return rc;
    /* buffers a reset clears (mod.rs:2451-2460) */
    size_t nc = (size_t)s->W * s->H;
    memset(s->pres, 0, nc * sizeof(V2));
    memset(s->p2keep, 0, nc * sizeof(float));
    memset(&s->S, 0, sizeof s->S);
    /* a new scene records the most until its frames say otherwise (mod.rs:2478-2483) */
    s->K.rec[0] = s->K.rec[1] = p->pressure_max_iters;
    s->K.rec[2] = p->viscosity_max_iters;
    for (int k = 0; k < 3; k++) {
        s->K.cap[k] = recorded_limit(s->K.rec[k], k == 2, p->viscosity_precond != 0);
        s->K.f_it[k] = s->K.f_un[k] = 0u;
    }
    memset(s->dheat, 0, nc * sizeof(V4));
    memset(s->ledger, 0, sizeof s->ledger);
    s->grid_valid = 0;
    s->since_sort = 0;
    s->sim_time = 0.0;
    return 0;
}

int osim_spawn(OSim* s, const OParticle* in, uint32_t n) {
    const OSimParams* p = &s->prm;
    uint32_t room = SPAWN_MAX - s->n_pending;
    OParticle* q = s->pending + s->n_pending;
    uint32_t m = 0;
    for (uint32_t k = 0; k < n && m < room; k++) {
        /* particles without a material are not queued (reset drops them too, mod.rs:1994) */
        uint32_t mat = in[k].kind & 255u;
        if (in[k].kind == KIND_DEAD || mat == 0u || mat > O_MAX_MATERIALS) continue;
        q[m] = in[k];
        q[m].id = s->next_id + m;
        if (settle(s, &q[m]) != 0) return -1;
        m++;
    }
    int present[O_MAX_MATERIALS] = {0};
    for (int k = 0; k < s->tank.nrows; k++) present[s->tank.rows[k]] = 1;
    int thermal = s->thermal;
    int before = 0;
    for (int r = 0; r < O_MAX_MATERIALS; r++) before += present[r];
    mark_materials(s, q, m, present, &thermal);
    int after = 0;
    for (int r = 0; r < O_MAX_MATERIALS; r++) after += present[r];
    if (after != before || thermal != s->thermal) {
        int rc = set_tank(s, present, thermal);
        if (rc == -2 || rc == -3) return 0;   /* they do not fit: none is accepted */
        if (rc != 0) return rc;
    }
    for (uint32_t k = 0; k < m; k++) {
        s->spawn_speed = maxf(s->spawn_speed, hypotf(q[k].vel[0], q[k].vel[1]));
        q[k].kind |= KIND_FRESH;
    }
    s->next_id += m;
    s->n_pending += m;
    return (int)m;
}

/* record (mod.rs:2486-2503) and claim.comp: queued particles fill fresh slots while there are
 * any, then dead slots, the k-th dead slot (in slot order) taking the k-th remaining entry;
 * entries beyond the dead slots are dropped. */
static void take_spawns(OSim* s) {
    uint32_t n = s->n_pending;
    if (n == 0) return;
    uint32_t fresh = n < s->capacity - s->n_slots ? n : s->capacity - s->n_slots;
    memcpy(s->particles + s->n_slots, s->pending, (size_t)fresh * sizeof(OParticle));
    s->n_slots += fresh;
    uint32_t k = fresh;
    for (uint32_t id = 0; id < s->n_slots && k < n; id++)
        if (s->particles[id].kind == KIND_DEAD) s->particles[id] = s->pending[k++];
    s->n_pending = 0;
}

long osim_cell_counts(const OSim* s, const int lo[2], const int hi[2], uint32_t* out, size_t cap) {
    if (lo[0] < 0 || lo[1] < 0 || hi[0] > s->W || hi[1] > s->H) return -1;
    int sw = hi[0] - lo[0] > 0 ? hi[0] - lo[0] : 0, sh = hi[1] - lo[1] > 0 ? hi[1] - lo[1] : 0;
    size_t n = (size_t)sw * sh;
    if (!out) return (long)n;
    if (cap < n) return -1;
    memset(out, 0, n * sizeof(uint32_t));
    /* count.comp:17-23 over the slots, then the queue (mod.rs:3380-3385) */
    for (uint32_t id = 0; id < s->n_slots; id++) {
        const OParticle* q = &s->particles[id];
        if ((q->kind & 255u) == 0u) continue;
        int cx = (int)floorf(q->pos[0]) - lo[0], cy = (int)floorf(q->pos[1]) - lo[1];
        if (cx >= 0 && cy >= 0 && cx < sw && cy < sh) out[(size_t)cy * sw + cx]++;
    }
    for (uint32_t k = 0; k < s->n_pending; k++) {
        const OParticle* q = &s->pending[k];
        int cx = (int)floorf(q->pos[0]) - lo[0], cy = (int)floorf(q->pos[1]) - lo[1];
        if (cx >= 0 && cy >= 0 && cx < sw && cy < sh) out[(size_t)cy * sw + cx]++;
    }
    return (long)n;
}

/* The iterations a frame records for a solve (mod.rs:2569, 2603-2606): its count rounded up
 * to even, the viscosity solve's to a multiple of 4 with the Jacobi preconditioner. */
static uint32_t recorded_limit(uint32_t rec, int viscosity, int mg_precond) {
    uint32_t q = (viscosity && !mg_precond) ? 4u : 2u;
    return (rec + q - 1u) / q * q;
}

/* poll_readbacks' adaptation (mod.rs:3100-3106). */
static uint32_t adapt_rec(uint32_t rec, uint32_t used, uint32_t unconverged, uint32_t max, float margin) {
    if (unconverged > 0u) {
        uint32_t v = rec + rec / 2u + 2u;
        return v < max ? v : max;
    }
    uint32_t v = used + (uint32_t)((float)used * margin) + 2u;
    return v < 2u ? 2u : (v > max ? max : v);
}

/* The end of a frame (a step call): the recorded counts adapted from the frame's solves as the
 * reference adapts them when the frame's read-back arrives (mod.rs:3093-3114), the limits of
 * the next frame, the frame's statistics cleared. */
static void frame_end(OSim* s) {
    SolveBuf* K = &s->K;
    float margin = maxf(s->prm.iters_margin, 0.0f);
    uint32_t pmax = s->prm.pressure_max_iters, vmax = s->prm.viscosity_max_iters;
    K->rec[0] = adapt_rec(K->rec[0], K->f_it[0], K->f_un[0], pmax, margin);
    if (s->visc_mode == 2 && s->prm.viscous_projection != 0)
        K->rec[1] = adapt_rec(K->rec[1], K->f_it[1], K->f_un[1], pmax, margin);
    else
        K->rec[1] = K->rec[0];
    K->rec[2] = adapt_rec(K->rec[2], K->f_it[2], K->f_un[2], vmax, 0.5f);
    for (int k = 0; k < 3; k++) {
        K->cap[k] = recorded_limit(K->rec[k], k == 2, s->prm.viscosity_precond != 0);
        K->f_it[k] = 0u;
        K->f_un[k] = 0u;
    }
}

void osim_recorded_iters(const OSim* s, uint32_t out[3]) {
    for (int k = 0; k < 3; k++) out[k] = s->K.rec[k];
}

int osim_step(OSim* s, uint32_t substeps, float target, const OTool* tool) {
    s->frame += 1u;
    take_spawns(s);
    build_params(s, tool);
    s->spawn_speed = 0.0f;
    if (substeps > 0) {
        s->S.frame_left = maxf(target, 0.0f);
        s->S.batch_steps = substeps;
        s->S.batch_done = 0;
    }
    for (uint32_t k = 0; k < substeps; k++) {
        substep(s, s->grid_valid);
        /* the particles sorted by cell after every substep, as the engine keeps them (the
         * reference sorts every 128 substeps, mod.rs:100, 2546; the order changes no physics:
         * the deposits are integer sums and every particle is updated on its own) */
        osim_sort(s);
        s->grid_valid = 1;
        s->substeps_done++;
    }
    if (substeps > 0) frame_end(s);
    s->sim_time = s->S.advanced;
    return 0;
}

uint32_t osim_particles(const OSim* s, OParticle* out, uint32_t cap) {
    uint32_t n = s->n_slots < cap ? s->n_slots : cap;
    memcpy(out, s->particles, (size_t)n * sizeof(OParticle));
    return s->n_slots;
}

/* ------------------------------------------------------------------------------------ */
/* The render side's cell passes: cell_optics.comp, light.comp, optics_blur.comp            */
/* (mod.rs:1626-1660), into layers of RGBA16F texels as the reference's image array holds   */
/* them. exp / log / pow, sin / cos and atan are the oracle's own (o_expf, o_logf, o_powf,   */
/* o_sincos, o_atan2). The dust field (layer 18) and the film tiles are left out, as in the  */
/* engine.                                                                                   */
/* ------------------------------------------------------------------------------------ */

typedef struct OOptics {   /* material.rs GpuOptics: 240 bytes */
    float absorb[4], solid[4], opt[4], sty[4];
    int idx[4];
    float fx[4], fx2[4], lum[4], hot[4], thermo[4], scat[4], opt2[4], dust[4], dust2[4], dcol[4];
} OOptics;

/* IEEE binary16 from binary32, rounded to nearest even; and back */
static uint16_t o_half(float f) {
    uint32_t x;
    memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t mant = x & 0x7fffffu;
    int e = (int)((x >> 23) & 255u);
    if (e == 255) return (uint16_t)(sign | 0x7c00u | (mant ? 0x200u : 0u));
    int he = e - 127 + 15;
    if (he >= 31) return (uint16_t)(sign | 0x7c00u);
    if (he <= 0) {   /* subnormal half (or zero) */
        if (he < -10) return (uint16_t)sign;
        uint32_t m = mant | 0x800000u;
        int shift = 14 - he;   /* 24 bits down to (10 + he) bits */
        uint32_t hm = m >> shift, rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (hm & 1u))) hm++;
        return (uint16_t)(sign | hm);
    }
    uint32_t hm = mant >> 13, rem = mant & 0x1fffu;
    uint32_t out = sign | ((uint32_t)he << 10) | hm;
    if (rem > 0x1000u || (rem == 0x1000u && (hm & 1u))) out++;   /* may carry into the exponent: right */
    return (uint16_t)out;
}
static float o_unhalf(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    int e = (h >> 10) & 31;
    uint32_t m = h & 0x3ffu, x;
    if (e == 0) {
        if (m == 0) x = sign;
        else {
            e = 1;
            while (!(m & 0x400u)) { m <<= 1; e--; }
            m &= 0x3ffu;
            x = sign | ((uint32_t)(e - 15 + 127) << 23) | (m << 13);
        }
    } else if (e == 31) {
        x = sign | 0x7f800000u | (m << 13);
    } else {
        x = sign | ((uint32_t)(e - 15 + 127) << 23) | (m << 13);
    }
    float f;
    memcpy(&f, &x, 4);
    return f;
}
static void put_texel(uint16_t* out, size_t i, V4 v) {
    out[4 * i + 0] = o_half(v.x);
    out[4 * i + 1] = o_half(v.y);
    out[4 * i + 2] = o_half(v.z);
    out[4 * i + 3] = o_half(v.w);
}
static V4 get_texel(const uint16_t* in, size_t i) {
    return v4(o_unhalf(in[4 * i + 0]), o_unhalf(in[4 * i + 1]), o_unhalf(in[4 * i + 2]), o_unhalf(in[4 * i + 3]));
}
static V4 v4add(V4 a, V4 b) { return v4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static V4 v4mul(float s, V4 a) { return v4(s * a.x, s * a.y, s * a.z, s * a.w); }
static V4 v4muls(V4 a, float s) { return v4(a.x * s, a.y * s, a.z * s, a.w * s); }
static V4 v4mix(V4 a, V4 b, float t) { return v4(mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t), mixf(a.w, b.w, t)); }
static V4 v4ld(const float* f) { return v4(f[0], f[1], f[2], f[3]); }

/* optics.glsl: to_srgb, deep_reflectance, film_colour, look_key */
static float o_srgb1(float v) {
    v = clampf(v, 0.0f, 1.0f);
    return mixf(v * 12.92f, 1.055f * o_powf(v, 1.0f / 2.4f) - 0.055f, v < 0.0031308f ? 0.0f : 1.0f);
}
static V4 o_look_key(V4 k) {
    const float film = 0.35f;
    float kk[3] = {k.x, k.y, k.z}, out[3];
    for (int c = 0; c < 3; c++) {
        float ext = kk[c] + k.w;
        float tv = o_expf(-2.0f * ext * film);
        float w = k.w / maxf(kk[c] + k.w, 1e-6f);
        float q = sqrtf(maxf(1.0f - w, 0.0f));
        float refl = (1.0f - q) / (1.0f + q) * (1.0f - tv);
        out[c] = o_srgb1(refl + 0.75f * tv * o_expf(-2.0f * kk[c] * film));
    }
    return v4(out[0], out[1], out[2], 1.0f);
}
/* cell_optics.comp glow: the colour and brightness of a grey body at T (deg C) */
static void o_glow(float T, float out[3]) {
    float K = T + 273.15f;
    if (K < 760.0f) { out[0] = out[1] = out[2] = 0.0f; return; }
    float rel = o_expf(23587.0f / 1300.0f - 23587.0f / K);
    float level = minf(o_logf(1.0f + 200.0f * rel) / o_logf(201.0f), 1.6f);
    float cr = 1.0f, cg = 1.677f * o_expf(-2573.0f / K), cb = 3.89f * o_expf(-7355.0f / K);
    float m = maxf(cr, maxf(cg, cb));
    out[0] = cr / m * level;
    out[1] = cg / m * level;
    out[2] = cb / m * level;
}
static float o_occ_of(const OSim* s, int x, int y) {
    if (x < 0 || y < 0 || x >= s->W || y >= s->H) return 0.0f;
    return minf((float)s->acc[(y * s->W + x) * s->tank.stride + 4] / MASS_SCALE * P_.inv_ppc, 1.0f);
}
static float o_sdf_cell(const OSim* s, int x, int y) {
    x = mini(maxi(x, 0), s->W - 1);
    y = mini(maxi(y, 0), s->H - 1);
    int w1 = s->W + 1, k = y * w1 + x;
    return 0.25f * (s->sdf[k] + s->sdf[k + 1] + s->sdf[k + w1] + s->sdf[k + w1 + 1]);
}
static float o_aq_share(const OSim* s, int x, int y) {
    if (x < 0 || y < 0 || x >= s->W || y >= s->H) return 0.0f;
    int kq = (y * s->W + x) * s->tank.stride;
    int cwq = s->acc[kq + 4];
    if (cwq <= 0) return 0.0f;
    int others = 0, aqw = 0;
    for (int j = 0; j < P_.n_present; j++) {
        const int* ia = s->mats[P_.present[j]].ia;
        if (ia[2] < 0) continue;
        int w = s->acc[kq + ia[2]];
        others += w;
        if (ia[0] == 0) aqw += w;
    }
    int rest = maxi(cwq - others, 0);
    if (s->mats[P_.present[0]].ia[0] == 0) aqw += rest;
    return clampf((float)aqw / (float)cwq, 0.0f, 1.0f);
}

/* sin and cos rounded once from FP64: reduction by the nearest multiple q of pi/2 (Cody and
 * Waite, pi/2 in 33 + 53 bits), Taylor series to r^15 / r^16 on [-pi/4, pi/4], the quadrant's
 * swap and signs. The same operations as the engine's, so the same bits. */
static void o_sincos(float af, float* s, float* c) {
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
/* atan(y, x) rounded once from FP64: two angle halvings, the series to u^25, the octant;
 * 0 at x = y = 0 (GLSL leaves it undefined). */
float o_atan2(float yf, float xf) {
    const double y = (double)yf, x = (double)xf, ay = fabs(y), ax = fabs(x);
    if (ax == 0.0 && ay == 0.0) return 0.0f;
    const int swap = ay > ax;
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
float o_sinf(float a) { float s, c; o_sincos(a, &s, &c); return s; }
float o_cosf(float a) { float s, c; o_sincos(a, &s, &c); return c; }

/* FluidSim::spike_params (mod.rs:1885-1899). */
static void o_spike_params(const OSim* s, float* gap, float* mc) {
    *gap = *mc = 0.0f;
    const OMat* best = NULL;
    for (int k = 0; k < s->tank.nrows; k++) {
        const OMat* m = &s->prm.mat[s->tank.rows[k]];
        if (m->susceptibility > 0.0f && (!best || m->susceptibility >= best->susceptibility)) best = m;
    }
    if (!best || s->n_magnets == 0) return;
    float g = maxf(s->prm.gravity, 1.0f);
    float rho = maxf(best->density, 1.0f), sigma = maxf(best->tension, 1e-4f);
    float gp = 2.0f * 3.14159265f * sqrtf(sigma / (rho * g)) / s->prm.cell_size;
    *gap = gp > 3.0f ? gp : 3.0f;
    const float mu0 = 1.2566371e-6f;
    *mc = sqrtf(2.0f * mu0 * (1.0f + 1.0f / (1.0f + best->susceptibility)) * sqrtf(rho * g * sigma));
}
/* cell_optics.comp:86-117: the spikes' height and where they stand */
static float o_spike_height(const OSim* s, float gap, float mc, float B) {
    if (gap <= 0.0f || P_.mag[1] <= 0.0f) return 0.0f;
    float chi = P_.mag[1], ce = chi / (1.0f + chi);
    float m = ce * B / (1.0f + ce * B / maxf(P_.mag[2], 1e-6f));
    float over = m * m / maxf(mc * mc, 1e-12f) - 1.0f;
    return over > 0.0f ? 0.85f * gap * (1.0f - o_expf(-over)) : 0.0f;
}
static V2 o_spike_phase(const OSim* s, float gap, float x, float y) {
    int best = 0;
    float bb = -1.0f;
    for (int k = 0; k < (int)P_.mag[0]; k++) {
        const float* mg = P_.magnet[k];
        float r = maxf(len2(v2(x - mg[0], y - mg[1])), mg[2]);
        float b = mg[3] * o_powf(mg[2] / r, 3.0f);
        if (b > bb) {
            bb = b;
            best = k;
        }
    }
    float dx = x - P_.magnet[best][0], dy = y - P_.magnet[best][1];
    float mx = P_.magnet_dir[best][0], my = P_.magnet_dir[best][1];
    float ang = o_atan2(mx * dy - my * dx, mx * dx + my * dy);
    float ph = 6.2831853f * len2(v2(dx, dy)) * ang / (maxf(gap, 1e-3f) * 4.0f);
    float sn, cs;
    o_sincos(ph, &sn, &cs);
    return v2(cs, sn);
}

static void o_cell_optics(const OSim* s, const OOptics* opt, float inv_speed, float spike_gap, float spike_mc,
                          const int32_t* dfield, float dust, int cx, int cy, uint16_t* raw) {
    const int i = cy * s->W + cx, k = i * s->tank.stride;
    const size_t nc = (size_t)s->W * s->H;
    const int cw = s->acc[k + 4];
    V4 o[20];
    for (int l = 0; l < 20; l++) o[l] = v4(0.0f, 0.0f, 0.0f, 0.0f);
    if (spike_gap > 0.0f) {   /* every cell: the spikes stand in the air */
        float px = (float)cx + 0.5f, py = (float)cy + 0.5f;
        V2 B = magnet_field(s, px, py);
        float b = len2(B), hgt = o_spike_height(s, spike_gap, spike_mc, b);
        o[13] = v4(b > 1e-9f ? B.x / b * hgt : 0.0f, b > 1e-9f ? B.y / b * hgt : 0.0f, 0.0f, spike_gap);
        V2 ph = o_spike_phase(s, spike_gap, px, py);
        o[14].x = ph.x;
        o[14].y = ph.y;
    }
    if (cw > 0) {
        int thermal = has_cap(s, CAP_THERMAL);
        float T = thermal ? s->therm[i].x : P_.heat[0];
        int others = 0;
        for (int j = 0; j < P_.n_present; j++) {
            int ch = s->mats[P_.present[j]].ia[2];
            if (ch >= 0) others += s->acc[k + ch];
        }
        int cl = maxi(cw, 1);
        float occ = minf((float)cw / MASS_SCALE * P_.inv_ppc, 1.0f);
        float Tg[GROUPS];
        {
            float Csh = 0.0f, Cg[GROUPS] = {0};
            if (thermal) {
                for (int j = 0; j < P_.n_present; j++) {
                    int r = P_.present[j];
                    const int* ia = s->mats[r].ia;
                    if (ia[2] < 0 && P_.primary >= 0 && r != P_.primary) continue;
                    int w = ia[2] >= 0 ? s->acc[k + ia[2]] : maxi(cw - others, 0);
                    if (w <= 0) continue;
                    float sh = w >= cw ? 1.0f : clampf((float)w / (float)cw, 0.0f, 1.0f);
                    float sc = (ia[1] >= 0 && ia[3] >= 0) ? clampf((float)s->acc[k + ia[3]] / (float)w, 0.0f, 1.0f) : 1.0f;
                    float cr = sh * thermal_of(s, (uint32_t)r, sc).w;
                    Csh += cr;
                    Cg[ia[0]] += cr;
                }
            }
            group_temperatures(s, k, cw, Csh, Cg, &T, Tg);
        }
        V4 aq = v4(0, 0, 0, 0), ot = aq, op_sum = aq, sty = aq, aq_plain = aq, aq_conc = aq, iaq = aq, iot = aq, fx = aq, fx2 = aq;
        V4 dense = aq;
        float c_aq = 0.0f, lum[3] = {0, 0, 0}, em[3] = {0, 0, 0}, ior_sum = 0.0f;
        V4 vi = s->vel[i];
        float vsx = face_live(vi.z) ? vi.x : 0.0f, vsy = face_live(vi.w) ? vi.y : 0.0f;
        float stirred = smoothstepf(1.5f, 12.0f, sqrtf(vsx * vsx + vsy * vsy));
        float best_sh = 0.0f, wden = 0.0f, fden = 0.0f, mag = 0.0f, fzx = 0.0f, fzy = 0.0f, waq = 0.0f, wot = 0.0f, skin = 0.0f;
        int best_row = -1;
        float waq_here = o_aq_share(s, cx, cy);
        for (int j = 0; j < P_.n_present; j++) {
            int r = P_.present[j];
            const int* ia = s->mats[r].ia;
            if (ia[2] < 0 && P_.primary >= 0 && r != P_.primary) continue;
            int w = ia[2] >= 0 ? s->acc[k + ia[2]] : maxi(cw - others, 0);
            if (w <= 0) continue;
            float sh = clampf((float)w / (float)cl, 0.0f, 1.0f);
            float sc = (ia[1] >= 0 && ia[3] >= 0) ? clampf((float)s->acc[k + ia[3]] / (float)w, 0.0f, 1.0f) : 1.0f;
            const OOptics* oo = &opt[r];
            V4 absorb = v4ld(oo->absorb);
            if (oo->thermo[1] > oo->thermo[0]) absorb = v4mix(absorb, v4ld(oo->hot), smoothstepf(oo->thermo[0], oo->thermo[1], Tg[ia[0]]));
            V4 lab = absorb, op = v4ld(oo->opt), st = v4ld(oo->sty), ef = v4ld(oo->fx), lm = v4ld(oo->lum);
            V4 e2 = v4(oo->fx2[0], oo->fx2[1], absorb.w * oo->scat[0], absorb.w * oo->scat[2]);
            float labs[3] = {oo->solid[0], oo->solid[1], oo->solid[2]};
            if (ia[1] >= 0) {
                const OOptics* dd = &opt[ia[1]];
                lab = v4mix(v4ld(dd->absorb), absorb, sc);
                for (int c = 0; c < 3; c++) labs[c] = mixf(dd->solid[c], labs[c], sc);
                op = v4mix(v4ld(dd->opt), op, sc);
                st = v4mix(v4ld(dd->sty), st, sc);
                ef = v4mix(v4ld(dd->fx), ef, sc);
                e2 = v4mix(v4(dd->fx2[0], dd->fx2[1], dd->absorb[3] * dd->scat[0], dd->absorb[3] * dd->scat[2]), e2, sc);
                lm = v4mix(v4ld(dd->lum), lm, sc);
            }
            V4 kl = absorb;
            if (absorb.w <= 1e-3f && oo->opt[0] < 0.2f) {
                float grey = kl.x * 0.3f + kl.y * 0.45f + kl.z * 0.25f;
                kl = v4(grey, grey, grey, kl.w);
            }
            if (ia[1] >= 0) {
                const OOptics* dd = &opt[ia[1]];
                V4 kd = v4ld(dd->absorb);
                if (dd->absorb[3] <= 1e-3f && dd->opt[0] < 0.2f) {
                    float grey = kd.x * 0.3f + kd.y * 0.45f + kd.z * 0.25f;
                    kd = v4(grey, grey, grey, kd.w);
                }
                kl = v4mix(kd, absorb, sc);
            }
            o[19] = v4add(o[19], v4mul(sh, kl));
            ior_sum += sh * (ia[1] >= 0 ? mixf(opt[ia[1]].opt2[0], oo->opt2[0], sc) : oo->opt2[0]);
            fx2 = v4add(fx2, v4mul(sh, e2));
            float sl = mixf(1.0f, stirred, lm.w);
            lum[0] += sh * lm.x * sl;
            lum[1] += sh * lm.y * sl;
            lum[2] += sh * lm.z * sl;
            mag += sh * s->mats[r].el[2];
            float Tm = Tg[ia[0]], fs = 0.0f;
            if (thermal) {
                V4 th = thermal_of(s, (uint32_t)r, sc);
                fs = th.y > -1e8f ? clampf((th.y - Tm) / maxf(th.y - th.x, 1e-3f), 0.0f, 1.0f) : 0.0f;
                op.w *= 1.0f - 0.6f * fs;
                op.x = mixf(op.x, maxf(op.x, 0.6f), fs);
            }
            if (oo->idx[1] == 0) {
                aq = v4add(aq, v4mul(sh, lab));
                if (ia[1] >= 0) {
                    aq_plain = v4add(aq_plain, v4mul(sh * (1.0f - sc), v4ld(opt[ia[1]].absorb)));
                    aq_conc = v4add(aq_conc, v4mul(sh * sc, absorb));
                    c_aq += sh * sc;
                } else {
                    aq_plain = v4add(aq_plain, v4mul(sh, absorb));
                }
                waq += sh;
                iaq = v4add(iaq, v4mul(sh * fs, v4(labs[0], labs[1], labs[2], 0.0f)));
                fzx += sh * fs;
            } else {
                if (oo->idx[1] == 1) ot = v4add(ot, v4mul(sh, lab));
                else {
                    dense = v4add(dense, v4mul(sh, lab));
                    wden += sh;
                    fden += sh * fs;
                }
                wot += sh;
                iot = v4add(iot, v4mul(sh * fs, v4(labs[0], labs[1], labs[2], 0.0f)));
                fzy += sh * fs;
            }
            if (thermal && ia[0] == 3 && ef.w > 0.01f && Tm > 0.0f) {
                V4 th = thermal_of(s, (uint32_t)r, sc);
                if (th.y > -1e8f) {
                    float g = 2.0f * s->mats[r].th[1];
                    float hc = P_.heat2[3], Tw = minf(Tg[0], 100.0f), Ta = P_.heat[0] + 273.15f;
                    float ts_w = (g * Tm + hc * Tw) / maxf(g + hc, 1e-12f), ts_a = Tm;
                    for (int it = 0; it < 4; it++) {
                        float Kk = ts_a + 273.15f;
                        float h = P_.heat[2] + st.w * P_.heat[3] * (Kk * Kk + Ta * Ta) * (Kk + Ta);
                        ts_a = (g * Tm + h * P_.heat[0]) / maxf(g + h, 1e-12f);
                    }
                    float range = maxf(th.y - th.x, 1e-3f);
                    float sk_w = clampf((th.y - ts_w) / range, 0.0f, 1.0f), sk_a = clampf((th.y - ts_a) / range, 0.0f, 1.0f);
                    float to_air = 0.0f, to_water = waq_here;
                    for (int q = 0; q < 4; q++) {
                        int nx = cx + (q == 0 ? -1 : q == 1 ? 1 : 0), ny = cy + (q == 2 ? -1 : q == 3 ? 1 : 0);
                        if (o_sdf_cell(s, nx, ny) < 0.0f) continue;
                        float on = o_occ_of(s, nx, ny);
                        to_air += 1.0f - on;
                        to_water += on * o_aq_share(s, nx, ny);
                    }
                    skin = maxf(skin, sh * maxf(sk_w * clampf(to_water, 0.0f, 1.0f), sk_a * clampf(to_air, 0.0f, 1.0f)));
                }
            }
            op_sum = v4add(op_sum, v4mul(sh, op));
            fx = v4add(fx, v4mul(sh, ef));
            if (sh > best_sh) { best_sh = sh; best_row = r; }
            sty = v4add(sty, v4mul(sh, st));
            float gl[3];
            o_glow(Tm, gl);
            for (int c = 0; c < 3; c++) em[c] += sh * gl[c] * st.w;
        }
        float speed = minf(sqrtf(vsx * vsx + vsy * vsy) * inv_speed, 1.5f);
        o[15] = v4muls(v4(aq_plain.x, aq_plain.y, aq_plain.z, maxf(waq - c_aq, 0.0f)), occ);
        if (waq > 0.0f) aq = v4add(v4muls(aq_plain, o_expf(-24.0f * c_aq / waq)), aq_conc);
        o[0] = v4muls(aq, occ);
        o[1] = v4muls(ot, occ);
        o[2] = v4muls(op_sum, occ);
        float sk = 1.0f - 0.6f * clampf(skin, 0.0f, 1.0f);
        for (int c = 0; c < 3; c++) em[c] *= sk;
        o[3] = v4muls(v4(em[0] + lum[0], em[1] + lum[1], em[2] + lum[2], speed), occ);
        float s_mean = aq.w + ot.w + dense.w;
        o[16] = v4(fx2.x * occ, fx2.y * occ, s_mean > 1e-5f ? fx2.z / s_mean : 1.0f, s_mean > 1e-5f ? fx2.w / s_mean : 1.0f);
        if (dust > 0.0f && occ > 0.02f) {   /* cell_optics.comp:387-390 */
            const float f = 1.0f / 1024.0f;
            o[18] = v4((float)dfield[4 * i] * f, (float)dfield[4 * i + 1] * f, (float)dfield[4 * i + 2] * f,
                       (float)dfield[4 * i + 3] * f);
            float cap = 200.0f * occ;
            o[18] = v4(minf(o[18].x, cap), minf(o[18].y, cap), minf(o[18].z, cap), minf(o[18].w, cap));
        }
        o[19] = v4add(v4muls(o[19], occ), o[18]);
        o[17] = v4muls(v4(lum[0], lum[1], lum[2], ior_sum), occ);
        o[4] = v4muls(v4(sty.x, sty.y, waq, waq + wot), occ);
        o[5] = v4muls(v4(iaq.x, iaq.y, iaq.z, wden), occ);
        o[6] = v4muls(v4(iot.x, iot.y, iot.z, fden), occ);
        o[11] = v4muls(dense, occ);
        int last = s->W * s->H - 1;
        V4 vr = s->vel[mini(i + 1, last)], vt = s->vel[mini(i + s->W, last)];
        float ucx = 0.5f * (vsx + (face_live(vr.z) ? vr.x : 0.0f)), ucy = 0.5f * (vsy + (face_live(vt.w) ? vt.y : 0.0f));
        o[7] = v4muls(v4(fzx, fzy, ucx, ucy), occ);
        o[8] = v4muls(fx, occ);
        o[9] = v4muls(v4(0.0f, 0.0f, 0.0f, skin), occ);
        o[10] = v4(fx.y * occ, 0.0f, 0.0f, 0.0f);
        o[13].z = fx.x * occ;
        o[14].w = (float)(best_row + 1);
        float wl = waq + wot;
        if (wl > 0.0f) {
            V4 sum = v4add(v4add(aq, ot), dense);
            o[12] = v4muls(o_look_key(v4(sum.x / wl, sum.y / wl, sum.z / wl, sum.w / wl)), occ);
        }
        o[14].z = P_.mag[1] > 0.0f ? mag / P_.mag[1] * occ : 0.0f;
    }
    for (int l = 0; l < 20; l++) put_texel(raw, (size_t)l * nc + i, o[l]);
}

static void o_light(const OSim* s, uint16_t* raw) {
    const int H = s->H, W = s->W;
    const size_t nc = (size_t)W * H;
    const int stretch = mini((H + 63) / 64, 32);
    for (int x = 0; x < W; x++) {
        float sums[64][3];
        for (int t = 0; t < 64; t++) {
            int top = H - 1 - t * stretch;
            float sm[3] = {0, 0, 0};
            for (int k = 0; k < stretch; k++) {
                int y = top - k;
                if (y < 0) break;
                V4 kv = get_texel(raw, (size_t)19 * nc + (size_t)y * W + x);
                float kk[3] = {kv.x, kv.y, kv.z};
                for (int c = 0; c < 3; c++) sm[c] += minf(sqrtf(maxf(kk[c] * (kk[c] + 3.0f * kv.w), 0.0f)), 0.25f);
            }
            for (int c = 0; c < 3; c++) sums[t][c] = sm[c];
        }
        for (int t = 0; t < 64; t++) {
            int top = H - 1 - t * stretch;
            float tau[3] = {0, 0, 0};
            for (int j = 0; j < t; j++)
                for (int c = 0; c < 3; c++) tau[c] += sums[j][c];
            for (int k = 0; k < stretch; k++) {
                int y = top - k;
                if (y < 0) break;
                V4 kv = get_texel(raw, (size_t)19 * nc + (size_t)y * W + x);
                float kk[3] = {kv.x, kv.y, kv.z}, a[3];
                for (int c = 0; c < 3; c++) a[c] = minf(sqrtf(maxf(kk[c] * (kk[c] + 3.0f * kv.w), 0.0f)), 0.25f);
                size_t at = (size_t)10 * nc + (size_t)y * W + x;
                V4 l10 = get_texel(raw, at);
                V4 il = v4(l10.x, o_expf(-0.35f * (tau[0] + 0.5f * a[0])), o_expf(-0.35f * (tau[1] + 0.5f * a[1])),
                           o_expf(-0.35f * (tau[2] + 0.5f * a[2])));
                put_texel(raw, at, il);
                for (int c = 0; c < 3; c++) tau[c] += a[c];
            }
        }
    }
}

static void o_optics_blur(const OSim* s, const uint16_t* raw, uint16_t* sm, int cx, int cy) {
    const int W = s->W, H = s->H;
    const size_t nc = (size_t)W * H;
    const float K[3] = {1.0f, 2.0f, 1.0f};
    V4 acc[20];
    for (int l = 0; l < 20; l++) acc[l] = v4(0, 0, 0, 0);
    float wsum = 0.0f, hx = (float)cx + 0.5f, hy = (float)cy + 0.5f;
    for (int b = -1; b <= 1; b++)
        for (int a = -1; a <= 1; a++) {
            int qx = cx + a, qy = cy + b;
            if (qx < 0 || qy < 0 || qx >= W || qy >= H) continue;
            if (a != 0 || b != 0) {
                int nx = mini(maxi((int)rintf(hx + 0.5f * (float)a), 0), W);
                int ny = mini(maxi((int)rintf(hy + 0.5f * (float)b), 0), H);
                if (s->sdf[ny * (W + 1) + nx] < 0.0f) continue;
            }
            float w = K[a + 1] * K[b + 1];
            wsum += w;
            size_t q = (size_t)qy * W + qx;
            for (int l = 0; l < 20; l++)
                if (l != 10) acc[l] = v4add(acc[l], v4mul(w, get_texel(raw, (size_t)l * nc + q)));
        }
    for (int l = 0; l < 20; l++) acc[l] = v4(acc[l].x / wsum, acc[l].y / wsum, acc[l].z / wsum, acc[l].w / wsum);
    {
        float il[3] = {0, 0, 0}, iw = 0.0f;
        for (int a = -14; a <= 14; a++) {
            int qx = cx + a;
            if (qx < 0 || qx >= W) continue;
            float w = o_expf(-0.5f * (float)(a * a) / (6.0f * 6.0f));
            V4 l10 = get_texel(raw, (size_t)10 * nc + (size_t)cy * W + qx);
            il[0] += w * l10.y;
            il[1] += w * l10.z;
            il[2] += w * l10.w;
            iw += w;
        }
        float iv = maxf(iw, 1e-6f);
        acc[9] = v4(il[0] / iv * acc[4].w, il[1] / iv * acc[4].w, il[2] / iv * acc[4].w, acc[9].w);
    }
    size_t i = (size_t)cy * W + cx;
    for (int l = 0; l < 20; l++)
        if (l != 10) put_texel(sm, (size_t)l * nc + i, acc[l]);
}

/* sss.comp: stage 0 prepares layers 22 (E, D) and 23 (s, kind) of co (and 20 in air), stage 1
 * a Jacobi iteration from layer src into the other of 20, 21 (whole grid, read before written) */
static void o_sss(const OSim* s, const uint16_t* raw, uint16_t* co, int stage, int src) {
    const int W = s->W, H = s->H;
    const size_t nc = (size_t)W * H;
    const float KA = -1.0f, KS = -2.0f;
    if (stage == 0) {
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                size_t i = (size_t)y * W + x;
                float occ = get_texel(co, (size_t)4 * nc + i).w;
                int w1 = W + 1, k = y * w1 + x;
                float sdc = 0.25f * (s->sdf[k] + s->sdf[k + 1] + s->sdf[k + w1] + s->sdf[k + w1 + 1]);
                if (sdc < -0.3f) {
                    put_texel(co, (size_t)22 * nc + i, v4(0, 0, 0, 0));
                    put_texel(co, (size_t)23 * nc + i, v4(0, 0, 0, KS));
                    continue;
                }
                if (occ < 0.05f) {
                    V4 r10 = get_texel(raw, (size_t)10 * nc + i);
                    put_texel(co, (size_t)22 * nc + i, v4(r10.y, r10.z, r10.w, 0.0f));
                    put_texel(co, (size_t)23 * nc + i, v4(0, 0, 0, KA));
                    put_texel(co, (size_t)20 * nc + i, v4(r10.y, r10.z, r10.w, 0.0f));
                    continue;
                }
                V4 k19 = get_texel(co, (size_t)19 * nc + i), l9 = get_texel(co, (size_t)9 * nc + i);
                V4 kk = v4(k19.x / occ, k19.y / occ, k19.z / occ, k19.w / occ);
                float lum_a = kk.x * 0.3f + kk.y * 0.45f + kk.z * 0.25f;
                float D = clampf(1.0f / (3.0f * (lum_a + kk.w) + 1e-4f), 0.04f, 1.6f);
                put_texel(co, (size_t)22 * nc + i, v4(l9.x / occ, l9.y / occ, l9.z / occ, D));
                put_texel(co, (size_t)23 * nc + i, v4(kk.x + 0.04f, kk.y + 0.04f, kk.z + 0.04f, occ));
            }
        return;
    }
    int dst = src == 20 ? 21 : 20;
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            size_t i = (size_t)y * W + x;
            V4 kc = get_texel(co, (size_t)23 * nc + i), ec = get_texel(co, (size_t)22 * nc + i);
            if (kc.w < 0.0f) {
                put_texel(co, (size_t)dst * nc + i, kc.w == KA ? v4(ec.x, ec.y, ec.z, 0.0f) : v4(0, 0, 0, 0));
                continue;
            }
            float num[3] = {kc.x * ec.x, kc.y * ec.y, kc.z * ec.z}, den[3] = {kc.x, kc.y, kc.z};
            for (int q = 0; q < 4; q++) {
                int qx = x + (q == 0 ? -1 : q == 1 ? 1 : 0), qy = y + (q == 2 ? -1 : q == 3 ? 1 : 0);
                if (qx < 0 || qy < 0 || qx >= W || qy >= H) continue;
                size_t n = (size_t)qy * W + qx;
                float kind = get_texel(co, (size_t)23 * nc + n).w;
                if (kind == KS) continue;
                float Dn = kind == KA ? ec.w : get_texel(co, (size_t)22 * nc + n).w;
                float Df = 2.0f * ec.w * Dn / maxf(ec.w + Dn, 1e-6f);
                V4 pn = get_texel(co, (size_t)src * nc + n);
                num[0] += Df * pn.x;
                num[1] += Df * pn.y;
                num[2] += Df * pn.z;
                for (int c = 0; c < 3; c++) den[c] += Df;
            }
            put_texel(co, (size_t)dst * nc + i, v4(num[0] / den[0], num[1] / den[1], num[2] / den[2], 0.0f));
        }
}

/* glow.comp: the 2 x 2 means of raw layer 3's emission blurred across into ga, then down into gb */
static void o_glow_pass(const OSim* s, const uint16_t* raw, uint16_t* ga, uint16_t* gb, int dir) {
    const int W = s->W, H = s->H, hw = (W + 1) / 2, hh = (H + 1) / 2;
    const size_t nc = (size_t)W * H;
    for (int hy = 0; hy < hh; hy++)
        for (int hx = 0; hx < hw; hx++) {
            V4 sum = v4(0, 0, 0, 0);
            float norm = 0.0f;
            for (int t = -9; t <= 9; t++) {
                float w = o_expf(-0.5f * (float)(t * t) / (3.0f * 3.0f));
                norm += w;
                int qx = hx + (dir == 0 ? t : 0), qy = hy + (dir == 0 ? 0 : t);
                if (qx < 0 || qy < 0 || qx >= hw || qy >= hh) continue;
                V4 v;
                if (dir == 0) {
                    V4 sm = v4(0, 0, 0, 0);
                    for (int j = 0; j < 2; j++)
                        for (int i = 0; i < 2; i++) {
                            int cx = 2 * qx + i, cy = 2 * qy + j;
                            if (cx >= W || cy >= H) continue;
                            V4 e = get_texel(raw, (size_t)3 * nc + (size_t)cy * W + cx);
                            sm = v4add(sm, v4(e.x, e.y, e.z, 0.0f));
                        }
                    v = v4mul(0.25f, sm);
                } else {
                    v = get_texel(ga, (size_t)qy * hw + qx);
                }
                sum = v4add(sum, v4mul(w, v));
            }
            sum = v4(sum.x / norm, sum.y / norm, sum.z / norm, sum.w / norm);
            put_texel(dir == 0 ? ga : gb, (size_t)hy * hw + hx, sum);
        }
}

/* The passes over the oracle's current grid: raw holds 20 x W x H texels of four half words,
 * smooth 24 (layer-major; its layer 10 is left as it was, its layer 20 is the warm start of
 * sss.comp), ga and gb ceil(W / 2) x ceil(H / 2). */
long osim_render(const OSim* s, const void* optics, float inv_speed, int sss_iters, uint16_t* raw, uint16_t* smooth,
                 uint16_t* ga, uint16_t* gb) {
    const OOptics* opt = (const OOptics*)optics;
    float gap, mc;
    o_spike_params(s, &gap, &mc);
    /* the last frame's dust field, once the pool has run (mod.rs:1653) */
    float dust = (s->d_seen && s->has_dust && s->dfield) ? 1.0f : 0.0f;
    for (int y = 0; y < s->H; y++)
        for (int x = 0; x < s->W; x++) o_cell_optics(s, opt, inv_speed, gap, mc, s->dfield, dust, x, y, raw);
    o_light(s, raw);
    for (int y = 0; y < s->H; y++)
        for (int x = 0; x < s->W; x++) o_optics_blur(s, raw, smooth, x, y);
    int iters = (sss_iters + 1) / 2 * 2;
    if (iters > 0) {
        o_sss(s, raw, smooth, 0, 20);
        for (int k = 0; k < iters; k++) o_sss(s, raw, smooth, 1, k % 2 == 0 ? 20 : 21);
    }
    o_glow_pass(s, raw, ga, gb, 0);
    o_glow_pass(s, raw, ga, gb, 1);
    return 0;
}

/* flow_map.comp:54-72 on every cell of the grid: the displacement carried by the smoothed
 * velocity (layer 7 zw over the occupancy of layer 4 w, capped at SPEED_MAX = 30 cells/s) from
 * copy `src` of the map into the other, grown by u dt; each pair restarted (zero) when
 * floor(now / period + o) changed over the step (o = 0 for xy, 0.5 for zw). Periods
 * FLOW_PERIOD_SHORT = 4 s and FLOW_PERIOD_LONG = 12 s (mod.rs:431-432). sample_at
 * (flow_map.comp:41-50): bilinear at a cell-centred position, clamped to the grid. */
long osim_flow_map(const OSim* s, const uint16_t* smooth, uint16_t* flow, float dt, float now, uint32_t src) {
    const size_t nc = (size_t)s->W * s->H;
    const int sl = 2 * (int)src, dl = 2 * (1 - (int)src);
    for (int cy = 0; cy < s->H; cy++)
        for (int cx = 0; cx < s->W; cx++) {
            const size_t i = (size_t)cy * s->W + cx;
            float occ = get_texel(smooth, 4 * nc + i).w;
            V2 u = v2(0.0f, 0.0f);
            if (occ > 0.02f) {
                V4 v = get_texel(smooth, 7 * nc + i);
                u = v2(v.z / occ, v.w / occ);
            }
            float sp = len2(u);
            if (sp > 30.0f) {
                float k = 30.0f / sp;
                u = v2(u.x * k, u.y * k);
            }
            V2 from = v2(((float)cx + 0.5f) - u.x * dt, ((float)cy + 0.5f) - u.y * dt);
            V2 q = v2(clampf(from.x - 0.5f, 0.0f, (float)(s->W - 1)), clampf(from.y - 0.5f, 0.0f, (float)(s->H - 1)));
            int i0x = q.x == q.x ? (int)floorf(q.x) : 0, i0y = q.y == q.y ? (int)floorf(q.y) : 0;
            int i1x = mini(i0x + 1, s->W - 1), i1y = mini(i0y + 1, s->H - 1);
            V2 f = v2(q.x - (float)i0x, q.y - (float)i0y);
            for (int k = 0; k < 2; k++) {
                float period = k == 0 ? 4.0f : 12.0f;
                const uint16_t* L = flow + 4 * (size_t)(sl + k) * nc;
                V4 a = v4mix(get_texel(L, (size_t)i0y * s->W + i0x), get_texel(L, (size_t)i0y * s->W + i1x), f.x);
                V4 b = v4mix(get_texel(L, (size_t)i1y * s->W + i0x), get_texel(L, (size_t)i1y * s->W + i1x), f.x);
                V4 sa = v4mix(a, b, f.y);
                V4 d = v4(sa.x + u.x * dt, sa.y + u.y * dt, sa.z + u.x * dt, sa.w + u.y * dt);
                if (floorf(now / period + 0.0f) != floorf((now - dt) / period + 0.0f)) d.x = d.y = 0.0f;
                if (floorf(now / period + 0.5f) != floorf((now - dt) / period + 0.5f)) d.z = d.w = 0.0f;
                put_texel(flow + 4 * (size_t)(dl + k) * nc, i, d);
            }
        }
    return 0;
}

/* spray.comp (main 171-494; mod.rs:1739-1773): bubbles, foam and spray in a pool of 65536.
 * Stage 0 (make, per cell) where liquid traps air, folds in, crests, or fizzes; stage 1 (move,
 * per entry) as bubble, foam or spray, the foam counted per cell, the live entries listed.
 * The pool is handed out in one deterministic order the reference's atomics allow: the
 * frame's emissions ranked by cell and by their order in it take the free stack's top first,
 * then unused entries; freed entries go onto the stack, and live ones into the list, in entry
 * order. Not restated: the specks (not carried) and a droplet's splat into the film map's
 * intake (film_lay.glsl; no film map): the droplet is removed as the reference removes it. */
typedef struct ODiffuse { float px, py, vx, vy, life, r; uint32_t info; float z; } ODiffuse;
#define D_MAX 65536u       /* DIFFUSE_MAX */
#define D_DUST 131072u     /* DUST_MAX */
#define D_POOL (D_MAX + D_DUST)
static int d_alloc(OSim* s) {
    if (s->dpool) return 0;
    const size_t nc = (size_t)s->W * s->H;
    s->dpool = (ODiffuse*)calloc(D_POOL, sizeof(ODiffuse));
    s->dstack = (uint32_t*)calloc(D_MAX, sizeof(uint32_t));
    s->dstack1 = (uint32_t*)calloc(D_DUST, sizeof(uint32_t));
    s->dlist = (uint32_t*)calloc(D_POOL, sizeof(uint32_t));
    s->dcount = (uint32_t*)calloc(4 * nc, sizeof(uint32_t));
    s->dfield = (int32_t*)calloc(4 * nc, sizeof(int32_t));
    return (s->dpool && s->dstack && s->dstack1 && s->dlist && s->dcount && s->dfield) ? 0 : -2;
}
void osim_set_dust(OSim* s, int has_dust) { s->has_dust = has_dust; }
enum { D_FREE = 0, D_BUBBLE = 1, D_FOAM = 2, D_SPRAY = 3 };
static float d_rnd(uint32_t h) { return (float)(h >> 8) / 16777216.0f; }
static float d_ramp(float x, float lo, float hi) { return clampf((x - lo) / (hi - lo), 0.0f, 1.0f); }
static float d_occ_cell(const OSim* s, int x, int y) {
    if (x < 0 || y < 0 || x >= s->W || y >= s->H) return 0.0f;
    return clampf(s->cell[y * s->W + x].x, 0.0f, 1.5f);
}
static float d_occ_at(const OSim* s, float px, float py) {
    float gx = px - 0.5f, gy = py - 0.5f;
    int bx = (int)floorf(gx), by = (int)floorf(gy);
    float fx = gx - (float)bx, fy = gy - (float)by;
    return mixf(mixf(d_occ_cell(s, bx, by), d_occ_cell(s, bx + 1, by), fx),
                mixf(d_occ_cell(s, bx, by + 1), d_occ_cell(s, bx + 1, by + 1), fx), fy);
}
static V2 d_centre_vel(const OSim* s, int i) {
    int n = s->W * s->H;
    V4 v = s->vel[i];
    float ux = face_live(v.z) ? v.x : 0.0f, uy = face_live(v.w) ? v.y : 0.0f;
    V4 vr = s->vel[mini(i + 1, n - 1)], vt = s->vel[mini(i + s->W, n - 1)];
    return v2(0.5f * (ux + (face_live(vr.z) ? vr.x : 0.0f)), 0.5f * (uy + (face_live(vt.w) ? vt.y : 0.0f)));
}
/* air.glsl sample_vel at an entry: a face's cell by its linear index, zeros off the buffer */
static V4 d_vel_lin(const OSim* s, int x, int y) {
    long long k = (long long)y * s->W + x;
    return (k >= 0 && k < (long long)s->W * s->H) ? s->vel[k] : v4(0.0f, 0.0f, 0.0f, 0.0f);
}
static V2 d_sample_vel_fb(const OSim* s, float x, float y, V2 fb) {
    float o[2] = {fb.x, fb.y};
    for (int comp = 0; comp < 2; comp++) {
        float gx = comp == 0 ? x : x - 0.5f, gy = comp == 0 ? y - 0.5f : y;
        int bx = (int)floorf(gx), by = (int)floorf(gy);
        float fx = gx - (float)bx, fy = gy - (float)by;
        float sw = 0.0f, su = 0.0f;
        for (int b = 0; b < 2; b++)
            for (int a = 0; a < 2; a++) {
                V4 q = d_vel_lin(s, bx + a, by + b);
                if (face_live(comp == 0 ? q.z : q.w)) {
                    float wt = (a == 0 ? 1.0f - fx : fx) * (b == 0 ? 1.0f - fy : fy);
                    sw += wt;
                    su += wt * (comp == 0 ? q.x : q.y);
                }
            }
        if (sw > 1e-3f) o[comp] = su / sw;
    }
    return v2(o[0], o[1]);
}
static float d_crowd(const OSim* s, int x, int y, uint32_t copy) {
    x = clampi(x, 0, s->W - 1);
    y = clampi(y, 0, s->H - 1);
    return (float)s->dcount[(size_t)copy * s->W * s->H + (size_t)y * s->W + x];
}
static int d_dominant_row(const OSim* s, int i) {
    int k = i * s->tank.stride, cw = s->acc[k + 4];
    if (cw <= 0) return -1;
    int others = 0;
    for (int j = 0; j < P_.n_present; j++) {
        int ch = s->mats[P_.present[j]].ia[2];
        if (ch >= 0) others += s->acc[k + ch];
    }
    int best = -1, bw = 0;
    for (int j = 0; j < P_.n_present; j++) {
        int r = P_.present[j];
        const int* ia = s->mats[r].ia;
        if (ia[2] < 0 && P_.primary >= 0 && r != P_.primary) continue;
        int w = ia[2] >= 0 ? s->acc[k + ia[2]] : maxi(cw - others, 0);
        if (w > bw) {
            bw = w;
            best = r;
        }
    }
    return best;
}
static ODiffuse d_bubble(int cx, int cy, uint32_t h, int k, float r0, uint32_t grows, float ux, float uy, float spread,
                         int row) {
    uint32_t hk = hash32(h + (uint32_t)k * 0x9e3779b9u);
    ODiffuse e;
    e.px = (float)cx + d_rnd(hk);
    e.py = (float)cy + d_rnd(hash32(hk ^ 0x51ed270bu));
    float a = 6.2831853f * d_rnd(hash32(hk ^ 0x2545f491u));
    float sn, cs;
    o_sincos(a, &sn, &cs);
    float j = d_rnd(hash32(hk ^ 0x27d4eb2fu));
    e.vx = ux + spread * cs * j;
    e.vy = uy + spread * sn * j;
    float sr = d_rnd(hash32(hk ^ 0x165667b1u));
    e.r = r0 * (0.45f + 1.1f * sr * sr);
    e.info = (uint32_t)D_BUBBLE | grows | ((uint32_t)(row + 1) << 8) | (hash32(hk ^ 0x68e31da4u) & 0xffff8000u);
    e.life = 40.0f;
    e.z = d_rnd(hash32(hk ^ 0xb5297a4du));
    return e;
}
static int d_take(const OSim* s, uint32_t r, uint32_t top0, uint32_t hw0) {
    if (r < top0) return (int)s->dstack[top0 - 1u - r];
    uint32_t hw = hw0 + (r - top0);
    return hw < D_MAX ? (int)hw : -1;
}
/* make(): the cell's emissions, each into the slot of its rank (from *rank on) */
static void d_make(OSim* s, const uint16_t* sm, int cx, int cy, float dt, float amount, uint32_t* rank, uint32_t top0,
                   uint32_t hw0) {
    const size_t nc = (size_t)s->W * s->H;
    int W = s->W, H = s->H, i = cy * W + cx;
    float occ = d_occ_cell(s, cx, cy);
    if (occ < 0.08f) return;
    V4 l4 = get_texel(sm, 4 * nc + i);
    if (l4.w < 0.02f) return;
    float foam_k = l4.y / l4.w;
    float fizz = get_texel(sm, 16 * nc + i).y / l4.w;
    float cs = P_.misc[2];
    V2 u = d_centre_vel(s, i);
    float ta = 0.0f, gx = 0.0f, gy = 0.0f;
    for (int q = 0; q < 4; q++) {
        int dx = q == 0 ? -1 : q == 1 ? 1 : 0, dy = q == 2 ? -1 : q == 3 ? 1 : 0;
        int nx = cx + dx, ny = cy + dy;
        float on = d_occ_cell(s, nx, ny);
        gx += (float)dx * on;
        gy += (float)dy * on;
        if (on < 0.08f || nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
        V2 un = d_centre_vel(s, ny * W + nx);
        float dvx = u.x - un.x, dvy = u.y - un.y;
        float m = len2(v2(dvx, dvy));
        if (m < 1e-4f) continue;
        ta += m * (1.0f - (dvx / m * -(float)dx + dvy / m * -(float)dy));
    }
    float ul = len2(u);
    float speed = ul * cs;
    float energy = d_ramp(speed, 0.6f, 3.0f), trapped = d_ramp(ta * cs, 1.0f, 5.0f);
    float g = len2(v2(gx, gy));
    float crest = 0.0f, plunge = 0.0f;
    if (g > 0.15f && speed > 0.05f) {
        float nox = -gx / g, noy = -gy / g;
        float along = u.x / ul * nox + u.y / ul * noy;
        crest = d_ramp(along, 0.6f, 0.95f) * d_ramp(speed, 1.0f, 3.5f);
        plunge = d_ramp(-along, 0.4f, 0.9f) * d_ramp(speed, 0.08f, 1.2f) * smoothstepf(0.15f, 0.6f, g);
    }
    float tension = maxf(s->sprop[i].x, 0.0f) * cs * cs * cs / 7.2e-5f;
    float r0 = clampf(1.2e-3f * sqrtf(clampf(tension, 0.05f, 4.0f)) / cs, 0.03f, 0.4f);
    uint32_t h = hash32((uint32_t)i * 0x85ebca6bu ^ hash32(s->frame * 0x9e3779b1u + 0x3c6ef372u));
    float rate = amount * (40.0f * trapped * energy + 30.0f * plunge + 25.0f * crest * foam_k);
    float fn = floorf(rate * dt + d_rnd(h));
    int n = fn >= 6.0f ? 6 : (fn >= 1.0f ? (int)fn : 0);
    int row = (n > 0 || fizz > 0.0f) ? d_dominant_row(s, i) : -1;
    for (int k = 0; k < n; k++) {
        int slot = d_take(s, (*rank)++, top0, hw0);
        if (slot >= 0) s->dpool[slot] = d_bubble(cx, cy, h, k, r0, 0u, u.x, u.y, 0.3f * ul, row);
    }
    if (fizz > 0.0f) {
        int w1 = W + 1, kk = cy * w1 + cx;
        float sd = 0.25f * (s->sdf[kk] + s->sdf[kk + 1] + s->sdf[kk + w1] + s->sdf[kk + w1 + 1]);
        float wall = 1.0f - d_ramp(sd, 0.5f, 2.0f);
        float fr = amount * 1.6f * fizz * minf(occ, 1.0f) * (1.0f + 5.0f * wall);
        uint32_t h2 = hash32(h ^ 0x7feb352du);
        float ff = floorf(fr * dt + d_rnd(h2));
        int nf = ff >= 2.0f ? 2 : (ff >= 1.0f ? (int)ff : 0);
        float r0f = clampf(0.25e-3f / cs, 0.02f, 0.2f);
        for (int k = 0; k < nf; k++) {
            int slot = d_take(s, (*rank)++, top0, hw0);
            if (slot >= 0) s->dpool[slot] = d_bubble(cx, cy, h2, k, r0f, 4u, u.x, u.y, 0.0f, row);
        }
    }
}
/* hemi-octahedral flake normals (look.comp pack_n, spray.comp unpack_n) */
static uint32_t d_quant10(float v, uint32_t h) {
    const float m = 1023.0f;
    return (uint32_t)clampf(floorf(clampf(v, 0.0f, 1.0f) * m + d_rnd(h)), 0.0f, m);
}
static uint32_t d_pack_n(float nx, float ny, float nz, uint32_t h) {
    if (nz < 0.0f) {
        nx = -nx;
        ny = -ny;
        nz = -nz;
    }
    float den = maxf(fabsf(nx) + fabsf(ny) + nz, 1e-6f);
    float px = nx / den, py = ny / den;
    float qx = (px + py) * 0.5f + 0.5f, qy = (px - py) * 0.5f + 0.5f;
    return d_quant10(qx, hash32(h)) | (d_quant10(qy, hash32(h ^ 0x68e31da4u)) << 10);
}
static void d_normalize3(float* x, float* y, float* z) {
    float l = sqrtf(*x * *x + *y * *y + *z * *z);
    *x = *x / l;
    *y = *y / l;
    *z = *z / l;
}
static void d_unpack_n(uint32_t b, float* x, float* y, float* z) {
    float qx = (float)(b & 1023u) / 1023.0f * 2.0f - 1.0f, qy = (float)((b >> 10) & 1023u) / 1023.0f * 2.0f - 1.0f;
    *x = (qx + qy) * 0.5f;
    *y = (qx - qy) * 0.5f;
    *z = maxf(1.0f - fabsf(*x) - fabsf(*y), 0.0f);
    d_normalize3(x, y, z);
}
/* spray.comp move_dust (lines 272-367): a speck suspended, resting or falling; resting ones
 * counted per cell (copies 2, 3), its share of the colour into the dust field */
static int d_move_dust(OSim* s, const OOptics* opt, uint32_t i, float dt) {
    const size_t nc = (size_t)s->W * s->H;
    ODiffuse e = s->dpool[i];
    uint32_t st = e.info & 3u;
    int W = s->W, H = s->H;
    uint32_t copy_in = 1u - s->d_parity, copy_out = s->d_parity;
    int row = (int)((e.info >> 8) & 127u) - 1;
    if (row < 0) {
        s->dpool[i].info = 0u;
        return 1;
    }
    const OOptics* o = &opt[row];
    float rho_p = o->dust2[1] / 998.0f;
    float aspect = o->dust2[2];
    float rr = e.r;
    float d_eq = 2.0f * rr * (aspect < 0.6667f ? o_powf(1.5f * maxf(aspect, 0.005f), 1.0f / 3.0f) : 1.0f);
    float pack = maxf(o->dcol[3], 1.0f);
    float Bc = (aspect * aspect - 1.0f) / (aspect * aspect + 1.0f);
    float nx, ny, nz;
    uint32_t lb;
    memcpy(&lb, &e.life, 4);
    d_unpack_n(lb, &nx, &ny, &nz);
    uint32_t h0 = hash32(e.info ^ hash32(s->frame * 0x9e3779b1u + i));
    float sf = ceilf(dt * 120.0f);
    int steps = sf >= 8.0f ? 8 : (sf >= 1.0f ? (int)sf : 1);
    float h = dt / (float)steps;
    for (int k = 0; k < steps && st != D_FREE; k++) {
        int cx = clampi((int)e.px, 0, W - 1), cy = clampi((int)e.py, 0, H - 1), ci = cy * W + cx;
        float occ = d_occ_at(s, e.px, e.py);
        V4 cf = s->cell[ci];
        float rho = maxf(cf.y, 0.3f), nu = maxf(cf.z / rho, 1e-6f);
        float drho = rho_p - rho;
        float down = drho >= 0.0f ? 1.0f : -1.0f;
        float ux_ = e.px - 0.0f, uy_ = e.py - down * (rr + 0.35f);
        V2 gu;
        float sd_u = sample_sdf(s, v2(ux_, uy_), &gu);
        int cux = clampi((int)ux_, 0, W - 1), cuy = clampi((int)uy_, 0, H - 1);
        float packed = (float)s->dcount[(size_t)(2u + copy_in) * nc + (size_t)cuy * W + cux];
        int held = sd_u < 0.0f || ((cux != cx || cuy != cy) && packed >= pack) || uy_ < 0.0f;
        int wet = occ > 0.30f;
        V2 uf = d_sample_vel_fb(s, e.px, e.py, v2(0.0f, 0.0f));
        float u_crit = 8.0f * sqrtf(0.05f * fabsf(drho) * P_.gravity * d_eq / rho);
        if (st == D_FOAM) {
            if (!held) st = wet ? D_BUBBLE : D_SPRAY;
            else if (wet && len2(uf) > u_crit) {
                st = D_BUBBLE;
                e.vx = uf.x;
                e.vy = uf.y;
            } else {
                float bx = 0.0f, by = 1.0f, bz = 0.0f;
                if (sd_u < 0.0f) {
                    bx = gu.x + 0.0f;
                    by = gu.y + 1e-4f;
                    float l = sqrtf(bx * bx + by * by);
                    bx = bx / l;
                    by = by / l;
                }
                float sg = signf(nx * bx + ny * by + nz * bz + 1e-4f);
                float t = 1.0f - o_expf(-h / 0.3f);
                nx = mixf(nx, bx * sg, t);
                ny = mixf(ny, by * sg, t);
                nz = mixf(nz, bz * sg, t);
                d_normalize3(&nx, &ny, &nz);
                e.vx = wet ? 0.0f : e.vx + h;
                e.vy = 0.0f;
                if (e.vx > 30.0f) st = D_FREE;
                continue;
            }
        }
        if (st == D_SPRAY && wet) st = D_BUBBLE;
        if (st == D_BUBBLE && !wet) st = D_SPRAY;
        if (st == D_BUBBLE) {
            float vt = terminal(s, drho, rho, nu, d_eq);
            float tx = uf.x - 0.0f, ty = uf.y - down * vt;
            float tau = clampf(rho_p * d_eq * d_eq / (18.0f * rho * nu), 0.004f, 0.5f);
            float t = 1.0f - o_expf(-h / tau);
            e.vx = mixf(e.vx, tx, t);
            e.vy = mixf(e.vy, ty, t);
            if (aspect < 0.6667f) {
                V2 ux1 = d_sample_vel_fb(s, e.px + 0.5f, e.py + 0.0f, uf), ux0 = d_sample_vel_fb(s, e.px - 0.5f, e.py - 0.0f, uf);
                V2 uy1 = d_sample_vel_fb(s, e.px + 0.0f, e.py + 0.5f, uf), uy0 = d_sample_vel_fb(s, e.px - 0.0f, e.py - 0.5f, uf);
                float gxx = ux1.x - ux0.x, gxy = ux1.y - ux0.y, gyx = uy1.x - uy0.x, gyy = uy1.y - uy0.y;
                float w = 0.5f * (gxy - gyx);
                float dv = 0.5f * (gxx + gyy);
                float exx = gxx - dv, eyy = gyy - dv, exy = 0.5f * (gyx + gxy);
                float wnx = -w * ny, wny = w * nx, wnz = 0.0f;
                float enx = exx * nx + exy * ny, eny = exy * nx + eyy * ny, enz = 0.0f;
                float ne = nx * enx + ny * eny + nz * enz;
                nx = nx + h * (wnx + Bc * (enx - ne * nx));
                ny = ny + h * (wny + Bc * (eny - ne * ny));
                nz = nz + h * (wnz + Bc * (enz - ne * nz));
                d_normalize3(&nx, &ny, &nz);
            }
            if (held && (e.vx - uf.x) * 0.0f + (e.vy - uf.y) * -down >= 0.0f && len2(uf) < u_crit) {
                st = D_FOAM;
                e.vx = 0.0f;
                e.vy = 0.0f;
            }
        } else if (st == D_SPRAY) {
            e.vx += 0.0f - e.vx * 1.2f * h;
            e.vy += -P_.gravity * h - e.vy * 1.2f * h;
        }
        e.px += e.vx * h;
        e.py += e.vy * h;
        V2 gs;
        float sd = sample_sdf(s, v2(e.px, e.py), &gs);
        float rim = rr + 0.05f;
        if (sd < rim) {
            float gl = maxf(len2(gs), 1e-6f);
            float nrx = gs.x / gl, nry = gs.y / gl;
            e.px += nrx * (rim - sd);
            e.py += nry * (rim - sd);
            float vn = minf(e.vx * nrx + e.vy * nry, 0.0f);
            e.vx -= nrx * vn;
            e.vy -= nry * vn;
            if (st == D_SPRAY) {
                st = D_FOAM;
                e.vx = 0.0f;
                e.vy = 0.0f;
            }
        }
        if (e.px < 0.0f || e.py < -1.0f || e.px >= (float)W || e.py >= (float)H) st = D_FREE;
    }
    uint32_t nb = d_pack_n(nx, ny, nz, h0);
    memcpy(&e.life, &nb, 4);
    e.info = (e.info & ~3u) | st;
    s->dpool[i] = e;
    if (st == D_FREE) return 1;
    int cx = clampi((int)e.px, 0, W - 1), cy = clampi((int)e.py, 0, H - 1), ci = cy * W + cx;
    if (st == D_FOAM) s->dcount[(size_t)(2u + copy_out) * nc + ci] += 1u;
    if (o->dust[3] > 0.0f && d_occ_cell(s, cx, cy) > 0.05f) {
        int qx = (int)(o->dust[0] * 1024.0f + 0.5f), qy = (int)(o->dust[1] * 1024.0f + 0.5f);
        int qz = (int)(o->dust[2] * 1024.0f + 0.5f), qw = (int)(o->dust[3] * 1024.0f + 0.5f);
        if (qx > 0) s->dfield[4 * ci] += qx;
        if (qy > 0) s->dfield[4 * ci + 1] += qy;
        if (qz > 0) s->dfield[4 * ci + 2] += qz;
        s->dfield[4 * ci + 3] += qw;
    }
    return 2;
}
/* move(): entry i; 0 nothing, 1 freed, 2 live */
static int d_move(OSim* s, const uint16_t* sm, const OOptics* opt, uint32_t i, float dt) {
    const size_t nc = (size_t)s->W * s->H;
    ODiffuse e = s->dpool[i];
    uint32_t st = e.info & 3u;
    if (st == D_FREE) return 0;
    if ((e.info & 8u) != 0u) return d_move_dust(s, opt, i, dt);
    int W = s->W, H = s->H;
    uint32_t copy_in = 1u - s->d_parity, copy_out = s->d_parity;
    float cs = P_.misc[2];
    float sf = ceilf(dt * 120.0f);
    int steps = sf >= 8.0f ? 8 : (sf >= 1.0f ? (int)sf : 1);
    float h = dt / (float)steps;
    for (int k = 0; k < steps && st != D_FREE; k++) {
        int cx = clampi((int)e.px, 0, W - 1), cy = clampi((int)e.py, 0, H - 1), ci = cy * W + cx;
        float occ = d_occ_at(s, e.px, e.py);
        V2 uf = d_sample_vel_fb(s, e.px, e.py, v2(0.0f, 0.0f));
        float crowd = d_crowd(s, cx, cy, copy_in);
        float gcx = d_crowd(s, cx + 1, cy, copy_in) - d_crowd(s, cx - 1, cy, copy_in);
        float gcy = d_crowd(s, cx, cy + 1, copy_in) - d_crowd(s, cx, cy - 1, copy_in);
        uint32_t want = occ > 0.62f ? D_BUBBLE : (occ + 0.06f * crowd > 0.10f ? D_FOAM : D_SPRAY);
        V4 l4 = get_texel(sm, 4 * nc + ci);
        float wl = maxf(l4.w, 1e-3f);
        if (want != st) {
            if (want == D_FOAM || (want == D_BUBBLE && st == D_SPRAY)) {
                float foam_k = l4.w > 0.02f ? l4.y / wl : 0.0f;
                float froth = l4.w > 0.02f ? get_texel(sm, 16 * nc + ci).x / wl : 0.0f;
                if (st == D_SPRAY && foam_k < 0.05f) { st = D_FREE; break; }
                if (want == D_FOAM && st == D_BUBBLE && (crowd > 5.0f || foam_k < 0.05f)) { st = D_FREE; break; }
                if (want == D_FOAM) {
                    e.life = maxf(froth, 0.05f) * (0.5f + d_rnd(hash32(e.info ^ (uint32_t)k)));
                    e.z = e.life;
                }
                if (want == D_BUBBLE) e.life = 40.0f;
            }
            if (want == D_SPRAY) e.life = minf(e.life, 1.5f);
            if (want == D_BUBBLE && st == D_FOAM) e.z = d_rnd(hash32(e.info ^ 0xb5297a4du));
            st = want;
        }
        float tx, ty, tau;
        if (st == D_BUBBLE) {
            V4 cf = s->cell[ci];
            float rho = maxf(cf.y, 0.3f), nu = maxf(cf.z / rho, 1e-6f);
            float vt = terminal(s, rho, rho, nu, 2.0f * e.r);
            tx = uf.x + 0.0f;
            ty = uf.y + vt;
            tau = 0.03f;
            if ((e.info & 4u) != 0u) e.r = minf(e.r + 0.5e-3f / cs * h, 0.35f);
            e.life -= h;
        } else if (st == D_FOAM) {
            float sub = clampf(occ * 2.0f, 0.0f, 1.0f);
            tx = uf.x * sub;
            ty = uf.y * sub;
            float below = d_occ_at(s, e.px - 0.0f, e.py - 0.7f) + 0.25f * d_crowd(s, cx, cy - 1, copy_in);
            int held = occ > 0.25f || below > 0.45f;
            float push = d_ramp(crowd, 2.0f * 0.7f, 2.0f * 2.0f);
            float gl = len2(v2(gcx, gcy));
            if (gl > 1e-3f) {
                float spx = -gcx / gl * 6.0f * push, spy = -gcy / gl * 6.0f * push;
                if (!held) spy = minf(spy, 0.0f);
                tx += spx;
                ty += spy;
            }
            ty -= held ? 1.5f * (1.0f - d_ramp(occ, 0.1f, 0.4f)) : 8.0f;
            if (occ > 0.45f) ty += 4.0f * (occ - 0.45f);
            tau = 0.06f;
            e.life -= h * (crowd < 2.0f ? 2.5f : 1.0f);
        } else {
            tx = e.vx + 0.0f - e.vx * 1.2f * h;
            ty = e.vy + -P_.gravity * h - e.vy * 1.2f * h;
            tau = 0.0f;
            e.life -= h;
        }
        if (tau > 0.0f) {
            float t = 1.0f - o_expf(-h / tau);
            e.vx = mixf(e.vx, tx, t);
            e.vy = mixf(e.vy, ty, t);
        } else {
            e.vx = tx;
            e.vy = ty;
        }
        e.px += e.vx * h;
        e.py += e.vy * h;
        V2 gs;
        float sd = sample_sdf(s, v2(e.px, e.py), &gs);
        float rim = e.r + 0.1f;
        int drow = (int)((e.info >> 8) & 127u) - 1;
        if (st == D_SPRAY && sd < rim && drow >= 0) { st = D_FREE; break; }
        if (sd < rim) {
            float gl = maxf(len2(gs), 1e-6f);
            float nx = gs.x / gl, ny = gs.y / gl;
            e.px += nx * (rim - sd);
            e.py += ny * (rim - sd);
            float vn = minf(e.vx * nx + e.vy * ny, 0.0f);
            e.vx -= nx * vn;
            e.vy -= ny * vn;
        }
        if (e.life <= 0.0f || e.px < 0.0f || e.py < 0.0f || e.px >= (float)W || e.py >= (float)H) st = D_FREE;
    }
    e.info = (e.info & ~3u) | st;
    s->dpool[i] = e;
    if (st == D_FREE) return 1;
    if (st == D_FOAM) {
        int cx = clampi((int)e.px, 0, W - 1), cy = clampi((int)e.py, 0, H - 1);
        s->dcount[(size_t)copy_out * nc + (size_t)cy * W + cx] += 1u;
    }
    return 2;
}
/* record_spray: once a liquid that foams or fizzes (optics sty.y, fx2.y) has been in the tank
 * with bubbles on: the foam counts of this frame's copy cleared, stage 0 when one is and
 * dt > 0, stage 1, the copies swapped. The smoothed layers are osim_render's. */
long osim_spray(OSim* s, const uint16_t* smooth, const void* optics, float dt, float amount) {
    const size_t nc = (size_t)s->W * s->H;
    const OOptics* opt = (const OOptics*)optics;
    int makes = 0;
    if (amount > 0.0f)
        for (int k = 0; k < s->tank.nrows; k++) {
            const OOptics* o = &opt[s->tank.rows[k]];
            if (o->sty[1] > 0.0f || o->fx2[1] > 0.0f) makes = 1;
        }
    if (makes || s->has_dust) s->d_seen = 1;
    if (!s->d_seen) return 0;
    if (d_alloc(s)) return -2;
    memset(s->dcount + (size_t)s->d_parity * nc, 0, nc * sizeof(uint32_t));
    memset(s->dcount + (size_t)(2 + s->d_parity) * nc, 0, nc * sizeof(uint32_t));
    memset(s->dfield, 0, 4 * nc * sizeof(int32_t));
    if (makes && dt > 0.0f) {
        uint32_t rank = 0, top0 = s->d_top, hw0 = s->d_hw;
        for (int cy = 0; cy < s->H; cy++)
            for (int cx = 0; cx < s->W; cx++) d_make(s, smooth, cx, cy, dt, amount, &rank, top0, hw0);
        s->d_top = rank < top0 ? top0 - rank : 0u;
        s->d_hw += rank > top0 ? rank - top0 : 0u;
    }
    uint32_t listed = 0;
    for (uint32_t i = 0; i < D_POOL; i++) {
        int f = d_move(s, smooth, opt, i, dt);
        if (f == 1) {
            if (i < D_MAX) s->dstack[s->d_top++] = i;
            else s->dstack1[s->d_top1++] = i;
        } else if (f == 2) s->dlist[listed++] = i;
    }
    s->d_listed = listed;
    s->d_parity ^= 1u;
    return (long)listed;
}
/* The pool (196608 entries of 8 words), its free stacks and list, the counts (foam x 2,
 * resting specks x 2, W x H each) and the counters (bubbles never handed out, their stack's
 * height, listed, the copy counted next, specks never handed out, their stack's height). */
long osim_spray_state(const OSim* s, void* pool, uint32_t* stack, uint32_t* stack1, uint32_t* list, uint32_t* counts,
                      uint32_t state[8]) {
    state[0] = s->d_hw;
    state[1] = s->d_top;
    state[2] = s->d_listed;
    state[3] = s->d_parity;
    state[4] = s->d_hw1;
    state[5] = s->d_top1;
    state[6] = state[7] = 0u;
    if (!s->dpool) return 0;
    if (pool) memcpy(pool, s->dpool, D_POOL * sizeof(ODiffuse));
    if (stack) memcpy(stack, s->dstack, (size_t)s->d_top * 4);
    if (stack1) memcpy(stack1, s->dstack1, (size_t)s->d_top1 * 4);
    if (list) memcpy(list, s->dlist, (size_t)s->d_listed * 4);
    if (counts) memcpy(counts, s->dcount, 4 * (size_t)s->W * s->H * 4);
    return 1;
}

/* look.comp (main, 93-171) over the particle slots in order, from the optics table `optics`,
 * FluidSim's frame counter and `dt`, the simulated time since the last optics call: the
 * second moment A of the platelets' normals of each particle of a liquid with platelets,
 * Jeffery's equation with the quadratic closure on the shear part of its APIC gradient, in
 * sub = clamp(ceil(rate dt / 0.15), 1, 8) steps, then rotational diffusion (mix towards I / 3
 * by 1 - exp(-6 Dr dt)), kept at 10 bits each rounded stochastically (quant, pack_a); a slot
 * whose stored id differs holds a new particle, which starts at I / 3. The listed slots (in
 * slot order) go to `list` (at most `cap`); returns how many were listed. The specks' part
 * (a new particle's specks into spray.comp's pool) is not restated: no pool (dust_cap 0). */
static float o_rnd24(uint32_t h) { return (float)(h >> 8) / 16777216.0f; }
static uint32_t o_quant10(float v, uint32_t h) {
    const float m = 1023.0f;
    return (uint32_t)clampf(floorf(clampf(v, 0.0f, 1.0f) * m + o_rnd24(h)), 0.0f, m);
}
static uint32_t o_pack_a(float ax, float ay, float az, uint32_t h) {
    return o_quant10(ax, hash32(h ^ 0x1b873593u)) | (o_quant10(ay, hash32(h ^ 0xcc9e2d51u)) << 10) |
           (o_quant10(az + 0.5f, hash32(h ^ 0xe6546b64u)) << 20);
}
long osim_look(OSim* s, const void* optics, float dt, uint32_t* list, uint32_t cap) {
    const OOptics* opt = (const OOptics*)optics;
    if (!s->plook) {
        s->plook = (uint32_t*)calloc((size_t)s->capacity * 4, sizeof(uint32_t));
        if (!s->plook) return -2;
    }
    if (s->has_dust && d_alloc(s)) return -2;
    long listed = 0;
    const float third = 1.0f / 3.0f;
    uint32_t speck_rank = 0, top1 = s->d_top1, hw1 = s->d_hw1;
    for (uint32_t i = 0; i < s->n_slots; i++) {
        const OParticle* p = &s->particles[i];
        uint32_t low = p->kind & 255u;
        if (p->kind == KIND_DEAD || low == 0u || low > 96u) continue;   /* rows of the table */
        uint32_t row = low - 1u;
        const OOptics* o = &opt[row];
        float lx = o->opt[1], ly = o->fx2[2];   /* look_of */
        if (o->idx[0] >= 0) {
            const OOptics* dl = &opt[o->idx[0]];
            float t = clampf(p->s, 0.0f, 1.0f);
            lx = mixf(dl->opt[1], lx, t);
            ly = mixf(dl->fx2[2], ly, t);
        }
        if (maxf(lx, ly) <= 0.0f) continue;
        uint32_t* st = s->plook + 4 * (size_t)i;
        int fresh = st[0] != p->id;
        uint32_t h = hash32(p->id * 0x9e3779b1u ^ hash32(s->frame * 0x85ebca6bu + 0x165667b1u));
        /* look.comp:103-128: the specks a new particle brings into the pool's second part, in
         * slot order, the k-th of the frame taking what the k-th take gets */
        if (fresh && ly > 0.0f && s->dpool) {
            int src = o->fx2[2] > 0.0f ? (int)row : o->idx[0];
            float e = ly * P_.inv_ppc;
            float fn = floorf(e + o_rnd24(hash32(h ^ 0x2545f491u)));
            uint32_t n = fn >= 8.0f ? 8u : (fn >= 1.0f ? (uint32_t)fn : 0u);
            const OOptics* ds = &opt[src > 0 ? src : 0];
            for (uint32_t k = 0; k < n; k++) {
                uint32_t r = speck_rank + k;
                int slot;
                if (r < top1) slot = (int)s->dstack1[top1 - 1u - r];
                else {
                    uint32_t hw = hw1 + (r - top1);
                    slot = hw < D_DUST ? (int)(D_MAX + hw) : -1;
                }
                if (slot < 0) break;
                uint32_t hk = hash32(h + k * 0x9e3779b9u);
                float u1 = o_rnd24(hash32(hk ^ 0x2c1b3c6du)), u2 = o_rnd24(hash32(hk ^ 0x297a2d39u));
                float z = u1, a = 6.2831853f * u2, rr = sqrtf(maxf(1.0f - z * z, 0.0f));
                float sn, cs;
                o_sincos(a, &sn, &cs);
                ODiffuse d;
                d.px = p->pos[0] + (o_rnd24(hash32(hk ^ 0x51ed270bu)) - 0.5f) * 0.9f;
                d.py = p->pos[1] + (o_rnd24(hash32(hk ^ 0x7feb352du)) - 0.5f) * 0.9f;
                d.vx = p->vel[0];
                d.vy = p->vel[1];
                uint32_t nb = d_pack_n(rr * cs, rr * sn, z, hk);
                memcpy(&d.life, &nb, 4);
                d.r = ds->dust2[0] / P_.misc[2];
                d.info = 1u | 8u | ((uint32_t)((src > 0 ? src : 0) + 1) << 8) | (hash32(hk ^ 0x68e31da4u) & 0xffff8000u);
                d.z = o_rnd24(hash32(hk ^ 0xb5297a4du));
                s->dpool[slot] = d;
            }
            speck_rank += n;
        }
        if (lx <= 0.0f) {
            if (fresh) {
                st[0] = p->id; st[1] = 0u; st[2] = o_pack_a(third, third, 0.0f, h); st[3] = 0u;
            }
            continue;
        }
        float ax = third, ay = third, az = 0.0f;
        if (!fresh) {
            ax = (float)(st[2] & 1023u) / 1023.0f;
            ay = (float)((st[2] >> 10) & 1023u) / 1023.0f;
            az = (float)((st[2] >> 20) & 1023u) / 1023.0f - 0.5f;
            if (dt > 0.0f) {
                float Bc = o->opt2[2];
                float w = 0.5f * (p->c[2] - p->c[1]);
                float dv = 0.5f * (p->c[0] + p->c[3]);
                float exx = p->c[0] - dv, eyy = p->c[3] - dv, exy = 0.5f * (p->c[1] + p->c[2]);
                float rate = fabsf(w) + fabsf(exx) + fabsf(eyy) + fabsf(exy);
                float sf = ceilf(rate * dt / 0.15f);
                int sub = sf >= 8.0f ? 8 : (sf >= 1.0f ? (int)sf : 1);
                float h1 = dt / (float)sub;
                float ezz = 0.0f;
                for (int k = 0; k < sub; k++) {
                    float a = ax, b = ay, c = az, z = 1.0f - a - b;
                    float AE = exx * a + eyy * b + 2.0f * exy * c + ezz * z;
                    float rx = -2.0f * w * c, ry = 2.0f * w * c, rz = w * (a - b);
                    float e2 = 2.0f * AE;
                    float sx = 2.0f * (exx * a + exy * c) - e2 * a;
                    float sy = 2.0f * (exy * c + eyy * b) - e2 * b;
                    float sz = c * (exx + eyy) + exy * (a + b) - e2 * c;
                    ax = ax + h1 * (rx + Bc * sx);
                    ay = ay + h1 * (ry + Bc * sy);
                    az = az + h1 * (rz + Bc * sz);
                }
                float t = 1.0f - o_expf(-6.0f * o->opt2[1] * dt);
                ax = mixf(ax, third, t);
                ay = mixf(ay, third, t);
                az = mixf(az, 0.0f, t);
                ax = clampf(ax, 0.0f, 1.0f);
                ay = clampf(ay, 0.0f, 1.0f);
                az = clampf(az, -0.5f, 0.5f);
            }
        }
        st[0] = p->id; st[1] = 0u; st[2] = o_pack_a(ax, ay, az, h); st[3] = 0u;
        if ((uint32_t)listed < cap) list[listed] = i;
        listed++;
    }
    if (s->dpool) {   /* the takes' effect on the specks' counters */
        s->d_top1 = speck_rank < top1 ? top1 - speck_rank : 0u;
        s->d_hw1 += speck_rank > top1 ? speck_rank - top1 : 0u;
    }
    return listed;
}
/* look.comp's state per slot (4 words each, n_slots slots); returns the slots. */
long osim_look_state(const OSim* s, uint32_t* out, size_t cap) {
    if (!s->plook) return 0;
    if (out && cap >= 4 * (size_t)s->n_slots) memcpy(out, s->plook, (size_t)s->n_slots * 4 * sizeof(uint32_t));
    return (long)s->n_slots;
}

long osim_field(const OSim* s, const char* name, void* out, size_t cap) {
    size_t nc = (size_t)s->W * s->H;
    const void* src = NULL;
    size_t bytes = 0;
#define F(nm, ptr, sz) else if (strcmp(name, nm) == 0) { src = (ptr); bytes = (sz); }
    if (0) {}
    F("acc", s->acc, nc * (size_t)s->P.acc_stride * 4)
    F("vel", s->vel, nc * 16)
    F("vel0", s->vel0, nc * 8)
    F("cell", s->cell, nc * 16)
    F("comp", s->comp, nc * 16)
    F("coef", s->coef, nc * 16)
    F("sprop", s->sprop, nc * 16)
    F("surf", s->surf, nc * 16)
    F("pjump", s->pjump, nc * 8)
    F("therm", s->therm, nc * 16)
    F("dheat", s->dheat, nc * 16)
    F("hcell", s->hcell, nc * 8)
    F("vw", s->vw, nc * 16)
    F("vs", s->vs, nc * 16)
    F("pres", s->pres, nc * 8)
    F("prhs", s->prhs, nc * 16)
    F("mga", s->mga, (size_t)s->lv.total * 16)
    F("mgd", s->mgd, (size_t)s->lv.total * 4)
    F("mgz", s->mgz, (size_t)s->lv.total * 8)
    F("ptile", s->ptile, (size_t)s->lv.tiles * 4)
    F("p2keep", s->p2keep, nc * 4)
    F("mixb", s->mixb, nc * 4 * (size_t)(s->P.n_fam > 1 ? s->P.n_fam - 1 : 0))
    F("aux", s->aux, nc * 16)
    F("grho", s->grho, nc * 16)
    F("gbase", s->gbase, nc * 16)
    F("rh", s->rh, nc * 16)
    F("magc", s->magc, nc * 8)
    F("estr", s->estr, nc * 16)
    F("rl", s->rl, nc * 8)
    F("famocc", s->famocc, nc * 4 * (size_t)s->settle_fams)
    F("dsettle", s->dsettle, nc * 8 * (size_t)s->settle_fams)
    F("surf2", s->surf2, nc * 16)
    F("tiles", s->tiles, (size_t)s->nwg * 4)
    F("vtile", s->vtile, (size_t)s->lv.tiles * 4)
    F("vd", s->vd, nc * 8)
    F("vma", s->vma, (size_t)s->lv.total * 16)
    F("vmb", s->vmb, (size_t)s->lv.total * 16)
    F("vmd", s->vmd, (size_t)s->lv.total * 8)
    F("ledger", s->ledger, sizeof s->ledger)
    F("region_air", &s->region_air, 4)
    F("step", &s->S, sizeof s->S)
#undef F
    if (!src) return -1;
    if (out && cap >= bytes) memcpy(out, src, bytes);
    return (long)bytes;
}

/* Self-check of the implicit viscosity restatement: the level-0 matrix that visc_diag writes
 * out (vma, vmb, vmd, applied as vmg.glsl's offd) against the matrix-free operator of
 * visc_iter.comp (M d + G^T W G d through the weighted strain), for x on the unknown faces.
 * Writes both products to y_mg and y_free (2 floats per cell); returns the unknown count. */
long osim_visc_operator(OSim* s, const float* x, float* y_mg, float* y_free) {
    int n = s->W * s->H;
    Lv L0 = lev(s, 0);
    V2* X = (V2*)calloc((size_t)n, sizeof(V2));
    long unknowns = 0;
    for (int i = 0; i < n; i++) {
        V2 d = s->vmd[i];
        X[i] = v2(d.x > 0.0f ? x[2 * i] : 0.0f, d.y > 0.0f ? x[2 * i + 1] : 0.0f);
        unknowns += (d.x > 0.0f) + (d.y > 0.0f);
    }
    V2* keep = (V2*)malloc((size_t)n * sizeof(V2));
    memcpy(keep, s->vd, (size_t)n * sizeof(V2));
    memcpy(s->vd, X, (size_t)n * sizeof(V2));
    for (int cy = 0; cy < s->H; cy++)
        for (int cx = 0; cx < s->W; cx++) {
            int i = cidx(s, cx, cy);
            V2 d = s->vmd[i];
            V2 o = voffd(s, L0, X, cx, cy);
            y_mg[2 * i] = d.x * X[i].x + o.x;
            y_mg[2 * i + 1] = d.y * X[i].y + o.y;
            y_free[2 * i] = y_free[2 * i + 1] = 0.0f;
            if (!interior_c(s, cx, cy) || !tile_active_c(s, cx, cy)) continue;
            V2 g = v2(0, 0);
            int W = s->W;
            if (live_u(s, i)) {
                float c1 = closed_u(s, i - W) ? 1.0f : 0.5f, c2 = closed_u(s, i + W) ? -1.0f : -0.5f;
                V4 sl = strain_of_dir(s, cx - 1, cy), sc = strain_of_dir(s, cx, cy), su = strain_of_dir(s, cx, cy + 1);
                g.x = sl.x - sc.x + sc.z * c1 + su.z * c2;
            }
            if (live_v(s, i)) {
                float d1 = closed_v(s, i - 1) ? 1.0f : 0.5f, d2 = closed_v(s, i + 1) ? -1.0f : -0.5f;
                V4 sd = strain_of_dir(s, cx, cy - 1), sc = strain_of_dir(s, cx, cy), sr = strain_of_dir(s, cx + 1, cy);
                g.y = sd.y - sc.y + sc.z * d1 + sr.z * d2;
            }
            V4 cf = s->coef[i];
            y_free[2 * i] = live_u(s, i) ? cf.z * X[i].x + g.x : 0.0f;
            y_free[2 * i + 1] = live_v(s, i) ? cf.w * X[i].y + g.y : 0.0f;
        }
    memcpy(s->vd, keep, (size_t)n * sizeof(V2));
    free(keep);
    free(X);
    return unknowns;
}

/* Test hook: the assembled viscosity matrix of multigrid level l (vmg.glsl's diagonal and
 * offd) applied to x (2 floats per cell of that level, zeroed where no unknown); returns the
 * level's cell count. */
long osim_vmg_apply(OSim* s, int l, const float* x, float* y) {
    if (l < 0 || l >= s->lv.n) return -1;
    Lv L = lev(s, l);
    int n = L.w * L.h;
    V2* X = (V2*)calloc((size_t)n, sizeof(V2));
    for (int t = 0; t < n; t++) {
        V2 d = s->vmd[L.off + t];
        X[t] = v2(d.x > 0.0f ? x[2 * t] : 0.0f, d.y > 0.0f ? x[2 * t + 1] : 0.0f);
    }
    for (int t = 0; t < n; t++) {
        V2 d = s->vmd[L.off + t];
        V2 o = voffd(s, L, X, t % L.w, t / L.w);
        y[2 * t] = d.x * X[t].x + o.x;
        y[2 * t + 1] = d.y * X[t].y + o.y;
    }
    free(X);
    return n;
}

void osim_stats(const OSim* s, OStats* o) {
    memset(o, 0, sizeof *o);
    o->substeps = s->substeps_done;
    o->sim_time = s->S.advanced;
    o->dt = s->S.dt;
    o->dt_prev = s->S.dt_prev;
    o->p_iters[0] = s->K.p1_iters[0];
    o->p_iters[1] = s->K.p1_iters[1];
    o->p2_iters = s->K.p2_last;
    o->p_done[0] = s->K.p_done[0];
    o->p_done[1] = s->K.p_done[1];
    o->p_it_max = s->K.p_it_max;
    o->p_unconv = s->K.p_unconv;
    o->p2_it_max = s->K.p2_it_max;
    o->p2_unconv = s->K.p2_unconv;
    o->solves = s->K.solves;
    o->p_res_max = s->K.p_res_max;
    o->p_rr[0] = s->K.p_rr[0];
    o->p_rr[1] = s->K.p_rr[1];
    o->p_bb[0] = s->K.p_bb[0];
    o->p_bb[1] = s->K.p_bb[1];
    o->v_iters = s->K.v_iters;
    o->v_done = s->K.v_done;
    o->v_it_max = s->K.v_it_max;
    o->v_unconv = s->K.v_unconv;
    o->v_res_max = s->K.v_res_max;
    o->v_rr = s->K.v_rr;
    o->v_r0 = s->K.v_r0;
    o->umax_grid = bitsf(s->S.umax_grid);
    o->umax_part = bitsf(s->S.umax_part);
    o->n_slots = s->n_slots;
    o->caps = s->caps;
    o->acc_stride = (uint32_t)(s->tank.stride > ACC_MIN ? s->tank.stride : ACC_MIN);
    o->thermal = (uint32_t)s->thermal;
    o->viscosity_mode = (uint32_t)s->visc_mode;
    o->levels = (uint32_t)s->lv.n;
    o->tail = (uint32_t)s->lv.tail;
}

// Scene geometry and initial particle placement on the host, the inputs of a tank:
// Shape::sdf, Scene::rasterize with union_depth / seal_pockets / regions
// (src/scene.rs:60-470) and maps::fill_rect with its xorshift jitter (src/maps.rs:455-492).
#include "scene.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace sprout {

namespace {

constexpr float kWall = 3.0f;
constexpr float kNoTemp = -1e9f;

float shape_sdf(const Shape& s, float px, float py) {
    if (s.kind == Shape::Circle) return std::hypot(px - s.cx, py - s.cy) - s.r;
    float sn = std::sin(s.angle), cs = std::cos(s.angle);
    float x = px - s.cx, y = py - s.cy;
    float qx = cs * x + sn * y, qy = -sn * x + cs * y;
    float dx = std::fabs(qx) - s.hx, dy = std::fabs(qy) - s.hy;
    return std::hypot(std::max(dx, 0.0f), std::max(dy, 0.0f)) + std::min(std::max(dx, dy), 0.0f);
}

float shape_bound(const Shape& s) { return s.kind == Shape::Circle ? s.r : std::hypot(s.hx, s.hy); }

float open_fraction(float d0, float d1) {
    float f;
    if (d0 > 0.0f && d1 > 0.0f) f = 1.0f;
    else if (d0 <= 0.0f && d1 <= 0.0f) f = 0.0f;
    else f = std::max(d0, d1) / (std::max(d0, d1) - std::min(d0, d1));
    return f < 0.05f ? 0.0f : f;
}

struct Raster {
    int w, h, nw, nh;
    std::vector<float> sdf, open;

    void faces(int i, int j, float out[2]) const {
        bool here = open[j * w + i] > 0.0f;
        bool left = here && i > 0 && open[j * w + i - 1] > 0.0f;
        bool below = here && j > 0 && open[(j - 1) * w + i] > 0.0f;
        out[0] = left ? open_fraction(sdf[j * nw + i], sdf[(j + 1) * nw + i]) : 0.0f;
        out[1] = below ? open_fraction(sdf[j * nw + i], sdf[j * nw + i + 1]) : 0.0f;
    }

    // Inside the solids, depths measured to the outline of the union (chamfer 1 / sqrt 2).
    void union_depth() {
        const float FAR = 1e9f, D = 1.41421354f;
        std::vector<float> depth(sdf.size(), 0.0f);
        for (int j = 0; j < nh; j++)
            for (int i = 0; i < nw; i++) {
                int k = j * nw + i;
                if (!(sdf[k] < 0.0f)) continue;
                bool edge = false;
                for (int di = -1; di <= 1 && !edge; di++)
                    for (int dj = -1; dj <= 1; dj++) {
                        if (di == 0 && dj == 0) continue;
                        int a = i + di, b = j + dj;
                        if (a >= 0 && b >= 0 && a < nw && b < nh && !(sdf[b * nw + a] < 0.0f)) { edge = true; break; }
                    }
                depth[k] = edge ? -sdf[k] : FAR;
            }
        auto relax = [&](int k, int n, float st) { if (depth[n] + st < depth[k]) depth[k] = depth[n] + st; };
        for (int j = 0; j < nh; j++)
            for (int i = 0; i < nw; i++) {
                int k = j * nw + i;
                if (depth[k] == 0.0f) continue;
                if (i > 0) relax(k, k - 1, 1.0f);
                if (j > 0) {
                    relax(k, k - nw, 1.0f);
                    if (i > 0) relax(k, k - nw - 1, D);
                    if (i + 1 < nw) relax(k, k - nw + 1, D);
                }
            }
        for (int j = nh - 1; j >= 0; j--)
            for (int i = nw - 1; i >= 0; i--) {
                int k = j * nw + i;
                if (depth[k] == 0.0f) continue;
                if (i + 1 < nw) relax(k, k + 1, 1.0f);
                if (j + 1 < nh) {
                    relax(k, k + nw, 1.0f);
                    if (i + 1 < nw) relax(k, k + nw + 1, D);
                    if (i > 0) relax(k, k + nw - 1, D);
                }
            }
        for (size_t k = 0; k < sdf.size(); k++)
            if (sdf[k] < 0.0f && depth[k] < FAR) sdf[k] = std::min(sdf[k], -depth[k]);
    }

    // Enclosed groups of fewer than 16 open cells become solid.
    void seal_pockets() {
        size_t n = (size_t)w * h;
        std::vector<uint32_t> label(n, 0xffffffffu);
        std::vector<int> stack, members;
        for (int start = 0; start < (int)n; start++) {
            if (open[start] == 0.0f || label[start] != 0xffffffffu) continue;
            members.clear();
            label[start] = (uint32_t)start;
            stack.push_back(start);
            while (!stack.empty()) {
                int k = stack.back();
                stack.pop_back();
                members.push_back(k);
                int i = k % w, j = k / w;
                float lb[2], fr[2], fa[2];
                faces(i, j, lb);
                float right = 0.0f, above = 0.0f;
                if (i + 1 < w) { faces(i + 1, j, fr); right = fr[0]; }
                if (j + 1 < h) { faces(i, j + 1, fa); above = fa[1]; }
                const int nb[4] = {k - 1, k + 1, k - w, k + w};
                const float a[4] = {lb[0], right, lb[1], above};
                for (int q = 0; q < 4; q++)
                    if (a[q] > 0.0f && label[nb[q]] == 0xffffffffu) {
                        label[nb[q]] = (uint32_t)start;
                        stack.push_back(nb[q]);
                    }
            }
            if (members.size() < 16) {
                for (int k : members) {
                    open[k] = 0.0f;
                    int i = k % w, j = k / w;
                    const int nodes[4] = {j * nw + i, j * nw + i + 1, (j + 1) * nw + i, (j + 1) * nw + i + 1};
                    for (int nd : nodes) sdf[nd] = std::min(sdf[nd], -0.5f);
                }
            }
        }
    }
};

}  // namespace

float Scene::sdf(float x, float y) const {
    float W = (float)w, H = (float)h;
    float d = std::min(std::min(std::min(x - kWall, W - kWall - x), y - kWall), H - kWall - y);
    for (const Shape& s : shapes) d = std::min(d, shape_sdf(s, x, y));
    return d;
}

bool Scene::rasterize(float* sdf_out, float* solid4, uint32_t* region, float* temp) const {
    Raster R;
    R.w = w;
    R.h = h;
    R.nw = w + 1;
    R.nh = h + 1;
    R.sdf.resize((size_t)R.nw * R.nh);
    float W = (float)w, H = (float)h;
    for (int j = 0; j < R.nh; j++)
        for (int i = 0; i < R.nw; i++) {
            float x = (float)i, y = (float)j;
            R.sdf[j * R.nw + i] = std::min(std::min(std::min(x - kWall, W - kWall - x), y - kWall), H - kWall - y);
        }
    for (const Shape& s : shapes) {
        float r = shape_bound(s) + 6.0f;
        int i0 = (int)std::max(std::floor(s.cx - r), 0.0f);
        int i1 = std::min(std::max((int)std::ceil(s.cx + r), 0), R.nw - 1);
        int j0 = (int)std::max(std::floor(s.cy - r), 0.0f);
        int j1 = std::min(std::max((int)std::ceil(s.cy + r), 0), R.nh - 1);
        int jend = std::min(std::max(j1, j0), R.nh - 1), iend = std::min(std::max(i1, i0), R.nw - 1);
        for (int j = j0; j <= jend; j++)
            for (int i = i0; i <= iend; i++) {
                float& d = R.sdf[j * R.nw + i];
                d = std::min(d, shape_sdf(s, (float)i, (float)j));
            }
    }
    R.union_depth();
    R.open.assign((size_t)w * h, 0.0f);
    static const float FX[4][2] = {{0.25f, 0.25f}, {0.75f, 0.25f}, {0.25f, 0.75f}, {0.75f, 0.75f}};
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            const float d[4] = {R.sdf[j * R.nw + i], R.sdf[j * R.nw + i + 1], R.sdf[(j + 1) * R.nw + i], R.sdf[(j + 1) * R.nw + i + 1]};
            float acc = 0.0f;
            for (auto& f : FX) {
                float fx = f[0], fy = f[1];
                float v = (d[0] * (1.0f - fx) + d[1] * fx) * (1.0f - fy) + (d[2] * (1.0f - fx) + d[3] * fx) * fy;
                acc += std::min(std::max(v / 0.5f + 0.5f, 0.0f), 1.0f);
            }
            R.open[j * w + i] = acc * 0.25f < 0.1f ? 0.0f : acc * 0.25f;
        }
    R.seal_pockets();
    static const float K[3] = {1.0f / 6.0f, 2.0f / 3.0f, 1.0f / 6.0f};
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            float occ = 0.0f;
            for (int b = 0; b < 3; b++)
                for (int a = 0; a < 3; a++) {
                    int ii = i + a - 1, jj = j + b - 1;
                    float sv = (ii < 0 || jj < 0 || ii >= w || jj >= h) ? 1.0f : 1.0f - R.open[jj * w + ii];
                    occ += K[a] * K[b] * sv;
                }
            float f[2];
            R.faces(i, j, f);
            float* o = &solid4[4 * (j * w + i)];
            o[0] = f[0];
            o[1] = f[1];
            o[2] = occ;
            o[3] = R.open[j * w + i];
        }
    std::memcpy(sdf_out, R.sdf.data(), R.sdf.size() * sizeof(float));
    // Regions of open cells connected through open faces; the vent of each is the
    // leftmost cell of its top row.
    size_t n = (size_t)w * h;
    std::vector<int> stack;
    for (size_t k = 0; k < n; k++) region[k] = 0xffffffffu;
    uint32_t count = 0;
    for (int start = 0; start < (int)n; start++) {
        if (solid4[4 * start + 3] == 0.0f || region[start] != 0xffffffffu) continue;
        uint32_t id = std::min(count, 31u);
        count++;
        int vent = start;
        region[start] = id;
        stack.push_back(start);
        while (!stack.empty()) {
            int k = stack.back();
            stack.pop_back();
            if (k / w > vent / w || (k / w == vent / w && k < vent)) vent = k;
            int i = k % w, j = k / w;
            const bool ok[4] = {i > 0, i + 1 < w, j > 0, j + 1 < h};
            const int nb[4] = {k - 1, k + 1, k - w, k + w};
            const float a[4] = {solid4[4 * k], ok[1] ? solid4[4 * (k + 1)] : 0.0f, solid4[4 * k + 1],
                                ok[3] ? solid4[4 * (k + w) + 1] : 0.0f};
            for (int q = 0; q < 4; q++)
                if (ok[q] && a[q] > 0.0f && region[nb[q]] == 0xffffffffu) {
                    region[nb[q]] = id;
                    stack.push_back(nb[q]);
                }
        }
        region[vent] |= 256u;
    }
    for (size_t k = 0; k < n; k++)
        if (region[k] == 0xffffffffu) region[k] = 0;
    bool any = false;
    for (const Shape& s : shapes) any |= s.held;
    if (any && temp) {
        for (size_t k = 0; k < n; k++) temp[k] = kNoTemp;
        for (const Shape& s : shapes) {
            if (!s.held) continue;
            float r = shape_bound(s) + 2.0f;
            int i0 = (int)std::max(std::floor(s.cx - r), 0.0f);
            int i1 = std::min((int)std::max(std::ceil(s.cx + r), 0.0f), w);
            int j0 = (int)std::max(std::floor(s.cy - r), 0.0f);
            int j1 = std::min((int)std::max(std::ceil(s.cy + r), 0.0f), h);
            for (int j = j0; j < j1; j++)
                for (int i = i0; i < i1; i++)
                    if (shape_sdf(s, (float)i + 0.5f, (float)j + 0.5f) < 0.75f) temp[j * w + i] = s.temp;
        }
    }
    return any;
}

uint32_t Scene::fill_rect(const float rect[4], uint32_t material, uint32_t n_before, SproutParticleHost* out,
                          uint32_t cap) const {
    const float step = 0.5f;   // PPC = 4: a 2 x 2 sub-lattice per cell
    float W = (float)w, H = (float)h;
    int x0 = (int)std::round(std::max(rect[0], kWall) / step);
    int x1 = (int)std::round(std::min(rect[2], W - kWall) / step);
    int y0 = (int)std::round(std::max(rect[1], kWall) / step);
    int y1 = (int)std::round(std::min(rect[3], H - kWall) / step);
    uint32_t rng = 0x9E3779B9u ^ (n_before * 747796405u + 1u);
    auto next = [&]() {
        rng ^= rng << 13;
        rng ^= rng >> 17;
        rng ^= rng << 5;
        return (float)(rng >> 8) / (float)(1u << 24);
    };
    uint32_t n = 0;
    for (int j = y0; j < y1; j++)
        for (int i = x0; i < x1; i++) {
            float px = ((float)i + 0.5f + (next() - 0.5f) * 0.5f) * step;
            float py = ((float)j + 0.5f + (next() - 0.5f) * 0.5f) * step;
            if (sdf(px, py) > 0.1f) {
                if (n < cap && out) {
                    SproutParticleHost& p = out[n];
                    std::memset(&p, 0, sizeof p);
                    p.pos[0] = px;
                    p.pos[1] = py;
                    p.s = -1.0f;          // SPAWN_S: settled at reset
                    p.kind = material + 1u;
                    p.t = -1.0e4f;        // SPAWN_TEMP: settled at reset
                }
                n++;
            }
        }
    return n;
}

}  // namespace sprout

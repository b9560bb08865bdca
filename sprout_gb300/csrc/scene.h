// Host-side scene: analytic solids and their rasterisation into the fields a tank needs
// (Scene, src/scene.rs), and the rest-lattice particle fill (maps::fill_rect, src/maps.rs).
#pragma once

#include <cstdint>
#include <vector>

namespace sprout {

// Layout-identical to SproutParticle (48 bytes).
struct SproutParticleHost {
    float pos[2], vel[2], c[4], s;
    uint32_t kind, id;
    float t;
};
static_assert(sizeof(SproutParticleHost) == 48, "particle is 48 bytes");

struct Shape {
    enum Kind { Circle = 0, Box = 1 } kind = Box;
    float cx = 0, cy = 0, hx = 0, hy = 0, r = 0, angle = 0;
    bool held = false;   // held at `temp` (Scene::temps)
    float temp = 0;
};

struct Scene {
    int w = 0, h = 0;
    std::vector<Shape> shapes;
    float sdf(float x, float y) const;
    // Returns whether any shape is held at a temperature.
    bool rasterize(float* sdf, float* solid4, uint32_t* region, float* temp) const;
    uint32_t fill_rect(const float rect[4], uint32_t material, uint32_t n_before, SproutParticleHost* out,
                       uint32_t cap) const;
};

}  // namespace sprout

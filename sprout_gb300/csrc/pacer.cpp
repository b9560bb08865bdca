// Frame pacing (src/pacing.rs): how much simulated time each rendered frame covers and in
// how many substeps. The device sizes every substep itself (step.comp); the pacer asks for a
// span of simulated time and enough substeps to cover it at the last known step length.
// Substep counts follow the measured device cost of a substep with hysteresis (a heavy tank
// runs the same count every frame and simulated time slows down, rather than alternating
// n and n + 1), and frames much shorter than a substep bank their time until a full-length
// substep is due. Single precision throughout, as the reference computes it.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <new>

#include "../../include/sprout_gpu.h"

namespace {

constexpr uint32_t kUnmeasuredSubsteps = 2;   // pacing.rs:20
constexpr float kSlack = 0.1f;                // pacing.rs:23

}  // namespace

struct SproutPacer {
    float bank = 0.0f;        // simulated time owed, s
    uint32_t cap = kUnmeasuredSubsteps;
    float delivered = 0.0f, asked = 0.0f;
    uint32_t last = 0;
    float idle_frame = 0.0f;

    float speed() const { return asked > 0.0f ? delivered / asked : 1.0f; }

    // Pacer::plan (pacing.rs:67-112)
    SproutPlan plan(float frame_dt, float dt, bool fixed, float time_scale, float cost, float budget) {
        if (cost > 0.0f) {
            // raise the cap only when one more substep clearly fits, lower it as soon as the
            // current count does not
            if ((float)(cap + 1) * cost < 0.85f * budget) cap += 1;
            while (cap > 1 && (float)cap * cost > budget) cap -= 1;
            cap = std::min(cap, (uint32_t)SPROUT_MAX_SUBSTEPS_PER_FRAME);
        }
        const float wanted = std::min(frame_dt, 0.1f) * time_scale;
        bank += wanted;
        const float idle = std::max(std::min(frame_dt, 0.1f) - (float)last * cost, 1e-4f);
        idle_frame = idle_frame == 0.0f ? idle : idle_frame + 0.25f * (idle - idle_frame);
        SproutPlan p{};
        if (fixed) {
            const uint32_t n = std::min((uint32_t)(bank / dt), cap);
            const float t = (float)n * dt;
            p = SproutPlan{n, t, t};
        } else {
            const float r = bank / dt;
            // step once a full substep is owed, or when waiting for the next frame would owe
            // more than one
            const bool due = r >= 1.0f || bank + idle_frame * time_scale > dt;
            const uint32_t n = due ? std::min((uint32_t)std::max(std::ceil(r - kSlack), 1.0f), cap) : 0u;
            const float t = std::min(bank, (float)n * dt);
            p = SproutPlan{n, t, t};
        }
        // time that cannot be simulated this frame is dropped, not carried as debt
        const float kept = std::min(bank - p.expected, dt);
        const float dropped = bank - p.expected - kept;
        bank = kept;
        const float keep = 1.0f - std::min(frame_dt * 2.0f, 1.0f);
        delivered = delivered * keep + wanted - dropped;
        asked = asked * keep + wanted;
        last = p.substeps;
        return p;
    }
};

extern "C" {

int sprout_pacer_new(SproutPacer** out) {
    if (!out) return SPROUT_E_ARG;
    *out = new (std::nothrow) SproutPacer();
    return *out ? SPROUT_OK : SPROUT_E_NOMEM;
}

int sprout_pacer_free(SproutPacer* p) {
    delete p;
    return SPROUT_OK;
}

int sprout_pacer_reset(SproutPacer* p) {
    if (!p) return SPROUT_E_ARG;
    p->bank = 0.0f;
    return SPROUT_OK;
}

int sprout_pacer_speed(const SproutPacer* p, float* speed) {
    if (!p || !speed) return SPROUT_E_ARG;
    *speed = p->speed();
    return SPROUT_OK;
}

int sprout_pacer_plan(SproutPacer* p, float frame_dt, float dt, int fixed, float time_scale, float cost, float budget,
                      SproutPlan* out) {
    if (!p || !out || !(dt > 0.0f)) return SPROUT_E_ARG;
    *out = p->plan(frame_dt, dt, fixed != 0, time_scale, cost, budget);
    return SPROUT_OK;
}

}  // extern "C"

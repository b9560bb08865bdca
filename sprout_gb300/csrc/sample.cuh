// Samplers of the grid shared by the particle pass (particles.comp) and spray.comp: the
// solids' signed distance bilinear between nodes with its gradient, and the MAC velocity
// bilinear over live faces (common.glsl's sample_sdf / sample_vel).
#pragma once

#include "dev_common.cuh"

namespace sprout {

struct Grid {
    const float4* vel;
    const float* sdf;
    int W, H;
    DEV float4 v(int x, int y) const { return __ldg(&vel[y * W + x]); }
};

DEV float sample_sdf(const Grid& g, float x, float y, float* gx_out, float* gy_out) {
    float gx = clampf(x, 0.0f, (float)g.W - 0.001f), gy = clampf(y, 0.0f, (float)g.H - 0.001f);
    int ix = (int)gx, iy = (int)gy;
    float fx = gx - (float)ix, fy = gy - (float)iy;
    int w1 = g.W + 1;
    int k = iy * w1 + ix;
    float d00 = __ldg(&g.sdf[k]), d10 = __ldg(&g.sdf[k + 1]), d01 = __ldg(&g.sdf[k + w1]), d11 = __ldg(&g.sdf[k + w1 + 1]);
    *gx_out = mixf(d10 - d00, d11 - d01, fy);
    *gy_out = mixf(d01 - d00, d11 - d10, fx);
    return mixf(mixf(d00, d10, fx), mixf(d01, d11, fx), fy);
}

// Bilinear grid velocity over live faces; components without a live face keep the fallback.
DEV float2 sample_vel(const Grid& g, float x, float y, float2 fb) {
    float2 o = fb;
    {
        float gx = x, gy = y - 0.5f;
        int bx = (int)floorf(gx), by = (int)floorf(gy);
        float fx = gx - (float)bx, fy = gy - (float)by;
        float sw = 0.0f, su = 0.0f;
#pragma unroll
        for (int b = 0; b < 2; b++)
#pragma unroll
            for (int a = 0; a < 2; a++) {
                float4 q = g.v(bx + a, by + b);
                if (face_live(q.z)) {
                    float wt = (a == 0 ? 1.0f - fx : fx) * (b == 0 ? 1.0f - fy : fy);
                    sw += wt;
                    su += wt * q.x;
                }
            }
        if (sw > 1e-3f) o.x = su / sw;
    }
    {
        float gx = x - 0.5f, gy = y;
        int bx = (int)floorf(gx), by = (int)floorf(gy);
        float fx = gx - (float)bx, fy = gy - (float)by;
        float sw = 0.0f, su = 0.0f;
#pragma unroll
        for (int b = 0; b < 2; b++)
#pragma unroll
            for (int a = 0; a < 2; a++) {
                float4 q = g.v(bx + a, by + b);
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

}  // namespace sprout

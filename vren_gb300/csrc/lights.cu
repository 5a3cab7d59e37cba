// Point-light bouncer (vren_demo/resources/shaders/bounce_point_lights.comp:33-73, host
// vren_demo/vren_demo/point_light_bouncer.cpp:17-57): the per-frame producer of the light positions
// that construct_point_light_bvh reads.  Each light is clamped into an axis-aligned box and moves
// speed * dt along its direction, reflecting off the box faces (at most 32 bounces).
//
// One thread per light, 128-bit loads and stores of the position and direction (32 B read and 32 B
// written per light).  The arithmetic is the canonical one of this library: every operation rounded
// on its own (no FMA contraction: this unit is compiled with --fmad=false and uses the _rn
// intrinsics), IEEE division, GLSL min/max (min(x, y) = y < x ? y : x), so the result is bit-identical
// to the CPU restatement.
#include "common.cuh"

namespace vren_gb300 {

VREN_DEFINE_ERROR_WORD(lights)

__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }

constexpr float kBounceInf = 1e35f;
constexpr float kBounceEps = 1e-5f;
constexpr int kBounceMaxIter = 32;

struct BounceBox {
    float mn[3];
    float mx[3];
};

__global__ void __launch_bounds__(256) bounce_point_lights_kernel(float4* __restrict__ positions,
                                                                  float4* __restrict__ directions, uint32_t L,
                                                                  BounceBox box, float speed, float dt)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x) {
        const float4 p4 = positions[i], d4 = directions[i];
        float p[3] = {p4.x, p4.y, p4.z}, d[3] = {d4.x, d4.y, d4.z};
#pragma unroll
        for (int c = 0; c < 3; ++c) p[c] = gmin(gmax(p[c], box.mn[c]), box.mx[c]);
        float rem = fmul(speed, dt);
        for (int j = 0; j < kBounceMaxIter && rem > 0.0f; ++j) {
            float t1[3], t2[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                t1[c] = fdiv(fsub(box.mn[c], p[c]), d[c]);
                t1[c] = t1[c] <= 0.0f ? kBounceInf : t1[c];
                t2[c] = fdiv(fsub(box.mx[c], p[c]), d[c]);
                t2[c] = t2[c] <= 0.0f ? kBounceInf : t2[c];
            }
            const float min_t = gmin(t1[0], gmin(t2[0], gmin(t1[1], gmin(t2[1], gmin(t1[2], t2[2])))));
            const float step = gmin(fsub(min_t, kBounceEps), rem);
#pragma unroll
            for (int c = 0; c < 3; ++c) p[c] = fadd(p[c], fmul(step, d[c]));
            if (min_t < rem) {
#pragma unroll
                for (int c = 0; c < 3; ++c) d[c] = fmul(d[c], (t1[c] == min_t || t2[c] == min_t) ? -1.0f : 1.0f);
            }
            rem = fsub(rem, step);
        }
        positions[i] = make_float4(p[0], p[1], p[2], 1.0f);
        directions[i] = make_float4(d[0], d[1], d[2], 0.0f);
    }
}

}  // namespace vren_gb300

using namespace vren_gb300;

extern "C" int vren_bounce_point_lights(vren_stream_t s, float* light_positions, float* light_directions,
                                        uint32_t light_count, const float* aabb_min, const float* aabb_max,
                                        float speed, float dt)
{
    if (light_count == 0) return VREN_OK;
    if (!light_positions || !light_directions || !aabb_min || !aabb_max) return VREN_ERR_ARG;
    if (((uintptr_t)light_positions | (uintptr_t)light_directions) & 15u) return VREN_ERR_ARG;
    BounceBox box;
    for (int c = 0; c < 3; ++c) {
        box.mn[c] = aabb_min[c];
        box.mx[c] = aabb_max[c];
    }
    uint32_t grid = (light_count + 255) / 256;
    if (grid > (uint32_t)kNumSMsHint * 16) grid = kNumSMsHint * 16;
    launch_kernel(bounce_point_lights_kernel, grid, 256, 0, as_stream(s), reinterpret_cast<float4*>(light_positions),
                  reinterpret_cast<float4*>(light_directions), light_count, box, speed, dt);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

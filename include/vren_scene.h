/*
 * vren_scene.h — seeded synthetic inputs for the vren_gb300 benchmarks and tests.
 *
 * All randomness comes from PCG32 (M. O'Neill, "PCG: A Family of Simple Fast Space-Efficient
 * Statistically Good Algorithms for Random Number Generation", 2014): 64-bit LCG state,
 * XSH-RR output.  (seed, stream) select the sequence; every function is deterministic and
 * single-valued for a given seed whatever the thread count.
 *
 * The scene follows the reference's camera conventions (vren/vren/camera.cpp:32-50): view space
 * is x right, y up, +z forward; the projection maps view z in [near, far] to depth [0, 1]
 * with m[2][2] = f/(f-n), m[3][2] = -f*n/(f-n), m[2][3] = 1.
 */
#ifndef VREN_SCENE_H_
#define VREN_SCENE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* PCG32 */
typedef struct vren_pcg32 { uint64_t state, inc; } vren_pcg32;
void vren_pcg32_seed(vren_pcg32* rng, uint64_t seed, uint64_t stream);
uint32_t vren_pcg32_next(vren_pcg32* rng);
void vren_pcg32_advance(vren_pcg32* rng, uint64_t delta);

/* out[i] = i-th output of PCG32(seed, stream), i in [0, n) (parallel via jump-ahead). */
void vren_gen_u32(uint64_t seed, uint64_t stream, uint32_t* out, uint64_t n, int threads);
/* out[i] = (i-th output) & mask */
void vren_gen_u32_masked(uint64_t seed, uint64_t stream, uint32_t* out, uint64_t n, uint32_t mask, int threads);

/* Camera used by the scenes: origin, yaw = pitch = 0, vertical fov, near/far planes. */
typedef struct vren_scene_camera {
    float fov_y;       /* radians */
    float near_plane;
    float far_plane;
    uint32_t width, height;
} vren_scene_camera;

/* Depth buffer from `num_planes` random oriented planar discs (centre in the frustum, view z
 * log-uniform in [1, 0.9 far], normal facing the camera, radius 20-80 % of the frustum half-height
 * at that depth): per pixel the nearest positive hit of the ray through the pixel centre, view z
 * clamped to [near, far] (a miss gives far), stored as NDC depth (f32[W*H], row-major).  normals
 * (f32x3[W*H]) receive the hit plane's unit normal (misses: (0, 0, -1)).  Either output may be NULL. */
void vren_gen_depth_planes(uint64_t seed, const vren_scene_camera* cam, uint32_t num_planes,
                           float* depth, float* normals, int threads);

/* Point lights: positions uniform in the frustum's bounding box (x within +-far*tan(fov/2)*aspect,
 * y within +-far*tan(fov/2), z in [near, far]), w = 1; colour uniform [0,1]^3; radius (the
 * reference's point_light.intensity) lognormal(mu = ln 2, sigma = 0.5).
 * positions: vec4[L]; lights: {r, g, b, radius}[L]. */
void vren_gen_lights(uint64_t seed, const vren_scene_camera* cam, uint32_t count, float* positions,
                     float* lights);

/* Point lights placed on visible surfaces of a depth buffer (a random pixel closer than the far
 * plane, pulled towards the camera by 10-60 % of the light's radius); radius lognormal(ln 2, 0.5),
 * colour uniform [0,1]^3.  Used by the differentiable-shading workload, where lights spread over the
 * whole frustum box would leave most gradients zero. */
void vren_gen_lights_near_surfaces(uint64_t seed, const vren_scene_camera* cam, const float* depth, uint32_t count,
                                   float* positions, float* lights);

/* G-buffer material channels: normals uniform on the hemisphere facing the camera (n.z <= 0),
 * albedo uniform [0,1]^3, roughness uniform [0.05, 1], metallic Bernoulli(0.5) in {0, 1}.
 * Any output may be NULL. */
void vren_gen_gbuffer(uint64_t seed, uint32_t width, uint32_t height, float* normals, float* albedo,
                      float* roughness, float* metallic, int threads);

/* n standard normal f32 values (Box-Muller). */
void vren_gen_normal01(uint64_t seed, uint64_t stream, float* out, uint64_t n, int threads);

#ifdef __cplusplus
}
#endif

#endif /* VREN_SCENE_H_ */

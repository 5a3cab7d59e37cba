/* Seeded synthetic scenes (host C).  See include/vren_scene.h for the contract. */
#include "vren_scene.h"

#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PCG_MULT 6364136223846793005ULL

void vren_pcg32_seed(vren_pcg32* rng, uint64_t seed, uint64_t stream)
{
    rng->state = 0u;
    rng->inc = (stream << 1u) | 1u;
    vren_pcg32_next(rng);
    rng->state += seed;
    vren_pcg32_next(rng);
}

uint32_t vren_pcg32_next(vren_pcg32* rng)
{
    uint64_t old = rng->state;
    rng->state = old * PCG_MULT + rng->inc;
    uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((-rot) & 31u));
}

/* Jump-ahead for the LCG (F. Brown, "Random number generation with arbitrary strides", 1994). */
void vren_pcg32_advance(vren_pcg32* rng, uint64_t delta)
{
    uint64_t cur_mult = PCG_MULT, cur_plus = rng->inc;
    uint64_t acc_mult = 1u, acc_plus = 0u;
    while (delta > 0) {
        if (delta & 1u) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1u) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1u;
    }
    rng->state = acc_mult * rng->state + acc_plus;
}

static int clamp_threads(int threads)
{
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
    return threads;
#else
    (void)threads;
    return 1;
#endif
}

void vren_gen_u32_masked(uint64_t seed, uint64_t stream, uint32_t* out, uint64_t n, uint32_t mask, int threads)
{
    const uint64_t chunk = 1u << 20;
    const int64_t nchunks = (int64_t)((n + chunk - 1) / chunk);
    threads = clamp_threads(threads);
#pragma omp parallel for schedule(static) num_threads(threads) if (nchunks > 1)
    for (int64_t c = 0; c < nchunks; ++c) {
        vren_pcg32 rng;
        vren_pcg32_seed(&rng, seed, stream);
        vren_pcg32_advance(&rng, (uint64_t)c * chunk);
        uint64_t end = ((uint64_t)c + 1) * chunk < n ? ((uint64_t)c + 1) * chunk : n;
        for (uint64_t i = (uint64_t)c * chunk; i < end; ++i) out[i] = vren_pcg32_next(&rng) & mask;
    }
}

void vren_gen_u32(uint64_t seed, uint64_t stream, uint32_t* out, uint64_t n, int threads)
{
    vren_gen_u32_masked(seed, stream, out, n, 0xFFFFFFFFu, threads);
}

/* uniform double in [0, 1) from 53 random bits */
static double uniform01(vren_pcg32* rng)
{
    uint64_t a = vren_pcg32_next(rng) >> 5, b = vren_pcg32_next(rng) >> 6;
    return (double)(a * 67108864ULL + b) * (1.0 / 9007199254740992.0);
}

static double std_normal(vren_pcg32* rng)
{
    double u1 = 1.0 - uniform01(rng); /* (0, 1] */
    double u2 = uniform01(rng);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

static void unit_sphere(vren_pcg32* rng, double n[3])
{
    double z = 2.0 * uniform01(rng) - 1.0;
    double phi = 6.283185307179586 * uniform01(rng);
    double r = sqrt(fmax(0.0, 1.0 - z * z));
    n[0] = r * cos(phi);
    n[1] = r * sin(phi);
    n[2] = z;
}

void vren_gen_depth_planes(uint64_t seed, const vren_scene_camera* cam, uint32_t num_planes, float* depth,
                           float* normals, int threads)
{
    /* Oriented planar discs: centre inside the frustum (view z log-uniform in [1, 0.9 far], x/y
     * uniform in the cross-section), unit normal uniform on the hemisphere facing the camera,
     * radius 20-80 % of the frustum's half-height at the centre's depth.  Unbounded planes would
     * let the nearest one cover almost the whole view. */
    enum { kMaxPlanes = 1024 };
    double pn[kMaxPlanes][3], pc[kMaxPlanes], ctr[kMaxPlanes][3], rad2[kMaxPlanes];
    if (num_planes > kMaxPlanes) num_planes = kMaxPlanes;
    const double W = cam->width, H = cam->height;
    const double aspect = W / H;
    const double t = tan((double)cam->fov_y * 0.5);
    const double n_ = cam->near_plane, f_ = cam->far_plane;

    vren_pcg32 rng;
    vren_pcg32_seed(&rng, seed, 101u);
    for (uint32_t i = 0; i < num_planes; ++i) {
        double nn[3];
        unit_sphere(&rng, nn);
        if (nn[2] > 0.0) { nn[0] = -nn[0]; nn[1] = -nn[1]; nn[2] = -nn[2]; } /* face the camera */
        double z0 = exp(uniform01(&rng) * log(0.9 * f_));
        if (z0 < 1.0) z0 = 1.0;
        double x0 = (2.0 * uniform01(&rng) - 1.0) * z0 * t * aspect;
        double y0 = (2.0 * uniform01(&rng) - 1.0) * z0 * t;
        double r = (0.2 + 0.6 * uniform01(&rng)) * z0 * t;
        pn[i][0] = nn[0]; pn[i][1] = nn[1]; pn[i][2] = nn[2];
        ctr[i][0] = x0; ctr[i][1] = y0; ctr[i][2] = z0;
        rad2[i] = r * r;
        pc[i] = nn[0] * x0 + nn[1] * y0 + nn[2] * z0;
    }
    const double m22 = f_ / (f_ - n_), m32 = -(f_ * n_) / (f_ - n_);
    threads = clamp_threads(threads);
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int64_t y = 0; y < (int64_t)cam->height; ++y) {
        for (uint32_t x = 0; x < cam->width; ++x) {
            const double ndc_x = 2.0 * ((double)x + 0.5) / W - 1.0;
            const double ndc_y = 1.0 - 2.0 * ((double)y + 0.5) / H;
            const double d[3] = {ndc_x * t * aspect, ndc_y * t, 1.0};
            double best = INFINITY;
            int hit = -1;
            for (uint32_t i = 0; i < num_planes; ++i) {
                double den = pn[i][0] * d[0] + pn[i][1] * d[1] + pn[i][2] * d[2];
                if (den == 0.0) continue;
                double tt = pc[i] / den;
                if (!(tt > 0.0 && tt < best)) continue;
                double q0 = tt * d[0] - ctr[i][0], q1 = tt * d[1] - ctr[i][1], q2 = tt * d[2] - ctr[i][2];
                if (q0 * q0 + q1 * q1 + q2 * q2 > rad2[i]) continue;
                best = tt;
                hit = (int)i;
            }
            double z = hit >= 0 ? best : f_;
            if (z < n_) z = n_;
            if (z > f_) z = f_;
            const size_t px = (size_t)y * cam->width + x;
            if (depth) depth[px] = (float)(m22 + m32 / z);
            if (normals) {
                if (hit >= 0) {
                    normals[3 * px + 0] = (float)pn[hit][0];
                    normals[3 * px + 1] = (float)pn[hit][1];
                    normals[3 * px + 2] = (float)pn[hit][2];
                } else {
                    normals[3 * px + 0] = 0.0f;
                    normals[3 * px + 1] = 0.0f;
                    normals[3 * px + 2] = -1.0f;
                }
            }
        }
    }
}

void vren_gen_lights(uint64_t seed, const vren_scene_camera* cam, uint32_t count, float* positions, float* lights)
{
    const double aspect = (double)cam->width / (double)cam->height;
    const double t = tan((double)cam->fov_y * 0.5);
    const double f_ = cam->far_plane, n_ = cam->near_plane;
    const double hx = f_ * t * aspect, hy = f_ * t;
    vren_pcg32 rng;
    vren_pcg32_seed(&rng, seed, 202u);
    for (uint32_t i = 0; i < count; ++i) {
        double x = (2.0 * uniform01(&rng) - 1.0) * hx;
        double y = (2.0 * uniform01(&rng) - 1.0) * hy;
        double z = n_ + uniform01(&rng) * (f_ - n_);
        double r = exp(log(2.0) + 0.5 * std_normal(&rng));
        double cr = uniform01(&rng), cg = uniform01(&rng), cb = uniform01(&rng);
        if (positions) {
            positions[4 * i + 0] = (float)x;
            positions[4 * i + 1] = (float)y;
            positions[4 * i + 2] = (float)z;
            positions[4 * i + 3] = 1.0f;
        }
        if (lights) {
            lights[4 * i + 0] = (float)cr;
            lights[4 * i + 1] = (float)cg;
            lights[4 * i + 2] = (float)cb;
            lights[4 * i + 3] = (float)r;
        }
    }
}

void vren_gen_gbuffer(uint64_t seed, uint32_t width, uint32_t height, float* normals, float* albedo, float* roughness,
                      float* metallic, int threads)
{
    threads = clamp_threads(threads);
    /* one PCG32 stream per row keeps the output independent of the thread count */
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int64_t y = 0; y < (int64_t)height; ++y) {
        vren_pcg32 rng;
        vren_pcg32_seed(&rng, seed, 1000003ULL + (uint64_t)y);
        for (uint32_t x = 0; x < width; ++x) {
            const size_t px = (size_t)y * width + x;
            double nn[3];
            unit_sphere(&rng, nn);
            if (nn[2] > 0.0) { nn[0] = -nn[0]; nn[1] = -nn[1]; nn[2] = -nn[2]; }
            double a0 = uniform01(&rng), a1 = uniform01(&rng), a2 = uniform01(&rng);
            double ro = 0.05 + 0.95 * uniform01(&rng);
            double me = (vren_pcg32_next(&rng) & 1u) ? 1.0 : 0.0;
            if (normals) { normals[3 * px] = (float)nn[0]; normals[3 * px + 1] = (float)nn[1]; normals[3 * px + 2] = (float)nn[2]; }
            if (albedo) { albedo[3 * px] = (float)a0; albedo[3 * px + 1] = (float)a1; albedo[3 * px + 2] = (float)a2; }
            if (roughness) roughness[px] = (float)ro;
            if (metallic) metallic[px] = (float)me;
        }
    }
}

void vren_gen_normal01(uint64_t seed, uint64_t stream, float* out, uint64_t n, int threads)
{
    const uint64_t chunk = 1u << 16;
    const int64_t nchunks = (int64_t)((n + chunk - 1) / chunk);
    threads = clamp_threads(threads);
#pragma omp parallel for schedule(static) num_threads(threads) if (nchunks > 1)
    for (int64_t c = 0; c < nchunks; ++c) {
        vren_pcg32 rng;
        vren_pcg32_seed(&rng, seed, stream + 7919ULL * (uint64_t)c);
        uint64_t end = ((uint64_t)c + 1) * chunk < n ? ((uint64_t)c + 1) * chunk : n;
        for (uint64_t i = (uint64_t)c * chunk; i < end; ++i) out[i] = (float)std_normal(&rng);
    }
}

void vren_gen_lights_near_surfaces(uint64_t seed, const vren_scene_camera* cam, const float* depth, uint32_t count,
                                   float* positions, float* lights)
{
    const double W = cam->width, H = cam->height;
    const double aspect = W / H;
    const double t = tan((double)cam->fov_y * 0.5);
    const double n_ = cam->near_plane, f_ = cam->far_plane;
    const double m22 = f_ / (f_ - n_), m32 = -(f_ * n_) / (f_ - n_);
    vren_pcg32 rng;
    vren_pcg32_seed(&rng, seed, 303u);
    for (uint32_t i = 0; i < count; ++i) {
        double p[3] = {0.0, 0.0, 0.5 * (n_ + f_)};
        for (int attempt = 0; attempt < 64; ++attempt) {
            const uint32_t x = vren_pcg32_next(&rng) % cam->width, y = vren_pcg32_next(&rng) % cam->height;
            const double D = depth[(size_t)y * cam->width + x];
            const double z = m32 / (D - m22);
            if (!(z < f_ * 0.999)) continue;
            const double ndc_x = 2.0 * ((double)x + 0.5) / W - 1.0, ndc_y = 1.0 - 2.0 * ((double)y + 0.5) / H;
            p[0] = ndc_x * t * aspect * z;
            p[1] = ndc_y * t * z;
            p[2] = z;
            break;
        }
        const double r = exp(log(2.0) + 0.5 * std_normal(&rng));
        /* pull the light towards the camera by 10-60 % of its radius so it lights the surface */
        const double len = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        const double back = (0.1 + 0.5 * uniform01(&rng)) * r;
        const double s = len > back ? (len - back) / len : 0.5;
        const double cr = uniform01(&rng), cg = uniform01(&rng), cb = uniform01(&rng);
        if (positions) {
            positions[4 * i + 0] = (float)(p[0] * s);
            positions[4 * i + 1] = (float)(p[1] * s);
            positions[4 * i + 2] = (float)(p[2] * s);
            positions[4 * i + 3] = 1.0f;
        }
        if (lights) {
            lights[4 * i + 0] = (float)cr;
            lights[4 * i + 1] = (float)cg;
            lights[4 * i + 2] = (float)cb;
            lights[4 * i + 3] = (float)r;
        }
    }
}

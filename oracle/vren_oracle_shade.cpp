// vren_oracle_shade.cpp — CPU oracle for clustered shading in FP64.  TEST INFRASTRUCTURE ONLY.
//
// Restates shade.comp:69-141 and pbr.glsl:6-112 (PI = 3.14, a = k = roughness) with the two falloffs
// (reference: 1 - min(d/r, 1)^1.5, pbr.glsl:89; windowed inverse square: saturate(1-(d/r)^4)^2/(d^2+1),
// Karis 2013), evaluated in double.  The reference gradient with respect to each light's position,
// colour and radius is obtained by forward-mode differentiation (dual numbers carrying 7 tangents),
// which is independent of the hand-written reverse-mode adjoint of the CUDA kernel.  Branch
// conventions: max(x, 0) passes the derivative only for x > 0, min(t, 1) only for t < 1,
// clamp(w, 0, 1) only for 0 < w < 1.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {
#include "vren_oracle.h"
}

namespace {

constexpr double kPi = 3.14;
constexpr int NT = 7;  // position xyz, colour rgb, radius

struct Dual {
    double v;
    double d[NT];
};

inline Dual cst(double v)
{
    Dual r;
    r.v = v;
    std::memset(r.d, 0, sizeof(r.d));
    return r;
}
inline Dual operator+(const Dual& a, const Dual& b)
{
    Dual r;
    r.v = a.v + b.v;
    for (int i = 0; i < NT; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
inline Dual operator-(const Dual& a, const Dual& b)
{
    Dual r;
    r.v = a.v - b.v;
    for (int i = 0; i < NT; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
inline Dual operator-(const Dual& a)
{
    Dual r;
    r.v = -a.v;
    for (int i = 0; i < NT; ++i) r.d[i] = -a.d[i];
    return r;
}
inline Dual operator*(const Dual& a, const Dual& b)
{
    Dual r;
    r.v = a.v * b.v;
    for (int i = 0; i < NT; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
inline Dual operator/(const Dual& a, const Dual& b)
{
    Dual r;
    r.v = a.v / b.v;
    for (int i = 0; i < NT; ++i) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) / (b.v * b.v);
    return r;
}
inline Dual operator*(double s, const Dual& a) { return cst(s) * a; }
inline Dual operator+(double s, const Dual& a) { return cst(s) + a; }
inline Dual operator-(double s, const Dual& a) { return cst(s) - a; }
inline Dual dsqrt(const Dual& a)
{
    Dual r;
    r.v = std::sqrt(a.v);
    for (int i = 0; i < NT; ++i) r.d[i] = a.d[i] / (2.0 * r.v);
    return r;
}
inline Dual max0(const Dual& a) { return a.v > 0.0 ? a : cst(0.0); }
inline Dual min1(const Dual& a) { return a.v < 1.0 ? a : cst(1.0); }
inline Dual clamp01(const Dual& a) { return a.v <= 0.0 ? cst(0.0) : (a.v >= 1.0 ? cst(1.0) : a); }

struct V3 {
    Dual x, y, z;
};
inline V3 v3(const Dual& x, const Dual& y, const Dual& z) { return {x, y, z}; }
inline V3 v3c(double x, double y, double z) { return {cst(x), cst(y), cst(z)}; }
inline Dual dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 sub(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 scale(const V3& a, const Dual& s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 divs(const V3& a, const Dual& s) { return {a.x / s, a.y / s, a.z / s}; }

struct Pixel {
    double p[3], N[3], V[3], alb[3], rough, metal;
};

// pbr_apply_point_light for one (pixel, light) pair, returns the three channels.
void point_light(const Pixel& q, const V3& lp, const V3& col, const Dual& r, int falloff, Dual out[3])
{
    const V3 p = v3c(q.p[0], q.p[1], q.p[2]);
    const V3 N = v3c(q.N[0], q.N[1], q.N[2]);
    const V3 V = v3c(q.V[0], q.V[1], q.V[2]);
    const V3 d = sub(p, lp);
    const Dual dist = dsqrt(dot(d, d));
    const V3 L = divs(d, dist);
    Dual att;
    if (falloff == 0) {
        const Dual u = min1(dist / r);
        att = 1.0 - u * dsqrt(u);
    } else {
        const Dual t = dist / r;
        const Dual t2 = t * t;
        const Dual w = clamp01(1.0 - t2 * t2);
        att = (w * w) / (dist * dist + cst(1.0));
    }
    const V3 hv = sub(V, L);
    const V3 H = divs(hv, dsqrt(dot(hv, hv)));
    const double a2 = q.rough * q.rough;
    const Dual NdotH = max0(dot(N, H));
    const Dual D = NdotH * NdotH * cst(a2 - 1.0) + cst(1.0);
    const Dual NDF = cst(a2) / (kPi * D * D);
    const double k = q.rough;
    const double NdotV = std::max(q.N[0] * q.V[0] + q.N[1] * q.V[1] + q.N[2] * q.V[2], 0.0);
    const Dual NdotL = max0(-dot(N, L));
    const double ggxV = NdotV / (NdotV * (1.0 - k) + k);
    const Dual ggxL = NdotL / (NdotL * cst(1.0 - k) + cst(k));
    const Dual G = cst(ggxV) * ggxL;
    const Dual HdotV = max0(dot(H, V));
    const Dual x = 1.0 - HdotV;
    const Dual f5 = x * x * x * x * x;
    const Dual spec = NDF * G / (cst(4.0 * NdotV) * NdotL + cst(0.0001));
    const Dual c3[3] = {col.x, col.y, col.z};
    for (int c = 0; c < 3; ++c) {
        const double F0 = 0.04 * (1.0 - q.metal) + q.alb[c] * q.metal;
        const Dual F = cst(F0) + cst(1.0 - F0) * f5;
        const Dual kD = (1.0 - F) * cst(1.0 - q.metal);
        out[c] = max0((kD * cst(q.alb[c] / kPi) + F * spec) * c3[c] * att * NdotL);
    }
}

bool load_pixel(const oracle_cs_view* v, uint32_t W, uint32_t H, uint32_t x, uint32_t y, const float* depth,
                const float* normals, const float* albedo, const float* rough, const float* metal, Pixel& q)
{
    const size_t px = (size_t)y * W + x;
    const double fx = (double)x / W, fy = (double)y / H;
    const double v0[4] = {fx * 2.0 - 1.0, (1.0 - fy) * 2.0 - 1.0, (double)depth[px], 1.0};
    double vv[4];
    for (int r = 0; r < 4; ++r)
        vv[r] = v->inv_proj[r] * v0[0] + v->inv_proj[4 + r] * v0[1] + v->inv_proj[8 + r] * v0[2] + v->inv_proj[12 + r] * v0[3];
    for (int r = 0; r < 4; ++r) vv[r] /= vv[3];
    if (!(vv[2] < (double)v->far_plane - 0.001)) return false;
    for (int r = 0; r < 3; ++r)
        q.p[r] = v->inv_view[r] * vv[0] + v->inv_view[4 + r] * vv[1] + v->inv_view[8 + r] * vv[2] + v->inv_view[12 + r] * vv[3];
    double e[3] = {v->eye[0] - q.p[0], v->eye[1] - q.p[1], v->eye[2] - q.p[2]};
    const double le = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    for (int c = 0; c < 3; ++c) {
        q.V[c] = e[c] / le;
        q.N[c] = normals[3 * px + c];
        q.alb[c] = albedo[3 * px + c];
    }
    q.rough = rough[px];
    q.metal = metal[px];
    return true;
}

struct LightParams {
    V3 lp, col;
    Dual r;
};

LightParams seed_light(const float* lpos, const float* lights, uint32_t l, bool tangents)
{
    LightParams P;
    Dual a[7];
    const double vals[7] = {lpos[4 * l], lpos[4 * l + 1], lpos[4 * l + 2], lights[4 * l], lights[4 * l + 1],
                            lights[4 * l + 2], lights[4 * l + 3]};
    for (int i = 0; i < 7; ++i) {
        a[i] = cst(vals[i]);
        if (tangents) a[i].d[i] = 1.0;
    }
    P.lp = v3(a[0], a[1], a[2]);
    P.col = v3(a[3], a[4], a[5]);
    P.r = a[6];
    return P;
}

}  // namespace

extern "C" void oracle_cs_shade_f64(const oracle_cs_view* v, uint32_t W, uint32_t H, const float* depth,
                                    const float* normals, const float* albedo, const float* rough, const float* metal,
                                    const uint32_t* refs, const uint32_t* counts, const uint32_t* offsets,
                                    const uint32_t* indices, const float* lpos, const float* lights, uint32_t L,
                                    int falloff, int mode, double* out, uint8_t* shaded, int threads)
{
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads > 0 ? threads : 1)
    for (int64_t y = 0; y < (int64_t)H; ++y) {
        for (uint32_t x = 0; x < W; ++x) {
            const size_t px = (size_t)y * W + x;
            Pixel q;
            shaded[px] = 0;
            if (!load_pixel(v, W, H, x, (uint32_t)y, depth, normals, albedo, rough, metal, q)) continue;
            shaded[px] = 1;
            double Lo[3] = {0, 0, 0};
            if (L > 0) {
                const uint32_t c = refs[px];
                for (uint32_t i = 0; i < counts[c]; ++i) {
                    const uint32_t l = indices[offsets[c] + i];
                    LightParams P = seed_light(lpos, lights, l, false);
                    Dual o[3];
                    point_light(q, P.lp, P.col, P.r, falloff, o);
                    for (int k = 0; k < 3; ++k) Lo[k] += o[k].v;
                }
            }
            for (int k = 0; k < 3; ++k) out[3 * px + k] = mode == 0 ? std::pow(0.03 * q.alb[k] + Lo[k], 1.0 / 2.2) : Lo[k];
        }
    }
}

// dLoss/dtheta for Loss = sum_px sum_c grad[px][c] * radiance[px][c]; outputs per light 7 values
// (position xyz, colour rgb, radius) in g7[7*L].
extern "C" void oracle_cs_shade_grad_f64(const oracle_cs_view* v, uint32_t W, uint32_t H, const float* depth,
                                         const float* normals, const float* albedo, const float* rough,
                                         const float* metal, const uint32_t* refs, const uint32_t* counts,
                                         const uint32_t* offsets, const uint32_t* indices, const float* lpos,
                                         const float* lights, uint32_t L, int falloff, const float* grad, double* g7,
                                         int threads)
{
    const int nt = threads > 0 ? threads : 1;
    std::vector<std::vector<double>> acc(nt, std::vector<double>((size_t)L * NT, 0.0));
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        const int tid = omp_get_thread_num();
#else
        const int tid = 0;
#endif
        std::vector<double>& mine = acc[tid];
#pragma omp for schedule(static)
        for (int64_t y = 0; y < (int64_t)H; ++y) {
            for (uint32_t x = 0; x < W; ++x) {
                const size_t px = (size_t)y * W + x;
                Pixel q;
                if (!load_pixel(v, W, H, x, (uint32_t)y, depth, normals, albedo, rough, metal, q)) continue;
                const uint32_t c = refs[px];
                for (uint32_t i = 0; i < counts[c]; ++i) {
                    const uint32_t l = indices[offsets[c] + i];
                    LightParams P = seed_light(lpos, lights, l, true);
                    Dual o[3];
                    point_light(q, P.lp, P.col, P.r, falloff, o);
                    for (int k = 0; k < 3; ++k)
                        for (int t = 0; t < NT; ++t) mine[(size_t)l * NT + t] += (double)grad[3 * px + k] * o[k].d[t];
                }
            }
        }
    }
    for (size_t i = 0; i < (size_t)L * NT; ++i) {
        double s = 0;
        for (int t = 0; t < nt; ++t) s += acc[t][i];
        g7[i] = s;
    }
}

// Loss restricted to the pairs of light `l`, with its 7 parameters replaced by theta (for central
// finite differences: only these pairs depend on the light).
extern "C" double oracle_cs_shade_light_loss_f64(const oracle_cs_view* v, uint32_t W, uint32_t H, const float* depth,
                                                 const float* normals, const float* albedo, const float* rough,
                                                 const float* metal, const uint32_t* refs, const uint32_t* counts,
                                                 const uint32_t* offsets, const uint32_t* indices, uint32_t l,
                                                 const double* theta, int falloff, const float* grad)
{
    double loss = 0.0;
    for (uint32_t y = 0; y < H; ++y) {
        for (uint32_t x = 0; x < W; ++x) {
            const size_t px = (size_t)y * W + x;
            Pixel q;
            if (!load_pixel(v, W, H, x, y, depth, normals, albedo, rough, metal, q)) continue;
            const uint32_t c = refs[px];
            for (uint32_t i = 0; i < counts[c]; ++i) {
                if (indices[offsets[c] + i] != l) continue;
                const V3 lp = v3c(theta[0], theta[1], theta[2]);
                const V3 col = v3c(theta[3], theta[4], theta[5]);
                Dual o[3];
                point_light(q, lp, col, cst(theta[6]), falloff, o);
                for (int k = 0; k < 3; ++k) loss += (double)grad[3 * px + k] * o[k].v;
            }
        }
    }
    return loss;
}

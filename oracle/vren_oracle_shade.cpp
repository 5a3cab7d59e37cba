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
// the same operations on plain doubles (values only: the finite differences)
inline double dsqrt(double a) { return std::sqrt(a); }
inline double max0(double a) { return a > 0.0 ? a : 0.0; }
inline double min1(double a) { return a < 1.0 ? a : 1.0; }
inline double clamp01(double a) { return a <= 0.0 ? 0.0 : (a >= 1.0 ? 1.0 : a); }
template <class T> inline T num(double v);
template <> inline Dual num<Dual>(double v) { return cst(v); }
template <> inline double num<double>(double v) { return v; }

template <class T> struct V3T {
    T x, y, z;
};
using V3 = V3T<Dual>;
inline V3 v3(const Dual& x, const Dual& y, const Dual& z) { return {x, y, z}; }
template <class T> inline V3T<T> v3n(double x, double y, double z) { return {num<T>(x), num<T>(y), num<T>(z)}; }
inline V3 v3c(double x, double y, double z) { return v3n<Dual>(x, y, z); }
template <class T> inline T dot(const V3T<T>& a, const V3T<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline V3T<T> sub(const V3T<T>& a, const V3T<T>& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3T<T> divs(const V3T<T>& a, const T& s) { return {a.x / s, a.y / s, a.z / s}; }

struct Pixel {
    double p[3], N[3], V[3], alb[3], rough, metal;
};

// pbr_apply_point_light for one (pixel, light) pair, returns the three channels; T = Dual carries the
// 7 tangents, T = double evaluates the value only.
template <class T>
void point_light(const Pixel& q, const V3T<T>& lp, const V3T<T>& col, const T& r, int falloff, T out[3])
{
    const V3T<T> p = v3n<T>(q.p[0], q.p[1], q.p[2]);
    const V3T<T> N = v3n<T>(q.N[0], q.N[1], q.N[2]);
    const V3T<T> V = v3n<T>(q.V[0], q.V[1], q.V[2]);
    const V3T<T> d = sub(p, lp);
    const T dist = dsqrt(dot(d, d));
    const V3T<T> L = divs(d, dist);
    T att;
    if (falloff == 0) {
        const T u = min1(dist / r);
        att = 1.0 - u * dsqrt(u);
    } else {
        const T t = dist / r;
        const T t2 = t * t;
        const T w = clamp01(1.0 - t2 * t2);
        att = (w * w) / (dist * dist + num<T>(1.0));
    }
    const V3T<T> hv = sub(V, L);
    const V3T<T> H = divs(hv, dsqrt(dot(hv, hv)));
    const double a2 = q.rough * q.rough;
    const T NdotH = max0(dot(N, H));
    const T D = NdotH * NdotH * num<T>(a2 - 1.0) + num<T>(1.0);
    const T NDF = num<T>(a2) / (kPi * D * D);
    const double k = q.rough;
    const double NdotV = std::max(q.N[0] * q.V[0] + q.N[1] * q.V[1] + q.N[2] * q.V[2], 0.0);
    const T NdotL = max0(-dot(N, L));
    const double ggxV = NdotV / (NdotV * (1.0 - k) + k);
    const T ggxL = NdotL / (NdotL * num<T>(1.0 - k) + num<T>(k));
    const T G = num<T>(ggxV) * ggxL;
    const T HdotV = max0(dot(H, V));
    const T x = 1.0 - HdotV;
    const T f5 = x * x * x * x * x;
    const T spec = NDF * G / (num<T>(4.0 * NdotV) * NdotL + num<T>(0.0001));
    const T c3[3] = {col.x, col.y, col.z};
    for (int c = 0; c < 3; ++c) {
        const double F0 = 0.04 * (1.0 - q.metal) + q.alb[c] * q.metal;
        const T F = num<T>(F0) + num<T>(1.0 - F0) * f5;
        const T kD = (1.0 - F) * num<T>(1.0 - q.metal);
        out[c] = max0((kD * num<T>(q.alb[c] / kPi) + F * spec) * c3[c] * att * NdotL);
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

// The FP64 gradient (forward mode) and the central finite differences with step h of the loss with
// respect to the 7 parameters of each light in `sel` only, evaluating only the (pixel, light) pairs of
// those lights: g7[7 * i + t] and fd7[7 * i + t] for light sel[i] (h <= 0: no differences, fd7 = 0).  The pairs are gathered once (one
// pass over the pixels' lists); each light's 1 + 14 evaluations then run over its own pairs.
extern "C" void oracle_cs_shade_grad_lights_f64(const oracle_cs_view* v, uint32_t W, uint32_t H, const float* depth,
                                                const float* normals, const float* albedo, const float* rough,
                                                const float* metal, const uint32_t* refs, const uint32_t* counts,
                                                const uint32_t* offsets, const uint32_t* indices, const float* lpos,
                                                const float* lights, uint32_t L, int falloff, const float* grad,
                                                const uint32_t* sel, uint32_t nsel, double h, double* g7, double* fd7,
                                                uint64_t* pair_counts, int threads)
{
    const int nt = threads > 0 ? threads : 1;
    std::vector<int32_t> slot(L, -1);
    for (uint32_t i = 0; i < nsel; ++i)
        if (sel[i] < L) slot[sel[i]] = (int32_t)i;
    // pairs per selected light, gathered per thread then merged in row order
    std::vector<std::vector<std::vector<uint32_t>>> part(nt, std::vector<std::vector<uint32_t>>(nsel));
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        const int tid = omp_get_thread_num();
#else
        const int tid = 0;
#endif
#pragma omp for schedule(static)
        for (int64_t y = 0; y < (int64_t)H; ++y)
            for (uint32_t x = 0; x < W; ++x) {
                const size_t px = (size_t)y * W + x;
                const uint32_t c = refs[px];
                for (uint32_t i = 0; i < counts[c]; ++i) {
                    const uint32_t l = indices[offsets[c] + i];
                    if (l < L && slot[l] >= 0) part[tid][slot[l]].push_back((uint32_t)px);
                }
            }
    }
    std::vector<std::vector<uint32_t>> pairs(nsel);
    for (uint32_t i = 0; i < nsel; ++i)
        for (int t = 0; t < nt; ++t) pairs[i].insert(pairs[i].end(), part[t][i].begin(), part[t][i].end());
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t i = 0; i < (int64_t)nsel; ++i) {
        const uint32_t l = sel[i];
        double g[NT] = {0, 0, 0, 0, 0, 0, 0};
        double fp[NT] = {0, 0, 0, 0, 0, 0, 0}, fm[NT] = {0, 0, 0, 0, 0, 0, 0};
        const double base[NT] = {lpos[4 * l], lpos[4 * l + 1], lpos[4 * l + 2], lights[4 * l], lights[4 * l + 1],
                                 lights[4 * l + 2], lights[4 * l + 3]};
        pair_counts[i] = pairs[i].size();
        for (uint32_t px : pairs[i]) {
            Pixel q;
            const uint32_t x = px % W, y = px / W;
            if (!load_pixel(v, W, H, x, y, depth, normals, albedo, rough, metal, q)) continue;
            LightParams P = seed_light(lpos, lights, l, true);
            Dual o[3];
            point_light(q, P.lp, P.col, P.r, falloff, o);
            for (int k = 0; k < 3; ++k)
                for (int t = 0; t < NT; ++t) g[t] += (double)grad[3 * px + k] * o[k].d[t];
            for (int t = 0; t < NT && h > 0.0; ++t) {
                for (int sgn = 0; sgn < 2; ++sgn) {
                    double th[NT];
                    for (int u = 0; u < NT; ++u) th[u] = base[u];
                    th[t] += sgn ? -h : h;
                    double e[3];
                    point_light<double>(q, v3n<double>(th[0], th[1], th[2]), v3n<double>(th[3], th[4], th[5]), th[6],
                                        falloff, e);
                    double s = 0.0;
                    for (int k = 0; k < 3; ++k) s += (double)grad[3 * px + k] * e[k];
                    (sgn ? fm : fp)[t] += s;
                }
            }
        }
        for (int t = 0; t < NT; ++t) {
            g7[7 * i + t] = g[t];
            fd7[7 * i + t] = (fp[t] - fm[t]) / (2.0 * h);
        }
    }
}

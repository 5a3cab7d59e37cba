// Clustered Cook-Torrance/GGX shading (vren/resources/shaders/clustered_shading/shade.comp:69-141,
// vren/resources/shaders/pbr.glsl:6-112) and its hand-written adjoint with respect to the point
// lights' positions, colours and radii (the light-to-cluster assignment held fixed).
//
// Both passes work tile by tile (one CTA per 32x32 tile).  The CTA stages the tile's pixels in
// shared memory (world position, normal, view vector, material, upstream gradient), then groups
// them by cluster with a stable compaction, so a warp always works on pixels that share one light
// list: no lane idles on another cluster's lights, and every light record a warp reads is the same
// for all its lanes.
// Forward: a warp takes 32 pixels of one cluster and walks the cluster's lights.
// Adjoint (deterministic, nothing stored per (pixel, light) pair):
//   1. a warp takes one (cluster, light) slot of the tile and sums the pair gradients over the
//      cluster's pixels - lanes stride them in pixel order, then a fixed butterfly reduction - into
//      one 7-float partial per slot;
//   2. the slots are grouped by light with the stable bucket sort of (light, slot) pairs;
//   3. one warp per light sums its slots' partials in slot order.
//
// The world position of a pixel is reconstructed as an unevaluated sum of two floats (about 44
// significant bits), and a light's offset is formed as (p_hi - light) + p_lo: lights sit within
// a fraction of a unit of surfaces hundreds of units from the camera, where rounding p to single
// precision first would cost the offset (and the gradient, which scales with 1 / distance) four
// significant digits.
#include "common.cuh"
#include "internal.h"

#include <cstring>

namespace vren_gb300 {

VREN_DEFINE_ERROR_WORD(shade)

constexpr float kPi = 3.14f;  // common.glsl:6

struct ShadeArgs {
    const vren_cs_frame* frame;
    uint32_t W, H;
    vren_cs_gbuffer g;
    vren_cs_light_lists lists;
    const float4* lpos;
    const float4* lights;
    uint32_t L;
    const float4* dir;  // {direction, pad}, {color, pad}
    uint32_t ndir;
    int falloff;
    int mode;
    float* out;
    int packed;  // forward: two lights per step in packed f32x2 arithmetic (VREN_TUNE_SHADE_PACKED)
};

// Per-pixel shading state: position (p + plo), geometry, and the terms of pbr_apply_light that
// depend on the pixel alone.
struct Px {
    float p[3], plo[3], N[3], V[3];
    float a2, k, k1, omn2, NdotV, ggxV, nv4;
    float F0[3], omF0[3], kdiff[3];  // Fresnel F0, 1 - F0, (1 - metallic) albedo / PI
};

__device__ __forceinline__ float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// a x b, each component one product and one fused multiply-add (accurate when the result is small).
__device__ __forceinline__ void cross3(const float* a, const float* b, float* c)
{
    c[0] = fmaf(a[1], b[2], -(a[2] * b[1]));
    c[1] = fmaf(a[2], b[0], -(a[0] * b[2]));
    c[2] = fmaf(a[0], b[1], -(a[1] * b[0]));
}

// Hardware approximations (PTX rcp/rsqrt/sqrt .approx, about one ulp): the shading is compared with
// an FP64 evaluation to 1e-5..1e-4, not bit for bit.
__device__ __forceinline__ float rcp_a(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_a(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sqrt_a(float x)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// ------------------------------------------------------------------------------------------------
// Double-float arithmetic: x = hi + lo with |lo| <= ulp(hi) / 2.  Knuth's two-sum and the fused
// multiply-add two-product are error-free transformations (Dekker 1971; Ogita, Rump, Oishi 2005).
// ------------------------------------------------------------------------------------------------
struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ ff two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, fmaf(a, b, -p)};
}

__device__ __forceinline__ ff ff_add(ff a, ff b)
{
    const ff s = two_sum(a.hi, b.hi);
    return two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ ff ff_mul_f(ff a, float c)
{
    const ff p = two_prod(a.hi, c);
    return two_sum(p.hi, fmaf(a.lo, c, p.lo));
}

__device__ __forceinline__ ff ff_div(ff a, ff b)
{
    const float q = __fdiv_rn(a.hi, b.hi);
    const ff qb = ff_mul_f(b, q);
    const ff r = ff_add(a, {-qb.hi, -qb.lo});
    return two_sum(q, __fdiv_rn(r.hi, b.hi));
}

// x / n as double-float for integers x, n < 2^24: the remainder of the correctly rounded quotient
// is exactly representable, so one fused multiply-add recovers it.
__device__ __forceinline__ ff ratio(uint32_t x, uint32_t n)
{
    const float fx = (float)x, fn = (float)n;
    const float q = __fdiv_rn(fx, fn);
    return {q, __fdiv_rn(fmaf(-q, fn, fx), fn)};
}

// World position of pixel (x, y) as p + plo; returns false when the pixel is not shaded
// (shade.comp:86: view depth at the far plane).  A non-finite depth takes the single-precision
// path of the same formulas (plo = 0).
__device__ __forceinline__ bool pixel_world(const vren_cs_frame* F, uint32_t x, uint32_t y, uint32_t W, uint32_t H,
                                            float D, float p[3], float plo[3])
{
    const float* ip = F->view.inv_proj;
    const float* iv = F->view.inv_view;
    if (!isfinite(D)) {
        const float nx = ((float)x / (float)W) * 2.0f - 1.0f, ny = (1.0f - (float)y / (float)H) * 2.0f - 1.0f;
        float v[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) v[r] = ip[r] * nx + ip[4 + r] * ny + ip[8 + r] * D + ip[12 + r];
#pragma unroll
        for (int r = 0; r < 3; ++r) v[r] = v[r] / v[3];
        if (!(v[2] < F->view.far_plane - 0.001f)) return false;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            p[r] = iv[r] * v[0] + iv[4 + r] * v[1] + iv[8 + r] * v[2] + iv[12 + r];
            plo[r] = 0.0f;
        }
        return true;
    }
    const ff fx = ratio(x, W), fy = ratio(y, H);
    // NDC: fx * 2 - 1 and (1 - fy) * 2 - 1 = 1 - 2 fy (doubling is exact)
    const ff nx = ff_add(two_sum(2.0f * fx.hi, -1.0f), {2.0f * fx.lo, 0.0f});
    const ff ny = ff_add(two_sum(1.0f, -2.0f * fy.hi), {-2.0f * fy.lo, 0.0f});
    ff v[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        ff acc = ff_add(two_prod(ip[8 + r], D), {ip[12 + r], 0.0f});
        acc = ff_add(acc, ff_mul_f(nx, ip[r]));
        v[r] = ff_add(acc, ff_mul_f(ny, ip[4 + r]));
    }
    ff vv[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) vv[r] = ff_div(v[r], v[3]);
    if (!(vv[2].hi < F->view.far_plane - 0.001f)) return false;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        ff acc = ff_add(ff_mul_f(vv[0], iv[r]), {iv[12 + r], 0.0f});
        acc = ff_add(acc, ff_mul_f(vv[1], iv[4 + r]));
        acc = ff_add(acc, ff_mul_f(vv[2], iv[8 + r]));
        p[r] = acc.hi;
        plo[r] = acc.lo;
    }
    return true;
}

// 1 - |n|^2 to within a few ulps of its own size: the squares as exact product pairs, summed with
// two-sum, then 1 - hi (exact for hi in [0.5, 2]) - lo.
__device__ __forceinline__ float one_minus_norm2(const float* n)
{
    float hi = 0.0f, lo = 0.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const ff sq = two_prod(n[c], n[c]);
        const ff s = two_sum(hi, sq.hi);
        hi = s.hi;
        lo = __fadd_rn(lo, __fadd_rn(s.lo, sq.lo));
    }
    return __fsub_rn(__fsub_rn(1.0f, hi), lo);
}

// View vector and the pixel-only terms, from p + plo, N, albedo, roughness and metallic.
__device__ __forceinline__ void px_terms(Px& q, const float* eye, const float alb[3], float rough, float metal)
{
    const float e[3] = {(eye[0] - q.p[0]) - q.plo[0], (eye[1] - q.p[1]) - q.plo[1], (eye[2] - q.p[2]) - q.plo[2]};
    const float le = sqrtf(dot3(e, e));
#pragma unroll
    for (int c = 0; c < 3; ++c) q.V[c] = e[c] / le;
    q.a2 = rough * rough;
    q.k = rough;  // pbr.glsl:14-22 uses k = roughness
    q.k1 = 1.0f - rough;
    q.omn2 = one_minus_norm2(q.N);
    q.NdotV = fmaxf(dot3(q.N, q.V), 0.0f);
    q.ggxV = q.NdotV / fmaf(q.NdotV, q.k1, q.k);
    q.nv4 = 4.0f * q.NdotV;
    const float m1 = 1.0f - metal;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        q.F0[c] = fmaf(alb[c], metal, 0.04f * m1);
        q.omF0[c] = 1.0f - q.F0[c];
        q.kdiff[c] = m1 * alb[c] / kPi;
    }
}

// Light offset d = p - light position with the low part of p folded in.
__device__ __forceinline__ void light_offset(const Px& q, float4 lp, float d[3])
{
    d[0] = (q.p[0] - lp.x) + q.plo[0];
    d[1] = (q.p[1] - lp.y) + q.plo[1];
    d[2] = (q.p[2] - lp.z) + q.plo[2];
}

// GGX denominator D = NdotH^2 (a2 - 1) + 1 (pbr.glsl:24-35) for NdotH = max(N.H, 0), H = hv / |hv|,
// given nhu = N.hv and rhl = 1 / |hv|.  Written as a2 h^2 + (1 - h^2) with Lagrange's identity
//     1 - (N.H)^2 = ((1 - |N|^2) |hv|^2 + |N x hv|^2) / |hv|^2,
// whose terms stay accurate near the specular peak, where 1 - (N.H)^2 computed from a rounded N.H
// would cancel (a2 = roughness^2 can be 0.0025, so D's relative error there would be ~1e-4).
__device__ __forceinline__ float ggx_den(const Px& q, const float* hv, float nhu, float hl2, float rhl)
{
    if (!(nhu > 0.0f)) return 1.0f;
    float c[3];
    cross3(q.N, hv, c);
    return (q.a2 * nhu * nhu + fmaf(hl2, q.omn2, dot3(c, c))) * (rhl * rhl);
}

// pbr_apply_light (pbr.glsl:42-73) for light direction L (from the light towards the point) and
// radiance; accumulates into out.
__device__ __forceinline__ void brdf_accumulate(const Px& q, const float L[3], const float rad[3], float out[3])
{
    const float hv[3] = {q.V[0] - L[0], q.V[1] - L[1], q.V[2] - L[2]};
    const float hl2 = dot3(hv, hv);
    const float rhl = rsqrt_a(hl2);
    const float H[3] = {hv[0] * rhl, hv[1] * rhl, hv[2] * rhl};
    const float D = ggx_den(q, hv, dot3(q.N, hv), hl2, rhl);
    const float NDF = q.a2 * rcp_a(kPi * D * D);
    const float NdotL = fmaxf(-dot3(q.N, L), 0.0f);
    const float G = q.ggxV * NdotL * rcp_a(fmaf(NdotL, q.k1, q.k));
    const float HdotV = fmaxf(dot3(H, q.V), 0.0f);
    const float x = 1.0f - HdotV;
    const float x2 = x * x;
    const float f5 = x2 * x2 * x;
    const float spec = NDF * G * rcp_a(fmaf(q.nv4, NdotL, 0.0001f));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float F = fmaf(q.omF0[c], f5, q.F0[c]);
        const float B = fmaf(1.0f - F, q.kdiff[c], F * spec);
        out[c] += fmaxf(B * rad[c] * NdotL, 0.0f);
    }
}

// Attenuation: reference 1 - min(d/r, 1)^1.5 (pbr.glsl:89) or windowed inverse square.
__device__ __forceinline__ float falloff_value(int mode, float dist, float dd, float rr)
{
    const float t = dist * rr;
    if (mode == VREN_CS_FALLOFF_REF) {
        const float u = fminf(t, 1.0f);
        return 1.0f - u * sqrt_a(u);
    }
    const float t2 = t * t;
    const float w = fminf(fmaxf(1.0f - t2 * t2, 0.0f), 1.0f);
    return w * w * rcp_a(dd + 1.0f);
}

// pbr_apply_point_light (pbr.glsl:75-93) for one light.
// ------------------------------------------------------------------------------------------------
// Two lights at once in packed single-precision pairs (Blackwell's f32x2 add / mul / fma: one
// instruction for both lights), the same operations as point_light_fwd per light; the contributions
// are added to `out` in list order (light 0, then light 1), as the one-light loop does.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 pk2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }
__device__ __forceinline__ float2 dot3x2(const float2* a, const float2* b)
{
    return fma2(a[2], b[2], fma2(a[1], b[1], mul2(a[0], b[0])));
}

__device__ __forceinline__ void point_light_fwd2(const Px& q, float4 lp0, float4 lc0, float4 lp1, float4 lc1,
                                                 int falloff, float out[3])
{
    float2 d[3];
    d[0] = add2(sub2(bc2(q.p[0]), pk2(lp0.x, lp1.x)), bc2(q.plo[0]));
    d[1] = add2(sub2(bc2(q.p[1]), pk2(lp0.y, lp1.y)), bc2(q.plo[1]));
    d[2] = add2(sub2(bc2(q.p[2]), pk2(lp0.z, lp1.z)), bc2(q.plo[2]));
    const float2 dd = dot3x2(d, d);
    const float2 rdist = pk2(rsqrt_a(dd.x), rsqrt_a(dd.y));
    const float2 L[3] = {mul2(d[0], rdist), mul2(d[1], rdist), mul2(d[2], rdist)};
    // falloff_value for both lights
    const float2 t = mul2(mul2(dd, rdist), pk2(rcp_a(lc0.w), rcp_a(lc1.w)));
    float2 att;
    if (falloff == VREN_CS_FALLOFF_REF) {
        const float2 u = pk2(fminf(t.x, 1.0f), fminf(t.y, 1.0f));
        att = sub2(bc2(1.0f), mul2(u, pk2(sqrt_a(u.x), sqrt_a(u.y))));
    } else {
        const float2 t2 = mul2(t, t);
        const float2 om = sub2(bc2(1.0f), mul2(t2, t2));
        const float2 w = pk2(fminf(fmaxf(om.x, 0.0f), 1.0f), fminf(fmaxf(om.y, 0.0f), 1.0f));
        const float2 den = add2(dd, bc2(1.0f));
        att = mul2(mul2(w, w), pk2(rcp_a(den.x), rcp_a(den.y)));
    }
    const float2 rad[3] = {mul2(pk2(lc0.x, lc1.x), att), mul2(pk2(lc0.y, lc1.y), att), mul2(pk2(lc0.z, lc1.z), att)};
    // brdf_accumulate for both lights
    const float2 N2[3] = {bc2(q.N[0]), bc2(q.N[1]), bc2(q.N[2])};
    const float2 V2[3] = {bc2(q.V[0]), bc2(q.V[1]), bc2(q.V[2])};
    const float2 hv[3] = {sub2(V2[0], L[0]), sub2(V2[1], L[1]), sub2(V2[2], L[2])};
    const float2 hl2 = dot3x2(hv, hv);
    const float2 rhl = pk2(rsqrt_a(hl2.x), rsqrt_a(hl2.y));
    const float2 H[3] = {mul2(hv[0], rhl), mul2(hv[1], rhl), mul2(hv[2], rhl)};
    const float2 nhu = dot3x2(N2, hv);
    // ggx_den: a2 h^2 + ((1 - |N|^2) |hv|^2 + |N x hv|^2) / |hv|^2 where N.hv > 0, else 1
    float2 c[3];
    c[0] = fma2(N2[1], hv[2], mul2(bc2(-q.N[2]), hv[1]));
    c[1] = fma2(N2[2], hv[0], mul2(bc2(-q.N[0]), hv[2]));
    c[2] = fma2(N2[0], hv[1], mul2(bc2(-q.N[1]), hv[0]));
    const float2 gd = mul2(fma2(mul2(bc2(q.a2), nhu), nhu, fma2(hl2, bc2(q.omn2), dot3x2(c, c))), mul2(rhl, rhl));
    const float2 D = pk2(nhu.x > 0.0f ? gd.x : 1.0f, nhu.y > 0.0f ? gd.y : 1.0f);
    const float2 dpi = mul2(mul2(bc2(kPi), D), D);
    const float2 NDF = mul2(bc2(q.a2), pk2(rcp_a(dpi.x), rcp_a(dpi.y)));
    const float2 nl = dot3x2(N2, L);
    const float2 NdotL = pk2(fmaxf(-nl.x, 0.0f), fmaxf(-nl.y, 0.0f));
    const float2 gden = fma2(NdotL, bc2(q.k1), bc2(q.k));
    const float2 G = mul2(mul2(bc2(q.ggxV), NdotL), pk2(rcp_a(gden.x), rcp_a(gden.y)));
    const float2 hdv = dot3x2(H, V2);
    const float2 x = sub2(bc2(1.0f), pk2(fmaxf(hdv.x, 0.0f), fmaxf(hdv.y, 0.0f)));
    const float2 x2 = mul2(x, x);
    const float2 f5 = mul2(mul2(x2, x2), x);
    const float2 sden = fma2(bc2(q.nv4), NdotL, bc2(0.0001f));
    const float2 spec = mul2(mul2(NDF, G), pk2(rcp_a(sden.x), rcp_a(sden.y)));
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const float2 F = fma2(bc2(q.omF0[ch]), f5, bc2(q.F0[ch]));
        const float2 B = fma2(sub2(bc2(1.0f), F), bc2(q.kdiff[ch]), mul2(F, spec));
        const float2 v = mul2(mul2(B, rad[ch]), NdotL);
        out[ch] += fmaxf(v.x, 0.0f);
        out[ch] += fmaxf(v.y, 0.0f);
    }
}

__device__ __forceinline__ void point_light_fwd(const Px& q, float4 lp, float4 lc, int falloff, float out[3])
{
    float d[3];
    light_offset(q, lp, d);
    const float dd = dot3(d, d);
    const float rdist = rsqrt_a(dd);
    const float Ld[3] = {d[0] * rdist, d[1] * rdist, d[2] * rdist};
    const float att = falloff_value(falloff, dd * rdist, dd, rcp_a(lc.w));
    const float rad[3] = {lc.x * att, lc.y * att, lc.z * att};
    brdf_accumulate(q, Ld, rad, out);
}

// ------------------------------------------------------------------------------------------------
// Adjoint of one (pixel, light) pair: accumulates dLoss/d(position, colour, radius) into g7 for the
// upstream gradient gin of the pair's radiance (reverse mode through pbr_apply_point_light).
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ void pair_backward(const Px& q, float4 lp, float4 lc, int falloff, const float gin[3],
                                              float g7[7])
{
    const float rr = rcp_a(lc.w);
    float d[3];
    light_offset(q, lp, d);
    const float dd = dot3(d, d);
    const float rdist = rsqrt_a(dd);
    const float dist = dd * rdist;
    const float L[3] = {d[0] * rdist, d[1] * rdist, d[2] * rdist};
    const float t = dist * rr;
    float att, datt_dt, datt_ddist_direct = 0.0f;
    if (falloff == VREN_CS_FALLOFF_REF) {
        const float u = fminf(t, 1.0f);
        const float su = sqrt_a(u);
        att = 1.0f - u * su;
        datt_dt = t < 1.0f ? -1.5f * su : 0.0f;
    } else {
        const float t2 = t * t;
        const float wr = 1.0f - t2 * t2;
        const float w = fminf(fmaxf(wr, 0.0f), 1.0f);
        const float rden = rcp_a(dd + 1.0f);
        att = w * w * rden;
        const float dw_dt = (wr > 0.0f && wr < 1.0f) ? -4.0f * t2 * t : 0.0f;
        datt_dt = 2.0f * w * rden * dw_dt;
        datt_ddist_direct = -w * w * 2.0f * dist * rden * rden;
    }
    const float col[3] = {lc.x, lc.y, lc.z};

    const float hv[3] = {q.V[0] - L[0], q.V[1] - L[1], q.V[2] - L[2]};
    const float hl2 = dot3(hv, hv);
    const float rhl = rsqrt_a(hl2);
    const float H[3] = {hv[0] * rhl, hv[1] * rhl, hv[2] * rhl};
    const float nhu = dot3(q.N, hv);  // |hv| (N.H)
    const float NdotH = fmaxf(nhu * rhl, 0.0f);
    const float D = ggx_den(q, hv, nhu, hl2, rhl);
    const float rD = rcp_a(D);
    const float NDF = q.a2 * (rD * rD) * (1.0f / kPi);
    const float nl_raw = -dot3(q.N, L);
    const float NdotL = fmaxf(nl_raw, 0.0f);
    const float rdl = rcp_a(fmaf(NdotL, q.k1, q.k));
    const float G = q.ggxV * NdotL * rdl;
    const float hvr = dot3(H, q.V);
    const float HdotV = fmaxf(hvr, 0.0f);
    const float x = 1.0f - HdotV;
    const float x2 = x * x;
    const float x4 = x2 * x2;
    const float f5 = x4 * x;
    const float rs = rcp_a(fmaf(q.nv4, NdotL, 0.0001f));
    const float spec = NDF * G * rs;

    const float an = att * NdotL;
    float gatt = 0.0f, gNdotL = 0.0f, gspec = 0.0f, gf5 = 0.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float F = fmaf(q.omF0[c], f5, q.F0[c]);
        const float B = fmaf(1.0f - F, q.kdiff[c], F * spec);
        const float gv = B * col[c] * an > 0.0f ? gin[c] : 0.0f;
        const float gvB = gv * B;
        const float gB = gv * col[c] * an;
        g7[3 + c] += gvB * an;  // colour
        gatt += gvB * col[c] * NdotL;
        gNdotL += gvB * col[c] * att;
        gspec += gB * F;
        gf5 += gB * (spec - q.kdiff[c]) * q.omF0[c];
    }
    const float gHdotV = -5.0f * gf5 * x4;
    const float gNDF = gspec * G * rs;
    const float gG = gspec * NDF * rs;
    gNdotL += -gspec * spec * rs * q.nv4;             // through the specular denominator
    gNdotL += gG * q.ggxV * q.k * (rdl * rdl);        // d(NdotL / (NdotL (1 - k) + k))
    const float gNdotH = gNDF * (-4.0f * (q.a2 - 1.0f) * NdotH) * NDF * rD;
    const float gnl = nl_raw > 0.0f ? gNdotL : 0.0f;
    const float gnh = nhu > 0.0f ? gNdotH : 0.0f;
    const float ghv = hvr > 0.0f ? gHdotV : 0.0f;
    // Through H = hv / |hv| and hv = V - L: d(N.H)/dhv = (N - (N.H) H) / |hv|, written as
    // hv x (N x hv) / |hv|^3 (no cancellation near the peak); d(H.V)/dhv = (V - (H.V) H) / |hv|.
    float nxh[3], tri[3];
    cross3(q.N, hv, nxh);
    cross3(hv, nxh, tri);
    const float sn = gnh * rhl * rhl * rhl, sv = ghv * rhl;
    float gL[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) gL[c] = -gnl * q.N[c] - sn * tri[c] - sv * (q.V[c] - H[c] * hvr);
    // attenuation: t = dist / r
    const float gt = gatt * datt_dt;
    const float gdist = gatt * datt_ddist_direct + gt * rr;
    g7[6] += -gt * dist * rr * rr;  // radius
    const float gLL = dot3(gL, L);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float gd = (gL[c] - L[c] * gLL) * rdist + gdist * L[c];
        g7[c] += -gd;  // d = p - light position
    }
}

// pair_backward for two lights at once (same pixel) in packed f32x2 arithmetic: the same operations
// per light; g7a and g7b receive the two lights' partials.
__device__ __forceinline__ float2 sel2(bool cx, float2 a, float ax, bool cy, float ay)
{
    return make_float2(cx ? a.x : ax, cy ? a.y : ay);
}

__device__ __forceinline__ void cross3x2(const float2* a, const float2* b, float2* c)
{
    c[0] = fma2(a[1], b[2], mul2(make_float2(-a[2].x, -a[2].y), b[1]));
    c[1] = fma2(a[2], b[0], mul2(make_float2(-a[0].x, -a[0].y), b[2]));
    c[2] = fma2(a[0], b[1], mul2(make_float2(-a[1].x, -a[1].y), b[0]));
}

__device__ __forceinline__ void pair_backward2(const Px& q, float4 lp0, float4 lc0, float4 lp1, float4 lc1,
                                               int falloff, const float gin[3], float g7a[7], float g7b[7])
{
    const float2 rr = pk2(rcp_a(lc0.w), rcp_a(lc1.w));
    float2 d[3];
    d[0] = add2(sub2(bc2(q.p[0]), pk2(lp0.x, lp1.x)), bc2(q.plo[0]));
    d[1] = add2(sub2(bc2(q.p[1]), pk2(lp0.y, lp1.y)), bc2(q.plo[1]));
    d[2] = add2(sub2(bc2(q.p[2]), pk2(lp0.z, lp1.z)), bc2(q.plo[2]));
    const float2 dd = dot3x2(d, d);
    const float2 rdist = pk2(rsqrt_a(dd.x), rsqrt_a(dd.y));
    const float2 dist = mul2(dd, rdist);
    const float2 L[3] = {mul2(d[0], rdist), mul2(d[1], rdist), mul2(d[2], rdist)};
    const float2 t = mul2(dist, rr);
    float2 att, datt_dt, datt_ddist_direct = bc2(0.0f);
    if (falloff == VREN_CS_FALLOFF_REF) {
        const float2 u = pk2(fminf(t.x, 1.0f), fminf(t.y, 1.0f));
        const float2 su = pk2(sqrt_a(u.x), sqrt_a(u.y));
        att = sub2(bc2(1.0f), mul2(u, su));
        const float2 m = mul2(bc2(-1.5f), su);
        datt_dt = sel2(t.x < 1.0f, m, 0.0f, t.y < 1.0f, 0.0f);
    } else {
        const float2 t2 = mul2(t, t);
        const float2 wr = sub2(bc2(1.0f), mul2(t2, t2));
        const float2 w = pk2(fminf(fmaxf(wr.x, 0.0f), 1.0f), fminf(fmaxf(wr.y, 0.0f), 1.0f));
        const float2 den = add2(dd, bc2(1.0f));
        const float2 rden = pk2(rcp_a(den.x), rcp_a(den.y));
        const float2 ww = mul2(w, w);
        att = mul2(ww, rden);
        const float2 dw = mul2(mul2(bc2(-4.0f), t2), t);
        const float2 dw_dt = sel2(wr.x > 0.0f && wr.x < 1.0f, dw, 0.0f, wr.y > 0.0f && wr.y < 1.0f, 0.0f);
        datt_dt = mul2(mul2(mul2(bc2(2.0f), w), rden), dw_dt);
        datt_ddist_direct = mul2(mul2(mul2(mul2(make_float2(-ww.x, -ww.y), bc2(2.0f)), dist), rden), rden);
    }
    const float2 col[3] = {pk2(lc0.x, lc1.x), pk2(lc0.y, lc1.y), pk2(lc0.z, lc1.z)};

    const float2 N2[3] = {bc2(q.N[0]), bc2(q.N[1]), bc2(q.N[2])};
    const float2 V2[3] = {bc2(q.V[0]), bc2(q.V[1]), bc2(q.V[2])};
    const float2 hv[3] = {sub2(V2[0], L[0]), sub2(V2[1], L[1]), sub2(V2[2], L[2])};
    const float2 hl2 = dot3x2(hv, hv);
    const float2 rhl = pk2(rsqrt_a(hl2.x), rsqrt_a(hl2.y));
    const float2 H[3] = {mul2(hv[0], rhl), mul2(hv[1], rhl), mul2(hv[2], rhl)};
    const float2 nhu = dot3x2(N2, hv);
    const float2 nh = mul2(nhu, rhl);
    const float2 NdotH = pk2(fmaxf(nh.x, 0.0f), fmaxf(nh.y, 0.0f));
    float2 nxh[3];
    cross3x2(N2, hv, nxh);
    const float2 gd = mul2(fma2(mul2(bc2(q.a2), nhu), nhu, fma2(hl2, bc2(q.omn2), dot3x2(nxh, nxh))), mul2(rhl, rhl));
    const float2 D = sel2(nhu.x > 0.0f, gd, 1.0f, nhu.y > 0.0f, 1.0f);
    const float2 rD = pk2(rcp_a(D.x), rcp_a(D.y));
    const float2 NDF = mul2(mul2(bc2(q.a2), mul2(rD, rD)), bc2(1.0f / kPi));
    const float2 nl_raw = mul2(bc2(-1.0f), dot3x2(N2, L));
    const float2 NdotL = pk2(fmaxf(nl_raw.x, 0.0f), fmaxf(nl_raw.y, 0.0f));
    const float2 gden = fma2(NdotL, bc2(q.k1), bc2(q.k));
    const float2 rdl = pk2(rcp_a(gden.x), rcp_a(gden.y));
    const float2 G = mul2(mul2(bc2(q.ggxV), NdotL), rdl);
    const float2 hvr = dot3x2(H, V2);
    const float2 HdotV = pk2(fmaxf(hvr.x, 0.0f), fmaxf(hvr.y, 0.0f));
    const float2 x = sub2(bc2(1.0f), HdotV);
    const float2 x2 = mul2(x, x);
    const float2 x4 = mul2(x2, x2);
    const float2 f5 = mul2(x4, x);
    const float2 sden = fma2(bc2(q.nv4), NdotL, bc2(0.0001f));
    const float2 rs = pk2(rcp_a(sden.x), rcp_a(sden.y));
    const float2 spec = mul2(mul2(NDF, G), rs);

    const float2 an = mul2(att, NdotL);
    float2 gatt = bc2(0.0f), gNdotL = bc2(0.0f), gspec = bc2(0.0f), gf5 = bc2(0.0f);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float2 F = fma2(bc2(q.omF0[c]), f5, bc2(q.F0[c]));
        const float2 B = fma2(sub2(bc2(1.0f), F), bc2(q.kdiff[c]), mul2(F, spec));
        const float2 bca = mul2(mul2(B, col[c]), an);
        const float2 gv = pk2(bca.x > 0.0f ? gin[c] : 0.0f, bca.y > 0.0f ? gin[c] : 0.0f);
        const float2 gvB = mul2(gv, B);
        const float2 gB = mul2(mul2(gv, col[c]), an);
        const float2 gcol = mul2(gvB, an);
        g7a[3 + c] += gcol.x;  // colour
        g7b[3 + c] += gcol.y;
        gatt = fma2(mul2(gvB, col[c]), NdotL, gatt);
        gNdotL = fma2(mul2(gvB, col[c]), att, gNdotL);
        gspec = fma2(gB, F, gspec);
        gf5 = fma2(mul2(gB, sub2(spec, bc2(q.kdiff[c]))), bc2(q.omF0[c]), gf5);
    }
    const float2 gHdotV = mul2(mul2(bc2(-5.0f), gf5), x4);
    const float2 gNDF = mul2(mul2(gspec, G), rs);
    const float2 gG = mul2(mul2(gspec, NDF), rs);
    gNdotL = add2(gNdotL, mul2(mul2(mul2(mul2(make_float2(-gspec.x, -gspec.y), spec), rs), bc2(1.0f)), bc2(q.nv4)));
    gNdotL = add2(gNdotL, mul2(mul2(mul2(gG, bc2(q.ggxV)), bc2(q.k)), mul2(rdl, rdl)));
    const float2 gNdotH = mul2(mul2(mul2(gNDF, mul2(bc2(-4.0f * (q.a2 - 1.0f)), NdotH)), NDF), rD);
    const float2 gnl = sel2(nl_raw.x > 0.0f, gNdotL, 0.0f, nl_raw.y > 0.0f, 0.0f);
    const float2 gnh = sel2(nhu.x > 0.0f, gNdotH, 0.0f, nhu.y > 0.0f, 0.0f);
    const float2 ghv = sel2(hvr.x > 0.0f, gHdotV, 0.0f, hvr.y > 0.0f, 0.0f);
    float2 tri[3];
    cross3x2(hv, nxh, tri);
    const float2 rhl3 = mul2(mul2(rhl, rhl), rhl);
    const float2 sn = mul2(gnh, rhl3), sv = mul2(ghv, rhl);
    float2 gL[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float2 vh = sub2(V2[c], mul2(H[c], hvr));
        gL[c] = sub2(sub2(mul2(make_float2(-gnl.x, -gnl.y), N2[c]), mul2(sn, tri[c])), mul2(sv, vh));
    }
    const float2 gt = mul2(gatt, datt_dt);
    const float2 gdist = fma2(gatt, datt_ddist_direct, mul2(gt, rr));
    const float2 grad_r = mul2(mul2(mul2(make_float2(-gt.x, -gt.y), dist), rr), rr);
    g7a[6] += grad_r.x;  // radius
    g7b[6] += grad_r.y;
    const float2 gLL = dot3x2(gL, L);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float2 gd = fma2(sub2(gL[c], mul2(L[c], gLL)), rdist, mul2(gdist, L[c]));
        g7a[c] -= gd.x;  // d = p - light position
        g7b[c] -= gd.y;
    }
}

// Per-pixel record staged in shared memory by the adjoint (96 bytes).
struct PxRec {
    float4 p_ref;     // p.xyz, cluster reference (bits; 0xFFFFFFFF = not shaded)
    float4 n_rough;   // N.xyz, roughness
    float4 v_metal;   // V.xyz, metallic
    float4 alb_nv;    // albedo.xyz, NdotV
    float4 g;         // upstream gradient, 1 - |N|^2
    float4 plo;       // low part of p, ggxV
};

__device__ __forceinline__ void rec_to_px(const PxRec& rec, Px& q)
{
    q.p[0] = rec.p_ref.x; q.p[1] = rec.p_ref.y; q.p[2] = rec.p_ref.z;
    q.plo[0] = rec.plo.x; q.plo[1] = rec.plo.y; q.plo[2] = rec.plo.z;
    q.N[0] = rec.n_rough.x; q.N[1] = rec.n_rough.y; q.N[2] = rec.n_rough.z;
    q.V[0] = rec.v_metal.x; q.V[1] = rec.v_metal.y; q.V[2] = rec.v_metal.z;
    const float rough = rec.n_rough.w, metal = rec.v_metal.w;
    q.a2 = rough * rough;
    q.k = rough;
    q.k1 = 1.0f - rough;
    q.omn2 = rec.g.w;
    q.NdotV = rec.alb_nv.w;
    q.ggxV = rec.plo.w;
    q.nv4 = 4.0f * q.NdotV;
    const float m1 = 1.0f - metal;
    const float alb[3] = {rec.alb_nv.x, rec.alb_nv.y, rec.alb_nv.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        q.F0[c] = fmaf(alb[c], metal, 0.04f * m1);
        q.omF0[c] = 1.0f - q.F0[c];
        q.kdiff[c] = m1 * alb[c] * (1.0f / kPi);
    }
}

// ------------------------------------------------------------------------------------------------
// Tile staging shared by both passes.  Dynamic shared memory layout:
//   uint32 cstart[1025] | uint32 aux[1025] | uint16 lc[1024] | uint16 order[1024] | PxRec px[1024]
// (the last only for the adjoint).  cstart[c] = first position in order[] of local cluster c;
// order[] lists the tile's shaded pixels grouped by cluster, in pixel order.
// ------------------------------------------------------------------------------------------------
constexpr int kTileThreads = 256;
constexpr uint32_t kNoCluster = 0xFFFFu;
constexpr size_t kGroupBytes = (2 * 1025 * 4 + 2 * 1024 * 2 + 15) / 16 * 16;
constexpr size_t kStageBytes = kGroupBytes + 1024 * sizeof(PxRec);

struct Stage {
    uint32_t* cstart;
    uint32_t* aux;
    uint16_t* lc;
    uint16_t* order;
    PxRec* px;
    uint32_t cmin, nc;
};

__device__ __forceinline__ Stage stage_layout(float4* dyn)
{
    Stage S;
    char* base = reinterpret_cast<char*>(dyn);
    S.cstart = reinterpret_cast<uint32_t*>(base);
    S.aux = S.cstart + 1025;
    S.lc = reinterpret_cast<uint16_t*>(S.aux + 1025);
    S.order = S.lc + 1024;
    S.px = reinterpret_cast<PxRec*>(base + kGroupBytes);
    S.cmin = S.nc = 0;
    return S;
}

// Exclusive scan of v[0, n) in place (n <= 1280), all threads of the CTA; returns the total.
__device__ __forceinline__ uint32_t block_scan_1025(uint32_t* v, uint32_t n, uint32_t* s_warp)
{
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    // thread t owns entries 5t .. 5t+4 (5 * 256 >= 1025)
    uint32_t x[5], run = 0;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const uint32_t i = 5 * tid + k;
        x[k] = i < n ? v[i] : 0u;
        run += x[k];
    }
    uint32_t incl = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= (uint32_t)d) incl += y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    uint32_t base = incl - run, total = 0;
#pragma unroll
    for (int w = 0; w < kTileThreads / 32; ++w) {
        const uint32_t t = s_warp[w];
        if (w < (int)warp) base += t;
        total += t;
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const uint32_t i = 5 * tid + k;
        if (i < n) v[i] = base;
        base += x[k];
    }
    __syncthreads();
    return total;
}

// Groups tile (tx, ty)'s shaded pixels by cluster; with RECORDS also stages their records (and the
// upstream gradient).  Returns false (uniformly) when the tile has no shaded pixel.
template <bool RECORDS>
__device__ __forceinline__ bool stage_tile(const ShadeArgs& a, const float* __restrict__ grad, uint32_t tx, uint32_t ty,
                                           Stage& S, uint32_t* s_misc)
{
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) {
        s_misc[8] = 0xFFFFFFFFu;
        s_misc[9] = 0u;
    }
    __syncthreads();
    uint32_t cmin = 0xFFFFFFFFu, cmax = 0u, refs[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t i = tid + k * kTileThreads;
        const uint32_t x = tx * 32 + (i & 31u), y = ty * 32 + (i >> 5);
        uint32_t ref = 0xFFFFFFFFu;
        Px q;
        const bool shaded =
            x < a.W && y < a.H && pixel_world(a.frame, x, y, a.W, a.H, a.g.depth[(size_t)y * a.W + x], q.p, q.plo);
        if (shaded) {
            const size_t px = (size_t)y * a.W + x;
            ref = a.lists.cluster_refs[px];
            cmin = min(cmin, ref);
            cmax = max(cmax, ref);
            if (RECORDS) {
                float alb[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    q.N[c] = a.g.normals[3 * px + c];
                    alb[c] = a.g.albedo[3 * px + c];
                }
                const float rough = a.g.roughness[px], metal = a.g.metallic[px];
                px_terms(q, a.frame->view.eye, alb, rough, metal);
                PxRec rec;
                rec.p_ref = make_float4(q.p[0], q.p[1], q.p[2], __uint_as_float(ref));
                rec.n_rough = make_float4(q.N[0], q.N[1], q.N[2], rough);
                rec.v_metal = make_float4(q.V[0], q.V[1], q.V[2], metal);
                rec.alb_nv = make_float4(alb[0], alb[1], alb[2], q.NdotV);
                rec.g = make_float4(grad[3 * px], grad[3 * px + 1], grad[3 * px + 2], q.omn2);
                rec.plo = make_float4(q.plo[0], q.plo[1], q.plo[2], q.ggxV);
                S.px[i] = rec;
            }
        }
        refs[k] = ref;
    }
    cmin = __reduce_min_sync(0xFFFFFFFFu, cmin);
    cmax = __reduce_max_sync(0xFFFFFFFFu, cmax);
    if (lane == 0) {
        atomicMin(&s_misc[8], cmin);
        atomicMax(&s_misc[9], cmax);
    }
    __syncthreads();
    cmin = s_misc[8];
    cmax = s_misc[9];
    if (cmin > cmax) return false;
    const uint32_t nc = cmax - cmin + 1;  // <= 1024: a tile's clusters are consecutive in the key list
    if (nc > 1024u) {  // references that no find_unique_cluster_list output can hold
        if (tid == 0) VREN_RECORD_ERROR(VREN_ERR_ARG);
        return false;
    }
    S.cmin = cmin;
    S.nc = nc;
    for (uint32_t c = tid; c <= nc; c += kTileThreads) {
        S.cstart[c] = 0u;
        S.aux[c] = 0u;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t i = tid + k * kTileThreads;
        const uint32_t l = refs[k] == 0xFFFFFFFFu ? kNoCluster : refs[k] - cmin;
        S.lc[i] = (uint16_t)l;
        if (l != kNoCluster) atomicAdd(&S.cstart[l], 1u);
    }
    __syncthreads();
    block_scan_1025(S.cstart, nc + 1, s_misc);
    // Stable grouping: warp 0 walks the 32 rows of pixels in order; peers of one cluster within a
    // row are ranked by lane, and a per-cluster running count (aux) carries the earlier rows.
    if (warp == 0) {
        for (uint32_t row = 0; row < 32; ++row) {
            const uint32_t i = row * 32 + lane;
            const uint32_t l = S.lc[i];
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, l);
            const uint32_t before = peers & lanemask_lt();
            if (l != kNoCluster) S.order[S.cstart[l] + S.aux[l] + __popc(before)] = (uint16_t)i;
            __syncwarp();
            if (l != kNoCluster && before == 0u) S.aux[l] += __popc(peers);
            __syncwarp();
        }
    }
    __syncthreads();
    return true;
}

// ------------------------------------------------------------------------------------------------
// Forward
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kTileThreads) shade_forward_kernel(ShadeArgs a)
{
    extern __shared__ float4 s_dyn[];
    __shared__ uint32_t s_misc[16];
    Stage S = stage_layout(s_dyn);
    const uint32_t TX = (a.W + 31) / 32;
    const uint32_t tx = blockIdx.x % TX, ty = blockIdx.x / TX;
    if (!stage_tile<false>(a, nullptr, tx, ty, S, s_misc)) return;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t nc = S.nc;
    // tasks: (cluster, chunk of 32 of its pixels); aux[c] = first task of cluster c
    for (uint32_t c = tid; c <= nc; c += kTileThreads)
        S.aux[c] = c < nc ? (S.cstart[c + 1] - S.cstart[c] + 31u) / 32u : 0u;
    __syncthreads();
    const uint32_t ntasks = block_scan_1025(S.aux, nc + 1, s_misc);
    const float* eye = a.frame->view.eye;
    for (uint32_t task = warp; task < ntasks; task += kTileThreads / 32) {
        uint32_t lo = 0, hi = nc - 1;  // last cluster whose first task <= task
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (S.aux[mid] <= task) lo = mid;
            else hi = mid - 1;
        }
        const uint32_t c = lo;
        const uint32_t j = (task - S.aux[c]) * 32u + lane;
        const bool valid = j < S.cstart[c + 1] - S.cstart[c];
        const uint32_t pix = valid ? S.order[S.cstart[c] + j] : S.order[S.cstart[c]];
        const uint32_t x = tx * 32 + (pix & 31u), y = ty * 32 + (pix >> 5);
        const size_t px = (size_t)y * a.W + x;
        Px q;
        pixel_world(a.frame, x, y, a.W, a.H, a.g.depth[px], q.p, q.plo);
        float alb[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            q.N[k] = a.g.normals[3 * px + k];
            alb[k] = a.g.albedo[3 * px + k];
        }
        px_terms(q, eye, alb, a.g.roughness[px], a.g.metallic[px]);
        float Lo[3] = {0.0f, 0.0f, 0.0f};
        if (a.L) {
            const uint32_t cref = S.cmin + c;
            const uint32_t off = a.lists.offsets[cref], cap = a.lists.index_capacity;
            uint32_t cnt = a.lists.counts[cref];
            if (off >= cap || cnt > cap - off) {  // a list cut by the assignment's index capacity
                cnt = off >= cap ? 0u : cap - off;
                if (lane == 0) VREN_RECORD_ERROR(VREN_ERR_CAPACITY);
            }
            const uint32_t* idx = a.lists.indices + off;
            uint32_t i = 0;
            if (a.packed) {
                for (; i + 1 < cnt; i += 2) {
                    const uint32_t l0 = idx[i], l1 = idx[i + 1];
                    point_light_fwd2(q, a.lpos[l0], a.lights[l0], a.lpos[l1], a.lights[l1], a.falloff, Lo);
                }
            }
            for (; i < cnt; ++i) {
                const uint32_t l = idx[i];
                point_light_fwd(q, a.lpos[l], a.lights[l], a.falloff, Lo);
            }
        }
        for (uint32_t i = 0; i < a.ndir; ++i) {
            const float4 dd = a.dir[2 * i], dc = a.dir[2 * i + 1];
            const float Ld[3] = {dd.x, dd.y, dd.z};
            const float rad[3] = {dc.x, dc.y, dc.z};
            brdf_accumulate(q, Ld, rad, Lo);
        }
        if (!valid) continue;
#pragma unroll
        for (int k = 0; k < 3; ++k)
            a.out[3 * px + k] = a.mode == VREN_CS_SHADE_COLOR ? powf(0.03f * alb[k] + Lo[k], 1.0f / 2.2f) : Lo[k];
    }
}

// ------------------------------------------------------------------------------------------------
// Adjoint, step 1: per-slot partials
// ------------------------------------------------------------------------------------------------
// The warp's sum of a slot's seven partials, stored by lane 0 as two float4 (the eighth word zero).
__device__ __forceinline__ void write_slot_partial(float g7[7], float* __restrict__ slot_grad, uint32_t s, uint32_t lane)
{
#pragma unroll
    for (int k = 0; k < 7; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) g7[k] += __shfl_xor_sync(0xFFFFFFFFu, g7[k], o);
    if (lane == 0) {
        float4* dst = reinterpret_cast<float4*>(slot_grad + 8 * (size_t)s);
        dst[0] = make_float4(g7[0], g7[1], g7[2], g7[3]);
        dst[1] = make_float4(g7[4], g7[5], g7[6], 0.0f);
    }
}

__global__ void __launch_bounds__(kTileThreads, 2) shade_backward_slots_kernel(ShadeArgs a, const float* __restrict__ grad,
                                                                            float* __restrict__ slot_grad,
                                                                            uint32_t n_slots)
{
    extern __shared__ float4 s_dyn[];
    __shared__ uint32_t s_misc[16];
    Stage S = stage_layout(s_dyn);
    const uint32_t TX = (a.W + 31) / 32;
    const uint32_t tx = blockIdx.x % TX, ty = blockIdx.x / TX;
    if (!stage_tile<true>(a, grad, tx, ty, S, s_misc)) return;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t nc = S.nc, cmin = S.cmin, cmax = cmin + nc - 1;
    // aux[c] = first slot of cluster c (list offsets); aux[nc] = end of the tile's slots
    for (uint32_t c = tid; c <= nc; c += kTileThreads)
        S.aux[c] = c < nc ? a.lists.offsets[cmin + c] : a.lists.offsets[cmax] + a.lists.counts[cmax];
    __syncthreads();
    const uint32_t s_begin = S.aux[0];
    uint32_t s_end = S.aux[nc];
    if (s_end > n_slots) {  // the caller's assignment count does not cover these lists
        if (tid == 0) VREN_RECORD_ERROR(VREN_ERR_CAPACITY);
        s_end = n_slots;
    }
    // A warp takes slots two at a time (packed: both lights of one cluster against the same pixels) or
    // one at a time.
    const uint32_t per = a.packed ? 2u : 1u;
    for (uint32_t s0 = s_begin + per * warp; s0 < s_end; s0 += per * (kTileThreads / 32)) {
        uint32_t lo = 0, hi = nc - 1;  // cluster owning slot s0: last c with aux[c] <= s0
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (S.aux[mid] <= s0) lo = mid;
            else hi = mid - 1;
        }
        const uint32_t c = lo;
        const uint32_t b = S.cstart[c], n = S.cstart[c + 1] - b;
        if (per == 2u && s0 + 1 < s_end && s0 + 1 < S.aux[c + 1]) {
            // slots s0 and s0 + 1 of the same cluster
            const uint32_t l0 = a.lists.indices[s0], l1 = a.lists.indices[s0 + 1];
            const float4 lp0 = a.lpos[l0], lc0 = a.lights[l0], lp1 = a.lpos[l1], lc1 = a.lights[l1];
            float g7a[7] = {0, 0, 0, 0, 0, 0, 0}, g7b[7] = {0, 0, 0, 0, 0, 0, 0};
            for (uint32_t j = lane; j < n; j += 32) {
                const PxRec& rec = S.px[S.order[b + j]];
                Px q;
                rec_to_px(rec, q);
                const float gin[3] = {rec.g.x, rec.g.y, rec.g.z};
                pair_backward2(q, lp0, lc0, lp1, lc1, a.falloff, gin, g7a, g7b);
            }
            write_slot_partial(g7a, slot_grad, s0, lane);
            write_slot_partial(g7b, slot_grad, s0 + 1, lane);
            continue;
        }
        for (uint32_t s = s0; s < s0 + per && s < s_end; ++s) {
            // a slot alone (or each of two slots of different clusters)
            uint32_t cs = c;
            if (s != s0) {
                lo = 0, hi = nc - 1;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi + 1) >> 1;
                    if (S.aux[mid] <= s) lo = mid;
                    else hi = mid - 1;
                }
                cs = lo;
            }
            const uint32_t bs = S.cstart[cs], ns = S.cstart[cs + 1] - bs;
            const uint32_t l = a.lists.indices[s];
            const float4 lp = a.lpos[l], lc = a.lights[l];
            float g7[7] = {0, 0, 0, 0, 0, 0, 0};
            for (uint32_t j = lane; j < ns; j += 32) {
                const PxRec& rec = S.px[S.order[bs + j]];
                Px q;
                rec_to_px(rec, q);
                const float gin[3] = {rec.g.x, rec.g.y, rec.g.z};
                pair_backward(q, lp, lc, a.falloff, gin, g7);
            }
            write_slot_partial(g7, slot_grad, s, lane);
        }
    }
}

__global__ void slot_pairs_kernel(const uint32_t* __restrict__ indices, uint32_t n, uint2* __restrict__ pairs)
{
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
        pairs[s] = make_uint2(indices[s], s);
}

// One warp per light: its slots (sorted, stable) summed in slot order.
__global__ void light_reduce_kernel(const uint2* __restrict__ sorted, const uint32_t* __restrict__ ends, uint32_t L,
                                    const float* __restrict__ slot_grad, float* __restrict__ gpos,
                                    float* __restrict__ gcol, float* __restrict__ grad_r)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t l = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (l >= L) return;
    const uint32_t begin = l == 0 ? 0u : ends[l - 1], end = ends[l];
    float g7[7] = {0, 0, 0, 0, 0, 0, 0};
    for (uint32_t i = begin + lane; i < end; i += 32) {
        const float4* src = reinterpret_cast<const float4*>(slot_grad + 8 * (size_t)sorted[i].y);
        const float4 a = src[0], b = src[1];
        g7[0] += a.x; g7[1] += a.y; g7[2] += a.z; g7[3] += a.w;
        g7[4] += b.x; g7[5] += b.y; g7[6] += b.z;
    }
#pragma unroll
    for (int j = 0; j < 7; ++j)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) g7[j] += __shfl_xor_sync(0xFFFFFFFFu, g7[j], o);
    if (lane == 0) {
        gpos[3 * l + 0] = g7[0]; gpos[3 * l + 1] = g7[1]; gpos[3 * l + 2] = g7[2];
        gcol[3 * l + 0] = g7[3]; gcol[3 * l + 1] = g7[4]; gcol[3 * l + 2] = g7[5];
        grad_r[l] = g7[6];
    }
}

static uint32_t light_key_bits(uint32_t L)
{
    uint32_t b = 1;
    while (b < 16 && (1u << b) < L) ++b;
    return b;
}

struct BwdLayout {
    size_t slots, pairs, bout, bscratch, total;
};

static BwdLayout bwd_layout(uint32_t L, uint32_t n)
{
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    const uint32_t kb = light_key_bits(L);
    BwdLayout b;
    b.slots = 0;
    b.pairs = up((size_t)(n ? n : 1) * 32);
    b.bout = b.pairs + up((size_t)(n ? n : 1) * 8);
    b.bscratch = b.bout + up(vren_bucket_sort_output_bytes(n, kb));
    b.total = b.bscratch + up(vren_bucket_sort_scratch_bytes(n, kb));
    return b;
}

}  // namespace vren_gb300

using namespace vren_gb300;

static bool shade_args(const vren_cs_frame* frame, uint32_t W, uint32_t H, const vren_cs_gbuffer* g,
                       const vren_cs_light_lists* lists, const float* lpos, const float* lights, uint32_t L,
                       ShadeArgs& a)
{
    if (!frame || !g || !lists || W == 0 || H == 0) return false;
    if (!g->depth || !g->normals || !g->albedo || !g->roughness || !g->metallic || !lists->cluster_refs) return false;
    if (L > 0 && (!lpos || !lights || !lists->counts || !lists->offsets || !lists->indices || !lists->index_capacity))
        return false;
    if (((uintptr_t)lpos | (uintptr_t)lights) & 15u) return false;
    std::memset(&a, 0, sizeof(a));
    a.frame = frame;
    a.W = W;
    a.H = H;
    a.g = *g;
    a.lists = *lists;
    a.lpos = reinterpret_cast<const float4*>(lpos);
    a.lights = reinterpret_cast<const float4*>(lights);
    a.L = L;
    return true;
}

extern "C" int vren_cs_shade(vren_stream_t s, const vren_cs_frame* frame, uint32_t width, uint32_t height,
                             const vren_cs_gbuffer* gbuffer, const vren_cs_light_lists* lists,
                             const float* light_positions, const float* point_lights, uint32_t light_count,
                             const float* directional_lights, uint32_t directional_count, int falloff, int output_mode,
                             float* out_rgb)
{
    ShadeArgs a;
    if (!out_rgb || !shade_args(frame, width, height, gbuffer, lists, light_positions, point_lights, light_count, a))
        return VREN_ERR_ARG;
    if (falloff != VREN_CS_FALLOFF_REF && falloff != VREN_CS_FALLOFF_WINDOWED_INV_SQ) return VREN_ERR_ARG;
    if (output_mode != VREN_CS_SHADE_COLOR && output_mode != VREN_CS_SHADE_RADIANCE) return VREN_ERR_ARG;
    if (directional_count > 0 && (!directional_lights || ((uintptr_t)directional_lights & 15u))) return VREN_ERR_ARG;
    a.dir = reinterpret_cast<const float4*>(directional_lights);
    a.ndir = directional_count;
    a.falloff = falloff;
    a.mode = output_mode;
    a.out = out_rgb;
    a.packed = tuning(VREN_TUNE_SHADE_PACKED);
    const uint32_t tiles = ((width + 31) / 32) * ((height + 31) / 32);
    shade_forward_kernel<<<tiles, kTileThreads, kGroupBytes, as_stream(s)>>>(a);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

extern "C" size_t vren_cs_shade_backward_scratch_bytes(uint32_t light_count, uint32_t assignments)
{
    return bwd_layout(light_count, assignments).total;
}

extern "C" int vren_cs_shade_backward(vren_stream_t s, const vren_cs_frame* frame, uint32_t width, uint32_t height,
                                      const vren_cs_gbuffer* gbuffer, const vren_cs_light_lists* lists,
                                      uint32_t assignments, const float* light_positions, const float* point_lights,
                                      uint32_t light_count, int falloff, const float* grad_radiance,
                                      float* grad_positions, float* grad_colors, float* grad_radii, void* scratch)
{
    ShadeArgs a;
    if (!shade_args(frame, width, height, gbuffer, lists, light_positions, point_lights, light_count, a))
        return VREN_ERR_ARG;
    if (falloff != VREN_CS_FALLOFF_REF && falloff != VREN_CS_FALLOFF_WINDOWED_INV_SQ) return VREN_ERR_ARG;
    if (light_count > 65536 || !grad_radiance || !scratch || ((uintptr_t)scratch & 255u)) return VREN_ERR_ARG;
    if (light_count > 0 && (!grad_positions || !grad_colors || !grad_radii)) return VREN_ERR_ARG;
    if (light_count == 0) return VREN_OK;
    // the slots are the index entries [0, assignments): lists cut by the assignment's capacity cannot
    // be differentiated
    if (assignments > lists->index_capacity) return VREN_ERR_CAPACITY;
    a.falloff = falloff;
    a.packed = tuning(VREN_TUNE_SHADE_PACKED);
    cudaStream_t st = as_stream(s);
    const BwdLayout lay = bwd_layout(light_count, assignments);
    char* sc = static_cast<char*>(scratch);
    float* slot_grad = reinterpret_cast<float*>(sc + lay.slots);
    uint2* pairs = reinterpret_cast<uint2*>(sc + lay.pairs);
    char* bout = sc + lay.bout;
    const uint32_t kb = light_key_bits(light_count);
    VREN_CUDA_TRY(cudaMemsetAsync(slot_grad, 0, (size_t)(assignments ? assignments : 1) * 32, st));
    const uint32_t tiles = ((width + 31) / 32) * ((height + 31) / 32);
    VREN_CUDA_TRY(cudaFuncSetAttribute(shade_backward_slots_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kStageBytes));
    if (assignments > 0) {
        shade_backward_slots_kernel<<<tiles, kTileThreads, kStageBytes, st>>>(a, grad_radiance, slot_grad,
                                                                               assignments);
        VREN_LAUNCH_CHECK();
        uint32_t g = (assignments + 255) / 256;
        if (g > 4096) g = 4096;
        slot_pairs_kernel<<<g, 256, 0, st>>>(lists->indices, assignments, pairs);
        VREN_LAUNCH_CHECK();
    }
    int rc = vren_bucket_sort_u32x2(s, reinterpret_cast<const uint32_t*>(pairs), assignments, bout, kb,
                                    sc + lay.bscratch);
    if (rc != VREN_OK) return rc;
    const uint32_t* ends = reinterpret_cast<const uint32_t*>(bout + ((size_t)assignments * 8 + 255) / 256 * 256);
    light_reduce_kernel<<<(light_count * 32 + 255) / 256, 256, 0, st>>>(
        reinterpret_cast<const uint2*>(bout), ends, light_count, slot_grad, grad_positions, grad_colors, grad_radii);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

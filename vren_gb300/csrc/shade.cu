// Clustered Cook-Torrance/GGX shading (vren/resources/shaders/clustered_shading/shade.comp:69-141,
// vren/resources/shaders/pbr.glsl:6-112) and its hand-written adjoint with respect to the point
// lights' positions, colours and radii (the light-to-cluster assignment held fixed).
//
// Forward: one thread per pixel, the loop over its cluster's lights.
// Adjoint (deterministic, nothing stored per (pixel, light) pair):
//   1. one CTA per 32x32 tile stages the tile's G-buffer and upstream gradient in shared memory;
//      each warp takes (cluster, light) slots of the tile and sums the pair gradients over the
//      tile's pixels of that cluster — lanes stride the pixels in a fixed order, then a fixed
//      butterfly reduction — into one 7-float partial per slot;
//   2. the slots are grouped by light with the stable bucket sort of (light, slot) pairs;
//   3. one warp per light sums its slots' partials in slot order.
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
};

struct Px {
    float p[3], N[3], V[3], alb[3];
    float rough, metal, NdotV;
    float omn2;  // 1 - |N|^2
};

__device__ __forceinline__ float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// a x b, each component one product and one fused multiply-add (accurate when the result is small).
__device__ __forceinline__ void cross3(const float* a, const float* b, float* c)
{
    c[0] = fmaf(a[1], b[2], -(a[2] * b[1]));
    c[1] = fmaf(a[2], b[0], -(a[0] * b[2]));
    c[2] = fmaf(a[0], b[1], -(a[1] * b[0]));
}

// 1 - |n|^2 to within a few ulps of its own size: the squares as exact product pairs, summed with
// error-free transformations (Knuth's two-sum), then 1 - hi (exact for hi in [0.5, 2]) - lo.
__device__ __forceinline__ float one_minus_norm2(const float* n)
{
    float hi = 0.0f, lo = 0.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float ph = __fmul_rn(n[c], n[c]);
        const float pl = fmaf(n[c], n[c], -ph);
        const float s = __fadd_rn(hi, ph);
        const float bb = __fsub_rn(s, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(ph, bb));
        hi = s;
        lo = __fadd_rn(lo, __fadd_rn(err, pl));
    }
    return __fsub_rn(__fsub_rn(1.0f, hi), lo);
}

// GGX denominator D = NdotH^2 (a2 - 1) + 1 (pbr.glsl:24-35) for NdotH = max(N.H, 0), H = hv / |hv|.
// Written as a2 h^2 + (1 - h^2) with Lagrange's identity
//     1 - (N.H)^2 = ((1 - |N|^2) |hv|^2 + |N x hv|^2) / |hv|^2,
// whose terms stay accurate near the specular peak, where 1 - (N.H)^2 computed from a rounded N.H
// would cancel (a2 = roughness^2 can be 0.0025, so D's relative error there would be ~1e-4).
__device__ __forceinline__ float ggx_den(const float* N, const float* hv, float nhu, float hl2, float omn2, float a2)
{
    if (!(nhu > 0.0f)) return 1.0f;
    float c[3];
    cross3(N, hv, c);
    return (a2 * nhu * nhu + fmaf(hl2, omn2, dot3(c, c))) / hl2;
}

// World position of pixel (x, y); returns false when the pixel is not shaded (shade.comp:86).
// Each row starts from the constant column and adds the depth term with one fused multiply-add:
// the homogeneous w of a perspective inverse is m[11] * D + m[15] with D close to 1 for distant
// pixels (about -9.999 * D + 10), and rounding m[11] * D on its own before the sum would cost
// three to four significant digits of the view depth there.
__device__ __forceinline__ bool pixel_world(const vren_cs_frame* F, uint32_t x, uint32_t y, uint32_t W, uint32_t H,
                                            float D, float p[3])
{
    const float fx = (float)x / (float)W, fy = (float)y / (float)H;
    const float nx = fx * 2.0f - 1.0f, ny = (1.0f - fy) * 2.0f - 1.0f;
    const float* ip = F->view.inv_proj;
    float v[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) v[r] = fmaf(ip[4 + r], ny, fmaf(ip[r], nx, fmaf(ip[8 + r], D, ip[12 + r])));
#pragma unroll
    for (int r = 0; r < 3; ++r) v[r] = v[r] / v[3];
    if (!(v[2] < F->view.far_plane - 0.001f)) return false;
    const float* iv = F->view.inv_view;
#pragma unroll
    for (int r = 0; r < 3; ++r) p[r] = fmaf(iv[8 + r], v[2], fmaf(iv[4 + r], v[1], fmaf(iv[r], v[0], iv[12 + r])));
    return true;
}

__device__ __forceinline__ void load_px(const ShadeArgs& a, uint32_t x, uint32_t y, const float p[3], Px& q)
{
    const size_t px = (size_t)y * a.W + x;
    const float* eye = a.frame->view.eye;
    float v[3] = {eye[0] - p[0], eye[1] - p[1], eye[2] - p[2]};
    const float lv = sqrtf(dot3(v, v));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        q.p[c] = p[c];
        q.V[c] = v[c] / lv;
        q.N[c] = a.g.normals[3 * px + c];
        q.alb[c] = a.g.albedo[3 * px + c];
    }
    q.rough = a.g.roughness[px];
    q.metal = a.g.metallic[px];
    q.NdotV = fmaxf(dot3(q.N, q.V), 0.0f);
    q.omn2 = one_minus_norm2(q.N);
}

// pbr_apply_light (pbr.glsl:184-215) for light direction L (from the light towards the point) and
// radiance; accumulates into out.
__device__ __forceinline__ void apply_light(const Px& q, const float L[3], const float rad[3], float out[3])
{
    float hv[3] = {q.V[0] - L[0], q.V[1] - L[1], q.V[2] - L[2]};
    const float hl2 = dot3(hv, hv);
    const float hl = sqrtf(hl2);
    const float H[3] = {hv[0] / hl, hv[1] / hl, hv[2] / hl};
    const float a2 = q.rough * q.rough;
    const float D = ggx_den(q.N, hv, dot3(q.N, hv), hl2, q.omn2, a2);
    const float NDF = a2 / (kPi * D * D);
    const float k = q.rough;
    const float nl = -dot3(q.N, L);
    const float NdotL = fmaxf(nl, 0.0f);
    const float ggxV = q.NdotV / (q.NdotV * (1.0f - k) + k);
    const float ggxL = NdotL / (NdotL * (1.0f - k) + k);
    const float G = ggxV * ggxL;
    const float HdotV = fmaxf(dot3(H, q.V), 0.0f);
    const float x = 1.0f - HdotV;
    const float f5 = x * x * x * x * x;
    const float spec = NDF * G / (4.0f * q.NdotV * NdotL + 0.0001f);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float F0 = 0.04f * (1.0f - q.metal) + q.alb[c] * q.metal;
        const float F = F0 + (1.0f - F0) * f5;
        const float kD = (1.0f - F) * (1.0f - q.metal);
        out[c] += fmaxf((kD * q.alb[c] / kPi + F * spec) * rad[c] * NdotL, 0.0f);
    }
}

__device__ __forceinline__ float falloff_value(int mode, float dist, float r)
{
    if (mode == VREN_CS_FALLOFF_REF) {
        const float u = fminf(dist / r, 1.0f);
        return 1.0f - u * sqrtf(u);
    }
    const float t = dist / r;
    const float t2 = t * t;
    const float w = fminf(fmaxf(1.0f - t2 * t2, 0.0f), 1.0f);
    return w * w / (dist * dist + 1.0f);
}

__global__ void __launch_bounds__(256) shade_forward_kernel(ShadeArgs a)
{
    const uint32_t x = blockIdx.x * 32 + (threadIdx.x & 31u);
    const uint32_t y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= a.W || y >= a.H) return;
    const size_t px = (size_t)y * a.W + x;
    float p[3];
    if (!pixel_world(a.frame, x, y, a.W, a.H, a.g.depth[px], p)) return;
    Px q;
    load_px(a, x, y, p, q);
    float Lo[3] = {0.0f, 0.0f, 0.0f};
    const uint32_t c = a.lists.cluster_refs[px];
    const uint32_t cnt = a.L ? a.lists.counts[c] : 0u;
    const uint32_t off = a.L ? a.lists.offsets[c] : 0u;
    for (uint32_t i = 0; i < cnt; ++i) {
        const uint32_t l = a.lists.indices[off + i];
        const float4 lp = a.lpos[l], lc = a.lights[l];
        float d[3] = {p[0] - lp.x, p[1] - lp.y, p[2] - lp.z};
        const float dist = sqrtf(dot3(d, d));
        const float Ld[3] = {d[0] / dist, d[1] / dist, d[2] / dist};
        const float att = falloff_value(a.falloff, dist, lc.w);
        const float rad[3] = {lc.x * att, lc.y * att, lc.z * att};
        apply_light(q, Ld, rad, Lo);
    }
    for (uint32_t i = 0; i < a.ndir; ++i) {
        const float4 dd = a.dir[2 * i], dc = a.dir[2 * i + 1];
        const float Ld[3] = {dd.x, dd.y, dd.z};
        const float rad[3] = {dc.x, dc.y, dc.z};
        apply_light(q, Ld, rad, Lo);
    }
    float o[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
        o[k] = a.mode == VREN_CS_SHADE_COLOR ? powf(0.03f * q.alb[k] + Lo[k], 1.0f / 2.2f) : Lo[k];
    a.out[3 * px + 0] = o[0];
    a.out[3 * px + 1] = o[1];
    a.out[3 * px + 2] = o[2];
}

// ------------------------------------------------------------------------------------------------
// Adjoint of one (pixel, light) pair: accumulates dLoss/d(position, colour, radius) into g7 for the
// upstream gradient gin of the pair's radiance (reverse mode through pbr_apply_point_light).
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ void pair_backward(const Px& q, float4 lp, float4 lc, int falloff, const float gin[3],
                                              float g7[7])
{
    const float r = lc.w;
    float d[3] = {q.p[0] - lp.x, q.p[1] - lp.y, q.p[2] - lp.z};
    const float dd = dot3(d, d);
    const float dist = sqrtf(dd);
    const float L[3] = {d[0] / dist, d[1] / dist, d[2] / dist};
    const float t = dist / r;
    float att, datt_dt, datt_ddist_direct = 0.0f;
    if (falloff == VREN_CS_FALLOFF_REF) {
        const float u = fminf(t, 1.0f);
        att = 1.0f - u * sqrtf(u);
        datt_dt = t < 1.0f ? -1.5f * sqrtf(t) : 0.0f;
    } else {
        const float t2 = t * t;
        const float wr = 1.0f - t2 * t2;
        const float w = fminf(fmaxf(wr, 0.0f), 1.0f);
        const float den = dd + 1.0f;
        att = w * w / den;
        const float dw_dt = (wr > 0.0f && wr < 1.0f) ? -4.0f * t2 * t : 0.0f;
        datt_dt = 2.0f * w / den * dw_dt;
        datt_ddist_direct = -w * w * 2.0f * dist / (den * den);
    }
    const float col[3] = {lc.x, lc.y, lc.z};

    float hv[3] = {q.V[0] - L[0], q.V[1] - L[1], q.V[2] - L[2]};
    const float hl2 = dot3(hv, hv);
    const float hl = sqrtf(hl2);
    const float H[3] = {hv[0] / hl, hv[1] / hl, hv[2] / hl};
    const float a2 = q.rough * q.rough;
    const float nhu = dot3(q.N, hv);  // |hv| (N.H)
    const float NdotH = fmaxf(nhu / hl, 0.0f);
    const float D = ggx_den(q.N, hv, nhu, hl2, q.omn2, a2);
    const float NDF = a2 / (kPi * D * D);
    const float k = q.rough;
    const float nl_raw = -dot3(q.N, L);
    const float NdotL = fmaxf(nl_raw, 0.0f);
    const float ggxV = q.NdotV / (q.NdotV * (1.0f - k) + k);
    const float dl = NdotL * (1.0f - k) + k;
    const float ggxL = NdotL / dl;
    const float G = ggxV * ggxL;
    const float hvr = dot3(H, q.V);
    const float HdotV = fmaxf(hvr, 0.0f);
    const float x = 1.0f - HdotV;
    const float x4 = x * x * x * x;
    const float f5 = x4 * x;
    const float sden = 4.0f * q.NdotV * NdotL + 0.0001f;
    const float spec = NDF * G / sden;

    float gatt = 0.0f, gNdotL = 0.0f, gspec = 0.0f, gf5 = 0.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float F0 = 0.04f * (1.0f - q.metal) + q.alb[c] * q.metal;
        const float F = F0 + (1.0f - F0) * f5;
        const float kD = (1.0f - F) * (1.0f - q.metal);
        const float B = kD * q.alb[c] / kPi + F * spec;
        const float val = B * col[c] * att * NdotL;
        const float gv = val > 0.0f ? gin[c] : 0.0f;
        const float gB = gv * col[c] * att * NdotL;
        g7[3 + c] += gv * B * att * NdotL;  // colour
        gatt += gv * B * col[c] * NdotL;
        gNdotL += gv * B * col[c] * att;
        const float gF = gB * (spec - (1.0f - q.metal) * q.alb[c] / kPi);
        gspec += gB * F;
        gf5 += gF * (1.0f - F0);
    }
    const float gHdotV = -gf5 * 5.0f * x4;
    const float gNDF = gspec * G / sden;
    const float gG = gspec * NDF / sden;
    const float gsden = -gspec * NDF * G / (sden * sden);
    gNdotL += gsden * 4.0f * q.NdotV;
    gNdotL += gG * ggxV * k / (dl * dl);
    const float gNdotH = gNDF * (-4.0f * a2 * NdotH * (a2 - 1.0f) / (kPi * D * D * D));
    const float gnl = nl_raw > 0.0f ? gNdotL : 0.0f;
    const float gnh = nhu > 0.0f ? gNdotH : 0.0f;
    const float ghv = hvr > 0.0f ? gHdotV : 0.0f;
    // Through H = hv / |hv| and hv = V - L: d(N.H)/dhv = (N - (N.H) H) / |hv|, written as
    // hv x (N x hv) / |hv|^3 (no cancellation near the peak); d(H.V)/dhv = (V - (H.V) H) / |hv|.
    float nxh[3], tri[3];
    cross3(q.N, hv, nxh);
    cross3(hv, nxh, tri);
    const float sn = gnh / (hl2 * hl), sv = ghv / hl;
    float gL[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) gL[c] = -gnl * q.N[c] - sn * tri[c] - sv * (q.V[c] - H[c] * hvr);
    // attenuation: t = dist / r
    const float gt = gatt * datt_dt;
    const float gdist = gatt * datt_ddist_direct + gt / r;
    g7[6] += -gt * dist / (r * r);  // radius
    const float gLL = dot3(gL, L);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float gd = (gL[c] - L[c] * gLL) / dist + gdist * L[c];
        g7[c] += -gd;  // d = p - light position
    }
}

// Per-pixel record staged in shared memory by the adjoint (80 bytes).
struct PxRec {
    float4 p_ref;     // p.xyz, cluster reference (bits; 0xFFFFFFFF = not shaded)
    float4 n_rough;   // N.xyz, roughness
    float4 v_metal;   // V.xyz, metallic
    float4 alb_nv;    // albedo.xyz, NdotV
    float4 g;         // upstream gradient, 1 - |N|^2
};

constexpr int kBwdThreads = 256;

__global__ void __launch_bounds__(kBwdThreads) shade_backward_slots_kernel(ShadeArgs a, const float* __restrict__ grad,
                                                                           float* __restrict__ slot_grad,
                                                                           uint32_t n_slots)
{
    extern __shared__ float4 s_dyn[];
    PxRec* s_px = reinterpret_cast<PxRec*>(s_dyn);
    __shared__ uint32_t s_coff[1025];
    __shared__ uint32_t s_cmin, s_cmax;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t TX = (a.W + 31) / 32;
    const uint32_t tx = blockIdx.x % TX, ty = blockIdx.x / TX;
    if (tid == 0) {
        s_cmin = 0xFFFFFFFFu;
        s_cmax = 0u;
    }
    __syncthreads();
    uint32_t cmin = 0xFFFFFFFFu, cmax = 0u;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t i = tid + k * kBwdThreads;
        const uint32_t x = tx * 32 + (i & 31u), y = ty * 32 + (i >> 5);
        PxRec rec;
        uint32_t ref = 0xFFFFFFFFu;
        float p[3];
        if (x < a.W && y < a.H && pixel_world(a.frame, x, y, a.W, a.H, a.g.depth[(size_t)y * a.W + x], p)) {
            const size_t px = (size_t)y * a.W + x;
            Px q;
            load_px(a, x, y, p, q);
            ref = a.lists.cluster_refs[px];
            rec.p_ref = make_float4(q.p[0], q.p[1], q.p[2], __uint_as_float(ref));
            rec.n_rough = make_float4(q.N[0], q.N[1], q.N[2], q.rough);
            rec.v_metal = make_float4(q.V[0], q.V[1], q.V[2], q.metal);
            rec.alb_nv = make_float4(q.alb[0], q.alb[1], q.alb[2], q.NdotV);
            rec.g = make_float4(grad[3 * px], grad[3 * px + 1], grad[3 * px + 2], q.omn2);
            cmin = min(cmin, ref);
            cmax = max(cmax, ref);
        } else {
            rec.p_ref = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0xFFFFFFFFu));
        }
        s_px[i] = rec;
    }
    cmin = __reduce_min_sync(0xFFFFFFFFu, cmin);
    cmax = __reduce_max_sync(0xFFFFFFFFu, cmax);
    if (lane == 0) {
        atomicMin(&s_cmin, cmin);
        atomicMax(&s_cmax, cmax);
    }
    __syncthreads();
    cmin = s_cmin;
    cmax = s_cmax;
    if (cmin > cmax) return;  // nothing shaded in this tile
    const uint32_t nc = cmax - cmin + 1;  // <= 1024 (keys of one tile)
    for (uint32_t c = tid; c <= nc; c += kBwdThreads)
        s_coff[c] = c < nc ? a.lists.offsets[cmin + c] : a.lists.offsets[cmax] + a.lists.counts[cmax];
    __syncthreads();
    const uint32_t s_begin = s_coff[0];
    uint32_t s_end = s_coff[nc];
    if (s_end > n_slots) {  // the caller's assignment count does not cover these lists
        if (tid == 0) VREN_RECORD_ERROR(VREN_ERR_CAPACITY);
        s_end = n_slots;
    }

    for (uint32_t s = s_begin + warp; s < s_end; s += kBwdThreads / 32) {
        // cluster owning slot s: last c with s_coff[c] <= s
        uint32_t lo = 0, hi = nc - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (s_coff[mid] <= s) lo = mid;
            else hi = mid - 1;
        }
        const uint32_t cref = cmin + lo;
        const uint32_t l = a.lists.indices[s];
        const float4 lp = a.lpos[l], lc = a.lights[l];
        float g7[7] = {0, 0, 0, 0, 0, 0, 0};
        for (uint32_t i = lane; i < 1024; i += 32) {
            const PxRec& rec = s_px[i];
            if (__float_as_uint(rec.p_ref.w) != cref) continue;
            Px q;
            q.p[0] = rec.p_ref.x; q.p[1] = rec.p_ref.y; q.p[2] = rec.p_ref.z;
            q.N[0] = rec.n_rough.x; q.N[1] = rec.n_rough.y; q.N[2] = rec.n_rough.z; q.rough = rec.n_rough.w;
            q.V[0] = rec.v_metal.x; q.V[1] = rec.v_metal.y; q.V[2] = rec.v_metal.z; q.metal = rec.v_metal.w;
            q.alb[0] = rec.alb_nv.x; q.alb[1] = rec.alb_nv.y; q.alb[2] = rec.alb_nv.z; q.NdotV = rec.alb_nv.w;
            q.omn2 = rec.g.w;
            const float gin[3] = {rec.g.x, rec.g.y, rec.g.z};
            pair_backward(q, lp, lc, a.falloff, gin, g7);
        }
#pragma unroll
        for (int j = 0; j < 7; ++j)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) g7[j] += __shfl_xor_sync(0xFFFFFFFFu, g7[j], o);
        if (lane == 0) {
            float4* dst = reinterpret_cast<float4*>(slot_grad + 8 * (size_t)s);
            dst[0] = make_float4(g7[0], g7[1], g7[2], g7[3]);
            dst[1] = make_float4(g7[4], g7[5], g7[6], 0.0f);
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
    if (L > 0 && (!lpos || !lights || !lists->counts || !lists->offsets || !lists->indices)) return false;
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
    dim3 grid((width + 31) / 32, (height + 7) / 8);
    shade_forward_kernel<<<grid, 256, 0, as_stream(s)>>>(a);
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
    a.falloff = falloff;
    cudaStream_t st = as_stream(s);
    const BwdLayout lay = bwd_layout(light_count, assignments);
    char* sc = static_cast<char*>(scratch);
    float* slot_grad = reinterpret_cast<float*>(sc + lay.slots);
    uint2* pairs = reinterpret_cast<uint2*>(sc + lay.pairs);
    char* bout = sc + lay.bout;
    const uint32_t kb = light_key_bits(light_count);
    VREN_CUDA_TRY(cudaMemsetAsync(slot_grad, 0, (size_t)(assignments ? assignments : 1) * 32, st));
    const uint32_t tiles = ((width + 31) / 32) * ((height + 31) / 32);
    const size_t smem = 1024 * sizeof(PxRec);
    VREN_CUDA_TRY(cudaFuncSetAttribute(shade_backward_slots_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    if (assignments > 0) {
        shade_backward_slots_kernel<<<tiles, kBwdThreads, smem, st>>>(a, grad_radiance, slot_grad, assignments);
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

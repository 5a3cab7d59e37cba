// Clustered light assignment — construct_point_light_bvh, find_unique_cluster_list and assign_lights
// (vren/vren/pipeline/clustered_shading.cpp:60-690 and the shaders under
// vren/resources/shaders/clustered_shading/).
//
// Arithmetic that decides a discrete outcome (Morton codes, depth slices, normal bins, cluster
// boxes, overlap tests) uses correctly rounded single-precision operations in a fixed order
// (__f*_rn intrinsics; this file is also compiled with --fmad=false), so the CPU oracle reproduces
// every key, list and index bit for bit.
#include "common.cuh"
#include "internal.h"
#include "bvh_common.cuh"

#include <cmath>
#include <cstring>

namespace vren_gb300 {

VREN_DEFINE_ERROR_WORD(cs)

// ================================================================================================
// Canonical float helpers
// ================================================================================================
// out[r] = ((m[0][r]*x + m[1][r]*y) + m[2][r]*z) + m[3][r]*w, m column-major.
__device__ __forceinline__ float mv_row(const float* m, int r, float x, float y, float z, float w)
{
    return fadd(fadd(fadd(fmul(m[r], x), fmul(m[4 + r], y)), fmul(m[8 + r], z)), fmul(m[12 + r], w));
}

__device__ __forceinline__ float glsl_min(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float glsl_max(float x, float y) { return x < y ? y : x; }

// clustered_shading.glsl:128-164.  The reference walks the three axes with t_i = sign(n_i) / n_i
// (= |rcp_rn(n_i)|, NaN for a zero or NaN component) and keeps the first strictly smaller t below
// 1e35; the cube face and the 3x3 cell on it follow from that axis and t.  Here with one correctly
// rounded reciprocal instead of three: rcp_rn is monotone non-increasing in |n|, so the smallest t
// over the usable components is rcp_rn(max |n_i|), and the first component whose t rounds to that
// value is the largest |n_i| or an earlier one within rounding of it (tested exactly, only when it is
// that close).  x / 2 and x * 0.5 are the same correctly rounded value.
__device__ __forceinline__ uint32_t discretize_normal(float nx, float ny, float nz)
{
    if (nx == 0.0f && ny == 0.0f && nz == 0.0f) return 0xFFFFFFFFu;
    const float ax = fabsf(nx), ay = fabsf(ny), az = fabsf(nz);
    const float M = fmaxf(fmaxf(ax, ay), az);  // NaN components drop out
    float min_t = 1e35f;
    uint32_t axis = 0, face = 0;
    if (M > 0.0f) {
        const float t = __frcp_rn(M);
        if (t < 1e35f) {
            // a < M rounds to the same reciprocal only within 2^-21 relative of M
            const float close = fmul(M, 0.9999f);
            if (ax == M || (ax >= close && __frcp_rn(ax) == t)) axis = 0;
            else if (ay == M || (ay >= close && __frcp_rn(ay) == t)) axis = 1;
            else axis = 2;
            const float na = axis == 0 ? nx : (axis == 1 ? ny : nz);
            min_t = t;
            face = (na > 0.0f ? 1u : 0u) * 3u + axis;
        }
    }
    const float n1 = axis == 0 ? ny : (axis == 1 ? nz : nx);
    const float n2 = axis == 0 ? nz : (axis == 1 ? nx : ny);
    const float u = fmul(n1, min_t);
    const float w = fmul(n2, min_t);
    const uint32_t du = floor_to_u32(fmul(fmul(fadd(u, 1.0f), 0.5f), 3.0f));
    const uint32_t dw = floor_to_u32(fmul(fmul(fadd(w, 1.0f), 0.5f), 3.0f));
    return (face * 9u + du * 3u + dw) & 0x3Fu;
}

// Largest k in [lo, hi] with bound[k] <= z, given bound[lo] <= z; bound is non-decreasing.
__device__ __forceinline__ uint32_t slice_search(float z, const float* __restrict__ bound, uint32_t lo, uint32_t hi)
{
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        if (__ldg(bound + mid) <= z) lo = mid;
        else hi = mid - 1u;
    }
    return lo;
}

// Largest k in [0, kmax] with bound[k] <= z (0 if none) for a non-decreasing, geometric table (bound[k] = bound[0] * r^k up to rounding, as both slicing modes
// build it): a logarithmic estimate, then at most two steps each way against the table before a
// binary search takes over, so the table alone decides the result.  inv_log2_r = 1 / log2(r).
__device__ __forceinline__ uint32_t slice_of_geometric(float z, const float* __restrict__ bound, uint32_t kmax, float b0,
                                                      float inv_log2_r)
{
    if (!(b0 <= z)) return 0u;
    if (kmax == 0u) return 0u;
    const float e = __log2f(__fdividef(z, b0)) * inv_log2_r;
    uint32_t k = e >= (float)kmax ? kmax : (e > 0.0f ? (uint32_t)e : 0u);
    if (__ldg(bound + k) <= z) {
        if (k < kmax && __ldg(bound + k + 1u) <= z) {
            ++k;
            if (k < kmax && __ldg(bound + k + 1u) <= z) k = slice_search(z, bound, k + 1u, kmax);
        }
    } else {
        // bound[0] <= z < bound[k], so k >= 1
        --k;
        if (!(__ldg(bound + k) <= z)) {
            --k;
            if (!(__ldg(bound + k) <= z)) k = slice_search(z, bound, 0u, k - 1u);
        }
    }
    return k;
}

struct Box {
    float mn[3], mx[3];
};

// clustered_shading.glsl:193-231 (cluster_min / cluster_max in view space).
__device__ __forceinline__ Box cluster_box(uint32_t key, const vren_cs_frame* __restrict__ F)
{
    const uint32_t ci = key & 0xFFu, cj = (key >> 8) & 0xFFu, ck = (key >> 16) & 0x3FFu;
    const float TX = (float)F->tiles_x, TY = (float)F->tiles_y;
    const float x0 = fdiv((float)ci, TX), y0 = fdiv((float)cj, TY);
    const float x1 = fdiv((float)(ci + 1u), TX), y1 = fdiv((float)(cj + 1u), TY);
    const float ax = fsub(fmul(x0, 2.0f), 1.0f), ay = fsub(fmul(fsub(1.0f, y0), 2.0f), 1.0f);
    const float bx = fsub(fmul(x1, 2.0f), 1.0f), by = fsub(fmul(fsub(1.0f, y1), 2.0f), 1.0f);
    const float* ip = F->view.inv_proj;
    float va[4], vb[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        va[r] = mv_row(ip, r, ax, ay, 0.0f, 1.0f);
        vb[r] = mv_row(ip, r, bx, by, 0.0f, 1.0f);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        va[c] = fdiv(va[c], va[3]);
        vb[c] = fdiv(vb[c], vb[3]);
    }
    const float la = fsqrt(fadd(fadd(fmul(va[0], va[0]), fmul(va[1], va[1])), fmul(va[2], va[2])));
    const float lb = fsqrt(fadd(fadd(fmul(vb[0], vb[0]), fmul(vb[1], vb[1])), fmul(vb[2], vb[2])));
    float d1[3], d2[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        d1[c] = fdiv(va[c], la);
        d2[c] = fdiv(vb[c], lb);
    }
    const float s1 = fdiv(F->slice_near[ck], d1[2]);
    const float s2 = fdiv(F->slice_far[ck], d2[2]);
    Box b;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        b.mn[c] = fmul(s1, d1[c]);
        b.mx[c] = fmul(s2, d2[c]);
    }
    return b;
}

// assign_lights.comp:84-94
__device__ __forceinline__ bool test_aabb_aabb(const Box& c, const NodeF& n)
{
    return c.mx[0] >= n.mn[0] && c.mn[0] <= n.mx[0] && c.mx[1] >= n.mn[1] && c.mn[1] <= n.mx[1] &&
           c.mx[2] >= n.mn[2] && c.mn[2] <= n.mx[2];
}

// assign_lights.comp:97-102
__device__ __forceinline__ bool test_sphere_aabb(float ox, float oy, float oz, float r, const Box& c)
{
    const float o[3] = {ox, oy, oz};
    float d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = fsub(glsl_max(c.mn[k], glsl_min(o[k], c.mx[k])), o[k]);
    const float len = fsqrt(fadd(fadd(fmul(d[0], d[0]), fmul(d[1], d[1])), fmul(d[2], d[2])));
    return len < r;
}

// ================================================================================================
// construct_point_light_bvh
// ================================================================================================
constexpr int kLbvhThreads = 256;
constexpr int kLbvhPerThread = 4;
constexpr uint32_t kLbvhPerCta = kLbvhThreads * kLbvhPerThread;

// Scratch layout (uint32 words): [0] ticket, [8, 14) final min/max keys, [16, 16 + 8*grid)
// per-CTA partial keys; then (256-byte aligned) Morton pairs, sort temporary, sort scratch.
struct LbvhLayout {
    size_t pairs, tmp, sort, total;
};

static LbvhLayout lbvh_layout(uint32_t L, uint32_t morton_bits, uint32_t digit_bits)
{
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    const uint32_t grid = (L + kLbvhPerCta - 1) / kLbvhPerCta;
    LbvhLayout l;
    l.pairs = up((16 + 8 * (size_t)(grid ? grid : 1)) * 4);
    l.tmp = l.pairs + up((size_t)L * 8);
    l.sort = l.tmp + up((size_t)L * 8);
    l.total = l.sort + up(sort_uvec2_scratch_bytes(L, morton_bits == 30 ? 30 : 16, digit_bits));
    return l;
}

__global__ void __launch_bounds__(kLbvhThreads) lbvh_transform_kernel(
    const float4* __restrict__ positions, uint32_t L, const vren_cs_frame* __restrict__ F,
    float4* __restrict__ view_pos, uint32_t* __restrict__ scratch)
{
    __shared__ uint32_t s_keys[kLbvhThreads / 32][6];
    __shared__ bool s_last;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const float* V = F->view.view;
    uint32_t kmin[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, kmax[3] = {0u, 0u, 0u};
#pragma unroll
    for (int k = 0; k < kLbvhPerThread; ++k) {
        const uint32_t i = blockIdx.x * kLbvhPerCta + k * kLbvhThreads + tid;
        if (i < L) {
            const float4 p = positions[i];
            float4 v;
            v.x = mv_row(V, 0, p.x, p.y, p.z, 1.0f);
            v.y = mv_row(V, 1, p.x, p.y, p.z, 1.0f);
            v.z = mv_row(V, 2, p.x, p.y, p.z, 1.0f);
            v.w = mv_row(V, 3, p.x, p.y, p.z, 1.0f);
            view_pos[i] = v;
            const float c[3] = {v.x, v.y, v.z};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const uint32_t key = fkey(c[a]);
                kmin[a] = key < kmin[a] ? key : kmin[a];
                kmax[a] = key > kmax[a] ? key : kmax[a];
            }
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        kmin[a] = __reduce_min_sync(0xFFFFFFFFu, kmin[a]);
        kmax[a] = __reduce_max_sync(0xFFFFFFFFu, kmax[a]);
    }
    if (lane == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            s_keys[warp][a] = kmin[a];
            s_keys[warp][3 + a] = kmax[a];
        }
    }
    __syncthreads();
    if (tid < 6) {
        uint32_t v = tid < 3 ? 0xFFFFFFFFu : 0u;
        for (int w = 0; w < kLbvhThreads / 32; ++w) {
            const uint32_t x = s_keys[w][tid];
            v = tid < 3 ? (x < v ? x : v) : (x > v ? x : v);
        }
        scratch[16 + 8 * blockIdx.x + tid] = v;
    }
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        s_last = atomicAdd(scratch, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    if (tid < 6) {
        uint32_t v = tid < 3 ? 0xFFFFFFFFu : 0u;
        for (uint32_t b = 0; b < gridDim.x; ++b) {
            const uint32_t x = ld_relaxed_u32(scratch + 16 + 8 * b + tid);
            v = tid < 3 ? (x < v ? x : v) : (x > v ? x : v);
        }
        scratch[8 + tid] = v;
    }
    if (tid == 0) scratch[0] = 0u;
}

// discretize_point_light_positions.comp:58-75
__global__ void lbvh_morton_kernel(const float4* __restrict__ view_pos, uint32_t L, const uint32_t* __restrict__ scratch,
                                   uint32_t bits, uint2* __restrict__ pairs)
{
    float mn[3], mx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        mn[a] = unkey(scratch[8 + a]);
        mx[a] = unkey(scratch[11 + a]);
    }
    const float scale = (float)(1u << bits);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x) {
        const float4 v = view_pos[i];
        const float c[3] = {v.x, v.y, v.z};
        uint32_t q[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) q[a] = floor_to_u32(fmul(fdiv(fsub(c[a], mn[a]), fsub(mx[a], mn[a])), scale));
        uint32_t code = 0;
        for (uint32_t b = 0; b < bits; ++b) {
            code |= ((q[0] >> b) & 1u) << (b * 3u);
            code |= ((q[1] >> b) & 1u) << (b * 3u + 1u);
            code |= ((q[2] >> b) & 1u) << (b * 3u + 2u);
        }
        pairs[i] = make_uint2(code, i);
    }
}

// init_light_array_bvh.comp:117-139 fused with the first one or two BuildBVH levels.
__global__ void __launch_bounds__(1024) lbvh_leaves_kernel(
    const uint2* __restrict__ light_index, const float4* __restrict__ view_pos, const float4* __restrict__ lights,
    uint32_t L, uint32_t P, vren_bvh_node* __restrict__ bvh, float4* __restrict__ spheres, int two_levels)
{
    __shared__ NodeF s_parent[32];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t i = blockIdx.x * blockDim.x + tid;
    NodeF leaf;
    float4 sph;
    if (i < L) {
        const uint32_t li = light_index[i].y;
        const float4 o = view_pos[li];
        const float r = lights[li].w;
        leaf.mn[0] = fsub(o.x, r); leaf.mn[1] = fsub(o.y, r); leaf.mn[2] = fsub(o.z, r);
        leaf.mx[0] = fadd(o.x, r); leaf.mx[1] = fadd(o.y, r); leaf.mx[2] = fadd(o.z, r);
        leaf.next = VREN_BVH_LEAF_NODE;
        sph = make_float4(o.x, o.y, o.z, fdiv(fsub(leaf.mx[0], leaf.mn[0]), 2.0f));
    } else {
        leaf.mn[0] = leaf.mn[1] = leaf.mn[2] = __int_as_float(0x7F800000);
        leaf.mx[0] = leaf.mx[1] = leaf.mx[2] = __int_as_float(0xFF800000);
        leaf.next = VREN_BVH_INVALID_NODE;
        sph = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    }
    leaf.pad = 0u;
    store_node(bvh, i, leaf);
    if (spheres) spheres[i] = sph;
    const NodeF p = warp_parent(leaf, true, i & ~31u);
    if (lane == 0) {
        store_node(bvh, P + (i >> 5), p);
        if (two_levels) s_parent[warp] = p;
    }
    if (!two_levels) return;
    __syncthreads();
    if (warp == 0) {
        const NodeF g = warp_parent(s_parent[lane], true, P + blockIdx.x * 32u);
        if (lane == 0) store_node(bvh, P + P / 32u + blockIdx.x, g);
    }
}

static int construct_light_bvh(cudaStream_t st, const float* positions, const float* lights, uint32_t L,
                               const vren_cs_frame* frame, uint32_t morton_bits, uint32_t digit_bits, float* view_pos,
                               vren_bvh_node* bvh, uint32_t* light_index, float* spheres, void* scratch)
{
    if (L == 0) return VREN_OK;
    const LbvhLayout lay = lbvh_layout(L, morton_bits, digit_bits);
    char* sc = static_cast<char*>(scratch);
    uint32_t* hdr = reinterpret_cast<uint32_t*>(sc);
    uint2* pairs = reinterpret_cast<uint2*>(sc + lay.pairs);
    uint32_t* tmp = reinterpret_cast<uint32_t*>(sc + lay.tmp);
    const uint32_t grid = (L + kLbvhPerCta - 1) / kLbvhPerCta;

    lbvh_transform_kernel<<<grid, kLbvhThreads, 0, st>>>(reinterpret_cast<const float4*>(positions), L, frame,
                                                         reinterpret_cast<float4*>(view_pos), hdr);
    VREN_LAUNCH_CHECK();
    const uint32_t bits = morton_bits == 30 ? 10u : 5u;
    uint32_t mgrid = (L + 255) / 256;
    if (mgrid > 1024) mgrid = 1024;
    lbvh_morton_kernel<<<mgrid, 256, 0, st>>>(reinterpret_cast<const float4*>(view_pos), L, hdr, bits, pairs);
    VREN_LAUNCH_CHECK();
    // bucket sort on the low 16 bits (bucket_sort.hpp:15-16); the 30-bit extension sorts 30 bits
    int rc = sort_uvec2(st, reinterpret_cast<const uint32_t*>(pairs), light_index, tmp, L, morton_bits == 30 ? 30 : 16,
                        digit_bits, sc + lay.sort);
    if (rc != VREN_OK) return rc;

    const uint32_t P = vren_calc_bvh_padded_leaf_count(L);
    const uint32_t threads = P < 1024 ? P : 1024;
    const int two = P >= 1024 ? 1 : 0;
    lbvh_leaves_kernel<<<P / threads, threads, 0, st>>>(
        reinterpret_cast<const uint2*>(light_index), reinterpret_cast<const float4*>(view_pos),
        reinterpret_cast<const float4*>(lights), L, P, bvh, reinterpret_cast<float4*>(spheres), two);
    VREN_LAUNCH_CHECK();
    if (P >= 32768) return build_bvh_levels(st, bvh, P + P / 32u, P / 1024u);
    return VREN_OK;
}

// ================================================================================================
// find_unique_cluster_list
// ================================================================================================
constexpr int kFucThreads = 256;
constexpr uint32_t kFucHeaderWords = 4;  // start ticket, done ticket, epoch, unused

__device__ __forceinline__ uint64_t make_status(uint32_t epoch, uint32_t flag, uint32_t value)
{
    return ((uint64_t)((epoch << 2) | flag) << 32) | value;
}

// One CTA per 32x32 tile (find_unique_clusters.comp:46-120).  The reference sorts the tile's 1024
// (key, pixel) pairs with a 55-stage bitonic network; here the 16 varying key bits (slice and
// normal; the tile coordinates are constant inside a tile) index a 65536-bit set in shared
// memory, so the sorted unique keys and every pixel's rank fall out of a popcount prefix.  A
// 2048-bit occupancy mask records which words of the set are non-zero, so the prefix visits only
// those (a tile holds a handful of distinct keys).  Thread t owns a strip of four horizontally
// adjacent pixels (row t / 8, columns 4 (t % 8) .. + 3), read with 128-bit loads when the row is
// 16-byte aligned; along a strip a pixel whose depth (normal) bits equal its left neighbour's
// reuses that neighbour's slice (normal bin), and only the first pixel of each run of equal
// sub-keys along a row touches the set.  Tiles are ordered by a dynamic ticket; decoupled
// look-back over the tiles gives each tile's offset in the key list (row-major tile order).
__global__ void __launch_bounds__(kFucThreads, 6) find_unique_kernel(
    const float* __restrict__ depth, const float* __restrict__ normals, uint32_t W, uint32_t H,
    const vren_cs_frame* __restrict__ F, uint32_t* __restrict__ keys, uint32_t key_cap,
    uint32_t* __restrict__ key_count, uint32_t* __restrict__ refs, uint32_t* __restrict__ scratch,
    uint32_t num_tiles, uint32_t wait_limit, uint32_t spin, int vec)
{
    __shared__ __align__(16) uint32_t s_bits[2048];
    __shared__ uint32_t s_prefix[2048];
    __shared__ uint32_t s_used[64];  // bit w: word w of s_bits is non-zero
    __shared__ uint32_t s_tile, s_epoch, s_offset;

    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) {
        s_tile = atomicAdd(scratch + 0, 1u);
        s_epoch = ld_relaxed_u32(scratch + 2) & 0x3FFFFFFFu;
    }
    reinterpret_cast<uint4*>(s_bits)[tid] = make_uint4(0u, 0u, 0u, 0u);
    reinterpret_cast<uint4*>(s_bits)[tid + kFucThreads] = make_uint4(0u, 0u, 0u, 0u);
    if (tid < 64) s_used[tid] = 0u;
    __syncthreads();
    const uint32_t tile = s_tile, epoch = s_epoch;
    const uint32_t TX = (W + 31) / 32;
    const uint32_t tx = tile % TX, ty = tile / TX;
    const uint32_t kmax = F->max_slice;
    const bool skip_offscreen = F->offscreen == VREN_CS_OFFSCREEN_SKIP;
    const float* ip = F->view.inv_proj;
    const float m2[4] = {ip[2], ip[6], ip[10], ip[14]};
    const float m3[4] = {ip[3], ip[7], ip[11], ip[15]};
    const float fW = (float)W, fH = (float)H;
    // For a perspective projection the z and w rows of its inverse have exact zeros in the x and y
    // columns and non-zero last coefficients.  Then X and Y only contribute signed zeros to a partial
    // sum that is either non-zero already or followed by the non-zero last term, so skipping them
    // leaves every bit of vz and vw unchanged (and the slice depends on the depth alone).
    const bool xy_free = m2[0] == 0.0f && m2[1] == 0.0f && m3[0] == 0.0f && m3[1] == 0.0f && m2[3] != 0.0f &&
                         m3[3] != 0.0f;
    const float* bound = F->slice_near;
    const float b0 = __ldg(bound);
    const float inv_log2_r = kmax ? __frcp_rn(__log2f(__fdividef(__ldg(bound + 1), b0))) : 0.0f;

    const uint32_t row = tid >> 3, strip = tid & 7u;
    const uint32_t gy = ty * 32u + row, gx0 = tx * 32u + strip * 4u;
    const bool full = vec && gy < H && gx0 + 3u < W;  // whole strip on screen, 16-byte aligned
    float D[4], N[4][3];
    bool on[4];
    if (full) {
        const size_t px0 = (size_t)gy * W + gx0;
        const float4 d4 = __ldg(reinterpret_cast<const float4*>(depth + px0));
        const float4* np = reinterpret_cast<const float4*>(normals + 3 * px0);
        const float4 a = __ldg(np), b = __ldg(np + 1), c = __ldg(np + 2);
        D[0] = d4.x; D[1] = d4.y; D[2] = d4.z; D[3] = d4.w;
        N[0][0] = a.x; N[0][1] = a.y; N[0][2] = a.z;
        N[1][0] = a.w; N[1][1] = b.x; N[1][2] = b.y;
        N[2][0] = b.z; N[2][1] = b.w; N[2][2] = c.x;
        N[3][0] = c.y; N[3][1] = c.z; N[3][2] = c.w;
#pragma unroll
        for (int j = 0; j < 4; ++j) on[j] = true;
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t gx = gx0 + j;
            on[j] = !(skip_offscreen && (gx >= W || gy >= H));
            // texel (x mod W, y mod H); a tile overhangs the image by less than 32 pixels
            const uint32_t xw = gx < W ? gx : gx % W, yw = gy < H ? gy : gy % H;
            const size_t px = (size_t)yw * W + xw;
            D[j] = on[j] ? __ldg(depth + px) : 0.0f;
#pragma unroll
            for (int c = 0; c < 3; ++c) N[j][c] = on[j] ? __ldg(normals + 3 * px + c) : 0.0f;
        }
    }

    uint32_t sub[4], k = 0, nd = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const bool same_d = j > 0 && xy_free && __float_as_uint(D[j]) == __float_as_uint(D[j - 1]);
        if (!same_d) {
            float vz, vw;
            if (xy_free) {
                vz = fadd(fmul(m2[2], D[j]), m2[3]);
                vw = fadd(fmul(m3[2], D[j]), m3[3]);
            } else {
                const float fx = fdiv((float)(gx0 + j), fW), fy = fdiv((float)gy, fH);
                const float X = fsub(fmul(fx, 2.0f), 1.0f), Y = fsub(fmul(fsub(1.0f, fy), 2.0f), 1.0f);
                vz = fadd(fadd(fadd(fmul(m2[0], X), fmul(m2[1], Y)), fmul(m2[2], D[j])), fmul(m2[3], 1.0f));
                vw = fadd(fadd(fadd(fmul(m3[0], X), fmul(m3[1], Y)), fmul(m3[2], D[j])), fmul(m3[3], 1.0f));
            }
            k = slice_of_geometric(fdiv(vz, vw), bound, kmax, b0, inv_log2_r);
        }
        const bool same_n = j > 0 && __float_as_uint(N[j][0]) == __float_as_uint(N[j - 1][0]) &&
                            __float_as_uint(N[j][1]) == __float_as_uint(N[j - 1][1]) &&
                            __float_as_uint(N[j][2]) == __float_as_uint(N[j - 1][2]);
        if (!same_n) nd = discretize_normal(N[j][0], N[j][1], N[j][2]);
        sub[j] = on[j] ? (((k & 0x3FFu) | (nd << 10)) & 0xFFFFu) : 0xFFFFFFFFu;
    }
    // One set insert per run of equal sub-keys along the row (lane - 1 holds the strip to the left).
    const uint32_t left3 = __shfl_up_sync(0xFFFFFFFFu, sub[3], 1);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t left = j ? sub[j - 1] : (strip ? left3 : 0xFFFFFFFFu);
        if (on[j] && sub[j] != left) {
            const uint32_t w = sub[j] >> 5;
            if (atomicOr(&s_bits[w], 1u << (sub[j] & 31u)) == 0u) atomicOr(&s_used[w >> 5], 1u << (w & 31u));
        }
    }
    __syncthreads();

    if (warp == 0) {
        // Lane l owns words [64 l, 64 l + 64): unique counts, exclusive scan, per-word prefixes.
        const uint32_t u0 = s_used[2 * lane], u1 = s_used[2 * lane + 1];
        uint32_t cnt = 0;
        for (uint32_t m = u0; m; m &= m - 1u) cnt += __popc(s_bits[64u * lane + __ffs(m) - 1u]);
        for (uint32_t m = u1; m; m &= m - 1u) cnt += __popc(s_bits[64u * lane + 32u + __ffs(m) - 1u]);
        uint32_t incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        const uint32_t excl = incl - cnt;
        const uint32_t tile_unique = __shfl_sync(0xFFFFFFFFu, incl, 31);
        {
            uint32_t run = excl;
            for (uint32_t m = u0; m; m &= m - 1u) {
                const uint32_t w = 64u * lane + __ffs(m) - 1u;
                s_prefix[w] = run;
                run += __popc(s_bits[w]);
            }
            for (uint32_t m = u1; m; m &= m - 1u) {
                const uint32_t w = 64u * lane + 32u + __ffs(m) - 1u;
                s_prefix[w] = run;
                run += __popc(s_bits[w]);
            }
        }

        // Decoupled look-back over tiles for this tile's offset.
        uint64_t* status = reinterpret_cast<uint64_t*>(scratch + kFucHeaderWords);
        uint32_t prefix = 0;
        if (tile == 0) {
            if (lane == 0) st_relaxed_u64(status, make_status(epoch, 2u, tile_unique));
        } else {
            if (lane == 0) st_relaxed_u64(status + tile, make_status(epoch, 1u, tile_unique));
            int64_t pos = (int64_t)tile - 1;
            bool timed_out = false;
            while (true) {
                const int64_t idx = pos - lane;
                uint32_t flag = 2u, val = 0u;
                if (idx >= 0) {
                    uint32_t ns = 32;
                    for (uint32_t round = 0;; ++round) {
                        const uint64_t w = ld_relaxed_u64(status + idx);
                        const uint32_t hi = (uint32_t)(w >> 32);
                        if ((hi >> 2) == epoch && (hi & 3u) != 0) {
                            flag = hi & 3u;
                            val = (uint32_t)w;
                            break;
                        }
                        if (round >= wait_limit) {
                            timed_out = true;
                            break;
                        }
                        if (round >= spin) {
                            __nanosleep(ns);
                            if (ns < 512) ns <<= 1;
                        }
                    }
                }
                const uint32_t pm = __ballot_sync(0xFFFFFFFFu, flag == 2u);
                const uint32_t stop = pm ? (uint32_t)(__ffs(pm) - 1) : 31u;
                uint32_t contrib = lane <= stop ? val : 0u;
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) contrib += __shfl_xor_sync(0xFFFFFFFFu, contrib, d);
                prefix += contrib;
                if (pm) break;
                pos -= 32;
            }
            if (__any_sync(0xFFFFFFFFu, timed_out) && lane == 0) VREN_RECORD_ERROR(VREN_ERR_TIMEOUT);
            if (lane == 0) st_relaxed_u64(status + tile, make_status(epoch, 2u, prefix + tile_unique));
        }
        if (lane == 0) {
            s_offset = prefix;
            if (tile == num_tiles - 1) {
                const uint32_t total = prefix + tile_unique;
                *key_count = total < key_cap ? total : key_cap;
                if (total > key_cap) VREN_RECORD_ERROR(VREN_ERR_CAPACITY);
            }
        }

        // Keys, ascending: word w bit b is the sub-key 32 w + b.
        const uint32_t low = ((ty & 0xFFu) << 8) | (tx & 0xFFu);
        uint32_t pos = prefix + excl;
        for (int h = 0; h < 2; ++h) {
            for (uint32_t m = h ? u1 : u0; m; m &= m - 1u) {
                const uint32_t w = 64u * lane + 32u * h + __ffs(m) - 1u;
                for (uint32_t bits = s_bits[w]; bits; bits &= bits - 1u) {
                    if (pos < key_cap) keys[pos] = ((w * 32u + __ffs(bits) - 1u) << 16) | low;
                    ++pos;
                }
            }
        }
    }
    __syncthreads();
    const uint32_t off = s_offset;

    // Per-pixel references (only on-screen pixels; the reference's imageStore drops the rest).
    uint32_t r[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t sj = sub[j];
        if (j > 0 && sj == sub[j - 1]) {
            r[j] = r[j - 1];
        } else if (sj != 0xFFFFFFFFu) {
            const uint32_t w = sj >> 5;
            r[j] = off + s_prefix[w] + __popc(s_bits[w] & ((1u << (sj & 31u)) - 1u));
        } else {
            r[j] = 0u;
        }
    }
    if (full) {
        *reinterpret_cast<uint4*>(refs + (size_t)gy * W + gx0) = make_uint4(r[0], r[1], r[2], r[3]);
    } else if (gy < H) {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (gx0 + j < W) refs[(size_t)gy * W + gx0 + j] = r[j];
    }

    if (tid == 0) {
        __threadfence();
        const uint32_t done = atomicAdd(scratch + 1, 1u);
        if (done == num_tiles - 1) {
            scratch[0] = 0u;
            scratch[1] = 0u;
            scratch[2] = (epoch + 1u) & 0x3FFFFFFFu;
        }
    }
}

static int launch_find_unique(cudaStream_t st, const float* depth, const float* normals, uint32_t W, uint32_t H,
                              const vren_cs_frame* frame, uint32_t* keys, uint32_t key_cap, uint32_t* key_count,
                              uint32_t* refs, uint32_t* scratch)
{
    const uint32_t tiles = ((W + 31) / 32) * ((H + 31) / 32);
    const int vec = (W % 4u == 0u) && ((uintptr_t)depth % 16u == 0u) && ((uintptr_t)normals % 16u == 0u) &&
                    ((uintptr_t)refs % 16u == 0u);
    find_unique_kernel<<<tiles, kFucThreads, 0, st>>>(depth, normals, W, H, frame, keys, key_cap, key_count, refs,
                                                      scratch, tiles, g_wait_limit,
                                                      (uint32_t)tuning(VREN_TUNE_SPIN_POLLS), vec);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

// ================================================================================================
// assign_lights
// ================================================================================================
struct LevelBase {
    uint32_t base[8];  // first node of each traversal level (0 = the root's children)
};

struct AssignArgs {
    const uint32_t* keys;
    const uint32_t* key_count;
    uint32_t key_cap;
    const vren_cs_frame* frame;
    const vren_bvh_node* bvh;
    const uint2* light_index;
    const float4* view_pos;
    const float4* spheres;
    uint32_t* counts;
    const uint32_t* offsets;
    uint32_t* indices;
    uint32_t index_cap;
};

// The reference walks the 32-ary tree with an explicit state machine over per-level overlap
// masks (assign_lights.comp:142-240): ENTERING tests the 32 nodes of a group with one ballot,
// ADVANCE clears the lowest set bit and descends into the next overlapping child.  The same
// depth-first order, written as a recursion over compile-time levels: the masks stay in
// registers and the group address is built incrementally (assign_lights.comp:108-119).
template <int LEVEL, int LC, bool WRITE, bool SPHERES>
__device__ __forceinline__ void visit(const AssignArgs& a, const LevelBase& lb, const Box& box, uint32_t rel,
                                      uint32_t lane, uint32_t& acc, uint32_t out_base)
{
    const uint32_t addr = lb.base[LEVEL] + rel;
    if constexpr (LEVEL == LC - 1) {
        bool hit = false;
        uint32_t li = 0;
        if constexpr (SPHERES) {
            const float4 s = __ldg(a.spheres + addr + lane);
            hit = test_sphere_aabb(s.x, s.y, s.z, s.w, box);
            if (WRITE && hit) li = __ldg(&a.light_index[addr + lane].y);
        } else {
            const NodeF n = load_node(a.bvh, addr + lane);
            if (n.next != VREN_BVH_INVALID_NODE) {
                li = a.light_index[addr + lane].y;
                const float4 o = a.view_pos[li];
                hit = test_sphere_aabb(o.x, o.y, o.z, fdiv(fsub(n.mx[0], n.mn[0]), 2.0f), box);
            }
        }
        const uint32_t mask = __ballot_sync(0xFFFFFFFFu, hit);
        if (WRITE && hit) {
            // assign_lights.comp:229: lanes of a group are written in descending order
            const uint32_t slot = __popc(mask & ~lanemask_lt()) - 1u;
            const uint32_t pos = out_base + acc + slot;
            if (pos < a.index_cap) a.indices[pos] = li;
            else VREN_RECORD_ERROR(VREN_ERR_CAPACITY);
        }
        acc += __popc(mask);
    } else {
        const NodeF n = load_node(a.bvh, addr + lane);
        const bool hit = n.next != VREN_BVH_INVALID_NODE && test_aabb_aabb(box, n);
        uint32_t mask = __ballot_sync(0xFFFFFFFFu, hit);
        while (mask) {
            const uint32_t ch = __ffs(mask) - 1;
            mask &= mask - 1u;
            visit<LEVEL + 1, LC, WRITE, SPHERES>(a, lb, box, 32u * (rel + ch), lane, acc, out_base);
        }
    }
}

template <int LC, bool WRITE, bool SPHERES>
__global__ void __launch_bounds__(256) assign_kernel(AssignArgs a, LevelBase lb)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps_per_cta = blockDim.x >> 5;
    const uint32_t gw = blockIdx.x * warps_per_cta + (threadIdx.x >> 5);
    const uint32_t nw = gridDim.x * warps_per_cta;
    uint32_t U = *a.key_count;
    if (U > a.key_cap) U = a.key_cap;
    for (uint32_t c = gw; c < U; c += nw) {
        const Box box = cluster_box(a.keys[c], a.frame);
        uint32_t acc = 0;
        const uint32_t out_base = WRITE ? a.offsets[c] : 0u;
        visit<0, LC, WRITE, SPHERES>(a, lb, box, 0u, lane, acc, out_base);
        if (!WRITE && lane == 0) a.counts[c] = acc;
    }
}

__global__ void zero_counts_kernel(const uint32_t* __restrict__ key_count, uint32_t key_cap, uint32_t* __restrict__ counts,
                                   uint32_t* __restrict__ offsets, uint32_t* __restrict__ total)
{
    uint32_t U = *key_count;
    if (U > key_cap) U = key_cap;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < U; c += gridDim.x * blockDim.x) {
        counts[c] = 0u;
        offsets[c] = 0u;
    }
    if (total && blockIdx.x == 0 && threadIdx.x == 0) *total = 0u;
}

template <bool WRITE, bool SPHERES>
static void launch_assign(cudaStream_t st, uint32_t lc, dim3 grid, dim3 block, const AssignArgs& a, const LevelBase& lb)
{
    switch (lc) {
    case 1: assign_kernel<1, WRITE, SPHERES><<<grid, block, 0, st>>>(a, lb); break;
    case 2: assign_kernel<2, WRITE, SPHERES><<<grid, block, 0, st>>>(a, lb); break;
    case 3: assign_kernel<3, WRITE, SPHERES><<<grid, block, 0, st>>>(a, lb); break;
    case 4: assign_kernel<4, WRITE, SPHERES><<<grid, block, 0, st>>>(a, lb); break;
    case 5: assign_kernel<5, WRITE, SPHERES><<<grid, block, 0, st>>>(a, lb); break;
    default: assign_kernel<6, WRITE, SPHERES><<<grid, block, 0, st>>>(a, lb); break;
    }
}

static int assign_lights(cudaStream_t st, const uint32_t* keys, const uint32_t* key_count, uint32_t key_cap,
                         const vren_cs_frame* frame, const vren_bvh_node* bvh, uint32_t L, const uint32_t* light_index,
                         const float* view_pos, const float* spheres, uint32_t* counts, uint32_t* offsets,
                         uint32_t* indices, uint32_t index_cap, uint32_t* total, void* scratch, uint32_t warps_per_cta)
{
    if (L == 0) {
        zero_counts_kernel<<<256, 256, 0, st>>>(key_count, key_cap, counts, offsets, total);
        VREN_LAUNCH_CHECK();
        return VREN_OK;
    }
    const uint32_t lc = vren_calc_bvh_level_count(L);
    if (lc < 1 || lc > 6) return VREN_ERR_ARG;
    LevelBase lb{};
    const uint32_t root = vren_calc_bvh_root_index(L);
    uint64_t sub = 0, pw = 32;
    for (uint32_t l = 0; l < lc; ++l) {
        sub += pw;
        pw *= 32;
        lb.base[l] = (uint32_t)((uint64_t)root - sub);
    }
    AssignArgs a{keys, key_count, key_cap, frame, bvh, reinterpret_cast<const uint2*>(light_index),
                 reinterpret_cast<const float4*>(view_pos), reinterpret_cast<const float4*>(spheres),
                 counts, offsets, indices, index_cap};
    if (warps_per_cta < 1 || warps_per_cta > 8) warps_per_cta = 8;
    const dim3 block(32 * warps_per_cta);
    const dim3 grid(kNumSMsHint * (64 / warps_per_cta));
    if (spheres) launch_assign<false, true>(st, lc, grid, block, a, lb);
    else launch_assign<false, false>(st, lc, grid, block, a, lb);
    VREN_LAUNCH_CHECK();
    int rc = scan_exclusive_u32(st, counts, offsets, key_cap, key_count, total, scratch);
    if (rc != VREN_OK) return rc;
    if (spheres) launch_assign<true, true>(st, lc, grid, block, a, lb);
    else launch_assign<true, false>(st, lc, grid, block, a, lb);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

__global__ void frame_upload_kernel(vren_cs_frame f, vren_cs_frame* __restrict__ dst)
{
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&f);
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
    for (uint32_t i = threadIdx.x; i < sizeof(vren_cs_frame) / 4; i += blockDim.x) d[i] = src[i];
}

}  // namespace vren_gb300

using namespace vren_gb300;

// ================================================================================================
// Host helpers: camera matrices and frame blocks
// ================================================================================================
namespace {

using M4 = double[4][4];  // [col][row], like glm

void m4_identity(M4 m)
{
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) m[c][r] = c == r ? 1.0 : 0.0;
}

void m4_mul(const M4 a, const M4 b, M4 out)
{
    M4 t;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            double s = 0;
            for (int k = 0; k < 4; ++k) s += a[k][r] * b[c][k];
            t[c][r] = s;
        }
    std::memcpy(out, t, sizeof(M4));
}

// Rotation by angle about a unit axis (right-handed, like glm::rotate).
void m4_rotate(double angle, double x, double y, double z, M4 out)
{
    const double c = std::cos(angle), s = std::sin(angle), t = 1.0 - c;
    m4_identity(out);
    out[0][0] = c + x * x * t;     out[0][1] = y * x * t + z * s; out[0][2] = z * x * t - y * s;
    out[1][0] = x * y * t - z * s; out[1][1] = c + y * y * t;     out[1][2] = z * y * t + x * s;
    out[2][0] = x * z * t + y * s; out[2][1] = y * z * t - x * s; out[2][2] = c + z * z * t;
}

bool m4_inverse(const M4 m, M4 out)
{
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = m[c][r];
            a[r][4 + c] = r == c ? 1.0 : 0.0;
        }
    for (int col = 0; col < 4; ++col) {
        int piv = col;
        for (int r = col + 1; r < 4; ++r)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        if (a[piv][col] == 0.0) return false;
        if (piv != col)
            for (int k = 0; k < 8; ++k) std::swap(a[piv][k], a[col][k]);
        const double inv = 1.0 / a[col][col];
        for (int k = 0; k < 8; ++k) a[col][k] *= inv;
        for (int r = 0; r < 4; ++r) {
            if (r == col || a[r][col] == 0.0) continue;
            const double f = a[r][col];
            for (int k = 0; k < 8; ++k) a[r][k] -= f * a[col][k];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c][r] = a[r][4 + c];
    return true;
}

void m4_store(const M4 m, float* dst)
{
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) dst[c * 4 + r] = (float)m[c][r];
}

}  // namespace

extern "C" void vren_cs_view_from_camera(const vren_camera* cam, uint32_t slicing, vren_cs_view* out)
{
    std::memset(out, 0, sizeof(*out));
    // camera.cpp:43-49: orientation = rotate(yaw, Y) * rotate(-pitch, X)
    M4 ry, rx, orient, inv_orient, inv_t, view, proj, inv_proj, inv_view;
    m4_rotate(cam->yaw, 0, 1, 0, ry);
    m4_rotate(-(double)cam->pitch, 1, 0, 0, rx);
    m4_mul(ry, rx, orient);
    m4_inverse(orient, inv_orient);
    // camera.cpp:66-72: view = inverse(orientation) * translate(-position)
    m4_identity(inv_t);
    inv_t[3][0] = -(double)cam->position[0];
    inv_t[3][1] = -(double)cam->position[1];
    inv_t[3][2] = -(double)cam->position[2];
    m4_mul(inv_orient, inv_t, view);
    // camera.cpp:74-84
    const double th = std::tan((double)cam->fov_y / 2.0);
    const double n = cam->near_plane, f = cam->far_plane;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) proj[c][r] = 0.0;
    proj[0][0] = 1.0 / (th * cam->aspect_ratio);
    proj[1][1] = 1.0 / th;
    proj[2][2] = f / (f - n);
    proj[2][3] = 1.0;
    proj[3][2] = -(f * n) / (f - n);
    m4_inverse(proj, inv_proj);
    m4_inverse(view, inv_view);
    m4_store(view, out->view);
    m4_store(inv_proj, out->inv_proj);
    m4_store(inv_view, out->inv_view);
    for (int i = 0; i < 3; ++i) out->eye[i] = cam->position[i];
    out->near_plane = cam->near_plane;
    out->far_plane = cam->far_plane;
    out->half_fov_y = cam->fov_y / 2.0f;
    out->slicing = slicing;
}

extern "C" int vren_cs_frame_build(const vren_cs_view* view, uint32_t width, uint32_t height, int offscreen,
                                   vren_cs_frame* out)
{
    if (!view || !out || width == 0 || height == 0) return VREN_ERR_ARG;
    if (offscreen != VREN_CS_OFFSCREEN_WRAP && offscreen != VREN_CS_OFFSCREEN_SKIP) return VREN_ERR_ARG;
    if (view->slicing != VREN_CS_SLICING_REF && view->slicing != VREN_CS_SLICING_FIXED32) return VREN_ERR_ARG;
    std::memset(out, 0, sizeof(*out));
    out->view = *view;
    out->width = width;
    out->height = height;
    out->tiles_x = (width + 31) / 32;
    out->tiles_y = (height + 31) / 32;
    out->offscreen = (uint32_t)offscreen;
    double bound[VREN_CS_SLICES + 1];
    const double nr = view->near_plane;
    if (view->slicing == VREN_CS_SLICING_FIXED32) {
        out->max_slice = 31;
        const double r = std::pow((double)view->far_plane / nr, 1.0 / 32.0);
        double p = 1.0;
        for (int k = 0; k <= VREN_CS_SLICES; ++k) {
            bound[k] = k <= 32 ? nr * p : INFINITY;
            p *= r;
        }
    } else {
        out->max_slice = VREN_CS_SLICES - 1;
        const double a = 1.0 + 2.0 * std::tan((double)view->half_fov_y) / (double)out->tiles_y;
        double p = 1.0;
        for (int k = 0; k <= VREN_CS_SLICES; ++k) {
            bound[k] = nr * p;
            p *= a;
        }
    }
    for (int k = 0; k < VREN_CS_SLICES; ++k) {
        out->slice_near[k] = (float)bound[k];
        out->slice_far[k] = (float)bound[k + 1];
    }
    return VREN_OK;
}

extern "C" int vren_cs_frame_upload(vren_stream_t s, const vren_cs_frame* host_frame, vren_cs_frame* device_frame)
{
    if (!host_frame || !device_frame || ((uintptr_t)device_frame & 15u)) return VREN_ERR_ARG;
    frame_upload_kernel<<<1, 256, 0, as_stream(s)>>>(*host_frame, device_frame);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

// ================================================================================================
// Stage entry points
// ================================================================================================
extern "C" size_t vren_cs_light_bvh_scratch_bytes(uint32_t light_count, uint32_t morton_bits)
{
    return lbvh_layout(light_count, morton_bits, 8).total;
}

extern "C" int vren_cs_construct_light_bvh(vren_stream_t s, const float* light_positions, const float* point_lights,
                                           uint32_t light_count, const vren_cs_frame* frame, uint32_t morton_bits,
                                           float* view_positions, vren_bvh_node* bvh, uint32_t* light_index,
                                           float* leaf_spheres, void* scratch)
{
    if (morton_bits != 15 && morton_bits != 30) return VREN_ERR_ARG;
    if (light_count == 0) return VREN_OK;
    if (light_count > (1u << 30) || !light_positions || !point_lights || !frame || !view_positions || !bvh ||
        !light_index || !scratch)
        return VREN_ERR_ARG;
    if (((uintptr_t)light_positions | (uintptr_t)point_lights | (uintptr_t)view_positions | (uintptr_t)bvh |
         (uintptr_t)leaf_spheres | (uintptr_t)light_index | (uintptr_t)scratch) & 15u)
        return VREN_ERR_ARG;
    return construct_light_bvh(as_stream(s), light_positions, point_lights, light_count, frame, morton_bits, 8,
                               view_positions, bvh, light_index, leaf_spheres, scratch);
}

extern "C" size_t vren_cs_unique_clusters_scratch_bytes(uint32_t width, uint32_t height)
{
    const uint64_t tiles = (uint64_t)((width + 31) / 32) * ((height + 31) / 32);
    return (size_t)(kFucHeaderWords * 4 + tiles * 8);
}

extern "C" int vren_cs_find_unique_clusters(vren_stream_t s, const float* depth, const float* normals, uint32_t width,
                                            uint32_t height, const vren_cs_frame* frame, uint32_t* cluster_keys,
                                            uint32_t key_capacity, uint32_t* key_count, uint32_t* cluster_refs,
                                            void* scratch)
{
    if (!depth || !normals || !frame || !cluster_keys || !key_count || !cluster_refs || !scratch) return VREN_ERR_ARG;
    if (width == 0 || height == 0 || width > 8192 || height > 8192) return VREN_ERR_ARG;
    if ((uintptr_t)scratch & 7u) return VREN_ERR_ARG;
    return launch_find_unique(as_stream(s), depth, normals, width, height, frame, cluster_keys, key_capacity,
                              key_count, cluster_refs, static_cast<uint32_t*>(scratch));
}

extern "C" size_t vren_cs_assign_lights_scratch_bytes(uint32_t key_capacity) { return scan_scratch_bytes(key_capacity); }

extern "C" int vren_cs_assign_lights(vren_stream_t s, const uint32_t* cluster_keys, const uint32_t* key_count,
                                     uint32_t key_capacity, const vren_cs_frame* frame, const vren_bvh_node* bvh,
                                     uint32_t light_count, const uint32_t* light_index, const float* view_positions,
                                     const float* leaf_spheres, uint32_t* counts, uint32_t* offsets, uint32_t* indices,
                                     uint32_t index_capacity, uint32_t* total, void* scratch)
{
    if (!cluster_keys || !key_count || !frame || !counts || !offsets || !scratch) return VREN_ERR_ARG;
    if (light_count > 0 && (!bvh || !light_index || !indices || (!view_positions && !leaf_spheres))) return VREN_ERR_ARG;
    if (((uintptr_t)bvh | (uintptr_t)leaf_spheres | (uintptr_t)view_positions | (uintptr_t)scratch) & 15u)
        return VREN_ERR_ARG;
    return assign_lights(as_stream(s), cluster_keys, key_count, key_capacity, frame, bvh, light_count, light_index,
                         view_positions, leaf_spheres, counts, offsets, indices, index_capacity, total, scratch, 8);
}

// ================================================================================================
// cluster_and_shade context (clustered_shading.cpp:817-1172): owns its buffers.
// ================================================================================================
struct vren_cluster_and_shade {
    uint32_t max_w = 0, max_h = 0, max_lights = 0, max_assign = 0;
    uint32_t key_cap = 0;
    vren_cs_options opt{15, 1, 8, 8};
    char* arena = nullptr;
    size_t arena_bytes = 0;
    // carved buffers
    vren_cs_frame* frame = nullptr;
    float* view_pos = nullptr;
    vren_bvh_node* bvh = nullptr;
    uint32_t* light_index = nullptr;
    float* spheres = nullptr;
    uint32_t* keys = nullptr;
    uint32_t* key_count = nullptr;
    uint32_t* refs = nullptr;
    uint32_t* counts = nullptr;
    uint32_t* offsets = nullptr;
    uint32_t* indices = nullptr;
    uint32_t* total = nullptr;
    void* lbvh_scratch = nullptr;
    void* fuc_scratch = nullptr;
    void* assign_scratch = nullptr;
    // host frame block (pinned) and the CUDA graph of the last frame shape
    vren_cs_frame* host_frame = nullptr;
    bool frame_valid = false;
    cudaGraphExec_t graph = nullptr;
    struct Key {
        uint32_t w, h, L, off;
        const void *depth, *normals, *pos, *lights;
        cudaStream_t stream;
        vren_cs_options opt;
    } graph_key{};
};

namespace {
size_t align256(size_t x) { return (x + 255) / 256 * 256; }

int cs_enqueue(vren_cluster_and_shade* cs, cudaStream_t st, uint32_t W, uint32_t H, const float* depth,
               const float* normals, const float* positions, const float* lights, uint32_t L)
{
    int rc = VREN_OK;
    if (L > 0) {
        rc = construct_light_bvh(st, positions, lights, L, cs->frame, cs->opt.morton_bits, cs->opt.sort_digit_bits,
                                 cs->view_pos, cs->bvh, cs->light_index, cs->spheres, cs->lbvh_scratch);
        if (rc != VREN_OK) return rc;
    }
    rc = launch_find_unique(st, depth, normals, W, H, cs->frame, cs->keys, cs->key_cap, cs->key_count, cs->refs,
                            static_cast<uint32_t*>(cs->fuc_scratch));
    if (rc != VREN_OK) return rc;
    return assign_lights(st, cs->keys, cs->key_count, cs->key_cap, cs->frame, cs->bvh, L, cs->light_index,
                         cs->view_pos, cs->spheres, cs->counts, cs->offsets, cs->indices, cs->max_assign, cs->total,
                         cs->assign_scratch, cs->opt.assign_warps);
}
}  // namespace

extern "C" int vren_cs_create(vren_cluster_and_shade** out, uint32_t max_width, uint32_t max_height,
                              uint32_t max_lights, uint32_t max_assignments)
{
    if (!out || max_width == 0 || max_height == 0 || max_width > 8192 || max_height > 8192 || max_lights > (1u << 24))
        return VREN_ERR_ARG;
    auto* cs = new vren_cluster_and_shade();
    cs->max_w = max_width;
    cs->max_h = max_height;
    cs->max_lights = max_lights;
    cs->max_assign = max_assignments;
    const uint32_t tiles = ((max_width + 31) / 32) * ((max_height + 31) / 32);
    cs->key_cap = tiles * 1024u;
    const uint32_t Lb = max_lights ? max_lights : 1;
    const uint32_t P = vren_calc_bvh_padded_leaf_count(Lb);
    size_t off = 0;
    auto carve = [&](size_t bytes) {
        size_t o = off;
        off += align256(bytes);
        return o;
    };
    const size_t o_frame = carve(sizeof(vren_cs_frame));
    const size_t o_vp = carve((size_t)Lb * 16);
    const size_t o_bvh = carve((size_t)vren_calc_bvh_buffer_length(Lb) * sizeof(vren_bvh_node));
    const size_t o_li = carve((size_t)Lb * 8);
    const size_t o_sph = carve((size_t)P * 16);
    const size_t o_keys = carve((size_t)cs->key_cap * 4);
    const size_t o_kc = carve(4);
    const size_t o_refs = carve((size_t)max_width * max_height * 4);
    const size_t o_counts = carve((size_t)cs->key_cap * 4);
    const size_t o_offs = carve((size_t)cs->key_cap * 4);
    const size_t o_idx = carve((size_t)(max_assignments ? max_assignments : 1) * 4);
    const size_t o_total = carve(4);
    size_t lbvh = 0;
    for (uint32_t db : {4u, 6u, 8u})
        for (uint32_t mb : {15u, 30u}) {
            const size_t b = lbvh_layout(Lb, mb, db).total;
            lbvh = b > lbvh ? b : lbvh;
        }
    const size_t o_lbvh = carve(lbvh);
    const size_t o_fuc = carve(vren_cs_unique_clusters_scratch_bytes(max_width, max_height));
    const size_t o_asg = carve(scan_scratch_bytes(cs->key_cap));
    cs->arena_bytes = off;
    if (cudaMalloc(&cs->arena, off) != cudaSuccess) {
        delete cs;
        return VREN_ERR_CUDA;
    }
    if (cudaMemset(cs->arena, 0, off) != cudaSuccess || cudaMallocHost(&cs->host_frame, sizeof(vren_cs_frame)) != cudaSuccess) {
        cudaFree(cs->arena);
        delete cs;
        return VREN_ERR_CUDA;
    }
    char* a = cs->arena;
    cs->frame = reinterpret_cast<vren_cs_frame*>(a + o_frame);
    cs->view_pos = reinterpret_cast<float*>(a + o_vp);
    cs->bvh = reinterpret_cast<vren_bvh_node*>(a + o_bvh);
    cs->light_index = reinterpret_cast<uint32_t*>(a + o_li);
    cs->spheres = reinterpret_cast<float*>(a + o_sph);
    cs->keys = reinterpret_cast<uint32_t*>(a + o_keys);
    cs->key_count = reinterpret_cast<uint32_t*>(a + o_kc);
    cs->refs = reinterpret_cast<uint32_t*>(a + o_refs);
    cs->counts = reinterpret_cast<uint32_t*>(a + o_counts);
    cs->offsets = reinterpret_cast<uint32_t*>(a + o_offs);
    cs->indices = reinterpret_cast<uint32_t*>(a + o_idx);
    cs->total = reinterpret_cast<uint32_t*>(a + o_total);
    cs->lbvh_scratch = a + o_lbvh;
    cs->fuc_scratch = a + o_fuc;
    cs->assign_scratch = a + o_asg;
    *out = cs;
    return VREN_OK;
}

extern "C" void vren_cs_destroy(vren_cluster_and_shade* cs)
{
    if (!cs) return;
    if (cs->graph) cudaGraphExecDestroy(cs->graph);
    cudaFree(cs->arena);
    cudaFreeHost(cs->host_frame);
    delete cs;
}

extern "C" int vren_cs_set_options(vren_cluster_and_shade* cs, const vren_cs_options* o)
{
    if (!cs || !o) return VREN_ERR_ARG;
    if (o->morton_bits != 15 && o->morton_bits != 30) return VREN_ERR_ARG;
    if (o->sort_digit_bits != 4 && o->sort_digit_bits != 6 && o->sort_digit_bits != 8) return VREN_ERR_ARG;
    if (o->assign_warps < 1 || o->assign_warps > 8) return VREN_ERR_ARG;
    cs->opt = *o;
    if (cs->graph) {
        cudaGraphExecDestroy(cs->graph);
        cs->graph = nullptr;
    }
    return VREN_OK;
}

extern "C" int vren_cs_cluster(vren_cluster_and_shade* cs, vren_stream_t s, const vren_cs_view* view, uint32_t width,
                               uint32_t height, int offscreen, const float* depth, const float* normals,
                               const float* light_positions, const float* point_lights, uint32_t light_count)
{
    if (!cs || !view || !depth || !normals) return VREN_ERR_ARG;
    if (width > cs->max_w || height > cs->max_h || light_count > cs->max_lights) return VREN_ERR_CAPACITY;
    if (light_count > 0 && (!light_positions || !point_lights)) return VREN_ERR_ARG;
    cudaStream_t st = as_stream(s);
    // The frame block lives in device memory and is read by every kernel; it is re-uploaded (from
    // pinned memory, outside the captured graph) only when the camera or the frame shape changes.
    static thread_local vren_cs_frame fresh;
    int rc = vren_cs_frame_build(view, width, height, offscreen, &fresh);
    if (rc != VREN_OK) return rc;
    if (!cs->frame_valid || std::memcmp(&fresh, cs->host_frame, sizeof(vren_cs_frame)) != 0) {
        VREN_CUDA_TRY(cudaStreamSynchronize(st));  // an earlier upload may still read host_frame
        std::memcpy(cs->host_frame, &fresh, sizeof(vren_cs_frame));
        VREN_CUDA_TRY(cudaMemcpyAsync(cs->frame, cs->host_frame, sizeof(vren_cs_frame), cudaMemcpyHostToDevice, st));
        cs->frame_valid = true;
    }
    const vren_cluster_and_shade::Key key{width, height, light_count, (uint32_t)offscreen, depth, normals,
                                          light_positions, point_lights, st, cs->opt};
    const bool use_graph = cs->opt.use_graph && st != nullptr;
    if (!use_graph) return cs_enqueue(cs, st, width, height, depth, normals, light_positions, point_lights, light_count);
    if (cs->graph && std::memcmp(&key, &cs->graph_key, sizeof(key)) == 0) {
        VREN_CUDA_TRY(cudaGraphLaunch(cs->graph, st));
        return VREN_OK;
    }
    if (cs->graph) {
        cudaGraphExecDestroy(cs->graph);
        cs->graph = nullptr;
    }
    cudaGraph_t g;
    VREN_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    rc = cs_enqueue(cs, st, width, height, depth, normals, light_positions, point_lights, light_count);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc != VREN_OK) {
        if (e == cudaSuccess) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return VREN_ERR_CUDA;
    e = cudaGraphInstantiate(&cs->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cs->graph = nullptr;
        return VREN_ERR_CUDA;
    }
    cs->graph_key = key;
    VREN_CUDA_TRY(cudaGraphLaunch(cs->graph, st));
    return VREN_OK;
}

extern "C" int vren_cs_get_outputs(const vren_cluster_and_shade* cs, vren_cs_outputs* o)
{
    if (!cs || !o) return VREN_ERR_ARG;
    o->view_positions = cs->view_pos;
    o->bvh = cs->bvh;
    o->light_index = cs->light_index;
    o->leaf_spheres = cs->spheres;
    o->cluster_keys = cs->keys;
    o->key_count = cs->key_count;
    o->cluster_refs = cs->refs;
    o->counts = cs->counts;
    o->offsets = cs->offsets;
    o->indices = cs->indices;
    o->total = cs->total;
    o->frame = cs->frame;
    o->key_capacity = cs->key_cap;
    o->index_capacity = cs->max_assign;
    return VREN_OK;
}

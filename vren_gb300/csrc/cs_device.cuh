// Device code shared by the per-frame clustered-shading kernels (clustered.cu) and their batched
// forms (batch.cu): the canonical float helpers, the per-light and per-tile bodies, and the BVH
// traversal.  Both translation units are compiled with --fmad=false and use the same functions, so a
// frame gives the same bits through either path.
//
// The including translation unit defines its device error word (VREN_DEFINE_ERROR_WORD) before
// including this header.
#pragma once

#include "common.cuh"
#include "bvh_common.cuh"
#include "lookback.cuh"

#include <cuda_fp16.h>

namespace vren_gb300 {

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

// clustered_shading.glsl:7-43.  The reference walks the three axes with t_i = sign(n_i) / n_i
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

// clustered_shading.glsl:72-110 (cluster_min / cluster_max in view space).
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
// construct_point_light_bvh bodies
// ================================================================================================
// point_light_position_to_view_space.comp:30: camera view matrix times (p, 1).
__device__ __forceinline__ float4 light_to_view(const float* V, float4 p)
{
    float4 v;
    v.x = mv_row(V, 0, p.x, p.y, p.z, 1.0f);
    v.y = mv_row(V, 1, p.x, p.y, p.z, 1.0f);
    v.z = mv_row(V, 2, p.x, p.y, p.z, 1.0f);
    v.w = mv_row(V, 3, p.x, p.y, p.z, 1.0f);
    return v;
}

// discretize_point_light_positions.comp:30-39: `bits` bits per axis, interleaved x, y, z from bit 0.
__device__ __forceinline__ uint32_t morton_code(float4 v, const float mn[3], const float mx[3], uint32_t bits)
{
    const float scale = (float)(1u << bits);
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
    return code;
}

// init_light_array_bvh.comp:42-65 fused with the first one or two BuildBVH levels, for one block of
// `threads` = min(P, 1024) leaves starting at leaf chunk * threads (all threads of the CTA call it;
// threads >= `threads` only return).  The leaf sphere is the light centre and the radius tested by
// the traversal ((max.x - min.x) / 2 of the leaf box, assign_lights.comp:214), -1 for padding.
__device__ __forceinline__ void light_leaves_block(uint32_t chunk, uint32_t threads, uint32_t L, uint32_t P,
                                                   const uint2* __restrict__ light_index,
                                                   const float4* __restrict__ view_pos, const float4* __restrict__ lights,
                                                   vren_bvh_node* __restrict__ bvh, float4* __restrict__ spheres,
                                                   NodeF* s_parent)
{
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid >= threads) return;
    const bool two_levels = threads == 1024u;
    const uint32_t i = chunk * threads + tid;
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
        const NodeF g = warp_parent(s_parent[lane], true, P + chunk * 32u);
        if (lane == 0) store_node(bvh, P + P / 32u + chunk, g);
    }
}

// ================================================================================================
// find_unique_cluster_list body
// ================================================================================================
constexpr int kFucThreads = 256;

// find_unique_cluster_list in two kernels, with no dependency between the tiles of the first:
//
// 1. One CTA per 32x32 tile (find_unique_clusters.comp:46-120).  The reference sorts the tile's 1024
//    (key, pixel) pairs with a 55-stage bitonic network; here the 16 varying key bits (slice and
//    normal; the tile coordinates are constant inside a tile) index a 65536-bit set in shared
//    memory, so the sorted unique keys and every pixel's rank fall out of a popcount prefix.  A
//    2048-bit occupancy mask records which words of the set are non-zero, so the prefix visits only
//    those (a tile holds a handful of distinct keys), and every warp computes it for itself, so only
//    one barrier separates the set inserts from the outputs.  Thread t owns a strip of four
//    horizontally adjacent pixels (row t / 8, columns 4 (t % 8) .. + 3), read with 128-bit loads when
//    the row is 16-byte aligned; along a strip a pixel whose depth (normal) bits equal its left
//    neighbour's reuses that neighbour's slice (normal bin), and only the first pixel of each run of
//    equal sub-keys along a row touches the set.  The tile writes its pixels' tile-local ranks into
//    the reference buffer, its sorted keys into its own 1024-entry slot and its key count.
// 2. One CTA scans the tile counts into tile offsets (row-major tile order) and the key count.
// 3. One CTA per tile adds the tile's offset to its references (still in L2) and copies its keys to
//    their place in the dense key list.
//
// One-kernel form (the context's device frames): the CTAs take their tiles by ticket, so every tile's
// predecessors have started; each tile publishes its key count as soon as its set is complete,
// resolves its offset among the tiles before it by decoupled look-back (warp 0), and writes its
// references and keys in their final places; the last tile writes the key count.  Stages 2 and 3 and
// their launches disappear, and the references are written once.
struct FucSmem {
    __align__(16) uint32_t bits[2048];
    uint32_t prefix[2048];
    uint32_t used[64];  // bit w: word w of bits is non-zero
    uint32_t offset;    // one-kernel form: the tile's offset in the dense key list
};

// Where one frame's find_unique_cluster_list reads and writes.
struct FucFrame {
    const float* depth;
    const float* normals;
    uint32_t W, H;
    const vren_cs_frame* F;
    uint32_t* keys;
    uint32_t key_cap;
    uint32_t* key_count;
    uint32_t* refs;
    uint32_t* tile_keys;    // [num_tiles][1024]: each tile's sorted keys
    uint32_t* tile_count;   // [num_tiles]: unique keys per tile
    uint32_t* tile_offset;  // [num_tiles]: exclusive prefix of tile_count
    uint32_t num_tiles;
    int vec;  // 128-bit accesses allowed (W % 4 == 0, 16-byte aligned depth, normals, refs)
    // one-kernel form only: look-back status per tile ([epoch:30 | flag:2 | value:32]), the polling
    // limit and the polls before back-off
    uint64_t* status;
    uint32_t wait_limit, spin;
    uint32_t* refs2;  // one-kernel form only: a second destination of the final references, or null
};

// Stage 1 for tile `tile` of frame `fr`, all threads of the CTA; sm.bits and sm.used must be zero
// (and synchronised) on entry.  FUSED: the one-kernel form (`epoch` from the tile's ticket).
template <bool FUSED = false>
__device__ __forceinline__ void find_unique_tile(const FucFrame& fr, uint32_t tile, FucSmem& sm, uint32_t epoch = 0)
{
    const float* __restrict__ depth = fr.depth;
    const float* __restrict__ normals = fr.normals;
    const uint32_t W = fr.W, H = fr.H;
    const vren_cs_frame* __restrict__ F = fr.F;
    uint32_t* __restrict__ refs = fr.refs;
    const int vec = fr.vec;
    uint32_t* s_bits = sm.bits;
    uint32_t* s_prefix = sm.prefix;
    uint32_t* s_used = sm.used;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
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
    // normals: f32x3, or RGBA16F (the reference's G-buffer format).  NR holds each pixel's raw normal
    // words (f32x3: the three floats' bits; RGBA16F: x | y << 16 and z), compared along the strip; a
    // normal is converted (half -> float is exact) and binned only where it differs from its left
    // neighbour's.
    const bool half_normals = F->normal_format == VREN_CS_NORMALS_RGBA16F;
    const unsigned short* __restrict__ hnormals = reinterpret_cast<const unsigned short*>(normals);
    float D[4];
    uint32_t NR[4][3];
    bool on[4];
    if (full) {
        const size_t px0 = (size_t)gy * W + gx0;
        const float4 d4 = __ldg(reinterpret_cast<const float4*>(depth + px0));
        D[0] = d4.x; D[1] = d4.y; D[2] = d4.z; D[3] = d4.w;
        if (half_normals) {
            const uint4* hp = reinterpret_cast<const uint4*>(hnormals + 4 * px0);
            const uint4 a = __ldg(hp), b = __ldg(hp + 1);
            NR[0][0] = a.x; NR[0][1] = a.y & 0xFFFFu;
            NR[1][0] = a.z; NR[1][1] = a.w & 0xFFFFu;
            NR[2][0] = b.x; NR[2][1] = b.y & 0xFFFFu;
            NR[3][0] = b.z; NR[3][1] = b.w & 0xFFFFu;
#pragma unroll
            for (int j = 0; j < 4; ++j) NR[j][2] = 0u;
        } else {
            const uint4* np = reinterpret_cast<const uint4*>(normals + 3 * px0);
            const uint4 a = __ldg(np), b = __ldg(np + 1), c = __ldg(np + 2);
            NR[0][0] = a.x; NR[0][1] = a.y; NR[0][2] = a.z;
            NR[1][0] = a.w; NR[1][1] = b.x; NR[1][2] = b.y;
            NR[2][0] = b.z; NR[2][1] = b.w; NR[2][2] = c.x;
            NR[3][0] = c.y; NR[3][1] = c.z; NR[3][2] = c.w;
        }
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
            if (!on[j]) {
                NR[j][0] = NR[j][1] = NR[j][2] = 0u;
            } else if (half_normals) {
                NR[j][0] = (uint32_t)__ldg(hnormals + 4 * px) | ((uint32_t)__ldg(hnormals + 4 * px + 1) << 16);
                NR[j][1] = __ldg(hnormals + 4 * px + 2);
                NR[j][2] = 0u;
            } else {
#pragma unroll
                for (int c = 0; c < 3; ++c) NR[j][c] = __float_as_uint(__ldg(normals + 3 * px + c));
            }
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
        const bool same_n =
            j > 0 && NR[j][0] == NR[j - 1][0] && NR[j][1] == NR[j - 1][1] && NR[j][2] == NR[j - 1][2];
        if (!same_n) {
            float nx, ny, nz;
            if (half_normals) {
                nx = __half2float(__ushort_as_half((unsigned short)(NR[j][0] & 0xFFFFu)));
                ny = __half2float(__ushort_as_half((unsigned short)(NR[j][0] >> 16)));
                nz = __half2float(__ushort_as_half((unsigned short)NR[j][1]));
            } else {
                nx = __uint_as_float(NR[j][0]);
                ny = __uint_as_float(NR[j][1]);
                nz = __uint_as_float(NR[j][2]);
            }
            nd = discretize_normal(nx, ny, nz);
        }
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

    // Every warp: lane l owns words [64 l, 64 l + 64); unique counts, exclusive scan over the lanes,
    // per-word prefixes (all warps store the same values).
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
    __syncwarp();
    uint32_t off = 0;  // one-kernel form: the tile's offset, added to its references
    if constexpr (FUSED) {
        if (warp == 0) {
            // publish the tile's count, find the keys before it, publish the inclusive prefix
            const uint32_t count = __shfl_sync(0xFFFFFFFFu, incl, 31);
            uint32_t prefix = 0;
            if (tile == 0) {
                if (lane == 0) st_relaxed_u64(fr.status, make_status(epoch, 2u, count));
            } else {
                if (lane == 0) st_relaxed_u64(fr.status + tile, make_status(epoch, 1u, count));
                bool timed_out = false;
                prefix = warp_lookback(fr.status, tile, 0u, epoch, lane, fr.wait_limit, fr.spin, timed_out);
                if (__any_sync(0xFFFFFFFFu, timed_out) && lane == 0) VREN_RECORD_ERROR(VREN_ERR_TIMEOUT);
                if (lane == 0) st_relaxed_u64(fr.status + tile, make_status(epoch, 2u, prefix + count));
            }
            // the tile's keys, ascending, at their place in the dense list
            const uint32_t low = ((ty & 0xFFu) << 8) | (tx & 0xFFu);
            uint32_t pos = prefix + excl;
            for (int h = 0; h < 2; ++h) {
                for (uint32_t m = h ? u1 : u0; m; m &= m - 1u) {
                    const uint32_t w = 64u * lane + 32u * h + __ffs(m) - 1u;
                    for (uint32_t bits = s_bits[w]; bits; bits &= bits - 1u, ++pos)
                        if (pos < fr.key_cap) fr.keys[pos] = ((w * 32u + __ffs(bits) - 1u) << 16) | low;
                }
            }
            if (lane == 0) {
                sm.offset = prefix;
                if (tile == fr.num_tiles - 1) {
                    const uint32_t total = prefix + count;
                    *fr.key_count = total < fr.key_cap ? total : fr.key_cap;
                    if (total > fr.key_cap) VREN_RECORD_ERROR(VREN_ERR_CAPACITY);
                }
            }
        }
        __syncthreads();
        off = sm.offset;
    } else if (warp == 0) {
        // the tile's keys, ascending (word w bit b is the sub-key 32 w + b), and their count
        const uint32_t low = ((ty & 0xFFu) << 8) | (tx & 0xFFu);
        uint32_t* out = fr.tile_keys + (size_t)tile * 1024u;
        uint32_t pos = excl;
        for (int h = 0; h < 2; ++h) {
            for (uint32_t m = h ? u1 : u0; m; m &= m - 1u) {
                const uint32_t w = 64u * lane + 32u * h + __ffs(m) - 1u;
                for (uint32_t bits = s_bits[w]; bits; bits &= bits - 1u) out[pos++] = ((w * 32u + __ffs(bits) - 1u) << 16) | low;
            }
        }
        if (lane == 31) fr.tile_count[tile] = incl;
    }

    // Tile-local ranks into the reference buffer (only on-screen pixels: the reference's imageStore
    // drops the rest).
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
        if constexpr (FUSED) {
            if (fr.refs2) *reinterpret_cast<uint4*>(fr.refs2 + (size_t)gy * W + gx0) = make_uint4(r[0], r[1], r[2], r[3]);
        }
    } else if (gy < H) {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (gx0 + j < W) {
                refs[(size_t)gy * W + gx0 + j] = r[j];
                if constexpr (FUSED) {
                    if (fr.refs2) fr.refs2[(size_t)gy * W + gx0 + j] = r[j];
                }
            }
    }

}

// Between the stages: one CTA of kFucScanThreads scans the frame's tile counts into offsets and
// writes the key count.  Thread t owns 16 consecutive counts of each 16384-tile chunk (unrolled
// loads, all in flight); chunks carry their running total.
constexpr int kFucScanThreads = 1024;
constexpr uint32_t kFucScanPer = 16;
// Tiles [t_begin, t_end) of the frame: offsets continue from the tile before t_begin (whose offset and
// count an earlier scan wrote); the key count is written when t_end is the last tile.
__device__ __forceinline__ void find_unique_scan(const FucFrame& fr, uint32_t* s_warp, uint32_t t_begin = 0,
                                                 uint32_t t_end = 0xFFFFFFFFu)
{
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t T = t_end < fr.num_tiles ? t_end : fr.num_tiles;
    uint32_t carry = t_begin ? fr.tile_offset[t_begin - 1] + fr.tile_count[t_begin - 1] : 0u;
    for (uint32_t chunk = t_begin; chunk < T; chunk += kFucScanThreads * kFucScanPer) {
        const uint32_t b0 = chunk + tid * kFucScanPer;
        uint32_t v[kFucScanPer], sum = 0;
#pragma unroll
        for (uint32_t k = 0; k < kFucScanPer; ++k) {
            v[k] = b0 + k < T ? fr.tile_count[b0 + k] : 0u;
            sum += v[k];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        __syncthreads();  // s_warp of the previous chunk has been read
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        uint32_t before = carry + incl - sum, total = 0;
#pragma unroll
        for (int w = 0; w < kFucScanThreads / 32; ++w) {
            if (w < (int)warp) before += s_warp[w];
            total += s_warp[w];
        }
#pragma unroll
        for (uint32_t k = 0; k < kFucScanPer; ++k) {
            if (b0 + k < T) fr.tile_offset[b0 + k] = before;
            before += v[k];
        }
        carry += total;
    }
    if (tid == 0 && T == fr.num_tiles) {
        *fr.key_count = carry < fr.key_cap ? carry : fr.key_cap;
        if (carry > fr.key_cap) VREN_RECORD_ERROR(VREN_ERR_CAPACITY);
    }
}

// Stages 2 and 3 together, for frames of at most kFucSelfScanTiles tiles: the CTA of tile `tile` sums
// the counts of the tiles before it (from L2) into its own offset, so no scan kernel runs between the
// tiles and the fix-up; the CTA of the last tile writes the key count.
constexpr uint32_t kFucSelfScanTiles = 16384;
__device__ __forceinline__ uint32_t find_unique_self_offset(const FucFrame& fr, uint32_t tile)
{
    __shared__ uint32_t s_part[kFucThreads / 32];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    uint32_t sum = 0;
#pragma unroll 8
    for (uint32_t i = tid; i < tile; i += kFucThreads) sum += fr.tile_count[i];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) sum += __shfl_xor_sync(0xFFFFFFFFu, sum, d);
    if (lane == 0) s_part[warp] = sum;
    __syncthreads();
    uint32_t off = 0;
#pragma unroll
    for (int w = 0; w < kFucThreads / 32; ++w) off += s_part[w];
    if (tid == 0 && tile == fr.num_tiles - 1) {
        const uint32_t total = off + fr.tile_count[tile];
        *fr.key_count = total < fr.key_cap ? total : fr.key_cap;
        if (total > fr.key_cap) VREN_RECORD_ERROR(VREN_ERR_CAPACITY);
    }
    return off;
}

// Stage 2 for tile `tile`: references += tile offset, keys to their place in the dense list (the
// offset from the scan, or summed here when SELF).
template <bool SELF = false>
__device__ __forceinline__ void find_unique_fixup(const FucFrame& fr, uint32_t tile)
{
    const uint32_t tid = threadIdx.x;
    const uint32_t off = SELF ? find_unique_self_offset(fr, tile) : fr.tile_offset[tile], n = fr.tile_count[tile];
    const uint32_t* src = fr.tile_keys + (size_t)tile * 1024u;
    for (uint32_t j = tid; j < n; j += kFucThreads)
        if (off + j < fr.key_cap) fr.keys[off + j] = src[j];
    const uint32_t W = fr.W, H = fr.H, TX = (W + 31) / 32;
    const uint32_t tx = tile % TX, ty = tile / TX;
    const uint32_t gy = ty * 32u + (tid >> 3), gx0 = tx * 32u + (tid & 7u) * 4u;
    if (gy >= H) return;
    uint32_t* row = fr.refs + (size_t)gy * W;
    if (fr.vec && gx0 + 3u < W) {
        uint4 v = *reinterpret_cast<uint4*>(row + gx0);
        v.x += off; v.y += off; v.z += off; v.w += off;
        *reinterpret_cast<uint4*>(row + gx0) = v;
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (gx0 + j < W) row[gx0 + j] += off;
    }
}

// ================================================================================================
// assign_lights traversal
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
    uint32_t* stage;       // optional: the count pass keeps each cluster's first kStageLights lights here
    uint32_t stage_slots;  // clusters c < stage_slots own stage[c * kStageLights ..]
};

// Lights a cluster can keep from the count pass for the write pass to copy instead of traversing again.
constexpr uint32_t kStageLights = 128;

// The reference walks the 32-ary tree with an explicit state machine over per-level overlap
// masks (assign_lights.comp:142-240): ENTERING tests the 32 nodes of a group with one ballot,
// ADVANCE clears the lowest set bit and descends into the next overlapping child.  The same
// depth-first order, written as a recursion over compile-time levels: the masks stay in
// registers and the group address is built incrementally (assign_lights.comp:108-119).
template <int LEVEL, int LC, bool WRITE, bool SPHERES, bool STAGE = false>
__device__ __forceinline__ void visit(const AssignArgs& a, const LevelBase& lb, const Box& box, uint32_t rel,
                                      uint32_t lane, uint32_t& acc, uint32_t out_base)  // STAGE: out_base = c * kStageLights
{
    const uint32_t addr = lb.base[LEVEL] + rel;
    if constexpr (LEVEL == LC - 1) {
        bool hit = false;
        uint32_t li = 0;
        if constexpr (SPHERES) {
            const float4 s = __ldg(a.spheres + addr + lane);
            hit = test_sphere_aabb(s.x, s.y, s.z, s.w, box);
            if ((WRITE || STAGE) && hit) li = __ldg(&a.light_index[addr + lane].y);
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
        if (STAGE && hit) {  // the same order, into the cluster's stage slots (the first kStageLights)
            const uint32_t local = acc + __popc(mask & ~lanemask_lt()) - 1u;
            if (local < kStageLights) a.stage[out_base + local] = li;
        }
        acc += __popc(mask);
    } else {
        const NodeF n = load_node(a.bvh, addr + lane);
        const bool hit = n.next != VREN_BVH_INVALID_NODE && test_aabb_aabb(box, n);
        uint32_t mask = __ballot_sync(0xFFFFFFFFu, hit);
        while (mask) {
            const uint32_t ch = __ffs(mask) - 1;
            mask &= mask - 1u;
            visit<LEVEL + 1, LC, WRITE, SPHERES, STAGE>(a, lb, box, 32u * (rel + ch), lane, acc, out_base);
        }
    }
}


// Traversal of one cluster (warp-wide): returns the number of lights assigned, and with WRITE writes
// them from out_base on.
template <int LC, bool WRITE, bool SPHERES, bool STAGE = false>
__device__ __forceinline__ uint32_t assign_cluster(const AssignArgs& a, const LevelBase& lb, uint32_t key,
                                                   uint32_t out_base, uint32_t lane)
{
    const Box box = cluster_box(key, a.frame);
    uint32_t acc = 0;
    visit<0, LC, WRITE, SPHERES, STAGE>(a, lb, box, 0u, lane, acc, out_base);
    return acc;
}

// Traversal level bases of the BVH over L lights: base[l] = first node of level l below the root
// (assign_lights.comp:108-119).  Returns the level count (0 for L == 0).
__host__ __device__ __forceinline__ uint32_t traversal_levels(uint32_t L, LevelBase& lb)
{
    if (L == 0) return 0u;
    uint64_t p = 32;  // padded leaf count (calc_bvh_padded_leaf_count)
    while (p < L) p <<= 5;
    uint64_t len = 0;
    uint32_t lc = 0;
    for (uint64_t q = p; q != 0; q >>= 5) len += q;
    for (uint64_t q = p; q > 1; q >>= 5) ++lc;
    const uint64_t root = len - 1;
    uint64_t sub = 0, pw = 32;
    for (uint32_t l = 0; l < lc && l < 8; ++l) {
        sub += pw;
        pw *= 32;
        lb.base[l] = (uint32_t)(root - sub);
    }
    return lc;
}

}  // namespace vren_gb300

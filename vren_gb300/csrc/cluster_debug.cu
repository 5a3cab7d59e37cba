// Headless cluster debug views (vren_demo/vren_demo/clustered_shading_debug.cpp:6-202):
//
//  - show_clusters (vren_demo/resources/shaders/show_clusters.comp:68-125): one RGBA float colour per
//    pixel of the cluster-reference image, by mode: a hash of the cluster key, the cluster's (i, j, k),
//    its normal bin, its light count, a hash of its light-list offset, a hash of the XOR of its light
//    indices.  Every mode's colour is a function of the pixel's cluster alone, so the kernel pair is:
//    one colour per cluster (a warp per cluster, the XOR of its list reduced across lanes), then one
//    gather per pixel (4 B reference read, 16 B colour from L2, 16 B written).
//  - show_clusters_geometry (show_clusters_geometry.comp:54-112, debug.glsl): per cluster, the 12 edges
//    of its view-space box and an arrow along its normal bin, 32 vertices of (vec3 position, u32 colour),
//    the reference's debug-renderer vertex layout.  The box is the one the light assignment tests.
//
// Arithmetic as the rest of the clustered path: every operation rounded on its own (this unit is
// compiled with --fmad=false), IEEE division and square root, GLSL min.
#include "common.cuh"

namespace vren_gb300 {
VREN_DEFINE_ERROR_WORD(cluster_debug)
}

#include "cs_device.cuh"

namespace vren_gb300 {
namespace {

constexpr uint32_t kNoNormal = 0x3Fu;
constexpr int kGeomVerticesPerCluster = 32;  // 12 box edges (24) + arrow (2 + 6)

// triple32 (show_clusters.comp:51-61): the integer hash with the three multiply-xorshift rounds
// published by C. Wellons ("hash prospector"), constants as in the shader.
__host__ __device__ __forceinline__ uint32_t triple32(uint32_t x)
{
    x ^= x >> 17;
    x *= 0xed5ad4bbu;
    x ^= x >> 11;
    x *= 0xac4c1b51u;
    x ^= x >> 15;
    x *= 0x31848babu;
    x ^= x >> 14;
    return x;
}

// float(triple32(x)) / float(0xffffffffu): both conversions round to nearest, IEEE division.
__device__ __forceinline__ float hash01(uint32_t x) { return fdiv(__uint2float_rn(triple32(x)), 4294967296.0f); }

__device__ __forceinline__ float4 grey(float c) { return make_float4(c, c, c, 1.0f); }

// Colour of cluster c for `mode` (show_clusters.comp:81-119).
__global__ void __launch_bounds__(256) show_clusters_colour_kernel(int mode, uint32_t tiles_x, uint32_t tiles_y,
                                                                   const uint32_t* __restrict__ keys,
                                                                   const uint32_t* __restrict__ key_count,
                                                                   uint32_t max_clusters,
                                                                   const uint32_t* __restrict__ counts,
                                                                   const uint32_t* __restrict__ offsets,
                                                                   const uint32_t* __restrict__ indices,
                                                                   uint32_t index_cap, float4* __restrict__ colours)
{
    const uint32_t U = min(*key_count, max_clusters);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < U; c += warps) {
        float4 col;
        const uint32_t key = keys[c];
        switch (mode) {
        case VREN_SHOW_CLUSTERS_KEY: col = grey(hash01(key)); break;
        case VREN_SHOW_CLUSTERS_IJK:
            col = make_float4(fdiv(__uint2float_rn(key & 0xFFu), __uint2float_rn(tiles_x)),
                              fdiv(__uint2float_rn((key >> 8) & 0xFFu), __uint2float_rn(tiles_y)),
                              fdiv(__uint2float_rn((key >> 16) & 0x3FFu), 1024.0f), 1.0f);
            break;
        case VREN_SHOW_CLUSTERS_NORMAL: {
            const uint32_t n = key >> 26;
            col = make_float4(fdiv(__uint2float_rn(n / 9u), 6.0f), fdiv(__uint2float_rn((n / 3u) % 3u), 3.0f),
                              fdiv(__uint2float_rn(n % 3u), 3.0f), 1.0f);
            break;
        }
        case VREN_SHOW_CLUSTERS_LIGHT_COUNTS: {
            const float v = fdiv(__uint2float_rn(counts[c]), 64.0f);
            col = grey(1.0f < v ? 1.0f : v);
            break;
        }
        case VREN_SHOW_CLUSTERS_LIGHT_OFFSETS: col = grey(hash01(offsets[c])); break;
        case VREN_SHOW_CLUSTERS_LIGHT_INDICES: {
            uint32_t n = counts[c];
            const uint32_t o = offsets[c];
            if (o >= index_cap || n > index_cap - o) {  // a list cut by the assignment's index capacity
                n = o >= index_cap ? 0u : index_cap - o;
                if (lane == 0) VREN_RECORD_ERROR(VREN_ERR_CAPACITY);
            }
            uint32_t h = 0;
            for (uint32_t i = lane; i < n; i += 32) h ^= indices[o + i];
#pragma unroll
            for (int s = 16; s > 0; s >>= 1) h ^= __shfl_xor_sync(0xffffffffu, h, s);
            col = grey(hash01(h));
            break;
        }
        default: col = make_float4(1.0f, 0.0f, 0.0f, 1.0f); break;
        }
        if (lane == 0) colours[c] = col;
    }
}

// Per pixel: the colour of its cluster; a reference outside the key list is drawn magenta.
__global__ void __launch_bounds__(256) show_clusters_pixels_kernel(uint32_t npix, const uint32_t* __restrict__ refs,
                                                                   const uint32_t* __restrict__ key_count,
                                                                   uint32_t max_clusters,
                                                                   const float4* __restrict__ colours,
                                                                   float4* __restrict__ out)
{
    const uint32_t U = min(*key_count, max_clusters);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        const uint32_t r = __ldcs(refs + p);
        const float4 c = r < U ? __ldg(colours + r) : make_float4(1.0f, 0.0f, 1.0f, 1.0f);
        __stcs(out + p, c);
    }
}

__device__ __forceinline__ void put_vertex(uint4* __restrict__ v, uint32_t& o, float x, float y, float z, uint32_t colour)
{
    v[o++] = make_uint4(__float_as_uint(x), __float_as_uint(y), __float_as_uint(z), colour);
}

__device__ __forceinline__ void put_line(uint4* __restrict__ v, uint32_t& o, const float a[3], const float b[3],
                                         uint32_t colour)
{
    put_vertex(v, o, a[0], a[1], a[2], colour);
    put_vertex(v, o, b[0], b[1], b[2], colour);
}

// show_clusters_geometry.comp:54-112 with debug.glsl's VREN_DEBUG_WRITE_AABB / _ARROW vertex order.
__global__ void __launch_bounds__(128) show_clusters_geometry_kernel(const vren_cs_frame* __restrict__ F,
                                                                     const uint32_t* __restrict__ keys,
                                                                     const uint32_t* __restrict__ key_count,
                                                                     uint32_t max_clusters,
                                                                     uint4* __restrict__ vertices)
{
    const uint32_t U = min(*key_count, max_clusters);
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < U; c += gridDim.x * blockDim.x) {
        const uint32_t key = keys[c];
        const Box b = cluster_box(key, F);
        const uint32_t n = key >> 26;
        uint4* v = vertices + (size_t)c * kGeomVerticesPerCluster;
        uint32_t o = 0;
        const float* m = b.mn;
        const float* M = b.mx;
        const uint32_t box_colour = n < kNoNormal ? 0xFFFFFFu : 0u;
        {
            const float p0[3] = {m[0], m[1], m[2]}, p1[3] = {M[0], m[1], m[2]}, p2[3] = {M[0], m[1], M[2]},
                        p3[3] = {m[0], m[1], M[2]};
            const float q0[3] = {m[0], M[1], m[2]}, q1[3] = {M[0], M[1], m[2]}, q2[3] = {M[0], M[1], M[2]},
                        q3[3] = {m[0], M[1], M[2]};
            put_line(v, o, p0, p1, box_colour);
            put_line(v, o, p1, p2, box_colour);
            put_line(v, o, p2, p3, box_colour);
            put_line(v, o, p3, p0, box_colour);
            put_line(v, o, q0, q1, box_colour);
            put_line(v, o, q1, q2, box_colour);
            put_line(v, o, q2, q3, box_colour);
            put_line(v, o, q3, q0, box_colour);
            put_line(v, o, p0, q0, box_colour);
            put_line(v, o, p1, q1, box_colour);
            put_line(v, o, p2, q2, box_colour);
            put_line(v, o, p3, q3, box_colour);
        }
        float pos[3], to[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) pos[k] = fdiv(fadd(m[k], M[k]), 2.0f);
        if (n < kNoNormal) {
            // the bin's direction (clustered_shading.glsl:45-54 decode, show_clusters_geometry.comp:84-96)
            const uint32_t face = n / 9u, axis = face % 3u, uc = (axis + 1u) % 3u, vc = (axis + 2u) % 3u;
            float d[3];
            d[axis] = (face / 3u) == 1u ? 1.0f : -1.0f;
            d[uc] = fsub(fmul(fdiv(fadd(__uint2float_rn((n / 3u) % 3u), 0.5f), 3.0f), 2.0f), 1.0f);
            d[vc] = fsub(fmul(fdiv(fadd(__uint2float_rn(n % 3u), 0.5f), 3.0f), 2.0f), 1.0f);
            const float len = fsqrt(fadd(fadd(fmul(d[0], d[0]), fmul(d[1], d[1])), fmul(d[2], d[2])));
#pragma unroll
            for (int k = 0; k < 3; ++k) to[k] = fadd(pos[k], fmul(fdiv(d[k], len), 0.01f));
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) to[k] = pos[k];
        }
        put_line(v, o, pos, to, 0x00FF00u);
        const float dx = fsub(pos[0], to[0]), dy = fsub(pos[1], to[1]), dz = fsub(pos[2], to[2]);
        const float h = fmul(fsqrt(fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz))), 0.1f);
        const float sgn[3][2][3] = {{{-1, -1, -1}, {1, 1, 1}}, {{1, 1, -1}, {-1, -1, 1}}, {{1, -1, -1}, {-1, 1, 1}}};
#pragma unroll
        for (int l = 0; l < 3; ++l) {
            float a[3], e[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                a[k] = fadd(to[k], fmul(sgn[l][0][k], h));
                e[k] = fadd(to[k], fmul(sgn[l][1][k], h));
            }
            put_line(v, o, a, e, 0xFF0000u);
        }
    }
}

}  // namespace
}  // namespace vren_gb300

using namespace vren_gb300;

extern "C" size_t vren_cs_show_clusters_scratch_bytes(uint32_t max_clusters)
{
    return (size_t)(max_clusters ? max_clusters : 1u) * sizeof(float4);
}

extern "C" int vren_cs_show_clusters(vren_stream_t s, int mode, uint32_t width, uint32_t height,
                                     const uint32_t* cluster_refs, const uint32_t* cluster_keys,
                                     const uint32_t* key_count, uint32_t max_clusters, const uint32_t* counts,
                                     const uint32_t* offsets, const uint32_t* indices, uint32_t index_capacity,
                                     float* rgba, void* scratch)
{
    if (width == 0 || height == 0) return VREN_OK;
    if (!cluster_refs || !cluster_keys || !key_count || !rgba || !scratch || max_clusters == 0) return VREN_ERR_ARG;
    if ((mode == VREN_SHOW_CLUSTERS_LIGHT_COUNTS || mode == VREN_SHOW_CLUSTERS_LIGHT_OFFSETS ||
         mode == VREN_SHOW_CLUSTERS_LIGHT_INDICES) &&
        (!counts || !offsets))
        return VREN_ERR_ARG;
    if (mode == VREN_SHOW_CLUSTERS_LIGHT_INDICES && (!indices || index_capacity == 0)) return VREN_ERR_ARG;
    if (((uintptr_t)rgba | (uintptr_t)scratch) & 15u) return VREN_ERR_ARG;
    const uint64_t npix = (uint64_t)width * height;
    if (npix > 0xFFFFFFFFull) return VREN_ERR_ARG;
    cudaStream_t st = as_stream(s);
    const uint32_t tiles_x = (width + 31) / 32, tiles_y = (height + 31) / 32;
    float4* colours = static_cast<float4*>(scratch);
    const uint32_t cgrid = min((max_clusters + 7) / 8, (uint32_t)kNumSMsHint * 16);
    launch_kernel(show_clusters_colour_kernel, cgrid, 256, 0, st, mode, tiles_x, tiles_y, cluster_keys, key_count,
                  max_clusters, counts, offsets, indices, index_capacity, colours);
    VREN_LAUNCH_CHECK();
    const uint64_t pblocks = (npix + 255) / 256;
    const uint32_t pgrid = pblocks < (uint64_t)kNumSMsHint * 16 ? (uint32_t)pblocks : (uint32_t)kNumSMsHint * 16;
    launch_kernel(show_clusters_pixels_kernel, pgrid, 256, 0, st, (uint32_t)npix, cluster_refs, key_count,
                  max_clusters, (const float4*)colours, reinterpret_cast<float4*>(rgba));
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

extern "C" int vren_cs_show_clusters_geometry(vren_stream_t s, const vren_cs_frame* frame,
                                              const uint32_t* cluster_keys, const uint32_t* key_count,
                                              uint32_t max_clusters, vren_debug_vertex* vertices)
{
    if (max_clusters == 0) return VREN_OK;
    if (!frame || !cluster_keys || !key_count || !vertices) return VREN_ERR_ARG;
    if ((uintptr_t)vertices & 15u) return VREN_ERR_ARG;
    const uint32_t grid = min((max_clusters + 127) / 128, (uint32_t)kNumSMsHint * 8);
    launch_kernel(show_clusters_geometry_kernel, grid, 128, 0, as_stream(s), frame, cluster_keys, key_count,
                  max_clusters, reinterpret_cast<uint4*>(vertices));
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

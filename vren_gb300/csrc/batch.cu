// Batched cluster assignment: many independent frames through one fixed kernel sequence.
//
// The plain path (clustered.cu) runs construct_point_light_bvh, find_unique_cluster_list and
// assign_lights per frame: eleven launches, most of them far too small to fill 152 SMs (a 16K-light
// BVH is a few CTAs).  Here every stage covers all frames at once, indexing its work by (frame, item)
// through a per-frame descriptor table and prefix arrays in device memory:
//
//   transform   1024-light chunks of every frame; per-frame min/max by the last chunk of the frame
//   morton      the same chunks; sort key (frame << 16) | code, value = the light's index in its frame
//   sort        one stable LSD radix sort of all frames' (key, index) pairs: within a frame the order
//               is exactly the per-frame stable sort by code
//   leaves      1024-leaf blocks of every frame's padded leaf range (+ first two BVH levels)
//   levels      one CTA per frame with >= 32768 padded leaves (the remaining one or two levels)
//   unique      every frame's 32x32 tiles, independent of each other
//   tile scan   one CTA per frame: tile counts -> tile offsets
//   fixup       tile offsets into the references, keys into each frame's dense list
//   bases       per-frame cluster counts -> dense cluster numbering over the batch
//   count       traversal over all clusters of all frames (warp per cluster)
//   scan        one exclusive scan of the dense counts
//   write       traversal again, writing light indices and frame-local offsets
//   totals      per-frame index bases and totals
//
// Every per-frame result is produced by the same device functions as the plain path
// (cs_device.cuh), so each frame's outputs are bit-identical to vren_cs_cluster on the same inputs.
// The whole sequence is captured once per batch shape and replayed as one CUDA graph.
#include "common.cuh"
#include "internal.h"

#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

namespace vren_gb300 {
VREN_DEFINE_ERROR_WORD(batch)
}  // namespace vren_gb300

#include "cs_device.cuh"

namespace vren_gb300 {

constexpr uint32_t kMaxBatchFrames = 1024;
constexpr uint32_t kChunkLights = 1024;   // lights per transform / morton CTA (256 threads x 4)
constexpr uint32_t kMaxBatchLights = 1u << 20;  // per frame: padded leaves <= 2^20 (<= 4 BVH levels)

struct BatchDesc {
    const float* depth;
    const float* normals;
    const float4* positions;
    const float4* lights;
    const vren_cs_frame* frame;
    uint32_t W, H, L, P;
    uint32_t lc;          // traversal levels (0 when L == 0)
    uint32_t tiles;
    int32_t vec;
    uint32_t light_base;  // first entry of the frame in the batch's light arrays
    uint64_t pixel_base;  // first cluster reference
    uint64_t key_base;    // first key slot (capacity tiles * 1024)
    uint64_t bvh_base;    // first BVH node
    uint64_t sphere_base; // first leaf sphere
    LevelBase lb;
};

// Last f with prefix[f] <= x (prefix non-decreasing, prefix[0] = 0, n entries).
__device__ __forceinline__ uint32_t frame_of(const uint32_t* __restrict__ prefix, uint32_t n, uint32_t x)
{
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(prefix + mid) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ------------------------------------------------------------------------------------------------
// Light BVH
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) batch_transform_kernel(const BatchDesc* d,
                                                              const uint32_t* chunk_prefix, uint32_t n,
                                                              float4* __restrict__ view_pos, uint32_t* __restrict__ part,
                                                              uint32_t* __restrict__ fmm, uint32_t* __restrict__ fticket)
{
    pdl_enter();
    __shared__ uint32_t s_keys[8][6];
    __shared__ bool s_last;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t f = frame_of(chunk_prefix, n, blockIdx.x);
    const uint32_t chunk = blockIdx.x - chunk_prefix[f];
    const uint32_t nchunks = chunk_prefix[f + 1] - chunk_prefix[f];
    const BatchDesc& fd = d[f];
    const float* V = fd.frame->view.view;
    uint32_t kmin[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, kmax[3] = {0u, 0u, 0u};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t i = chunk * kChunkLights + k * 256 + tid;
        if (i < fd.L) {
            const float4 v = light_to_view(V, fd.positions[i]);
            view_pos[fd.light_base + i] = v;
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
        for (int w = 0; w < 8; ++w) {
            const uint32_t x = s_keys[w][tid];
            v = tid < 3 ? (x < v ? x : v) : (x > v ? x : v);
        }
        part[8 * (size_t)blockIdx.x + tid] = v;
    }
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        s_last = atomicAdd(fticket + f, 1u) == nchunks - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    if (tid < 6) {
        uint32_t v = tid < 3 ? 0xFFFFFFFFu : 0u;
        for (uint32_t b = chunk_prefix[f]; b < chunk_prefix[f + 1]; ++b) {
            const uint32_t x = ld_relaxed_u32(part + 8 * (size_t)b + tid);
            v = tid < 3 ? (x < v ? x : v) : (x > v ? x : v);
        }
        fmm[8 * f + tid] = v;
    }
    if (tid == 0) fticket[f] = 0u;
}

__global__ void __launch_bounds__(256) batch_morton_kernel(const BatchDesc* d,
                                                           const uint32_t* chunk_prefix, uint32_t n,
                                                           const float4* view_pos,
                                                           const uint32_t* fmm, uint2* __restrict__ pairs)
{
    pdl_enter();
    const uint32_t f = frame_of(chunk_prefix, n, blockIdx.x);
    const uint32_t chunk = blockIdx.x - chunk_prefix[f];
    const BatchDesc& fd = d[f];
    float mn[3], mx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        mn[a] = unkey(fmm[8 * f + a]);
        mx[a] = unkey(fmm[8 * f + 3 + a]);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t i = chunk * kChunkLights + k * 256 + threadIdx.x;
        if (i < fd.L) {
            const uint32_t code = morton_code(view_pos[fd.light_base + i], mn, mx, 5u);
            pairs[fd.light_base + i] = make_uint2((f << 16) | (code & 0xFFFFu), i);
        }
    }
}

__global__ void __launch_bounds__(1024) batch_leaves_kernel(const BatchDesc* d,
                                                            const uint32_t* leaf_prefix, uint32_t n,
                                                            uint2* __restrict__ light_index,
                                                            const float4* view_pos,
                                                            vren_bvh_node* __restrict__ bvh, float4* __restrict__ spheres)
{
    pdl_enter();
    __shared__ NodeF s_parent[32];
    const uint32_t f = frame_of(leaf_prefix, n, blockIdx.x);
    const uint32_t chunk = blockIdx.x - leaf_prefix[f];
    const BatchDesc& fd = d[f];
    const uint32_t threads = fd.P < 1024u ? fd.P : 1024u;
    uint2* li = light_index + fd.light_base;
    const uint32_t i = chunk * threads + threadIdx.x;
    // the sorted pairs carry the frame in bits 16+ of the key: keep the Morton code only
    if (threadIdx.x < threads && i < fd.L) li[i].x &= 0xFFFFu;
    light_leaves_block(chunk, threads, fd.L, fd.P, li, view_pos + fd.light_base, fd.lights, bvh + fd.bvh_base,
                       spheres + fd.sphere_base, s_parent);
}

// Levels above the two built with the leaves (frames with at least 32768 padded leaves).
__global__ void __launch_bounds__(1024) batch_levels_kernel(const BatchDesc* d,
                                                            vren_bvh_node* __restrict__ bvh)
{
    pdl_enter();
    __shared__ NodeF s_parent[32];
    const BatchDesc& fd = d[blockIdx.x];
    if (fd.L == 0 || fd.P < 32768u) return;
    vren_bvh_node* b = bvh + fd.bvh_base;
    const uint32_t src = fd.P + fd.P / 32u, count = fd.P / 1024u;  // 32 or 1024 nodes
    if (count >= 1024u) bvh_levels_block(b, 0, src, count, src + count, src + count + count / 32u, true, s_parent);
    else bvh_levels_block(b, 0, src, count, src + count, 0, false, s_parent);
}

// ------------------------------------------------------------------------------------------------
// Unique clusters over all frames' tiles
// ------------------------------------------------------------------------------------------------
// References of at most this many bytes per unique-cluster group (they must stay in the 129 MB L2
// between the tile kernel and the fix-up).
constexpr uint64_t kFucGroupBytes = 48ull << 20;

struct BatchFuc {
    const BatchDesc* d;
    const uint32_t* tile_prefix;
    uint32_t n;
    uint32_t* keys;
    uint32_t* key_counts;
    uint32_t* refs;
    uint32_t* tile_keys;
    uint32_t* tile_count;
    uint32_t* tile_offset;
};

__device__ __forceinline__ FucFrame batch_fuc_frame(const BatchFuc& b, uint32_t f)
{
    const BatchDesc& fd = b.d[f];
    const uint32_t t0 = b.tile_prefix[f];
    return FucFrame{fd.depth,         fd.normals,          fd.W,          fd.H,
                    fd.frame,         b.keys + fd.key_base, fd.tiles * 1024u,
                    b.key_counts + f, b.refs + fd.pixel_base, b.tile_keys + (size_t)t0 * 1024u,
                    b.tile_count + t0, b.tile_offset + t0, fd.tiles, fd.vec};
}

// The tiles of a group of frames (global tile index = blockIdx.x + t0).
__global__ void __launch_bounds__(kFucThreads, 6) batch_find_unique_kernel(BatchFuc b, uint32_t t0)
{
    pdl_enter();
    __shared__ FucSmem sm;
    const uint32_t tid = threadIdx.x;
    reinterpret_cast<uint4*>(sm.bits)[tid] = make_uint4(0u, 0u, 0u, 0u);
    reinterpret_cast<uint4*>(sm.bits)[tid + kFucThreads] = make_uint4(0u, 0u, 0u, 0u);
    if (tid < 64) sm.used[tid] = 0u;
    __syncthreads();
    const uint32_t t = blockIdx.x + t0;
    const uint32_t f = frame_of(b.tile_prefix, b.n, t);
    find_unique_tile(batch_fuc_frame(b, f), t - b.tile_prefix[f], sm);
}

// One CTA per frame of the group (frame blockIdx.x + f0): its tile counts into offsets.
__global__ void __launch_bounds__(kFucScanThreads) batch_find_unique_scan_kernel(BatchFuc b, uint32_t f0)
{
    pdl_enter();
    __shared__ uint32_t s_warp[kFucScanThreads / 32];
    find_unique_scan(batch_fuc_frame(b, blockIdx.x + f0), s_warp);
}

__global__ void __launch_bounds__(kFucThreads) batch_find_unique_fixup_kernel(BatchFuc b, uint32_t t0)
{
    pdl_enter();
    const uint32_t t = blockIdx.x + t0;
    const uint32_t f = frame_of(b.tile_prefix, b.n, t);
    find_unique_fixup(batch_fuc_frame(b, f), t - b.tile_prefix[f]);
}

// Dense cluster numbering: base[f] = sum of the unique-cluster counts of frames < f; base[n] = total.
__global__ void __launch_bounds__(1024) batch_bases_kernel(const BatchDesc* d, uint32_t n,
                                                           const uint32_t* key_counts,
                                                           uint32_t* __restrict__ base)
{
    pdl_enter();
    __shared__ uint32_t s_warp[32];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    uint32_t u = 0;
    if (tid < n) {
        const uint32_t cap = d[tid].tiles * 1024u;
        u = key_counts[tid];
        u = u < cap ? u : cap;
    }
    uint32_t incl = u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (uint32_t w = 0; w < 32; ++w) {
        if (w < warp) before += s_warp[w];
        total += s_warp[w];
    }
    if (tid < n) base[tid] = before + incl - u;
    if (tid == 0) base[n] = total;
}

// ------------------------------------------------------------------------------------------------
// Traversal over all clusters of all frames (warp per cluster)
// ------------------------------------------------------------------------------------------------
struct BatchAssign {
    const BatchDesc* d;
    uint32_t n;
    const uint32_t* base;       // dense cluster bases [n + 1]
    const uint32_t* keys;
    uint32_t* counts;           // dense
    const uint32_t* goff;       // dense global offsets (write pass)
    uint32_t* offsets;          // dense frame-local offsets (write pass)
    uint32_t* indices;
    uint32_t index_cap;
    const uint2* light_index;
    const float4* view_pos;
    const float4* spheres;
    const vren_bvh_node* bvh;
};

template <bool WRITE>
__device__ __forceinline__ uint32_t batch_traverse(const AssignArgs& a, const LevelBase& lb, uint32_t lc, uint32_t key,
                                                   uint32_t out_base, uint32_t lane)
{
    switch (lc) {
    case 1: return assign_cluster<1, WRITE, true>(a, lb, key, out_base, lane);
    case 2: return assign_cluster<2, WRITE, true>(a, lb, key, out_base, lane);
    case 3: return assign_cluster<3, WRITE, true>(a, lb, key, out_base, lane);
    default: return assign_cluster<4, WRITE, true>(a, lb, key, out_base, lane);
    }
}

template <bool WRITE>
__global__ void __launch_bounds__(256) batch_assign_kernel(BatchAssign b)
{
    pdl_enter();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps_per_cta = blockDim.x >> 5;
    const uint32_t gw = blockIdx.x * warps_per_cta + (threadIdx.x >> 5);
    const uint32_t nw = gridDim.x * warps_per_cta;
    const uint32_t total = b.base[b.n];
    for (uint32_t c = gw; c < total; c += nw) {
        const uint32_t f = frame_of(b.base, b.n, c);
        const BatchDesc& fd = b.d[f];
        const uint32_t local = c - b.base[f];
        const uint32_t key = b.keys[fd.key_base + local];
        AssignArgs a{};
        a.frame = fd.frame;
        a.bvh = b.bvh + fd.bvh_base;
        a.light_index = b.light_index + fd.light_base;
        a.view_pos = b.view_pos + fd.light_base;
        a.spheres = b.spheres + fd.sphere_base;
        a.indices = b.indices;
        a.index_cap = b.index_cap;
        if (!WRITE) {
            const uint32_t acc = fd.lc ? batch_traverse<false>(a, fd.lb, fd.lc, key, 0u, lane) : 0u;
            if (lane == 0) b.counts[c] = acc;
        } else {
            const uint32_t out = b.goff[c];
            if (fd.lc && b.counts[c] != 0u) batch_traverse<true>(a, fd.lb, fd.lc, key, out, lane);  // skip empty
            if (lane == 0) b.offsets[c] = out - b.goff[b.base[f]];
        }
    }
}

// index_base[f] = first light index of frame f in the dense index array, totals[f] = its count.
__global__ void batch_totals_kernel(uint32_t n, const uint32_t* base, const uint32_t* goff,
                                    const uint32_t* grand_total, uint32_t* __restrict__ index_base,
                                    uint32_t* __restrict__ totals)
{
    pdl_enter();
    const uint32_t clusters = base[n];
    for (uint32_t f = threadIdx.x; f < n; f += blockDim.x) {
        const uint32_t b0 = base[f], b1 = base[f + 1];
        const uint32_t i0 = b0 < clusters ? goff[b0] : *grand_total;
        const uint32_t i1 = b1 < clusters ? goff[b1] : *grand_total;
        index_base[f] = i0;
        totals[f] = i1 - i0;
    }
}

}  // namespace vren_gb300

using namespace vren_gb300;

// ================================================================================================
// Host side
// ================================================================================================
struct vren_cs_batch {
    vren_cs_batch_options opt{8, 0, 8, 8, 1};
    // capacities of the reserved arena
    uint32_t cap_frames = 0, cap_chunks = 0, cap_leaf_blocks = 0, cap_tiles = 0;
    uint64_t cap_lights = 0, cap_pixels = 0, cap_keys = 0, cap_bvh = 0, cap_spheres = 0, cap_assign = 0;
    size_t cap_sort_scratch = 0, cap_scan_scratch = 0;
    char* arena = nullptr;
    size_t arena_bytes = 0;
    // carved device buffers
    BatchDesc* desc = nullptr;
    uint32_t* prefixes = nullptr;  // chunk [F+1] | leaf [F+1] | tile [F+1]
    vren_cs_frame* frames = nullptr;
    float4* view_pos = nullptr;
    uint2* pairs = nullptr;
    uint2* light_index = nullptr;
    uint2* sort_tmp = nullptr;
    void* sort_scratch = nullptr;
    uint32_t* part = nullptr;
    uint32_t* fmm = nullptr;
    uint32_t* fticket = nullptr;
    vren_bvh_node* bvh = nullptr;
    float4* spheres = nullptr;
    uint32_t* tile_count = nullptr;
    uint32_t* tile_offset = nullptr;
    uint32_t* tile_keys = nullptr;
    uint32_t* keys = nullptr;
    uint32_t* key_counts = nullptr;
    uint32_t* refs = nullptr;
    uint32_t* base = nullptr;
    uint32_t* counts = nullptr;
    uint32_t* goff = nullptr;
    uint32_t* offsets = nullptr;
    uint32_t* indices = nullptr;
    uint32_t* grand_total = nullptr;
    uint32_t* index_base = nullptr;
    uint32_t* totals = nullptr;
    void* scan_scratch = nullptr;
    // pinned staging of the descriptor table, prefixes and frame blocks
    char* host = nullptr;
    size_t host_bytes = 0;
    std::vector<char> uploaded;  // what the device copy currently holds
    // frame groups of the unique-cluster stage (boundaries, first = 0, last = n) and the host copy of
    // the tile prefix
    std::vector<uint32_t> fuc_groups;
    std::vector<uint32_t> fuc_tile_prefix;
    // second stream: the light BVHs are built beside the unique-cluster stage
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_bvh = nullptr;
    // the last upload of the staged block and the end of the last run, on whatever stream they were
    // enqueued: a new staging waits for both before it overwrites the pinned and the device copies
    cudaEvent_t ev_uploaded = nullptr, ev_done = nullptr;
    // layout of the current batch
    uint32_t n = 0, total_chunks = 0, total_leaf_blocks = 0, total_tiles = 0, total_lights = 0;
    uint64_t total_keys = 0;
    uint32_t frame_bits = 0;
    // graph of the last batch shape
    cudaGraphExec_t graph = nullptr;
    std::vector<char> graph_key;
    std::map<std::tuple<uint32_t, uint32_t, uint32_t>, vren_cs_batch_options> tuned;
};

namespace {

size_t up256(size_t x) { return (x + 255) / 256 * 256; }

uint32_t ceil_log2(uint64_t x)
{
    uint32_t b = 0;
    while ((1ull << b) < x) ++b;
    return b;
}

bool frame_ok(const vren_cs_batch_frame& f)
{
    if (f.width == 0 || f.height == 0 || f.width > 8192 || f.height > 8192) return false;
    if (!f.depth || !f.normals) return false;
    if (f.light_count > kMaxBatchLights) return false;
    if (f.light_count > 0) {
        if (!f.light_positions || !f.point_lights) return false;
        if (((uintptr_t)f.light_positions | (uintptr_t)f.point_lights) & 15u) return false;
    }
    if (f.normal_format != VREN_CS_NORMALS_F32X3 && f.normal_format != VREN_CS_NORMALS_RGBA16F) return false;
    return f.offscreen == VREN_CS_OFFSCREEN_WRAP || f.offscreen == VREN_CS_OFFSCREEN_SKIP;
}

struct Sizes {
    uint32_t chunks = 0, leaf_blocks = 0, tiles = 0;
    uint64_t lights = 0, pixels = 0, keys = 0, bvh = 0, spheres = 0;
};

Sizes sizes_of(const vren_cs_batch_frame* fr, uint32_t count)
{
    Sizes s;
    for (uint32_t i = 0; i < count; ++i) {
        const uint32_t L = fr[i].light_count;
        const uint32_t tiles = ((fr[i].width + 31) / 32) * ((fr[i].height + 31) / 32);
        s.chunks += (L + kChunkLights - 1) / kChunkLights;
        if (L > 0) {
            const uint32_t P = vren_calc_bvh_padded_leaf_count(L);
            s.leaf_blocks += P / (P < 1024u ? P : 1024u);
            s.bvh += vren_calc_bvh_buffer_length(L);
            s.spheres += P;
        }
        s.tiles += tiles;
        s.lights += L;
        s.pixels += (uint64_t)fr[i].width * fr[i].height;
        s.keys += (uint64_t)tiles * 1024u;
    }
    return s;
}

size_t sort_scratch_max(uint64_t lights, uint32_t key_bits)
{
    size_t m = 0;
    for (uint32_t db : {4u, 6u, 8u}) {
        const size_t b = sort_uvec2_scratch_bytes((uint32_t)(lights ? lights : 1), key_bits, db);
        m = b > m ? b : m;
    }
    return m;
}

// Builds the descriptor table, prefixes and frame blocks for `fr` in the pinned staging area and
// uploads it when it differs from what the device holds.
int stage_batch(vren_cs_batch* b, cudaStream_t st, const vren_cs_batch_frame* fr, uint32_t count)
{
    const size_t desc_bytes = (size_t)count * sizeof(BatchDesc);
    const size_t pref_bytes = (size_t)3 * (count + 1) * sizeof(uint32_t);
    const size_t frame_bytes = (size_t)count * sizeof(vren_cs_frame);
    std::vector<char> staged(desc_bytes + pref_bytes + frame_bytes);
    BatchDesc* desc = reinterpret_cast<BatchDesc*>(staged.data());
    uint32_t* pref = reinterpret_cast<uint32_t*>(staged.data() + desc_bytes);
    vren_cs_frame* frames = reinterpret_cast<vren_cs_frame*>(staged.data() + desc_bytes + pref_bytes);
    uint32_t chunk = 0, leaf = 0, tile = 0, light = 0;
    uint64_t pixel = 0, key = 0, node = 0, sphere = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const vren_cs_batch_frame& f = fr[i];
        int rc = vren_cs_frame_build(&f.view, f.width, f.height, f.offscreen, &frames[i]);
        if (rc != VREN_OK) return rc;
        frames[i].normal_format = f.normal_format;
        BatchDesc& d = desc[i];
        std::memset(&d, 0, sizeof(d));
        d.depth = f.depth;
        d.normals = f.normals;
        d.positions = reinterpret_cast<const float4*>(f.light_positions);
        d.lights = reinterpret_cast<const float4*>(f.point_lights);
        d.frame = b->frames + i;
        d.W = f.width;
        d.H = f.height;
        d.L = f.light_count;
        d.P = f.light_count ? vren_calc_bvh_padded_leaf_count(f.light_count) : 0u;
        d.lc = traversal_levels(f.light_count, d.lb);
        d.tiles = ((f.width + 31) / 32) * ((f.height + 31) / 32);
        d.vec = (f.width % 4u == 0u) && ((uintptr_t)f.depth % 16u == 0u) && ((uintptr_t)f.normals % 16u == 0u);
        d.light_base = light;
        d.pixel_base = pixel;
        d.key_base = key;
        d.bvh_base = node;
        d.sphere_base = sphere;
        pref[i] = chunk;
        pref[(count + 1) + i] = leaf;
        pref[2 * (count + 1) + i] = tile;
        chunk += (d.L + kChunkLights - 1) / kChunkLights;
        if (d.L) {
            leaf += d.P / (d.P < 1024u ? d.P : 1024u);
            node += vren_calc_bvh_buffer_length(d.L);
            sphere += d.P;
        }
        tile += d.tiles;
        light += d.L;
        pixel += (uint64_t)d.W * d.H;
        key += (uint64_t)d.tiles * 1024u;
    }
    pref[count] = chunk;
    pref[(count + 1) + count] = leaf;
    pref[2 * (count + 1) + count] = tile;
    // refs are written with 128-bit stores only when every frame's reference range is aligned
    for (uint32_t i = 0; i < count; ++i)
        if (desc[i].pixel_base % 4u != 0u) desc[i].vec = 0;
    // unique-cluster groups: consecutive frames whose references total at most kFucGroupBytes
    b->fuc_groups.assign(1, 0u);
    b->fuc_tile_prefix.assign(pref + 2 * (count + 1), pref + 2 * (count + 1) + count + 1);
    uint64_t group_bytes = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const uint64_t bytes = (uint64_t)desc[i].W * desc[i].H * 4u;
        if (group_bytes > 0 && group_bytes + bytes > kFucGroupBytes) {
            b->fuc_groups.push_back(i);
            group_bytes = 0;
        }
        group_bytes += bytes;
    }
    b->fuc_groups.push_back(count);
    b->n = count;
    b->total_chunks = chunk;
    b->total_leaf_blocks = leaf;
    b->total_tiles = tile;
    b->total_lights = light;
    b->total_keys = key;
    b->frame_bits = count > 1 ? ceil_log2(count) : 0u;
    if (b->uploaded.size() != staged.size() || std::memcmp(b->uploaded.data(), staged.data(), staged.size()) != 0) {
        VREN_CUDA_TRY(cudaEventSynchronize(b->ev_uploaded));  // an earlier upload may still read the pinned copy
        VREN_CUDA_TRY(cudaStreamWaitEvent(st, b->ev_done, 0));  // an earlier run may still read the device copy
        std::memcpy(b->host, staged.data(), staged.size());
        VREN_CUDA_TRY(cudaMemcpyAsync(b->desc, b->host, desc_bytes, cudaMemcpyHostToDevice, st));
        VREN_CUDA_TRY(cudaMemcpyAsync(b->prefixes, b->host + desc_bytes, pref_bytes, cudaMemcpyHostToDevice, st));
        VREN_CUDA_TRY(cudaMemcpyAsync(b->frames, b->host + desc_bytes + pref_bytes, frame_bytes,
                                      cudaMemcpyHostToDevice, st));
        VREN_CUDA_TRY(cudaEventRecord(b->ev_uploaded, st));
        b->uploaded.swap(staged);
    }
    return VREN_OK;
}

// The kernel sequence of one batch (capturable: no allocation, no host synchronisation).
int enqueue_batch(vren_cs_batch* b, cudaStream_t st)
{
    const PdlScope pdl(1);  // consecutive kernels of the sequence overlap their launches
    const uint32_t n = b->n;
    const uint32_t* chunk_prefix = b->prefixes;
    const uint32_t* leaf_prefix = b->prefixes + (n + 1);
    const uint32_t* tile_prefix = b->prefixes + 2 * (n + 1);
    // The light BVHs (on the second stream) and the unique clusters (on st) are independent; the
    // assignment waits for both.
    if (b->total_chunks > 0) {
        cudaStream_t ls = b->aux;
        VREN_CUDA_TRY(cudaEventRecord(b->ev_fork, st));
        VREN_CUDA_TRY(cudaStreamWaitEvent(ls, b->ev_fork, 0));
        int rc = VREN_OK;
        do {
            if (launch_kernel(batch_transform_kernel, b->total_chunks, 256, 0, ls, b->desc, chunk_prefix, n,
                              b->view_pos, b->part, b->fmm, b->fticket) != cudaSuccess ||
                launch_kernel(batch_morton_kernel, b->total_chunks, 256, 0, ls, b->desc, chunk_prefix, n, b->view_pos,
                              b->fmm, b->pairs) != cudaSuccess) {
                rc = VREN_ERR_CUDA;
                break;
            }
            rc = sort_uvec2(ls, reinterpret_cast<const uint32_t*>(b->pairs), reinterpret_cast<uint32_t*>(b->light_index),
                            reinterpret_cast<uint32_t*>(b->sort_tmp), b->total_lights, 16u + b->frame_bits,
                            b->opt.sort_digit_bits, b->sort_scratch);
            if (rc != VREN_OK) break;
            if (launch_kernel(batch_leaves_kernel, b->total_leaf_blocks, 1024, 0, ls, b->desc, leaf_prefix, n,
                              b->light_index, b->view_pos, b->bvh, b->spheres) != cudaSuccess ||
                launch_kernel(batch_levels_kernel, n, 1024, 0, ls, b->desc, b->bvh) != cudaSuccess)
                rc = VREN_ERR_CUDA;
        } while (false);
        const cudaError_t e1 = cudaEventRecord(b->ev_bvh, ls);
        if (rc != VREN_OK || e1 != cudaSuccess) {
            cudaStreamWaitEvent(st, b->ev_bvh, 0);  // rejoin before returning (a capture must end joined)
            return rc != VREN_OK ? rc : VREN_ERR_CUDA;
        }
    }
    const BatchFuc bf{b->desc, tile_prefix, n, b->keys, b->key_counts, b->refs, b->tile_keys, b->tile_count,
                      b->tile_offset};
    // tiles -> tile-count scan -> reference fix-up per group of frames, so that the group's references
    // are still in L2 when the fix-up adds the tile offsets
    cudaError_t fe = cudaSuccess;
    for (size_t g = 0; g + 1 < b->fuc_groups.size() && fe == cudaSuccess; ++g) {
        const uint32_t f0 = b->fuc_groups[g], f1 = b->fuc_groups[g + 1];
        const uint32_t t0 = b->fuc_tile_prefix[f0], t1 = b->fuc_tile_prefix[f1];
        fe = launch_kernel(batch_find_unique_kernel, t1 - t0, kFucThreads, 0, st, bf, t0);
        if (fe == cudaSuccess) fe = launch_kernel(batch_find_unique_scan_kernel, f1 - f0, kFucScanThreads, 0, st, bf, f0);
        if (fe == cudaSuccess) fe = launch_kernel(batch_find_unique_fixup_kernel, t1 - t0, kFucThreads, 0, st, bf, t0);
    }
    if (b->total_chunks > 0) VREN_CUDA_TRY(cudaStreamWaitEvent(st, b->ev_bvh, 0));  // join the light BVHs
    if (fe != cudaSuccess) return VREN_ERR_CUDA;
    launch_kernel(batch_bases_kernel, 1, 1024, 0, st, b->desc, n, b->key_counts, b->base);
    VREN_LAUNCH_CHECK();
    BatchAssign a{b->desc, n, b->base, b->keys, b->counts, b->goff, b->offsets, b->indices,
                  (uint32_t)(b->cap_assign < 0xFFFFFFFFull ? b->cap_assign : 0xFFFFFFFFull),
                  b->light_index, b->view_pos, b->spheres, b->bvh};
    uint32_t warps = b->opt.assign_warps;
    if (warps < 1 || warps > 8) warps = 8;
    const dim3 block(32 * warps), grid(kNumSMsHint * (64 / warps));
    launch_kernel(batch_assign_kernel<false>, grid, block, 0, st, a);
    VREN_LAUNCH_CHECK();
    int rc = scan_exclusive_u32(st, b->counts, b->goff, (uint32_t)b->total_keys, b->base + n, b->grand_total,
                                b->scan_scratch);
    if (rc != VREN_OK) return rc;
    launch_kernel(batch_assign_kernel<true>, grid, block, 0, st, a);
    VREN_LAUNCH_CHECK();
    launch_kernel(batch_totals_kernel, 1, 256, 0, st, n, b->base, b->goff, b->grand_total, b->index_base, b->totals);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

// Enqueues with the batch's tile variants in effect (the knobs are read at enqueue time).
int enqueue_with_options(vren_cs_batch* b, cudaStream_t st)
{
    const int saved_items = tuning(VREN_TUNE_RADIX_ITEMS), saved_slices = tuning(VREN_TUNE_SCAN_SLICES);
    vren_tuning_set(VREN_TUNE_RADIX_ITEMS, (int)b->opt.radix_items);
    vren_tuning_set(VREN_TUNE_SCAN_SLICES, (int)b->opt.scan_slices);
    const int rc = enqueue_batch(b, st);
    vren_tuning_set(VREN_TUNE_RADIX_ITEMS, saved_items);
    vren_tuning_set(VREN_TUNE_SCAN_SLICES, saved_slices);
    return rc;
}

void drop_graph(vren_cs_batch* b)
{
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->graph_key.clear();
}

bool options_ok(const vren_cs_batch_options& o)
{
    if (o.sort_digit_bits != 4 && o.sort_digit_bits != 6 && o.sort_digit_bits != 8) return false;
    if (o.radix_items > 1) return false;
    if (o.scan_slices != 4 && o.scan_slices != 8) return false;
    return o.assign_warps >= 1 && o.assign_warps <= 8;
}

}  // namespace

extern "C" int vren_cs_batch_create(vren_cs_batch** out)
{
    if (!out) return VREN_ERR_ARG;
    auto* b = new vren_cs_batch();
    if (cudaStreamCreateWithFlags(&b->aux, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_bvh, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_uploaded, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming) != cudaSuccess) {
        vren_cs_batch_destroy(b);
        return VREN_ERR_CUDA;
    }
    *out = b;
    return VREN_OK;
}

extern "C" void vren_cs_batch_destroy(vren_cs_batch* b)
{
    if (!b) return;
    drop_graph(b);
    if (b->aux) cudaStreamDestroy(b->aux);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_bvh) cudaEventDestroy(b->ev_bvh);
    if (b->ev_uploaded) cudaEventDestroy(b->ev_uploaded);
    if (b->ev_done) cudaEventDestroy(b->ev_done);
    cudaFree(b->arena);
    cudaFreeHost(b->host);
    delete b;
}

extern "C" int vren_cs_batch_reserve(vren_cs_batch* b, const vren_cs_batch_frame* fr, uint32_t count,
                                     uint64_t max_assignments)
{
    if (!b || (count > 0 && !fr) || count > kMaxBatchFrames) return VREN_ERR_ARG;
    for (uint32_t i = 0; i < count; ++i)
        if (!frame_ok(fr[i])) return VREN_ERR_ARG;
    const Sizes s = sizes_of(fr, count);
    if (s.lights > 0xFFFFFFFFull || s.keys > 0xFFFFFFFFull || s.bvh > 0xFFFFFFFFull) return VREN_ERR_CAPACITY;
    drop_graph(b);
    cudaFree(b->arena);
    cudaFreeHost(b->host);
    b->arena = nullptr;
    b->host = nullptr;
    b->uploaded.clear();
    const uint32_t F = count ? count : 1;
    const uint64_t Lb = s.lights ? s.lights : 1, Kb = s.keys ? s.keys : 1;
    const uint32_t fbits = count > 1 ? ceil_log2(count) : 0u;
    size_t off = 0;
    auto carve = [&](size_t bytes) {
        const size_t o = off;
        off += up256(bytes ? bytes : 1);
        return o;
    };
    const size_t o_desc = carve((size_t)F * sizeof(BatchDesc));
    const size_t o_pref = carve((size_t)3 * (F + 1) * 4);
    const size_t o_frames = carve((size_t)F * sizeof(vren_cs_frame));
    const size_t o_vp = carve(Lb * 16);
    const size_t o_pairs = carve(Lb * 8);
    const size_t o_li = carve(Lb * 8);
    const size_t o_tmp = carve(Lb * 8);
    const size_t sort_bytes = sort_scratch_max(Lb, 16u + fbits);
    const size_t o_sort = carve(sort_bytes);
    const size_t o_part = carve((size_t)(s.chunks ? s.chunks : 1) * 8 * 4);
    const size_t o_fmm = carve((size_t)F * 8 * 4);
    const size_t o_ftk = carve((size_t)F * 4);
    const size_t o_bvh = carve((size_t)(s.bvh ? s.bvh : 1) * sizeof(vren_bvh_node));
    const size_t o_sph = carve((size_t)(s.spheres ? s.spheres : 1) * 16);
    const size_t o_tcount = carve((size_t)(s.tiles ? s.tiles : 1) * 4);
    const size_t o_toff = carve((size_t)(s.tiles ? s.tiles : 1) * 4);
    const size_t o_tkeys = carve((size_t)(s.tiles ? s.tiles : 1) * 4096);
    const size_t o_keys = carve(Kb * 4);
    const size_t o_kc = carve((size_t)F * 4);
    const size_t o_refs = carve((s.pixels ? s.pixels : 1) * 4);
    const size_t o_base = carve((size_t)(F + 1) * 4);
    const size_t o_counts = carve(Kb * 4);
    const size_t o_goff = carve(Kb * 4);
    const size_t o_offs = carve(Kb * 4);
    const size_t o_idx = carve((max_assignments ? max_assignments : 1) * 4);
    const size_t o_gt = carve(4);
    const size_t o_ib = carve((size_t)F * 4);
    const size_t o_tot = carve((size_t)F * 4);
    const size_t scan_bytes = scan_scratch_bytes((uint32_t)Kb);
    const size_t o_scan = carve(scan_bytes);
    if (cudaMalloc(&b->arena, off) != cudaSuccess) {
        b->arena = nullptr;
        return VREN_ERR_CUDA;
    }
    b->host_bytes = (size_t)F * (sizeof(BatchDesc) + sizeof(vren_cs_frame)) + (size_t)3 * (F + 1) * 4;
    if (cudaMemset(b->arena, 0, off) != cudaSuccess || cudaMallocHost(&b->host, b->host_bytes) != cudaSuccess) {
        cudaFree(b->arena);
        b->arena = nullptr;
        b->host = nullptr;
        return VREN_ERR_CUDA;
    }
    b->arena_bytes = off;
    char* a = b->arena;
    b->desc = reinterpret_cast<BatchDesc*>(a + o_desc);
    b->prefixes = reinterpret_cast<uint32_t*>(a + o_pref);
    b->frames = reinterpret_cast<vren_cs_frame*>(a + o_frames);
    b->view_pos = reinterpret_cast<float4*>(a + o_vp);
    b->pairs = reinterpret_cast<uint2*>(a + o_pairs);
    b->light_index = reinterpret_cast<uint2*>(a + o_li);
    b->sort_tmp = reinterpret_cast<uint2*>(a + o_tmp);
    b->sort_scratch = a + o_sort;
    b->part = reinterpret_cast<uint32_t*>(a + o_part);
    b->fmm = reinterpret_cast<uint32_t*>(a + o_fmm);
    b->fticket = reinterpret_cast<uint32_t*>(a + o_ftk);
    b->bvh = reinterpret_cast<vren_bvh_node*>(a + o_bvh);
    b->spheres = reinterpret_cast<float4*>(a + o_sph);
    b->tile_count = reinterpret_cast<uint32_t*>(a + o_tcount);
    b->tile_offset = reinterpret_cast<uint32_t*>(a + o_toff);
    b->tile_keys = reinterpret_cast<uint32_t*>(a + o_tkeys);
    b->keys = reinterpret_cast<uint32_t*>(a + o_keys);
    b->key_counts = reinterpret_cast<uint32_t*>(a + o_kc);
    b->refs = reinterpret_cast<uint32_t*>(a + o_refs);
    b->base = reinterpret_cast<uint32_t*>(a + o_base);
    b->counts = reinterpret_cast<uint32_t*>(a + o_counts);
    b->goff = reinterpret_cast<uint32_t*>(a + o_goff);
    b->offsets = reinterpret_cast<uint32_t*>(a + o_offs);
    b->indices = reinterpret_cast<uint32_t*>(a + o_idx);
    b->grand_total = reinterpret_cast<uint32_t*>(a + o_gt);
    b->index_base = reinterpret_cast<uint32_t*>(a + o_ib);
    b->totals = reinterpret_cast<uint32_t*>(a + o_tot);
    b->scan_scratch = a + o_scan;
    b->cap_frames = F;
    b->cap_chunks = s.chunks;
    b->cap_leaf_blocks = s.leaf_blocks;
    b->cap_tiles = s.tiles;
    b->cap_lights = s.lights;
    b->cap_pixels = s.pixels;
    b->cap_keys = s.keys;
    b->cap_bvh = s.bvh;
    b->cap_spheres = s.spheres;
    b->cap_assign = max_assignments;
    b->cap_sort_scratch = sort_bytes;
    b->cap_scan_scratch = scan_bytes;
    return VREN_OK;
}

extern "C" int vren_cs_batch_set_options(vren_cs_batch* b, const vren_cs_batch_options* o)
{
    if (!b || !o || !options_ok(*o)) return VREN_ERR_ARG;
    b->opt = *o;
    drop_graph(b);
    return VREN_OK;
}

extern "C" int vren_cs_batch_get_options(const vren_cs_batch* b, vren_cs_batch_options* o)
{
    if (!b || !o) return VREN_ERR_ARG;
    *o = b->opt;
    return VREN_OK;
}

// Marks the end of a run on its stream (the next staging waits for it).
static int mark_done(vren_cs_batch* b, cudaStream_t st, int rc)
{
    if (rc == VREN_OK && cudaEventRecord(b->ev_done, st) != cudaSuccess) return VREN_ERR_CUDA;
    return rc;
}

extern "C" int vren_cs_batch_run(vren_cs_batch* b, vren_stream_t s, const vren_cs_batch_frame* fr, uint32_t count)
{
    if (!b || (count > 0 && !fr)) return VREN_ERR_ARG;
    if (count == 0) return VREN_OK;
    if (count > b->cap_frames || !b->arena) return VREN_ERR_CAPACITY;
    for (uint32_t i = 0; i < count; ++i)
        if (!frame_ok(fr[i])) return VREN_ERR_ARG;
    const Sizes sz = sizes_of(fr, count);
    if (sz.chunks > b->cap_chunks || sz.leaf_blocks > b->cap_leaf_blocks || sz.tiles > b->cap_tiles ||
        sz.lights > b->cap_lights || sz.pixels > b->cap_pixels || sz.keys > b->cap_keys || sz.bvh > b->cap_bvh ||
        sz.spheres > b->cap_spheres)
        return VREN_ERR_CAPACITY;
    const uint32_t fbits = count > 1 ? ceil_log2(count) : 0u;
    if (sort_scratch_max(sz.lights ? sz.lights : 1, 16u + fbits) > b->cap_sort_scratch) return VREN_ERR_CAPACITY;
    cudaStream_t st = as_stream(s);
    int rc = stage_batch(b, st, fr, count);
    if (rc != VREN_OK) return rc;
    const bool use_graph = b->opt.use_graph && st != nullptr;
    if (!use_graph) return mark_done(b, st, enqueue_with_options(b, st));
    // Graph key: every frame's shape and buffers, the options and the stream.  Cameras are not part
    // of it: the frame blocks the kernels read are uploaded above, outside the graph.
    struct FrameKey {
        uint32_t w, h, L;
        int32_t off;
        uint32_t normal_format, pad;
        const void *depth, *normals, *pos, *lights;
    };
    std::vector<char> key(sizeof(FrameKey) * count + sizeof(vren_cs_batch_options) + sizeof(st));
    for (uint32_t i = 0; i < count; ++i) {
        const FrameKey k{fr[i].width,         fr[i].height, fr[i].light_count, fr[i].offscreen,
                         fr[i].normal_format, 0u,           fr[i].depth,       fr[i].normals,
                         fr[i].light_positions, fr[i].point_lights};
        std::memcpy(key.data() + i * sizeof(FrameKey), &k, sizeof(k));
    }
    std::memcpy(key.data() + sizeof(FrameKey) * count, &b->opt, sizeof(b->opt));
    std::memcpy(key.data() + key.size() - sizeof(st), &st, sizeof(st));
    if (b->graph && key == b->graph_key)
        return mark_done(b, st, cudaGraphLaunch(b->graph, st) == cudaSuccess ? VREN_OK : VREN_ERR_CUDA);
    drop_graph(b);
    cudaGraph_t g;
    VREN_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    rc = enqueue_with_options(b, st);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc != VREN_OK) {
        if (e == cudaSuccess) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return VREN_ERR_CUDA;
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->graph = nullptr;
        return VREN_ERR_CUDA;
    }
    b->graph_key.swap(key);
    return mark_done(b, st, cudaGraphLaunch(b->graph, st) == cudaSuccess ? VREN_OK : VREN_ERR_CUDA);
}

extern "C" int vren_cs_batch_autotune(vren_cs_batch* b, vren_stream_t s, const vren_cs_batch_frame* fr, uint32_t count,
                                      uint32_t reps, vren_cs_batch_options* chosen)
{
    if (!b || !fr || count == 0) return VREN_ERR_ARG;
    cudaStream_t st = as_stream(s);
    const Sizes sz = sizes_of(fr, count);
    const auto bucket = std::make_tuple(count, ceil_log2(sz.pixels), ceil_log2(sz.lights ? sz.lights : 1));
    const auto hit = b->tuned.find(bucket);
    if (hit != b->tuned.end()) {
        const int rc = vren_cs_batch_set_options(b, &hit->second);
        if (rc == VREN_OK && chosen) *chosen = hit->second;
        return rc;
    }
    if (reps == 0) reps = 3;
    const vren_cs_batch_options start = b->opt;
    vren_cs_batch_options best = start;
    float best_ms = 0.0f;
    bool have = false;
    cudaEvent_t e0, e1;
    VREN_CUDA_TRY(cudaEventCreate(&e0));
    VREN_CUDA_TRY(cudaEventCreate(&e1));
    int rc = VREN_OK;
    for (uint32_t db : {4u, 6u, 8u})
        for (uint32_t items : {0u, 1u})
            for (uint32_t slices : {4u, 8u})
                for (uint32_t warps : {2u, 4u, 8u}) {
                    vren_cs_batch_options o{db, items, slices, warps, start.use_graph};
                    if ((rc = vren_cs_batch_set_options(b, &o)) != VREN_OK) goto out;
                    // first run captures (when graphs are on) and warms the caches
                    if ((rc = vren_cs_batch_run(b, s, fr, count)) != VREN_OK) goto out;
                    if (cudaEventRecord(e0, st) != cudaSuccess) { rc = VREN_ERR_CUDA; goto out; }
                    for (uint32_t r = 0; r < reps; ++r)
                        if ((rc = vren_cs_batch_run(b, s, fr, count)) != VREN_OK) goto out;
                    if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
                        rc = VREN_ERR_CUDA;
                        goto out;
                    }
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (!have || ms < best_ms) {
                        best = o;
                        best_ms = ms;
                        have = true;
                    }
                }
out:
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != VREN_OK) {
        vren_cs_batch_set_options(b, &start);
        return rc;
    }
    b->tuned[bucket] = best;
    rc = vren_cs_batch_set_options(b, &best);
    if (rc == VREN_OK && chosen) *chosen = best;
    return rc;
}

extern "C" int vren_cs_batch_frame_outputs(vren_cs_batch* b, vren_stream_t s, uint32_t f, vren_cs_outputs* o)
{
    if (!b || !o || f >= b->n || b->uploaded.empty()) return VREN_ERR_ARG;
    VREN_CUDA_TRY(cudaStreamSynchronize(as_stream(s)));
    uint32_t base = 0, ibase = 0;
    VREN_CUDA_TRY(cudaMemcpy(&base, b->base + f, 4, cudaMemcpyDeviceToHost));
    VREN_CUDA_TRY(cudaMemcpy(&ibase, b->index_base + f, 4, cudaMemcpyDeviceToHost));
    const BatchDesc& d = reinterpret_cast<const BatchDesc*>(b->uploaded.data())[f];
    o->view_positions = reinterpret_cast<const float*>(b->view_pos + d.light_base);
    o->bvh = b->bvh + d.bvh_base;
    o->light_index = reinterpret_cast<const uint32_t*>(b->light_index + d.light_base);
    o->leaf_spheres = reinterpret_cast<const float*>(b->spheres + d.sphere_base);
    o->cluster_keys = b->keys + d.key_base;
    o->key_count = b->key_counts + f;
    o->cluster_refs = b->refs + d.pixel_base;
    o->counts = b->counts + base;
    o->offsets = b->offsets + base;
    o->indices = b->indices + ibase;
    o->total = b->totals + f;
    o->frame = b->frames + f;
    o->key_capacity = d.tiles * 1024u;
    o->index_capacity = (uint32_t)(b->cap_assign - ibase);
    return VREN_OK;
}

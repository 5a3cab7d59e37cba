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

#include <algorithm>
#include <cmath>
#include <cstring>

namespace vren_gb300 {
VREN_DEFINE_ERROR_WORD(cs)
}  // namespace vren_gb300

#include "cs_device.cuh"
#include "lookback.cuh"

namespace vren_gb300 {

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
    const float4* positions, uint32_t L, const vren_cs_frame* F,
    float4* __restrict__ view_pos, uint32_t* __restrict__ scratch)
{
    pdl_enter();
    __shared__ uint32_t s_keys[kLbvhThreads / 32][6];
    __shared__ bool s_last;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const float* V = F->view.view;
    uint32_t kmin[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, kmax[3] = {0u, 0u, 0u};
#pragma unroll
    for (int k = 0; k < kLbvhPerThread; ++k) {
        const uint32_t i = blockIdx.x * kLbvhPerCta + k * kLbvhThreads + tid;
        if (i < L) {
            const float4 v = light_to_view(V, positions[i]);
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

// discretize_point_light_positions.comp:30-39
__global__ void lbvh_morton_kernel(const float4* view_pos, uint32_t L, const uint32_t* scratch,
                                   uint32_t bits, uint2* __restrict__ pairs)
{
    pdl_enter();
    float mn[3], mx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        mn[a] = unkey(scratch[8 + a]);
        mx[a] = unkey(scratch[11 + a]);
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x)
        pairs[i] = make_uint2(morton_code(view_pos[i], mn, mx, bits), i);
}

// Leaves and the two levels above them; with `done` (32768 <= P <= 2^20) the last CTA to finish also
// builds the one or two levels up to the root.
__global__ void __launch_bounds__(1024) lbvh_leaves_kernel(
    const uint2* light_index, const float4* view_pos, const float4* lights,
    uint32_t L, uint32_t P, vren_bvh_node* __restrict__ bvh, float4* __restrict__ spheres, uint32_t* __restrict__ done)
{
    pdl_enter();
    __shared__ NodeF s_parent[32];
    __shared__ bool s_last;
    light_leaves_block(blockIdx.x, blockDim.x, L, P, light_index, view_pos, lights, bvh, spheres, s_parent);
    if (!done) return;
    __syncthreads();
    if (threadIdx.x == 0) {  // thread 0 wrote this CTA's level-2 node
        __threadfence();
        s_last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const uint32_t src = P + P / 32u, count = P / 1024u;  // 32 or 1024 nodes
    bvh_levels_block(bvh, 0, src, count, src + count, src + count + count / 32u, count >= 1024u, s_parent);
    if (threadIdx.x == 0) *done = 0u;
}

// construct_point_light_bvh for few lights (up to kSmallPathLights, where the launches of the multi-CTA
// path cost more than its work) with 15-bit codes in one CTA: view transform and
// min/max, Morton codes, and the stable sort by code as two 8-bit LSD passes over (code << 16 | index)
// in shared memory (per-warp ballot ranking and digit counters, as in the multi-CTA onesweep passes;
// warp w takes a contiguous run of indices, so equal codes keep index order).  Writes view_pos and
// light_index exactly as the multi-kernel path does.
constexpr uint32_t kSmallLights = 16384;      // capacity of the kernel's shared-memory arrays
constexpr uint32_t kSmallPathLights = 2048;   // measured: at 16384 lights the multi-CTA path is faster
constexpr int kSmallThreads = 1024;
constexpr size_t kSmallSmem = (2 * kSmallLights + 32 * 256) * sizeof(uint32_t);

__global__ void __launch_bounds__(kSmallThreads) lbvh_small_kernel(const float4* positions, uint32_t L,
                                                                   const vren_cs_frame* F,
                                                                   float4* __restrict__ view_pos,
                                                                   uint2* __restrict__ light_index)
{
    pdl_enter();
    extern __shared__ uint32_t s_dyn[];
    uint32_t* A = s_dyn;                // keys (code << 16 | index), sorted result after two passes
    uint32_t* B = A + kSmallLights;     // pass temporary
    uint32_t* cnt = B + kSmallLights;   // [32 warps][256 digits]: counts, then scatter offsets
    __shared__ uint32_t s_mm[32][6];
    __shared__ uint32_t s_bound[6];
    __shared__ uint32_t s_wsum[32];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;

    // view positions and their min/max (order-preserving keys)
    const float* V = F->view.view;
    uint32_t kmin[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, kmax[3] = {0u, 0u, 0u};
    for (uint32_t i = tid; i < L; i += kSmallThreads) {
        const float4 v = light_to_view(V, positions[i]);
        view_pos[i] = v;
        const float c[3] = {v.x, v.y, v.z};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const uint32_t key = fkey(c[a]);
            kmin[a] = key < kmin[a] ? key : kmin[a];
            kmax[a] = key > kmax[a] ? key : kmax[a];
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
            s_mm[warp][a] = kmin[a];
            s_mm[warp][3 + a] = kmax[a];
        }
    }
    __syncthreads();
    if (tid < 6) {
        uint32_t v = tid < 3 ? 0xFFFFFFFFu : 0u;
        for (int w = 0; w < 32; ++w) {
            const uint32_t x = s_mm[w][tid];
            v = tid < 3 ? (x < v ? x : v) : (x > v ? x : v);
        }
        s_bound[tid] = v;
    }
    __syncthreads();
    float mn[3], mx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        mn[a] = unkey(s_bound[a]);
        mx[a] = unkey(s_bound[3 + a]);
    }
    // Morton codes (each thread reads back the view positions it wrote)
    for (uint32_t i = tid; i < L; i += kSmallThreads) A[i] = (morton_code(view_pos[i], mn, mx, 5u) << 16) | i;

    // two stable 8-bit passes over bits 16..31
    const uint32_t items = (L + kSmallThreads - 1) / kSmallThreads;  // <= 16
    const uint32_t chunk = items * 32u;                               // indices per warp
    for (uint32_t pass = 0; pass < 2; ++pass) {
        const uint32_t* src = pass ? B : A;
        uint32_t* dst = pass ? A : B;
        const uint32_t shift = 16u + 8u * pass;
#pragma unroll
        for (int k = 0; k < 8; ++k) cnt[tid * 8 + k] = 0u;
        __syncthreads();
        uint32_t rank[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const uint32_t idx = warp * chunk + (uint32_t)j * 32u + lane;
            const bool valid = (uint32_t)j < items && idx < L;
            const uint32_t d = valid ? (src[idx] >> shift) & 0xFFu : 0u;
            uint32_t peers = __ballot_sync(0xFFFFFFFFu, valid);
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const uint32_t m = __ballot_sync(0xFFFFFFFFu, (d >> b) & 1u);
                const uint32_t mine = (uint32_t)((int32_t)(d << (31 - b)) >> 31);
                peers &= ~(m ^ mine);
            }
            const uint32_t below = peers & lanemask_lt();
            const uint32_t before = valid ? cnt[warp * 256u + d] : 0u;
            __syncwarp();
            if (valid && below == 0) cnt[warp * 256u + d] = before + __popc(peers);
            __syncwarp();
            rank[j] = valid ? before + __popc(below) : 0xFFFFFFFFu;
        }
        __syncthreads();
        // exclusive scan of the counts in (digit, warp) order: entry f = 8 tid + k is (d = f / 32, w = f % 32)
        uint32_t c8[8], sum = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t f = tid * 8u + (uint32_t)k;
            c8[k] = cnt[(f & 31u) * 256u + (f >> 5)];
            sum += c8[k];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        if (lane == 31) s_wsum[warp] = incl;
        __syncthreads();
        uint32_t base = incl - sum;
        for (uint32_t w = 0; w < warp; ++w) base += s_wsum[w];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t f = tid * 8u + (uint32_t)k;
            cnt[(f & 31u) * 256u + (f >> 5)] = base;
            base += c8[k];
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            if (rank[j] != 0xFFFFFFFFu) {
                const uint32_t k = src[warp * chunk + (uint32_t)j * 32u + lane];
                dst[cnt[warp * 256u + ((k >> shift) & 0xFFu)] + rank[j]] = k;
            }
        }
        __syncthreads();
    }
    for (uint32_t i = tid; i < L; i += kSmallThreads) {
        const uint32_t k = A[i];
        light_index[i] = make_uint2(k >> 16, k & 0xFFFFu);
    }
}

// ------------------------------------------------------------------------------------------------
// construct_point_light_bvh for 2049..32768 lights (15-bit codes), whose padded tree always has 32768
// leaves: one kernel on a cluster of 16 CTAs (thread-block cluster, distributed shared memory).
// CTA r owns leaf slots [2048 r, 2048 r + 2048).  Hardware cluster barriers replace the kernel
// boundaries of the multi-kernel path:
//   1. each CTA transforms its lights to view space and publishes its min/max; every CTA reads all
//      sixteen (DSMEM) and computes the same bounds, then the Morton keys (code << 16 | light);
//   2. two stable 8-bit passes over bits 16..31: each CTA ranks its keys (ballots, per-warp digit
//      counters) and publishes its digit counts; each CTA reads the 16 x 256 counts and stores every
//      key straight into the shared memory of the CTA that owns its destination slot;
//   3. each CTA writes its slots' light index, leaves, spheres and their two parent levels
//      (light_leaves_block), and CTA 0 the root once all level-2 nodes are written.
// The output is the multi-kernel path's, bit for bit.
// ------------------------------------------------------------------------------------------------
constexpr int kClusterCtas = 16;
constexpr uint32_t kClusterSlots = 2048;
constexpr int kClusterThreads = 1024;
constexpr uint32_t kClusterMaxLights = kClusterCtas * kClusterSlots;  // 32768 = the padded leaf count
constexpr size_t kClusterSmem = (2 * kClusterSlots + 32 * 256) * sizeof(uint32_t);

__device__ __forceinline__ void cluster_barrier()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Address of `p` (this CTA's shared memory) in the shared memory of CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t dsmem_addr(const void* p, uint32_t rank)
{
    uint32_t out;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;"
                 : "=r"(out)
                 : "r"(static_cast<uint32_t>(__cvta_generic_to_shared(p))), "r"(rank));
    return out;
}
__device__ __forceinline__ uint32_t dsmem_ld(uint32_t addr)
{
    uint32_t v;
    asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
    return v;
}
__device__ __forceinline__ void dsmem_st(uint32_t addr, uint32_t v)
{
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

__global__ void __launch_bounds__(kClusterThreads) lbvh_cluster_kernel(
    const float4* positions, const float4* lights, uint32_t L,
    const vren_cs_frame* F, float4* __restrict__ view_pos, uint2* __restrict__ light_index,
    vren_bvh_node* __restrict__ bvh, float4* __restrict__ spheres)
{
    pdl_enter();
    extern __shared__ uint32_t s_dyn[];
    uint32_t* A = s_dyn;                 // this CTA's keys (code << 16 | light), by slot
    uint32_t* B = A + kClusterSlots;     // destination of a pass (written by every CTA)
    uint32_t* cnt = B + kClusterSlots;   // [32 warps][256 digits]
    __shared__ uint32_t s_mm[32][6];
    __shared__ uint32_t s_cta_mm[6];     // read by the other CTAs
    __shared__ uint32_t s_bound[6];
    __shared__ uint32_t s_hist[256];     // this CTA's digit counts, read by the other CTAs
    __shared__ uint32_t s_base[256];     // global first slot of each digit for this CTA's keys
    __shared__ uint32_t s_wsum[32];
    __shared__ NodeF s_parent[32];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t rank = blockIdx.x;  // the grid is one cluster
    const uint32_t base = rank * kClusterSlots;
    const uint32_t own = L > base ? (L - base < kClusterSlots ? L - base : kClusterSlots) : 0u;

    // 1. view positions, bounds, Morton keys
    const float* V = F->view.view;
    uint32_t kmin[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, kmax[3] = {0u, 0u, 0u};
    for (uint32_t j = tid; j < own; j += kClusterThreads) {
        const float4 v = light_to_view(V, positions[base + j]);
        view_pos[base + j] = v;
        const float c[3] = {v.x, v.y, v.z};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const uint32_t key = fkey(c[a]);
            kmin[a] = key < kmin[a] ? key : kmin[a];
            kmax[a] = key > kmax[a] ? key : kmax[a];
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
            s_mm[warp][a] = kmin[a];
            s_mm[warp][3 + a] = kmax[a];
        }
    }
    __syncthreads();
    if (tid < 6) {
        uint32_t v = tid < 3 ? 0xFFFFFFFFu : 0u;
        for (int w = 0; w < 32; ++w) {
            const uint32_t x = s_mm[w][tid];
            v = tid < 3 ? (x < v ? x : v) : (x > v ? x : v);
        }
        s_cta_mm[tid] = v;
    }
    cluster_barrier();
    if (tid < 6) {
        uint32_t v = tid < 3 ? 0xFFFFFFFFu : 0u;
        for (uint32_t c = 0; c < kClusterCtas; ++c) {
            const uint32_t x = dsmem_ld(dsmem_addr(&s_cta_mm[tid], c));
            v = tid < 3 ? (x < v ? x : v) : (x > v ? x : v);
        }
        s_bound[tid] = v;
    }
    __syncthreads();
    float mn[3], mx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        mn[a] = unkey(s_bound[a]);
        mx[a] = unkey(s_bound[3 + a]);
    }
    for (uint32_t j = tid; j < own; j += kClusterThreads)
        A[j] = (morton_code(view_pos[base + j], mn, mx, 5u) << 16) | (base + j);
    __syncthreads();
    // 2. two stable 8-bit passes over bits 16..31 across the cluster
    for (uint32_t pass = 0; pass < 2; ++pass) {
        const uint32_t* src = pass ? B : A;
        uint32_t* dst = pass ? A : B;
        const uint32_t shift = 16u + 8u * pass;
#pragma unroll
        for (int k = 0; k < 8; ++k) cnt[tid * 8 + k] = 0u;
        __syncthreads();
        uint32_t rnk[2], dig[2];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const uint32_t idx = warp * 64u + (uint32_t)j * 32u + lane;
            const bool valid = idx < own;
            const uint32_t d = valid ? (src[idx] >> shift) & 0xFFu : 0u;
            uint32_t peers = __ballot_sync(0xFFFFFFFFu, valid);
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const uint32_t m = __ballot_sync(0xFFFFFFFFu, (d >> b) & 1u);
                const uint32_t mine = (uint32_t)((int32_t)(d << (31 - b)) >> 31);
                peers &= ~(m ^ mine);
            }
            const uint32_t below = peers & lanemask_lt();
            const uint32_t before = valid ? cnt[warp * 256u + d] : 0u;
            __syncwarp();
            if (valid && below == 0) cnt[warp * 256u + d] = before + __popc(peers);
            __syncwarp();
            rnk[j] = valid ? before + __popc(below) : 0xFFFFFFFFu;
            dig[j] = d;
        }
        __syncthreads();
        // thread d: this CTA's count of digit d, and the warp prefixes of d in place
        if (tid < 256) {
            uint32_t run = 0;
            for (int w = 0; w < 32; ++w) {
                const uint32_t c = cnt[w * 256 + tid];
                cnt[w * 256 + tid] = run;
                run += c;
            }
            s_hist[tid] = run;
        }
        cluster_barrier();  // every CTA's digit counts are published
        if (warp < 8) {
            // thread d: the cluster's count of digit d and that of the lower-ranked CTAs
            uint32_t tot = 0, pre = 0;
            for (uint32_t c = 0; c < kClusterCtas; ++c) {
                const uint32_t h = dsmem_ld(dsmem_addr(&s_hist[tid], c));
                tot += h;
                pre += c < rank ? h : 0u;
            }
            uint32_t incl = tot;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= (uint32_t)o) incl += y;
            }
            if (lane == 31) s_wsum[warp] = incl;
            __syncwarp();
            s_base[tid] = incl - tot + pre;  // the other warps' sums are added below
        }
        __syncthreads();
        if (tid < 256) {
            uint32_t add = 0;
            for (uint32_t w = 0; w < warp; ++w) add += s_wsum[w];
            s_base[tid] += add;
        }
        __syncthreads();
        // every key straight into the slot it sorts to, in the CTA that owns that slot
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if (rnk[j] != 0xFFFFFFFFu) {
                const uint32_t idx = warp * 64u + (uint32_t)j * 32u + lane;
                const uint32_t slot = s_base[dig[j]] + cnt[warp * 256u + dig[j]] + rnk[j];
                dsmem_st(dsmem_addr(&dst[slot & (kClusterSlots - 1u)], slot / kClusterSlots), src[idx]);
            }
        }
        cluster_barrier();  // all keys have arrived; the counts may be reused
    }

    // 3. light index, leaves, spheres, levels 1 and 2 of this CTA's slots (as light_leaves_block),
    //    then the root over the 32 level-2 nodes
    constexpr uint32_t P = kClusterMaxLights;
#pragma unroll 1
    for (uint32_t h = 0; h < 2; ++h) {
        const uint32_t j = h * 1024u + tid, i = base + j;
        NodeF leaf;
        float4 sph;
        if (j < own) {
            const uint32_t key = A[j], li = key & 0xFFFFu;
            light_index[i] = make_uint2(key >> 16, li);
            const float4 o = __ldcg(view_pos + li);  // written by another CTA of this cluster
            const float r = __ldg(&lights[li].w);
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
            s_parent[warp] = p;
        }
        __syncthreads();
        if (warp == 0) {
            const uint32_t chunk = rank * 2u + h;
            const NodeF g = warp_parent(s_parent[lane], true, P + chunk * 32u);
            if (lane == 0) store_node(bvh, P + P / 32u + chunk, g);
        }
        __syncthreads();
    }
    cluster_barrier();  // every level-2 node is written
    if (rank == 0 && warp == 0) {
        const float4* q = reinterpret_cast<const float4*>(bvh + P + P / 32u + lane);
        const float4 lo = __ldcg(q), hi = __ldcg(q + 1);
        NodeF c;
        c.mn[0] = lo.x; c.mn[1] = lo.y; c.mn[2] = lo.z; c.next = __float_as_uint(lo.w);
        c.mx[0] = hi.x; c.mx[1] = hi.y; c.mx[2] = hi.z; c.pad = __float_as_uint(hi.w);
        const NodeF root = warp_parent(c, true, P + P / 32u);
        if (lane == 0) store_node(bvh, P + P / 32u + 32u, root);
    }
}

// Whether a 16-CTA cluster of lbvh_cluster_kernel can be resident on the current device (checked once).
static bool cluster_path_available()
{
    static int state = -1;
    if (state < 0) {
        bool ok = cudaFuncSetAttribute(lbvh_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                      cudaSuccess &&
                  cudaFuncSetAttribute(lbvh_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kClusterSmem) == cudaSuccess;
        int clusters = 0;
        if (ok) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(kClusterCtas);
            cfg.blockDim = dim3(kClusterThreads);
            cfg.dynamicSmemBytes = kClusterSmem;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = kClusterCtas;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            ok = cudaOccupancyMaxActiveClusters(&clusters, lbvh_cluster_kernel, &cfg) == cudaSuccess;
        }
        if (!ok) cudaGetLastError();  // clear: the multi-kernel path is used instead
        state = ok && clusters >= 1 ? 1 : 0;
    }
    return state == 1;
}

static int launch_lbvh_cluster(cudaStream_t st, const float* positions, const float* lights, uint32_t L,
                               const vren_cs_frame* frame, float* view_pos, vren_bvh_node* bvh, uint32_t* light_index,
                               float* spheres)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kClusterCtas);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.dynamicSmemBytes = kClusterSmem;
    cfg.stream = st;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kClusterCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (g_pdl) {
        attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[1].val.programmaticStreamSerializationAllowed = 1;
        cfg.numAttrs = 2;
    }
    cudaLaunchKernelEx(&cfg, lbvh_cluster_kernel, reinterpret_cast<const float4*>(positions),
                       reinterpret_cast<const float4*>(lights), L, frame, reinterpret_cast<float4*>(view_pos),
                       reinterpret_cast<uint2*>(light_index), bvh, reinterpret_cast<float4*>(spheres));
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

static int construct_light_bvh(cudaStream_t st, const float* positions, const float* lights, uint32_t L,
                               const vren_cs_frame* frame, uint32_t morton_bits, uint32_t digit_bits, float* view_pos,
                               vren_bvh_node* bvh, uint32_t* light_index, float* spheres, void* scratch)
{
    if (L == 0) return VREN_OK;
    const LbvhLayout lay = lbvh_layout(L, morton_bits, digit_bits);
    char* sc = static_cast<char*>(scratch);
    uint32_t* hdr = reinterpret_cast<uint32_t*>(sc);
    if (morton_bits != 30 && L > kSmallPathLights && L <= kClusterMaxLights &&
        tuning(VREN_TUNE_LIGHT_BVH_CLUSTER) != 0 && cluster_path_available())
        return launch_lbvh_cluster(st, positions, lights, L, frame, view_pos, bvh, light_index, spheres);
    if (morton_bits != 30 && L <= kSmallPathLights) {
        static bool attr_set = false;  // the attribute is per function, set once
        if (!attr_set) {
            VREN_CUDA_TRY(cudaFuncSetAttribute(lbvh_small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)kSmallSmem));
            attr_set = true;
        }
        launch_kernel(lbvh_small_kernel, 1, kSmallThreads, kSmallSmem, st, reinterpret_cast<const float4*>(positions),
                      L, frame, reinterpret_cast<float4*>(view_pos), reinterpret_cast<uint2*>(light_index));
        VREN_LAUNCH_CHECK();
    } else {
        uint2* pairs = reinterpret_cast<uint2*>(sc + lay.pairs);
        uint32_t* tmp = reinterpret_cast<uint32_t*>(sc + lay.tmp);
        const uint32_t grid = (L + kLbvhPerCta - 1) / kLbvhPerCta;
        launch_kernel(lbvh_transform_kernel, grid, kLbvhThreads, 0, st, reinterpret_cast<const float4*>(positions), L,
                      frame, reinterpret_cast<float4*>(view_pos), hdr);
        VREN_LAUNCH_CHECK();
        const uint32_t bits = morton_bits == 30 ? 10u : 5u;
        uint32_t mgrid = (L + 255) / 256;
        if (mgrid > 1024) mgrid = 1024;
        launch_kernel(lbvh_morton_kernel, mgrid, 256, 0, st, reinterpret_cast<const float4*>(view_pos), L, hdr, bits,
                      pairs);
        VREN_LAUNCH_CHECK();
        // bucket sort on the low 16 bits (bucket_sort.hpp:15-16); the 30-bit extension sorts 30 bits
        int rc = sort_uvec2(st, reinterpret_cast<const uint32_t*>(pairs), light_index, tmp, L,
                            morton_bits == 30 ? 30 : 16, digit_bits, sc + lay.sort);
        if (rc != VREN_OK) return rc;
    }
    const uint32_t P = vren_calc_bvh_padded_leaf_count(L);
    const uint32_t threads = P < 1024 ? P : 1024;
    uint32_t* done = (P >= 32768u && P <= (1u << 20)) ? hdr + 1 : nullptr;
    launch_kernel(lbvh_leaves_kernel, P / threads, threads, 0, st, reinterpret_cast<const uint2*>(light_index),
                  reinterpret_cast<const float4*>(view_pos), reinterpret_cast<const float4*>(lights), L, P, bvh,
                  reinterpret_cast<float4*>(spheres), done);
    VREN_LAUNCH_CHECK();
    if (P > (1u << 20)) return build_bvh_levels(st, bvh, P + P / 32u, P / 1024u);
    return VREN_OK;
}

// ================================================================================================
// find_unique_cluster_list
// ================================================================================================
__global__ void __launch_bounds__(kFucThreads, 6) find_unique_kernel(FucFrame fr, uint32_t tile_base)
{
    pdl_enter();
    __shared__ FucSmem sm;
    const uint32_t tid = threadIdx.x;
    reinterpret_cast<uint4*>(sm.bits)[tid] = make_uint4(0u, 0u, 0u, 0u);
    reinterpret_cast<uint4*>(sm.bits)[tid + kFucThreads] = make_uint4(0u, 0u, 0u, 0u);
    if (tid < 64) sm.used[tid] = 0u;
    __syncthreads();
    find_unique_tile(fr, tile_base + blockIdx.x, sm);
}

// The one-kernel form: tiles taken by ticket from the 64-bit word at `header` (zero-filled before
// the first use; the last ticket of every call re-opens it for the next).
__global__ void __launch_bounds__(kFucThreads, 6) find_unique_fused_kernel(FucFrame fr, uint32_t* header)
{
    pdl_enter();
    __shared__ FucSmem sm;
    __shared__ uint32_t s_tile, s_epoch;
    const uint32_t tid = threadIdx.x;
    reinterpret_cast<uint4*>(sm.bits)[tid] = make_uint4(0u, 0u, 0u, 0u);
    reinterpret_cast<uint4*>(sm.bits)[tid + kFucThreads] = make_uint4(0u, 0u, 0u, 0u);
    if (tid < 64) sm.used[tid] = 0u;
    if (tid == 0) {
        uint32_t e;
        s_tile = take_ticket(header, fr.num_tiles, e);
        s_epoch = e;
    }
    __syncthreads();
    if (s_tile >= fr.num_tiles) return;  // a header left inconsistent by a failed launch
    find_unique_tile<true>(fr, s_tile, sm, s_epoch);
}

__global__ void __launch_bounds__(kFucScanThreads) find_unique_scan_kernel(FucFrame fr, uint32_t t_begin,
                                                                          uint32_t t_end)
{
    pdl_enter();
    __shared__ uint32_t s_warp[kFucScanThreads / 32];
    find_unique_scan(fr, s_warp, t_begin, t_end);
}

__global__ void __launch_bounds__(kFucThreads) find_unique_fixup_kernel(FucFrame fr, uint32_t t_begin)
{
    pdl_enter();
    find_unique_fixup(fr, t_begin + blockIdx.x);
}

// The fix-up that sums its own tile offset (no scan kernel before it).
__global__ void __launch_bounds__(kFucThreads) find_unique_fixup_self_kernel(FucFrame fr, uint32_t t_begin)
{
    pdl_enter();
    find_unique_fixup<true>(fr, t_begin + blockIdx.x);
}

// Scratch of find_unique_cluster_list for T tiles (uint32 words): tile counts [T], tile offsets [T],
// then (16-byte aligned) the tiles' key slots [T][1024].
static size_t fuc_keys_offset_words(uint32_t T) { return (2ull * T + 3) / 4 * 4; }

static FucFrame fuc_frame(const float* depth, const float* normals, uint32_t W, uint32_t H, const vren_cs_frame* frame,
                          uint32_t* keys, uint32_t key_cap, uint32_t* key_count, uint32_t* refs, uint32_t* scratch)
{
    const uint32_t tiles = ((W + 31) / 32) * ((H + 31) / 32);
    const int vec = (W % 4u == 0u) && ((uintptr_t)depth % 16u == 0u) && ((uintptr_t)normals % 16u == 0u) &&
                    ((uintptr_t)refs % 16u == 0u);
    return FucFrame{depth, normals, W, H, frame, keys, key_cap, key_count, refs,
                    scratch ? scratch + fuc_keys_offset_words(tiles) : nullptr, scratch,
                    scratch ? scratch + tiles : nullptr, tiles, vec, nullptr, 0u, 0u, nullptr};
}

// Stage 1 over tiles [tile_begin, tile_begin + count).
static int launch_find_unique_tiles(cudaStream_t st, const FucFrame& fr, uint32_t tile_begin, uint32_t count)
{
    if (count == 0) return VREN_OK;
    launch_kernel(find_unique_kernel, count, kFucThreads, 0, st, fr, tile_begin);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

// Stages 2 and 3 for tiles [t_begin, t_end), after those tiles and after the stages of every tile
// before t_begin (the offsets continue from there); by default the whole frame.
static int launch_find_unique_finish(cudaStream_t st, const FucFrame& fr, uint32_t t_begin = 0,
                                     uint32_t t_end = 0xFFFFFFFFu)
{
    t_end = t_end < fr.num_tiles ? t_end : fr.num_tiles;
    if (t_end <= t_begin) return VREN_OK;
    if (fr.num_tiles <= kFucSelfScanTiles && tuning(VREN_TUNE_FUC_FUSED) == 0) {
        launch_kernel(find_unique_fixup_self_kernel, t_end - t_begin, kFucThreads, 0, st, fr, t_begin);
        VREN_LAUNCH_CHECK();
        return VREN_OK;
    }
    launch_kernel(find_unique_scan_kernel, 1, kFucScanThreads, 0, st, fr, t_begin, t_end);
    VREN_LAUNCH_CHECK();
    launch_kernel(find_unique_fixup_kernel, t_end - t_begin, kFucThreads, 0, st, fr, t_begin);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

static int launch_find_unique(cudaStream_t st, const float* depth, const float* normals, uint32_t W, uint32_t H,
                              const vren_cs_frame* frame, uint32_t* keys, uint32_t key_cap, uint32_t* key_count,
                              uint32_t* refs, uint32_t* scratch)
{
    const FucFrame fr = fuc_frame(depth, normals, W, H, frame, keys, key_cap, key_count, refs, scratch);
    const int rc = launch_find_unique_tiles(st, fr, 0, fr.num_tiles);
    return rc != VREN_OK ? rc : launch_find_unique_finish(st, fr);
}

// Look-back state of the one-kernel form for up to `tiles` tiles: a 16-byte header (ticket word),
// then one 64-bit status word per tile.
static size_t fuc_lookback_bytes(uint32_t tiles) { return 16u + 8ull * tiles; }

// find_unique_cluster_list in one launch (the one-kernel form); `lookback` as above, zero-filled
// before its first use.
static int launch_find_unique_fused(cudaStream_t st, const float* depth, const float* normals, uint32_t W, uint32_t H,
                                    const vren_cs_frame* frame, uint32_t* keys, uint32_t key_cap,
                                    uint32_t* key_count, uint32_t* refs, uint32_t* lookback,
                                    uint32_t* refs2 = nullptr)
{
    FucFrame fr = fuc_frame(depth, normals, W, H, frame, keys, key_cap, key_count, refs, nullptr);
    fr.refs2 = refs2;
    if ((uintptr_t)refs2 % 16u != 0u) fr.vec = 0;
    fr.status = reinterpret_cast<uint64_t*>(lookback + 4);
    fr.wait_limit = g_wait_limit;
    fr.spin = (uint32_t)tuning(VREN_TUNE_SPIN_POLLS);
    launch_kernel(find_unique_fused_kernel, fr.num_tiles, kFucThreads, 0, st, fr, lookback);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

// The light lists of a frame copied into page-locked host memory by the device (no host round trip
// for their lengths): out = [U, total, keys[U], counts[U], offsets[U], indices[total]], cut at cap
// words (VREN_ERR_CAPACITY recorded when it does not fit).  `total` is the number of index entries
// the device holds: the assignment's total, cut at its index capacity.
__global__ void lists_to_host_kernel(const uint32_t* key_count, uint32_t key_cap,
                                     const uint32_t* total_p, const uint32_t* keys,
                                     const uint32_t* counts, const uint32_t* offsets,
                                     const uint32_t* indices, uint32_t index_cap,
                                     uint32_t* __restrict__ out, uint64_t cap)
{
    pdl_enter();
    uint32_t U = *key_count;
    U = U < key_cap ? U : key_cap;
    const uint32_t total = *total_p < index_cap ? *total_p : index_cap;
    const uint64_t need = 2ull + 3ull * U + total;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (cap >= 2) {
            out[0] = U;
            out[1] = total;
        }
        if (need > cap) VREN_RECORD_ERROR(VREN_ERR_CAPACITY);
    }
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 3ull * U + total; i += stride) {
        const uint64_t o = 2 + i;
        if (o >= cap) break;
        uint32_t v;
        if (i < U) v = keys[i];
        else if (i < 2ull * U) v = counts[i - U];
        else if (i < 3ull * U) v = offsets[i - 2ull * U];
        else v = indices[i - 3ull * U];
        out[o] = v;
    }
}

// ================================================================================================
// assign_lights
// ================================================================================================
template <int LC, bool WRITE, bool SPHERES>
__global__ void __launch_bounds__(256) assign_kernel(AssignArgs a, LevelBase lb)
{
    pdl_enter();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps_per_cta = blockDim.x >> 5;
    const uint32_t gw = blockIdx.x * warps_per_cta + (threadIdx.x >> 5);
    const uint32_t nw = gridDim.x * warps_per_cta;
    uint32_t U = *a.key_count;
    if (U > a.key_cap) U = a.key_cap;
    for (uint32_t c = gw; c < U; c += nw) {
        const bool staged = a.stage != nullptr && c < a.stage_slots;
        if (WRITE) {
            const uint32_t n = a.counts[c];
            if (n == 0u) continue;  // nothing to write: skip the second traversal
            if (staged && n <= kStageLights) {
                // the count pass kept the whole list, in list order: copy it instead of traversing again
                const uint32_t o = a.offsets[c];
                for (uint32_t i = lane; i < n; i += 32u) {
                    const uint32_t pos = o + i;
                    if (pos < a.index_cap) a.indices[pos] = a.stage[(size_t)c * kStageLights + i];
                    else VREN_RECORD_ERROR(VREN_ERR_CAPACITY);
                }
                continue;
            }
            assign_cluster<LC, true, SPHERES>(a, lb, a.keys[c], a.offsets[c], lane);
        } else {
            const uint32_t acc = staged ? assign_cluster<LC, false, SPHERES, true>(a, lb, a.keys[c], c * kStageLights, lane)
                                        : assign_cluster<LC, false, SPHERES>(a, lb, a.keys[c], 0u, lane);
            if (lane == 0) a.counts[c] = acc;
        }
    }
}

// assign_lights in one kernel: every warp takes one cluster at a time by ticket, counts its lights
// (first traversal), publishes the count, resolves the cluster's first index by decoupled look-back
// over the counts of the preceding clusters (the count -> exclusive scan -> offsets step of
// assign_lights.comp and clustered_shading.cpp:612-640), then writes the list (second traversal).
// A warp holds one ticket at a time and publishes its count before it waits on anything, so the
// smallest unfinished cluster never waits on a later one.  One cluster per ticket keeps every warp
// on a single pair of traversals (chunks of 16 clusters per warp measured 3x slower: the traversals
// are chains of dependent loads).  Measured at 1920x1080 / 16384 lights: 31 us against 27 us for
// count kernel + scan + write kernel, whose scan costs less than this kernel's look-back chain over
// thousands of clusters, so the three-kernel form is the default (VREN_TUNE_ASSIGN_FUSED = 0).
// Scratch: [0..1] 64-bit [epoch | ticket], [2] completion counter, [3] unused, then one 64-bit status
// word per cluster; the last CTA to finish opens the next call's epoch.
constexpr uint32_t kAssignHeaderWords = 4;

size_t assign_fused_scratch_bytes(uint32_t key_cap)
{
    return (size_t)(kAssignHeaderWords * sizeof(uint32_t) + (uint64_t)(key_cap ? key_cap : 1) * sizeof(uint64_t));
}

template <int LC, bool SPHERES>
__global__ void __launch_bounds__(256) assign_fused_kernel(AssignArgs a, LevelBase lb, uint32_t* __restrict__ offsets,
                                                           uint32_t* __restrict__ scratch, uint32_t* __restrict__ total,
                                                           uint32_t wait_limit, uint32_t spin)
{
    pdl_enter();
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t U = *a.key_count;
    if (U > a.key_cap) U = a.key_cap;
    uint64_t* status = reinterpret_cast<uint64_t*>(scratch + kAssignHeaderWords);
    if (U == 0 && total && blockIdx.x == 0 && threadIdx.x == 0) *total = 0u;
    uint32_t epoch = 0;
    bool timed_out = false;
    for (;;) {
        unsigned long long w = 0;
        if (lane == 0) w = atomicAdd(reinterpret_cast<unsigned long long*>(scratch), 1ull);
        w = __shfl_sync(0xFFFFFFFFu, w, 0);
        const uint32_t c = (uint32_t)w;
        epoch = (uint32_t)(w >> 32) & 0x3FFFFFFFu;
        if (c >= U) break;
        const uint32_t key = a.keys[c];
        const uint32_t cnt = assign_cluster<LC, false, SPHERES>(a, lb, key, 0u, lane);
        uint32_t prefix = 0;
        if (c == 0) {
            if (lane == 0) st_relaxed_u64(status, make_status(epoch, 2u, cnt));
        } else {
            if (lane == 0) st_relaxed_u64(status + c, make_status(epoch, 1u, cnt));
            bool lb_timeout = false;
            prefix = warp_lookback(status, c, 0u, epoch, lane, wait_limit, spin, lb_timeout);
            if (lb_timeout) timed_out = true;
            if (lane == 0) st_relaxed_u64(status + c, make_status(epoch, 2u, prefix + cnt));
        }
        if (lane == 0) {
            a.counts[c] = cnt;
            offsets[c] = prefix;
            if (c == U - 1 && total) *total = prefix + cnt;
        }
        if (cnt) assign_cluster<LC, true, SPHERES>(a, lb, key, prefix, lane);
    }
    if (__any_sync(0xFFFFFFFFu, timed_out) && lane == 0) VREN_RECORD_ERROR(VREN_ERR_TIMEOUT);
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t done = atomicAdd(scratch + 2, 1u);
        if (done == gridDim.x - 1) {
            st_relaxed_u64(reinterpret_cast<uint64_t*>(scratch), (uint64_t)(epoch + 1u) << 32);
            scratch[2] = 0u;
        }
    }
}

__global__ void zero_counts_kernel(const uint32_t* key_count, uint32_t key_cap, uint32_t* __restrict__ counts,
                                   uint32_t* __restrict__ offsets, uint32_t* __restrict__ total)
{
    pdl_enter();
    uint32_t U = *key_count;
    if (U > key_cap) U = key_cap;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < U; c += gridDim.x * blockDim.x) {
        counts[c] = 0u;
        offsets[c] = 0u;
    }
    if (total && blockIdx.x == 0 && threadIdx.x == 0) *total = 0u;
}

// The count pass with the offsets step folded in (count -> exclusive scan of the counts -> offsets,
// clustered_shading.cpp:612-640): a fixed grid of CTAs takes tickets in start order; ticket t owns the
// clusters [t K, t K + K) with K = ceil(U / grid), its warps count (and keep) their lights, the CTA
// sums its counts, publishes the sum and resolves the counts before its range by a decoupled
// look-back over the preceding tickets (at most one per CTA of the grid, so the chain is short), then
// writes its clusters' offsets; the last ticket writes the total.  State: a 64-bit [epoch | ticket]
// word, then one 64-bit status word per CTA, at the end of the assignment scratch.  Measured at
// 1080p / 16,384 lights it is slower than count -> scan -> write (frame 0.0547 against 0.0513 ms):
// with all 1,216 ranges finishing their traversals together, the prefixes travel down the look-back
// chain 32 ranges per round trip, which costs more than the scan launch it saves; selectable
// (VREN_TUNE_ASSIGN_FUSED = 2).
constexpr uint32_t kCountScanMaxGrid = (uint32_t)kNumSMsHint * 8u;
constexpr uint32_t kCountScanThreads = 256;

size_t count_scan_state_bytes() { return 16u + 8ull * kCountScanMaxGrid; }

// The count-with-offsets state sits after the space of the other two forms, so that switching forms
// between calls never reads one form's words as another's.
size_t count_scan_state_offset(uint32_t key_capacity)
{
    const size_t a = scan_scratch_bytes(key_capacity), b = assign_fused_scratch_bytes(key_capacity);
    return ((a > b ? a : b) + 15) / 16 * 16;
}

template <int LC, bool SPHERES>
__global__ void __launch_bounds__(kCountScanThreads) assign_count_scan_kernel(AssignArgs a, LevelBase lb,
                                                                            uint32_t* offsets, uint32_t* total,
                                                                            uint32_t* state, uint32_t wait_limit,
                                                                            uint32_t spin)
{
    pdl_enter();
    constexpr uint32_t kWarps = kCountScanThreads / 32;
    __shared__ uint32_t s_ticket, s_epoch, s_prefix;
    __shared__ uint32_t s_warp[kWarps];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    uint32_t U = *a.key_count;
    if (U > a.key_cap) U = a.key_cap;
    if (tid == 0) {
        uint32_t e;
        s_ticket = take_ticket(state, gridDim.x, e);
        s_epoch = e;
    }
    __syncthreads();
    const uint32_t t = s_ticket, epoch = s_epoch;
    const uint32_t K = (U + gridDim.x - 1) / gridDim.x;
    const uint32_t c0 = t * K < U ? t * K : U, c1 = c0 + K < U ? c0 + K : U;

    // counts (a warp per cluster), the first kStageLights lights kept
    for (uint32_t c = c0 + warp; c < c1; c += kWarps) {
        const bool staged = a.stage != nullptr && c < a.stage_slots;
        const uint32_t acc = staged ? assign_cluster<LC, false, SPHERES, true>(a, lb, a.keys[c], c * kStageLights, lane)
                                    : assign_cluster<LC, false, SPHERES>(a, lb, a.keys[c], 0u, lane);
        if (lane == 0) a.counts[c] = acc;
    }
    __syncthreads();

    // the range's sum, published, and the counts before the range by look-back
    uint32_t sum = 0;
    for (uint32_t c = c0 + tid; c < c1; c += kCountScanThreads) sum += a.counts[c];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) sum += __shfl_xor_sync(0xFFFFFFFFu, sum, d);
    if (lane == 0) s_warp[warp] = sum;
    __syncthreads();
    uint64_t* status = reinterpret_cast<uint64_t*>(state + 4);
    if (warp == 0) {
        uint32_t range = lane < kWarps ? s_warp[lane] : 0u;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) range += __shfl_xor_sync(0xFFFFFFFFu, range, d);
        uint32_t prefix = 0;
        if (t == 0) {
            if (lane == 0) st_relaxed_u64(status, make_status(epoch, 2u, range));
        } else {
            if (lane == 0) st_relaxed_u64(status + t, make_status(epoch, 1u, range));
            bool timed_out = false;
            prefix = warp_lookback(status, t, 0u, epoch, lane, wait_limit, spin, timed_out);
            if (__any_sync(0xFFFFFFFFu, timed_out) && lane == 0) VREN_RECORD_ERROR(VREN_ERR_TIMEOUT);
            if (lane == 0) st_relaxed_u64(status + t, make_status(epoch, 2u, prefix + range));
        }
        if (lane == 0) {
            s_prefix = prefix;
            if (t == gridDim.x - 1 && total) *total = prefix + range;
        }
    }
    __syncthreads();

    // offsets of the range: block-wide exclusive scans of 256 counts at a time, from the prefix on
    uint32_t run = s_prefix;
    for (uint32_t seg = c0; seg < c1; seg += kCountScanThreads) {
        const uint32_t c = seg + tid;
        const uint32_t v = c < c1 ? a.counts[c] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        __syncthreads();  // s_warp of the previous segment has been read
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        uint32_t before = 0, seg_total = 0;
#pragma unroll
        for (uint32_t w = 0; w < kWarps; ++w) {
            const uint32_t x = s_warp[w];
            if (w < warp) before += x;
            seg_total += x;
        }
        if (c < c1) offsets[c] = run + before + incl - v;
        run += seg_total;
    }
}

template <bool SPHERES>
static void launch_count_scan(cudaStream_t st, uint32_t lc, uint32_t grid, const AssignArgs& a, const LevelBase& lb,
                              uint32_t* offsets, uint32_t* total, uint32_t* state)
{
    const uint32_t spin = (uint32_t)tuning(VREN_TUNE_SPIN_POLLS);
#define VREN_CS(LCV) launch_kernel(assign_count_scan_kernel<LCV, SPHERES>, grid, kCountScanThreads, 0, st, a, lb, offsets, \
                                   total, state, g_wait_limit, spin)
    switch (lc) {
    case 1: VREN_CS(1); break;
    case 2: VREN_CS(2); break;
    case 3: VREN_CS(3); break;
    case 4: VREN_CS(4); break;
    case 5: VREN_CS(5); break;
    default: VREN_CS(6); break;
    }
#undef VREN_CS
}

template <bool WRITE, bool SPHERES>
static void launch_assign(cudaStream_t st, uint32_t lc, dim3 grid, dim3 block, const AssignArgs& a, const LevelBase& lb)
{
    switch (lc) {
    case 1: launch_kernel(assign_kernel<1, WRITE, SPHERES>, grid, block, 0, st, a, lb); break;
    case 2: launch_kernel(assign_kernel<2, WRITE, SPHERES>, grid, block, 0, st, a, lb); break;
    case 3: launch_kernel(assign_kernel<3, WRITE, SPHERES>, grid, block, 0, st, a, lb); break;
    case 4: launch_kernel(assign_kernel<4, WRITE, SPHERES>, grid, block, 0, st, a, lb); break;
    case 5: launch_kernel(assign_kernel<5, WRITE, SPHERES>, grid, block, 0, st, a, lb); break;
    default: launch_kernel(assign_kernel<6, WRITE, SPHERES>, grid, block, 0, st, a, lb); break;
    }
}

static int assign_lights(cudaStream_t st, const uint32_t* keys, const uint32_t* key_count, uint32_t key_cap,
                         const vren_cs_frame* frame, const vren_bvh_node* bvh, uint32_t L, const uint32_t* light_index,
                         const float* view_pos, const float* spheres, uint32_t* counts, uint32_t* offsets,
                         uint32_t* indices, uint32_t index_cap, uint32_t* total, void* scratch, uint32_t warps_per_cta,
                         uint32_t* stage = nullptr, uint32_t stage_slots = 0)
{
    if (L == 0) {
        launch_kernel(zero_counts_kernel, 256, 256, 0, st, key_count, key_cap, counts, offsets, total);
        VREN_LAUNCH_CHECK();
        return VREN_OK;
    }
    LevelBase lb{};
    const uint32_t lc = traversal_levels(L, lb);
    if (lc < 1 || lc > 6) return VREN_ERR_ARG;
    AssignArgs a{keys, key_count, key_cap, frame, bvh, reinterpret_cast<const uint2*>(light_index),
                 reinterpret_cast<const float4*>(view_pos), reinterpret_cast<const float4*>(spheres),
                 counts, offsets, indices, index_cap, stage, stage ? stage_slots : 0u};
    if (warps_per_cta < 1 || warps_per_cta > 8) warps_per_cta = 8;
    const dim3 block(32 * warps_per_cta);
    const dim3 grid(kNumSMsHint * (64 / warps_per_cta));
    if (tuning(VREN_TUNE_ASSIGN_FUSED) == 1) {
        uint32_t* sc = static_cast<uint32_t*>(scratch);
        const uint32_t spin = (uint32_t)tuning(VREN_TUNE_SPIN_POLLS);
#define VREN_FUSED(LCV)                                                                                        \
    (spheres ? launch_kernel(assign_fused_kernel<LCV, true>, grid, block, 0, st, a, lb, offsets, sc, total,       \
                             g_wait_limit, spin)                                                                  \
             : launch_kernel(assign_fused_kernel<LCV, false>, grid, block, 0, st, a, lb, offsets, sc, total,      \
                             g_wait_limit, spin))
        switch (lc) {
        case 1: VREN_FUSED(1); break;
        case 2: VREN_FUSED(2); break;
        case 3: VREN_FUSED(3); break;
        case 4: VREN_FUSED(4); break;
        case 5: VREN_FUSED(5); break;
        default: VREN_FUSED(6); break;
        }
#undef VREN_FUSED
        VREN_LAUNCH_CHECK();
        return VREN_OK;
    }
    if (tuning(VREN_TUNE_ASSIGN_FUSED) == 2) {
        // count with the offsets folded in, then write
        uint32_t* state = reinterpret_cast<uint32_t*>(static_cast<char*>(scratch) + count_scan_state_offset(key_cap));
        const uint32_t cs_grid = key_cap < kCountScanMaxGrid ? (key_cap ? key_cap : 1u) : kCountScanMaxGrid;
        if (spheres) launch_count_scan<true>(st, lc, cs_grid, a, lb, offsets, total, state);
        else launch_count_scan<false>(st, lc, cs_grid, a, lb, offsets, total, state);
        VREN_LAUNCH_CHECK();
    } else {
        if (spheres) launch_assign<false, true>(st, lc, grid, block, a, lb);
        else launch_assign<false, false>(st, lc, grid, block, a, lb);
        VREN_LAUNCH_CHECK();
        int rc = scan_exclusive_u32(st, counts, offsets, key_cap, key_count, total, scratch);
        if (rc != VREN_OK) return rc;
    }
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
    // camera.cpp:9-15: orientation = rotate(yaw, Y) * rotate(-pitch, X)
    M4 ry, rx, orient, inv_orient, inv_t, view, proj, inv_proj, inv_view;
    m4_rotate(cam->yaw, 0, 1, 0, ry);
    m4_rotate(-(double)cam->pitch, 1, 0, 0, rx);
    m4_mul(ry, rx, orient);
    m4_inverse(orient, inv_orient);
    // camera.cpp:32-38: view = inverse(orientation) * translate(-position)
    m4_identity(inv_t);
    inv_t[3][0] = -(double)cam->position[0];
    inv_t[3][1] = -(double)cam->position[1];
    inv_t[3][2] = -(double)cam->position[2];
    m4_mul(inv_orient, inv_t, view);
    // camera.cpp:40-50
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
    return (size_t)((fuc_keys_offset_words((uint32_t)tiles) + tiles * 1024u) * 4);
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

extern "C" size_t vren_cs_assign_lights_scratch_bytes(uint32_t key_capacity)
{
    return count_scan_state_offset(key_capacity) + count_scan_state_bytes();
}

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
// Bands of tile rows the host-input frame uploads (and processes, and downloads) one after another.
constexpr uint32_t kHostBands = 4;

struct vren_cluster_and_shade {
    uint32_t max_w = 0, max_h = 0, max_lights = 0, max_assign = 0;
    uint32_t key_cap = 0;
    vren_cs_options opt{15, 1, 8, 8, VREN_CS_NORMALS_F32X3};
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
    uint32_t* stage = nullptr;  // the count pass's copy of each cluster's first kStageLights lights
    uint32_t stage_slots = 0;
    void* lbvh_scratch = nullptr;
    void* fuc_scratch = nullptr;
    uint32_t* fuc_lookback = nullptr;  // ticket word and tile statuses of the one-kernel unique clusters
    void* assign_scratch = nullptr;
    // host frame block (pinned) and the CUDA graph of the last frame shape
    vren_cs_frame* host_frame = nullptr;
    bool frame_valid = false;
    // what the frame block was last built from: the block is built again only when these change
    vren_cs_view last_view{};
    uint32_t last_w = 0, last_h = 0, last_fmt = 0;
    int last_off = 0;
    cudaGraphExec_t graph = nullptr;
    struct Key {
        uint32_t w, h, L, off;
        const void *depth, *normals, *pos, *lights;
        cudaStream_t stream;
        vren_cs_options opt;
    } graph_key{};
    // vren_cs_cluster_host: device copies of the host inputs, a second stream with its events, and
    // the graph of the last host-input frame shape
    char* inputs = nullptr;
    float *in_depth = nullptr, *in_normals = nullptr, *in_pos = nullptr, *in_lights = nullptr;
    cudaStream_t aux = nullptr, up = nullptr;  // light BVH and downloads; G-buffer uploads
    cudaEvent_t ev_fork = nullptr, ev_bvh = nullptr, ev_join = nullptr, ev_join_up = nullptr;
    cudaEvent_t ev_band[kHostBands] = {};  // a band of the G-buffer has arrived
    cudaEvent_t ev_done[kHostBands] = {};  // a band's references are final
    cudaGraphExec_t host_graph = nullptr;
    struct HostKey {
        Key k;
        void* refs_out;
        void* lists_out;
        uint64_t lists_cap;
        uint64_t zero_copy;  // the form the graph was captured with
    } host_key{};
    // vren_cs_cluster_and_shade: the graph of the last clustered-and-shaded frame shape
    cudaGraphExec_t shade_graph = nullptr;
    struct ShadeKey {
        Key k;
        vren_cs_gbuffer gb;
        const void* dir;
        uint32_t ndir;
        int falloff, mode;
        void* out;
    } shade_key{};
};

namespace {
size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// The key a captured frame graph is replayed under, compared byte for byte: zero-filled first so that
// padding bytes compare equal too.
void fill_key(vren_cluster_and_shade::Key& k, const vren_cluster_and_shade* cs, uint32_t W, uint32_t H, uint32_t L,
              int offscreen, const void* depth, const void* normals, const void* pos, const void* lights,
              cudaStream_t st)
{
    std::memset(&k, 0, sizeof(k));
    k.w = W;
    k.h = H;
    k.L = L;
    k.off = (uint32_t)offscreen;
    k.depth = depth;
    k.normals = normals;
    k.pos = pos;
    k.lights = lights;
    k.stream = st;
    k.opt = cs->opt;
}

int cs_enqueue(vren_cluster_and_shade* cs, cudaStream_t st, uint32_t W, uint32_t H, const float* depth,
               const float* normals, const float* positions, const float* lights, uint32_t L)
{
    const PdlScope pdl(1);  // consecutive kernels of the frame overlap their launches
    int rc = VREN_OK;
    // The light BVH and the unique clusters are independent: the BVH is built on the context's second
    // stream while the tiles run on st; the assignment waits for both.
    if (L > 0) {
        VREN_CUDA_TRY(cudaEventRecord(cs->ev_fork, st));
        VREN_CUDA_TRY(cudaStreamWaitEvent(cs->aux, cs->ev_fork, 0));
        rc = construct_light_bvh(cs->aux, positions, lights, L, cs->frame, cs->opt.morton_bits,
                                 cs->opt.sort_digit_bits, cs->view_pos, cs->bvh, cs->light_index, cs->spheres,
                                 cs->lbvh_scratch);
        VREN_CUDA_TRY(cudaEventRecord(cs->ev_bvh, cs->aux));
        if (rc != VREN_OK) {
            cudaStreamWaitEvent(st, cs->ev_bvh, 0);  // rejoin before returning (a capture must end joined)
            return rc;
        }
    }
    rc = tuning(VREN_TUNE_FUC_FUSED) == 2
             ? launch_find_unique_fused(st, depth, normals, W, H, cs->frame, cs->keys, cs->key_cap, cs->key_count,
                                        cs->refs, cs->fuc_lookback)
             : launch_find_unique(st, depth, normals, W, H, cs->frame, cs->keys, cs->key_cap, cs->key_count, cs->refs,
                                  static_cast<uint32_t*>(cs->fuc_scratch));
    if (L > 0) VREN_CUDA_TRY(cudaStreamWaitEvent(st, cs->ev_bvh, 0));
    if (rc != VREN_OK) return rc;
    return assign_lights(st, cs->keys, cs->key_count, cs->key_cap, cs->frame, cs->bvh, L, cs->light_index,
                         cs->view_pos, cs->spheres, cs->counts, cs->offsets, cs->indices, cs->max_assign, cs->total,
                         cs->assign_scratch, cs->opt.assign_warps, cs->stage, cs->stage_slots);
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
    // stage: one slot of kStageLights per cluster, up to the index capacity (the lists it can hold)
    const uint64_t stage_words = std::min<uint64_t>((uint64_t)max_assignments, (uint64_t)cs->key_cap * kStageLights);
    const size_t o_stage = carve((size_t)(stage_words ? stage_words : 1) * 4);
    size_t lbvh = 0;
    for (uint32_t db : {4u, 6u, 8u})
        for (uint32_t mb : {15u, 30u}) {
            const size_t b = lbvh_layout(Lb, mb, db).total;
            lbvh = b > lbvh ? b : lbvh;
        }
    const size_t o_lbvh = carve(lbvh);
    const size_t o_fuc = carve(vren_cs_unique_clusters_scratch_bytes(max_width, max_height));
    const size_t o_fuc_lb = carve(fuc_lookback_bytes(tiles));
    const size_t o_asg = carve(vren_cs_assign_lights_scratch_bytes(cs->key_cap));
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
    cs->stage = reinterpret_cast<uint32_t*>(a + o_stage);
    cs->stage_slots = (uint32_t)(stage_words / kStageLights);
    cs->lbvh_scratch = a + o_lbvh;
    cs->fuc_scratch = a + o_fuc;
    cs->fuc_lookback = reinterpret_cast<uint32_t*>(a + o_fuc_lb);
    cs->assign_scratch = a + o_asg;
    // the second and third streams (light BVH beside the tiles; banded uploads) and their events
    bool ok = cudaStreamCreateWithFlags(&cs->aux, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&cs->up, cudaStreamNonBlocking) == cudaSuccess;
    for (cudaEvent_t* e : {&cs->ev_fork, &cs->ev_bvh, &cs->ev_join, &cs->ev_join_up})
        ok = ok && cudaEventCreateWithFlags(e, cudaEventDisableTiming) == cudaSuccess;
    for (uint32_t b = 0; b < kHostBands; ++b)
        ok = ok && cudaEventCreateWithFlags(&cs->ev_band[b], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&cs->ev_done[b], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        vren_cs_destroy(cs);
        return VREN_ERR_CUDA;
    }
    *out = cs;
    return VREN_OK;
}

extern "C" void vren_cs_destroy(vren_cluster_and_shade* cs)
{
    if (!cs) return;
    if (cs->graph) cudaGraphExecDestroy(cs->graph);
    if (cs->host_graph) cudaGraphExecDestroy(cs->host_graph);
    if (cs->shade_graph) cudaGraphExecDestroy(cs->shade_graph);
    if (cs->aux) cudaStreamDestroy(cs->aux);
    if (cs->up) cudaStreamDestroy(cs->up);
    for (cudaEvent_t e : {cs->ev_fork, cs->ev_bvh, cs->ev_join, cs->ev_join_up})
        if (e) cudaEventDestroy(e);
    for (uint32_t b = 0; b < kHostBands; ++b) {
        if (cs->ev_band[b]) cudaEventDestroy(cs->ev_band[b]);
        if (cs->ev_done[b]) cudaEventDestroy(cs->ev_done[b]);
    }
    cudaFree(cs->inputs);
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
    if (o->normal_format != VREN_CS_NORMALS_F32X3 && o->normal_format != VREN_CS_NORMALS_RGBA16F) return VREN_ERR_ARG;
    cs->opt = *o;
    if (cs->graph) {
        cudaGraphExecDestroy(cs->graph);
        cs->graph = nullptr;
    }
    if (cs->host_graph) {
        cudaGraphExecDestroy(cs->host_graph);
        cs->host_graph = nullptr;
    }
    if (cs->shade_graph) {
        cudaGraphExecDestroy(cs->shade_graph);
        cs->shade_graph = nullptr;
    }
    return VREN_OK;
}

namespace {
// The frame block lives in device memory and is read by every kernel; it is re-uploaded (from pinned
// memory, outside any captured graph) only when the camera or the frame shape changes.
int refresh_frame(vren_cluster_and_shade* cs, cudaStream_t st, const vren_cs_view* view, uint32_t width,
                  uint32_t height, int offscreen)
{
    if (cs->frame_valid && width == cs->last_w && height == cs->last_h && offscreen == cs->last_off &&
        cs->opt.normal_format == cs->last_fmt && std::memcmp(view, &cs->last_view, sizeof(vren_cs_view)) == 0)
        return VREN_OK;  // same camera and frame shape: the block on the device is current
    static thread_local vren_cs_frame fresh;
    int rc = vren_cs_frame_build(view, width, height, offscreen, &fresh);
    if (rc != VREN_OK) return rc;
    fresh.normal_format = cs->opt.normal_format;
    if (!cs->frame_valid || std::memcmp(&fresh, cs->host_frame, sizeof(vren_cs_frame)) != 0) {
        VREN_CUDA_TRY(cudaStreamSynchronize(st));  // an earlier upload may still read host_frame
        std::memcpy(cs->host_frame, &fresh, sizeof(vren_cs_frame));
        VREN_CUDA_TRY(cudaMemcpyAsync(cs->frame, cs->host_frame, sizeof(vren_cs_frame), cudaMemcpyHostToDevice, st));
        cs->frame_valid = true;
    }
    cs->last_view = *view;
    cs->last_w = width;
    cs->last_h = height;
    cs->last_off = offscreen;
    cs->last_fmt = cs->opt.normal_format;
    return VREN_OK;
}

// The address under which the device reads or writes the host buffer `p` (page-locked and mapped,
// or any host memory when the device has pageable-memory access), or null when it cannot.
const void* device_view_of_host(const void* p)
{
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return p;
    int dev = 0, pageable = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return pageable ? p : nullptr;
}

// Band edges in tile rows for the host-input frame: band i gets a share bands - i of the rows (4/10,
// 3/10, 2/10, 1/10 for four bands), at least one row each, so that the last band, whose tiles,
// fix-up and download come after the last upload, is the smallest.
constexpr bool kHostBandTaper = true;
void host_band_edges(uint32_t rows, uint32_t bands, uint32_t* edge)
{
    const uint32_t total = kHostBandTaper ? bands * (bands + 1) / 2 : bands;
    uint32_t cum = 0;
    edge[0] = 0;
    for (uint32_t i = 0; i < bands; ++i) {
        cum += kHostBandTaper ? bands - i : 1u;
        uint32_t e = (uint32_t)(((uint64_t)rows * cum + total / 2) / total);
        if (e < edge[i] + 1u) e = edge[i] + 1u;               // at least one row
        if (e > rows - (bands - 1u - i)) e = rows - (bands - 1u - i);  // one row left for each later band
        edge[i + 1] = e;
    }
}

// One frame from host buffers: the lights go up and their BVH is built on the second stream while the
// depth and normals go up on `st` in bands of tile rows, each band's tiles processed as it arrives;
// then the references go down on the second stream while the light lists are assigned on `st`, and
// the lists are written into host memory by the device.
// zc_depth / zc_normals: the device's views of the host G-buffer for the zero-copy form (both null
// for the banded copies); zc_refs: the device's view of refs_out (null when no references go down).
int cs_enqueue_host(vren_cluster_and_shade* cs, cudaStream_t st, uint32_t W, uint32_t H, const float* depth,
                    const float* normals, const float* positions, const float* lights, uint32_t L, uint32_t* refs_out,
                    uint32_t* lists_out, uint64_t lists_cap, const float* zc_depth = nullptr,
                    const float* zc_normals = nullptr, uint32_t* zc_refs = nullptr)
{
    const PdlScope pdl(1);
    cudaStream_t aux = cs->aux, up = cs->up;
    VREN_CUDA_TRY(cudaEventRecord(cs->ev_fork, st));
    VREN_CUDA_TRY(cudaStreamWaitEvent(aux, cs->ev_fork, 0));
    VREN_CUDA_TRY(cudaStreamWaitEvent(up, cs->ev_fork, 0));
    int rc = VREN_OK;
    if (L > 0) {
        VREN_CUDA_TRY(cudaMemcpyAsync(cs->in_pos, positions, (size_t)L * 16, cudaMemcpyHostToDevice, aux));
        VREN_CUDA_TRY(cudaMemcpyAsync(cs->in_lights, lights, (size_t)L * 16, cudaMemcpyHostToDevice, aux));
        rc = construct_light_bvh(aux, cs->in_pos, cs->in_lights, L, cs->frame, cs->opt.morton_bits,
                                 cs->opt.sort_digit_bits, cs->view_pos, cs->bvh, cs->light_index, cs->spheres,
                                 cs->lbvh_scratch);
        if (rc != VREN_OK) return rc;
    }
    VREN_CUDA_TRY(cudaEventRecord(cs->ev_bvh, aux));
    if (zc_depth && zc_normals) {
        // Zero-copy: the one-kernel unique-cluster form reads the G-buffer over the link as its tiles
        // run (tiles in order, offsets by look-back), so the reads and the references going down
        // (written to both the context and refs_out as each tile finishes) share the link's two
        // directions for the whole kernel.
        VREN_CUDA_TRY(cudaEventRecord(cs->ev_join_up, up));
        rc = launch_find_unique_fused(st, zc_depth, zc_normals, W, H, cs->frame, cs->keys, cs->key_cap, cs->key_count,
                                      cs->refs, cs->fuc_lookback, zc_refs);
        if (rc != VREN_OK) return rc;
    } else {
        // G-buffer up in bands of tile rows, each band's tiles processed as soon as it has arrived (the last
        // tile row may wrap to the first rows, which arrive first)
        const FucFrame fr = fuc_frame(cs->in_depth, cs->in_normals, W, H, cs->frame, cs->keys, cs->key_cap,
                                      cs->key_count, cs->refs, static_cast<uint32_t*>(cs->fuc_scratch));
        const uint32_t TX = (W + 31) / 32, TY = (H + 31) / 32;
        const uint32_t bands = TY < kHostBands ? TY : kHostBands;
        uint32_t edge[kHostBands + 1];
        host_band_edges(TY, bands, edge);
        const size_t nbytes = cs->opt.normal_format == VREN_CS_NORMALS_RGBA16F ? 8 : 12;  // per pixel
        for (uint32_t band = 0; band < bands; ++band) {  // uploads on `up`, one event per band
            const uint32_t ty0 = edge[band], ty1 = edge[band + 1];
            const size_t y0 = (size_t)ty0 * 32, y1 = (size_t)ty1 * 32 < H ? (size_t)ty1 * 32 : H;
            VREN_CUDA_TRY(cudaMemcpyAsync(cs->in_depth + y0 * W, depth + y0 * W, (y1 - y0) * W * 4,
                                          cudaMemcpyHostToDevice, up));
            VREN_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char*>(cs->in_normals) + y0 * W * nbytes,
                                          reinterpret_cast<const char*>(normals) + y0 * W * nbytes, (y1 - y0) * W * nbytes,
                                          cudaMemcpyHostToDevice, up));
            VREN_CUDA_TRY(cudaEventRecord(cs->ev_band[band], up));
        }
        VREN_CUDA_TRY(cudaEventRecord(cs->ev_join_up, up));
        // Each band once it has arrived: its tiles, then its tile offsets (continuing from the band above)
        // and fix-up, after which its rows of references are final and go down on `aux` while the next
        // bands are still coming up.
        for (uint32_t band = 0; band < bands; ++band) {
            const uint32_t ty0 = edge[band], ty1 = edge[band + 1];
            VREN_CUDA_TRY(cudaStreamWaitEvent(st, cs->ev_band[band], 0));
            rc = launch_find_unique_tiles(st, fr, ty0 * TX, (ty1 - ty0) * TX);
            if (rc != VREN_OK) return rc;
            rc = launch_find_unique_finish(st, fr, ty0 * TX, ty1 * TX);
            if (rc != VREN_OK) return rc;
            if (refs_out) {
                const size_t y0 = (size_t)ty0 * 32, y1 = (size_t)ty1 * 32 < H ? (size_t)ty1 * 32 : H;
                VREN_CUDA_TRY(cudaEventRecord(cs->ev_done[band], st));
                VREN_CUDA_TRY(cudaStreamWaitEvent(aux, cs->ev_done[band], 0));
                VREN_CUDA_TRY(cudaMemcpyAsync(refs_out + y0 * W, cs->refs + y0 * W, (y1 - y0) * W * 4,
                                              cudaMemcpyDeviceToHost, aux));
            }
        }
    }
    VREN_CUDA_TRY(cudaStreamWaitEvent(st, cs->ev_bvh, 0));
    rc = assign_lights(st, cs->keys, cs->key_count, cs->key_cap, cs->frame, cs->bvh, L, cs->light_index,
                       cs->view_pos, cs->spheres, cs->counts, cs->offsets, cs->indices, cs->max_assign, cs->total,
                       cs->assign_scratch, cs->opt.assign_warps, cs->stage, cs->stage_slots);
    if (rc != VREN_OK) return rc;
    if (lists_out) {
        launch_kernel(lists_to_host_kernel, kNumSMsHint, 256, 0, st, cs->key_count, cs->key_cap, cs->total, cs->keys,
                      cs->counts, cs->offsets, cs->indices, cs->max_assign, lists_out, lists_cap);
        VREN_LAUNCH_CHECK();
    }
    VREN_CUDA_TRY(cudaEventRecord(cs->ev_join, aux));
    VREN_CUDA_TRY(cudaStreamWaitEvent(st, cs->ev_join, 0));
    VREN_CUDA_TRY(cudaStreamWaitEvent(st, cs->ev_join_up, 0));
    return VREN_OK;
}
}  // namespace

extern "C" int vren_cs_cluster(vren_cluster_and_shade* cs, vren_stream_t s, const vren_cs_view* view, uint32_t width,
                               uint32_t height, int offscreen, const float* depth, const float* normals,
                               const float* light_positions, const float* point_lights, uint32_t light_count)
{
    if (!cs || !view || !depth || !normals) return VREN_ERR_ARG;
    if (width > cs->max_w || height > cs->max_h || light_count > cs->max_lights) return VREN_ERR_CAPACITY;
    if (light_count > 0 && (!light_positions || !point_lights)) return VREN_ERR_ARG;
    cudaStream_t st = as_stream(s);
    int rc = refresh_frame(cs, st, view, width, height, offscreen);
    if (rc != VREN_OK) return rc;
    vren_cluster_and_shade::Key key;
    fill_key(key, cs, width, height, light_count, offscreen, depth, normals, light_positions, point_lights, st);
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
    std::memcpy(&cs->graph_key, &key, sizeof(key));
    VREN_CUDA_TRY(cudaGraphLaunch(cs->graph, st));
    return VREN_OK;
}

extern "C" int vren_cs_cluster_host(vren_cluster_and_shade* cs, vren_stream_t s, const vren_cs_view* view,
                                    uint32_t width, uint32_t height, int offscreen, const float* depth,
                                    const float* normals, const float* light_positions, const float* point_lights,
                                    uint32_t light_count, uint32_t* cluster_refs_out, uint32_t* lists_out,
                                    uint64_t lists_capacity)
{
    if (!cs || !view || !depth || !normals) return VREN_ERR_ARG;
    if (width > cs->max_w || height > cs->max_h || light_count > cs->max_lights) return VREN_ERR_CAPACITY;
    if (light_count > 0 && (!light_positions || !point_lights)) return VREN_ERR_ARG;
    cudaStream_t st = as_stream(s);
    if (!cs->inputs) {  // first use: device copies of the inputs
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        VREN_CUDA_TRY(cudaStreamIsCapturing(st, &cap));
        if (cap != cudaStreamCaptureStatusNone) return VREN_ERR_STATE;
        const size_t px = (size_t)cs->max_w * cs->max_h, Lb = cs->max_lights ? cs->max_lights : 1;
        const size_t o_n = align256(px * 4), o_p = o_n + align256(px * 12), o_l = o_p + align256(Lb * 16);
        const size_t bytes = o_l + align256(Lb * 16);
        if (cudaMalloc(&cs->inputs, bytes) != cudaSuccess) {
            cs->inputs = nullptr;
            return VREN_ERR_CUDA;
        }
        cs->in_depth = reinterpret_cast<float*>(cs->inputs);
        cs->in_normals = reinterpret_cast<float*>(cs->inputs + o_n);
        cs->in_pos = reinterpret_cast<float*>(cs->inputs + o_p);
        cs->in_lights = reinterpret_cast<float*>(cs->inputs + o_l);
    }
    int rc = refresh_frame(cs, st, view, width, height, offscreen);
    if (rc != VREN_OK) return rc;
    vren_cluster_and_shade::HostKey key;
    std::memset(&key, 0, sizeof(key));
    fill_key(key.k, cs, width, height, light_count, offscreen, depth, normals, light_positions, point_lights, st);
    key.refs_out = cluster_refs_out;
    key.lists_out = lists_out;
    key.lists_cap = lists_capacity;
    // The zero-copy form when it is selected and the device can address the G-buffer (and refs_out)
    const float* zc_depth = nullptr;
    const float* zc_normals = nullptr;
    uint32_t* zc_refs = nullptr;
    if (tuning(VREN_TUNE_HOST_ZERO_COPY) == 1) {
        zc_depth = static_cast<const float*>(device_view_of_host(depth));
        zc_normals = static_cast<const float*>(device_view_of_host(normals));
        zc_refs = cluster_refs_out ? static_cast<uint32_t*>(const_cast<void*>(device_view_of_host(cluster_refs_out)))
                                   : nullptr;
        if (!zc_depth || !zc_normals || (cluster_refs_out && !zc_refs)) zc_depth = zc_normals = nullptr, zc_refs = nullptr;
    }
    key.zero_copy = zc_depth ? 1u : 0u;
    const bool use_graph = cs->opt.use_graph && st != nullptr;
    if (!use_graph)
        return cs_enqueue_host(cs, st, width, height, depth, normals, light_positions, point_lights, light_count,
                               cluster_refs_out, lists_out, lists_capacity, zc_depth, zc_normals, zc_refs);
    if (cs->host_graph && std::memcmp(&key, &cs->host_key, sizeof(key)) == 0) {
        VREN_CUDA_TRY(cudaGraphLaunch(cs->host_graph, st));
        return VREN_OK;
    }
    if (cs->host_graph) {
        cudaGraphExecDestroy(cs->host_graph);
        cs->host_graph = nullptr;
    }
    cudaGraph_t g;
    VREN_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    rc = cs_enqueue_host(cs, st, width, height, depth, normals, light_positions, point_lights, light_count,
                         cluster_refs_out, lists_out, lists_capacity, zc_depth, zc_normals, zc_refs);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc != VREN_OK) {
        if (e == cudaSuccess) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return VREN_ERR_CUDA;
    e = cudaGraphInstantiate(&cs->host_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cs->host_graph = nullptr;
        return VREN_ERR_CUDA;
    }
    std::memcpy(&cs->host_key, &key, sizeof(key));
    VREN_CUDA_TRY(cudaGraphLaunch(cs->host_graph, st));
    return VREN_OK;
}

extern "C" int vren_cs_cluster_and_shade(vren_cluster_and_shade* cs, vren_stream_t s, const vren_cs_view* view,
                                         uint32_t width, uint32_t height, int offscreen, const vren_cs_gbuffer* gbuffer,
                                         const float* light_positions, const float* point_lights, uint32_t light_count,
                                         const float* directional_lights, uint32_t directional_count, int falloff,
                                         int output_mode, float* out_rgb)
{
    if (!cs || !view || !gbuffer || !gbuffer->depth || !gbuffer->normals || !out_rgb) return VREN_ERR_ARG;
    if (cs->opt.normal_format != VREN_CS_NORMALS_F32X3) return VREN_ERR_ARG;  // the shading kernels read f32x3
    if (width > cs->max_w || height > cs->max_h || light_count > cs->max_lights) return VREN_ERR_CAPACITY;
    if (light_count > 0 && (!light_positions || !point_lights)) return VREN_ERR_ARG;
    if (falloff != VREN_CS_FALLOFF_REF && falloff != VREN_CS_FALLOFF_WINDOWED_INV_SQ) return VREN_ERR_ARG;
    if (output_mode != VREN_CS_SHADE_COLOR && output_mode != VREN_CS_SHADE_RADIANCE) return VREN_ERR_ARG;
    cudaStream_t st = as_stream(s);
    int rc = refresh_frame(cs, st, view, width, height, offscreen);
    if (rc != VREN_OK) return rc;
    const vren_cs_light_lists lists{cs->refs, cs->counts, cs->offsets, cs->indices, cs->max_assign, 0u};
    auto enqueue = [&]() -> int {
        int r = cs_enqueue(cs, st, width, height, gbuffer->depth, gbuffer->normals, light_positions, point_lights,
                           light_count);
        if (r != VREN_OK) return r;
        return vren_cs_shade(st, cs->frame, width, height, gbuffer, &lists, light_positions, point_lights, light_count,
                             directional_lights, directional_count, falloff, output_mode, out_rgb);
    };
    if (!(cs->opt.use_graph && st != nullptr)) return enqueue();
    vren_cluster_and_shade::ShadeKey key;
    std::memset(&key, 0, sizeof(key));
    fill_key(key.k, cs, width, height, light_count, offscreen, gbuffer->depth, gbuffer->normals, light_positions,
             point_lights, st);
    key.gb = *gbuffer;
    key.dir = directional_lights;
    key.ndir = directional_count;
    key.falloff = falloff;
    key.mode = output_mode;
    key.out = out_rgb;
    if (cs->shade_graph && std::memcmp(&key, &cs->shade_key, sizeof(key)) == 0) {
        VREN_CUDA_TRY(cudaGraphLaunch(cs->shade_graph, st));
        return VREN_OK;
    }
    if (cs->shade_graph) {
        cudaGraphExecDestroy(cs->shade_graph);
        cs->shade_graph = nullptr;
    }
    cudaGraph_t g;
    VREN_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    rc = enqueue();
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc != VREN_OK) {
        if (e == cudaSuccess) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return VREN_ERR_CUDA;
    e = cudaGraphInstantiate(&cs->shade_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cs->shade_graph = nullptr;
        return VREN_ERR_CUDA;
    }
    std::memcpy(&cs->shade_key, &key, sizeof(key));
    VREN_CUDA_TRY(cudaGraphLaunch(cs->shade_graph, st));
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

// Karras binary radix tree over sorted leaves, and light assignment through it — an extension beside
// the reference's 32-ary BuildBVH (vren/vren/primitives/build_bvh.cpp, build_bvh.comp:32-55) and its
// traversal (assign_lights.comp:121-240).
//
// Build (T. Karras, "Maximizing Parallelism in the Construction of BVHs, Octrees, and k-d Trees",
// HPG 2012, section 4): one thread per internal node finds the range of leaves it covers from the
// longest common prefix of the augmented keys (key, leaf position) and splits it where that prefix
// grows; the boxes are then refitted bottom-up, one thread per leaf climbing until it is the first
// of two children to arrive (an atomic count per node, no waiting).  Unions are taken in IEEE total
// order, so the boxes do not depend on which child arrives last.
//
// Assignment: one thread per cluster walks the tree depth-first, left child first, so it meets the
// leaves in ascending order; the hits of one 32-leaf group are buffered and written back to front,
// which is the reference's list order.  With the tree built over the group boxes (level 1 of the
// 32-ary BVH) the assigned set is exactly the reference's (see vren_cs_assign_lights_lbvh).
#include "common.cuh"
#include "internal.h"

namespace vren_gb300 {
VREN_DEFINE_ERROR_WORD(lbvh)
}  // namespace vren_gb300

#include "cs_device.cuh"

namespace vren_gb300 {

constexpr uint32_t kLbvhNone = 0xFFFFFFFFu;
constexpr int kLbvhThreads = 256;
constexpr int kLbvhStack = 64;  // tree depth <= key bits (32) + position bits (24)

struct LbvhBox {
    float mn[3];
    float mx[3];
};

// Box of leaf i: boxes[i >> shift], or infinite without boxes.
__device__ __forceinline__ LbvhBox leaf_box(const vren_bvh_node* boxes, uint32_t shift, uint32_t i)
{
    LbvhBox b;
    if (boxes) {
        const NodeF n = load_node(boxes, i >> shift);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            b.mn[k] = n.mn[k];
            b.mx[k] = n.mx[k];
        }
    } else {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            b.mn[k] = __int_as_float(0xFF800000);  // -inf
            b.mx[k] = __int_as_float(0x7F800000);  // +inf
        }
    }
    return b;
}

// Longest common prefix of the augmented keys of leaves i and j; -1 outside [0, n).
__device__ __forceinline__ int lbvh_delta(const uint2* pairs, int64_t n, int64_t i, int64_t j)
{
    if (j < 0 || j >= n) return -1;
    const uint32_t a = pairs[i].x, b = pairs[j].x;
    if (a != b) return __clz(a ^ b);
    return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

// One thread per internal node i: its children (Karras 2012, Figure 4) and their parent links.
// parent[] holds the n - 1 internal nodes' parents, then the n leaves'; count[] is cleared here.
__global__ void __launch_bounds__(kLbvhThreads) lbvh_topology_kernel(const uint2* __restrict__ pairs, uint32_t n,
                                                                     vren_lbvh_node* __restrict__ nodes,
                                                                     uint32_t* __restrict__ parent,
                                                                     uint32_t* __restrict__ count)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i + 1 >= (int64_t)n) return;
    const int d = lbvh_delta(pairs, n, i, i + 1) - lbvh_delta(pairs, n, i, i - 1) >= 0 ? 1 : -1;
    const int dmin = lbvh_delta(pairs, n, i, i - d);
    int64_t lmax = 2;
    while (lbvh_delta(pairs, n, i, i + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0;
    for (int64_t t = lmax / 2; t >= 1; t /= 2)
        if (lbvh_delta(pairs, n, i, i + (l + t) * d) > dmin) l += t;
    const int64_t j = i + l * d;
    const int dnode = lbvh_delta(pairs, n, i, j);
    int64_t s = 0, t = l;
    do {
        t = (t + 1) / 2;
        if (lbvh_delta(pairs, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
    const bool left_leaf = (i < j ? i : j) == gamma, right_leaf = (i < j ? j : i) == gamma + 1;
    const uint32_t left = (uint32_t)gamma | (left_leaf ? VREN_LBVH_LEAF : 0u);
    const uint32_t right = (uint32_t)(gamma + 1) | (right_leaf ? VREN_LBVH_LEAF : 0u);
    nodes[i].left = left;
    nodes[i].right = right;
    parent[left_leaf ? (n - 1) + (uint32_t)gamma : (uint32_t)gamma] = (uint32_t)i;
    parent[right_leaf ? (n - 1) + (uint32_t)(gamma + 1) : (uint32_t)(gamma + 1)] = (uint32_t)i;
    if (i == 0) parent[0] = kLbvhNone;
    count[i] = 0u;
}

__device__ __forceinline__ LbvhBox lbvh_child_box(const vren_lbvh_node* nodes, const vren_bvh_node* boxes,
                                                  uint32_t shift, uint32_t child)
{
    if (child & VREN_LBVH_LEAF) return leaf_box(boxes, shift, child & ~VREN_LBVH_LEAF);
    // written by another thread of this kernel (ordered by the count atomic): read from L2
    const float4* p = reinterpret_cast<const float4*>(nodes + child);
    const float4 lo = __ldcg(p), hi = __ldcg(p + 1);
    LbvhBox b;
    b.mn[0] = lo.x; b.mn[1] = lo.y; b.mn[2] = lo.z;
    b.mx[0] = hi.x; b.mx[1] = hi.y; b.mx[2] = hi.z;
    return b;
}

// One thread per leaf: climb while this thread is the second child to arrive at the parent.
__global__ void __launch_bounds__(kLbvhThreads) lbvh_refit_kernel(const vren_bvh_node* __restrict__ boxes,
                                                                  uint32_t shift, uint32_t n,
                                                                  vren_lbvh_node* __restrict__ nodes,
                                                                  const uint32_t* __restrict__ parent,
                                                                  uint32_t* __restrict__ count)
{
    const uint32_t leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= n) return;
    uint32_t p = parent[(n - 1) + leaf];
    for (uint32_t steps = 0; p != kLbvhNone && steps < n; ++steps) {
        __threadfence();  // this thread's box writes are visible before the count says so
        if (atomicAdd(&count[p], 1u) == 0u) return;
        __threadfence();
        const uint32_t l = nodes[p].left, r = nodes[p].right;
        const LbvhBox a = lbvh_child_box(nodes, boxes, shift, l), b = lbvh_child_box(nodes, boxes, shift, r);
        float4* q = reinterpret_cast<float4*>(nodes + p);
        const float4 lo = make_float4(unkey(min(fkey(a.mn[0]), fkey(b.mn[0]))), unkey(min(fkey(a.mn[1]), fkey(b.mn[1]))),
                                      unkey(min(fkey(a.mn[2]), fkey(b.mn[2]))), __uint_as_float(l));
        const float4 hi = make_float4(unkey(max(fkey(a.mx[0]), fkey(b.mx[0]))), unkey(max(fkey(a.mx[1]), fkey(b.mx[1]))),
                                      unkey(max(fkey(a.mx[2]), fkey(b.mx[2]))), __uint_as_float(r));
        __stcg(q, lo);
        __stcg(q + 1, hi);
        p = parent[p];
    }
}

}  // namespace vren_gb300

using namespace vren_gb300;

extern "C" size_t vren_lbvh_scratch_bytes(uint32_t leaf_count)
{
    const uint64_t n = leaf_count ? leaf_count : 1;
    return (size_t)((2 * n - 1) + (n - 1) + 1) * sizeof(uint32_t);
}

namespace vren_gb300 {
int lbvh_build(cudaStream_t st, const uint32_t* sorted_pairs, uint32_t n, const vren_bvh_node* boxes, uint32_t shift,
               vren_lbvh_node* nodes, void* scratch)
{
    if (n < 2) return VREN_OK;
    uint32_t* parent = static_cast<uint32_t*>(scratch);
    uint32_t* count = parent + (2 * (uint64_t)n - 1);
    const uint32_t grid_i = (n - 1 + kLbvhThreads - 1) / kLbvhThreads;
    launch_kernel(lbvh_topology_kernel, grid_i, kLbvhThreads, 0, st, reinterpret_cast<const uint2*>(sorted_pairs), n,
                  nodes, parent, count);
    VREN_LAUNCH_CHECK();
    const uint32_t grid_l = (n + kLbvhThreads - 1) / kLbvhThreads;
    launch_kernel(lbvh_refit_kernel, grid_l, kLbvhThreads, 0, st, boxes, shift, n, nodes, parent, count);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}
}  // namespace vren_gb300

extern "C" int vren_build_lbvh(vren_stream_t s, const uint32_t* sorted_pairs, uint32_t leaf_count,
                               const vren_bvh_node* boxes, uint32_t box_shift, vren_lbvh_node* nodes, void* scratch)
{
    if (leaf_count > (1u << 24) || box_shift > 31) return VREN_ERR_ARG;
    if (leaf_count < 2) return VREN_OK;
    if (!sorted_pairs || !nodes || !scratch) return VREN_ERR_ARG;
    return lbvh_build(as_stream(s), sorted_pairs, leaf_count, boxes, box_shift, nodes, scratch);
}

// ================================================================================================
// Light assignment through the tree
// ================================================================================================
namespace vren_gb300 {

struct LbvhAssign {
    const uint32_t* keys;
    const uint32_t* key_count;
    uint32_t key_cap;
    const vren_cs_frame* frame;
    const vren_lbvh_node* nodes;
    const vren_bvh_node* bvh;     // level 0: leaf boxes (radii)
    const vren_bvh_node* groups;  // level 1 (group boxes), or null for at most 32 lights
    uint32_t L;
    const uint2* light_index;
    const float4* view_pos;
    const float4* spheres;
    uint32_t* counts;
    const uint32_t* offsets;
    uint32_t* indices;
    uint32_t index_cap;
};

__device__ __forceinline__ bool box_overlaps(const Box& c, const float mn[3], const float mx[3])
{
    return c.mx[0] >= mn[0] && c.mn[0] <= mx[0] && c.mx[1] >= mn[1] && c.mn[1] <= mx[1] && c.mx[2] >= mn[2] &&
           c.mn[2] <= mx[2];
}

// One cluster: returns the number of lights assigned; with WRITE writes them from out on.
template <bool WRITE>
__device__ uint32_t lbvh_cluster(const LbvhAssign& a, const Box& box, uint32_t out)
{
    uint32_t stack[kLbvhStack];
    uint32_t buf[32];
    int sp = 0, nb = 0;
    uint32_t cur = a.L == 1 ? VREN_LBVH_LEAF : 0u;
    uint32_t acc = 0, written = 0, grp = kLbvhNone;
    auto flush = [&]() {
        while (nb > 0) {
            const uint32_t pos = out + written++;
            if (pos < a.index_cap) a.indices[pos] = buf[--nb];
            else {
                --nb;
                VREN_RECORD_ERROR(VREN_ERR_CAPACITY);
            }
        }
    };
    for (;;) {
        bool descend = false;
        if (cur & VREN_LBVH_LEAF) {
            const uint32_t i = cur & ~VREN_LBVH_LEAF;
            const LbvhBox gb = leaf_box(a.groups, 5, i);
            if (box_overlaps(box, gb.mn, gb.mx)) {
                float4 s;
                uint32_t li;
                if (a.spheres) {
                    s = __ldg(a.spheres + i);
                    li = WRITE ? __ldg(&a.light_index[i].y) : 0u;
                } else {
                    const NodeF n = load_node(a.bvh, i);
                    li = a.light_index[i].y;
                    const float4 o = a.view_pos[li];
                    s = make_float4(o.x, o.y, o.z, fdiv(fsub(n.mx[0], n.mn[0]), 2.0f));
                }
                if (test_sphere_aabb(s.x, s.y, s.z, s.w, box)) {
                    if (WRITE) {
                        if ((i >> 5) != grp) {
                            flush();
                            grp = i >> 5;
                        }
                        buf[nb++] = li;
                    }
                    ++acc;
                }
            }
        } else {
            const float4* p = reinterpret_cast<const float4*>(a.nodes + cur);
            const float4 lo = __ldg(p), hi = __ldg(p + 1);
            const float mn[3] = {lo.x, lo.y, lo.z}, mx[3] = {hi.x, hi.y, hi.z};
            if (box_overlaps(box, mn, mx)) {
                if (sp == kLbvhStack) {  // deeper than any tree of at most 2^24 leaves
                    VREN_RECORD_ERROR(VREN_ERR_STATE);
                    break;
                }
                stack[sp++] = __float_as_uint(hi.w);
                cur = __float_as_uint(lo.w);
                descend = true;
            }
        }
        if (!descend) {
            if (sp == 0) break;
            cur = stack[--sp];
        }
    }
    if (WRITE) flush();
    return acc;
}

template <bool WRITE>
__global__ void __launch_bounds__(kLbvhThreads) lbvh_assign_kernel(LbvhAssign a)
{
    pdl_enter();
    const uint32_t kc = *a.key_count;
    const uint32_t U = kc < a.key_cap ? kc : a.key_cap;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < U; c += gridDim.x * blockDim.x) {
        const Box box = cluster_box(a.keys[c], a.frame);
        if (WRITE) lbvh_cluster<true>(a, box, a.offsets[c]);
        else a.counts[c] = lbvh_cluster<false>(a, box, 0u);
    }
}

__global__ void lbvh_zero_counts_kernel(const uint32_t* __restrict__ key_count, uint32_t key_cap,
                                        uint32_t* __restrict__ counts, uint32_t* __restrict__ offsets,
                                        uint32_t* __restrict__ total)
{
    const uint32_t kc = *key_count;
    const uint32_t U = kc < key_cap ? kc : key_cap;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < U; c += gridDim.x * blockDim.x) {
        counts[c] = 0u;
        offsets[c] = 0u;
    }
    if (total && blockIdx.x == 0 && threadIdx.x == 0) *total = 0u;
}

int lbvh_assign(cudaStream_t st, const uint32_t* keys, const uint32_t* key_count, uint32_t key_cap,
                const vren_cs_frame* frame, const vren_lbvh_node* nodes, const vren_bvh_node* bvh, uint32_t L,
                const uint32_t* light_index, const float* view_pos, const float* spheres, uint32_t* counts,
                uint32_t* offsets, uint32_t* indices, uint32_t index_cap, uint32_t* total, void* scratch)
{
    if (L == 0) {
        launch_kernel(lbvh_zero_counts_kernel, 256, 256, 0, st, key_count, key_cap, counts, offsets, total);
        VREN_LAUNCH_CHECK();
        return VREN_OK;
    }
    uint64_t P = 32;
    while (P < L) P <<= 5;
    LbvhAssign a{keys, key_count, key_cap, frame, nodes, bvh, L > 32 ? bvh + P : nullptr, L,
                 reinterpret_cast<const uint2*>(light_index), reinterpret_cast<const float4*>(view_pos),
                 reinterpret_cast<const float4*>(spheres), counts, offsets, indices, index_cap};
    const uint32_t grid = kNumSMsHint * 8;
    launch_kernel(lbvh_assign_kernel<false>, grid, kLbvhThreads, 0, st, a);
    VREN_LAUNCH_CHECK();
    int rc = scan_exclusive_u32(st, counts, offsets, key_cap, key_count, total, scratch);
    if (rc != VREN_OK) return rc;
    launch_kernel(lbvh_assign_kernel<true>, grid, kLbvhThreads, 0, st, a);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

}  // namespace vren_gb300

extern "C" int vren_cs_assign_lights_lbvh(vren_stream_t s, const uint32_t* cluster_keys, const uint32_t* key_count,
                                          uint32_t key_capacity, const vren_cs_frame* frame,
                                          const vren_lbvh_node* nodes, const vren_bvh_node* bvh, uint32_t light_count,
                                          const uint32_t* light_index, const float* view_positions,
                                          const float* leaf_spheres, uint32_t* counts, uint32_t* offsets,
                                          uint32_t* indices, uint32_t index_capacity, uint32_t* total, void* scratch)
{
    if (!cluster_keys || !key_count || !frame || !counts || !offsets || !scratch || light_count > (1u << 24))
        return VREN_ERR_ARG;
    if (light_count > 0 && (!bvh || !light_index || (!view_positions && !leaf_spheres) || !indices ||
                            (light_count > 1 && !nodes)))
        return VREN_ERR_ARG;
    return lbvh_assign(as_stream(s), cluster_keys, key_count, key_capacity, frame, nodes, bvh, light_count,
                       light_index, view_positions, leaf_spheres, counts, offsets, indices, index_capacity, total,
                       scratch);
}

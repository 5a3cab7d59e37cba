// Device helpers shared by the BVH builders (bvh.cu, clustered.cu).
#pragma once

#include "common.cuh"

namespace vren_gb300 {

// Order-preserving key of a float (IEEE-754 total order: -0 < +0, NaNs at the ends).
__device__ __forceinline__ uint32_t fkey(float f)
{
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float unkey(uint32_t k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

struct NodeF {
    float mn[3];
    uint32_t next;
    float mx[3];
    uint32_t pad;
};

// Reduce the 32 nodes held by the lanes of a warp into their parent (every lane returns it).
__device__ __forceinline__ NodeF warp_parent(const NodeF& c, bool present, uint32_t first_child_index)
{
    const bool valid = present && c.next != VREN_BVH_INVALID_NODE;
    const uint32_t vmask = __ballot_sync(0xFFFFFFFFu, valid);
    NodeF p;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const uint32_t kmin = __reduce_min_sync(0xFFFFFFFFu, valid ? fkey(c.mn[a]) : 0xFFFFFFFFu);
        const uint32_t kmax = __reduce_max_sync(0xFFFFFFFFu, valid ? fkey(c.mx[a]) : 0u);
        p.mn[a] = vmask ? unkey(kmin) : __int_as_float(0x7F800000);  // +inf
        p.mx[a] = vmask ? unkey(kmax) : __int_as_float(0xFF800000);  // -inf
    }
    p.next = vmask ? first_child_index : VREN_BVH_INVALID_NODE;
    p.pad = 0u;
    return p;
}

__device__ __forceinline__ NodeF load_node(const vren_bvh_node* b, uint32_t i)
{
    const float4* p = reinterpret_cast<const float4*>(b + i);
    float4 lo = p[0], hi = p[1];
    NodeF n;
    n.mn[0] = lo.x; n.mn[1] = lo.y; n.mn[2] = lo.z; n.next = __float_as_uint(lo.w);
    n.mx[0] = hi.x; n.mx[1] = hi.y; n.mx[2] = hi.z; n.pad = __float_as_uint(hi.w);
    return n;
}

__device__ __forceinline__ void store_node(vren_bvh_node* b, uint32_t i, const NodeF& n)
{
    float4* p = reinterpret_cast<float4*>(b + i);
    p[0] = make_float4(n.mn[0], n.mn[1], n.mn[2], __uint_as_float(n.next));
    p[1] = make_float4(n.mx[0], n.mx[1], n.mx[2], __uint_as_float(n.pad));
}

// One CTA of up to 1024 threads turns nodes [src_off + 1024 block, + 1024) of a level of `count`
// nodes into their parents at dst1_off and, when two_levels, the CTA's 32 parents into their parent
// at dst2_off + block.
__device__ __forceinline__ void bvh_levels_block(vren_bvh_node* __restrict__ bvh, uint32_t block, uint32_t src_off,
                                                 uint32_t count, uint32_t dst1_off, uint32_t dst2_off, bool two_levels,
                                                 NodeF* s_parent)
{
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t local = block * 1024u + tid;
    const bool present = local < count;
    NodeF c{};
    if (present) c = load_node(bvh, src_off + local);
    const uint32_t parent_local = local >> 5;
    NodeF p = warp_parent(c, present, src_off + (parent_local << 5));
    if (lane == 0 && present) {
        store_node(bvh, dst1_off + parent_local, p);
        if (two_levels) s_parent[warp] = p;
    }
    if (!two_levels) return;
    __syncthreads();
    if (warp == 0) {
        const uint32_t gp_local = block;
        const uint32_t parents_here = (count >> 5) - block * 32u < 32u ? (count >> 5) - block * 32u : 32u;
        const bool pres = lane < parents_here;
        NodeF q = pres ? s_parent[lane] : NodeF{};
        NodeF g = warp_parent(q, pres, dst1_off + (gp_local << 5));
        if (lane == 0) store_node(bvh, dst2_off + gp_local, g);
    }
}

}  // namespace vren_gb300

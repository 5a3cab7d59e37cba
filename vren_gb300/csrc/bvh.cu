// BuildBVH — vren::build_bvh (vren/vren/primitives/build_bvh.cpp:38-99, build_bvh.comp:32-55).
//
// The reference dispatches once per level; a 32-lane subgroup turns 32 children into one parent
// with subgroupMin/Max over the valid lanes.  Here one launch builds two levels: a 1024-thread CTA
// reads 1024 consecutive nodes, each warp reduces its 32 children into a parent (warp-wide
// redux.sync on order-preserving integer keys), and warp 0 reduces the CTA's 32 parents into the
// grandparent.  A 32^3-leaf light BVH therefore takes two launches instead of three dispatches and
// two barriers.
//
// Parents: next = index of the first child when at least one child is valid, else
// VREN_BVH_INVALID_NODE; the AABB is the min/max over the valid children (+inf/-inf when none);
// pad = 0.  min/max use IEEE-754 total order (-0 < +0), which makes them independent of the
// reduction order; the oracle states the same rule.
#include "common.cuh"
#include "internal.h"
#include "bvh_common.cuh"

namespace vren_gb300 {

VREN_DEFINE_ERROR_WORD(bvh)

// Level `src` (count nodes starting at src_off) -> parents at dst1_off (count/32 nodes) and, when
// two_levels, grandparents at dst2_off (count/1024 nodes).
__global__ void __launch_bounds__(1024) build_bvh_kernel(vren_bvh_node* __restrict__ bvh, uint32_t src_off,
                                                         uint32_t count, uint32_t dst1_off, uint32_t dst2_off,
                                                         int two_levels)
{
    pdl_enter();
    __shared__ NodeF s_parent[32];
    bvh_levels_block(bvh, blockIdx.x, src_off, count, dst1_off, dst2_off, two_levels != 0, s_parent);
}

}  // namespace vren_gb300

using namespace vren_gb300;

extern "C" uint32_t vren_calc_bvh_padded_leaf_count(uint32_t leaf_count)
{
    if (leaf_count <= 1) return 32u;
    uint64_t p = 32;
    while (p < leaf_count) p <<= 5;
    return p > 0xFFFFFFFFull ? 0u : (uint32_t)p;
}

extern "C" uint32_t vren_calc_bvh_buffer_length(uint32_t leaf_count)
{
    uint64_t p = vren_calc_bvh_padded_leaf_count(leaf_count);
    uint64_t len = 0;
    while (p != 0) {
        len += p;
        p >>= 5;
    }
    return len > 0xFFFFFFFFull ? 0u : (uint32_t)len;
}

extern "C" size_t vren_calc_bvh_buffer_size(uint32_t leaf_count)
{
    return (size_t)vren_calc_bvh_buffer_length(vren_calc_bvh_padded_leaf_count(leaf_count)) * sizeof(vren_bvh_node);
}

extern "C" uint32_t vren_calc_bvh_root_index(uint32_t leaf_count)
{
    uint32_t len = vren_calc_bvh_buffer_length(vren_calc_bvh_padded_leaf_count(leaf_count));
    return len ? len - 1 : 0u;
}

extern "C" uint32_t vren_calc_bvh_level_count(uint32_t leaf_count)
{
    uint32_t p = vren_calc_bvh_padded_leaf_count(leaf_count);
    uint32_t l = 0;
    while ((1ull << (l + 1)) <= p) ++l;  // integer log2
    return l / 5;
}

extern "C" int vren_build_bvh(vren_stream_t s, vren_bvh_node* bvh, uint32_t padded_leaf_count)
{
    // vren/primitives/build_bvh.cpp:45: leaf_count >= 32 and a power of 32.
    if (!bvh || padded_leaf_count < 32 || vren_calc_bvh_padded_leaf_count(padded_leaf_count) != padded_leaf_count)
        return VREN_ERR_ARG;
    if ((uintptr_t)bvh & 15u) return VREN_ERR_ARG;
    return build_bvh_levels(as_stream(s), bvh, 0, padded_leaf_count);
}

namespace vren_gb300 {
int build_bvh_levels(cudaStream_t st, vren_bvh_node* bvh, uint32_t src, uint32_t count)
{
    while (count > 1) {
        const uint32_t dst1 = src + count;
        if (count >= 1024) {
            const uint32_t dst2 = dst1 + count / 32;
            launch_kernel(build_bvh_kernel, count / 1024, 1024, 0, st, bvh, src, count, dst1, dst2, 1);
            VREN_LAUNCH_CHECK();
            src = dst1 + count / 32;
            count /= 1024;
        } else {
            launch_kernel(build_bvh_kernel, 1, count, 0, st, bvh, src, count, dst1, 0, 0);
            VREN_LAUNCH_CHECK();
            src = dst1;
            count /= 32;
        }
    }
    return VREN_OK;
}
}  // namespace vren_gb300

// k-d tree (vren/vren/base/kd_tree.{hpp,cpp}): a host build that gives the reference's node array
// bit for bit, the reference's single nearest-neighbour search on the host, and a batched search on
// the GPU (one thread per sample) that visits the nodes in the reference's order and so returns its
// results, ties included.
//
// Node (kd_tree.hpp:13-19): the reference's struct is 12 bytes, since its 2-bit axis field and the
// anonymous union of 30-bit fields after it cannot share a storage unit: word 0 = split (float) or
// point index; word 1 = axis (3 = leaf); word 2 = the distance to the right child (inner node) or the
// leaf count (first leaf of a run; the other leaves of the run hold 0x3FFFFFFF, ~0 cut to 30 bits).
//
// Build (vren/base/kd_tree.cpp:5-78): a run of at most max_leaf points becomes leaves; otherwise the Welford mean
// and (unnormalised) variance of the points in their current order, axis = (var0 > var1 ? 0 : var1 > var2
// ? 1 : 2) (the reference compares var0 with var1 twice), split = mean[axis], an in-place swap
// partition of the indices by point[axis] < split, the left subtree at offset + 1, the right one
// after it.  Nodes are laid out in pre-order, so the build here runs the same recursion with an
// explicit stack of pending right subtrees.  Where a split separates nothing (all points on one side:
// duplicates, NaN), the reference asserts (and recurses without end when asserts are off); here that
// node becomes one leaf run holding all its points.
#include "common.cuh"

#include <vector>

namespace vren_gb300 {

VREN_DEFINE_ERROR_WORD(kd_tree)

namespace {

constexpr uint32_t kKdLeafAxis = 3u;
constexpr uint32_t kKdCountMask = 0x3FFFFFFFu;
constexpr uint32_t kKdMaxStack = 128;  // pending far children on one root-to-leaf path

inline void kd_write_leaves(vren_kd_tree_node* tree, size_t offset, const uint32_t* indices, size_t count)
{
    for (size_t i = 0; i < count; ++i) {
        tree[offset + i].index = indices[i];
        tree[offset + i].axis = kKdLeafAxis;
        tree[offset + i].value = i == 0 ? (uint32_t)count & kKdCountMask : kKdCountMask;
    }
}

// Welford mean / variance over the run (vren/base/kd_tree.cpp:34-47), the axis choice (:52) and the partition
// (:53-66).  Returns the split point `middle`.
size_t kd_split(const float* points, size_t stride, uint32_t* indices, size_t count, uint32_t& axis, float& split)
{
    float mean[3] = {0.0f, 0.0f, 0.0f}, var[3] = {0.0f, 0.0f, 0.0f};
    float n = 1.0f;
    for (size_t i = 0; i < count; ++i, n += 1.0f) {
        const float* p = points + (size_t)indices[i] * stride;
        for (int j = 0; j < 3; ++j) {
            const float d = p[j] - mean[j];
            mean[j] += d / n;
            var[j] += (p[j] - mean[j]) * d;
        }
    }
    axis = (var[0] > var[1] && var[0] > var[1]) ? 0u : (var[1] > var[2] ? 1u : 2u);
    split = mean[axis];
    size_t middle = 0;
    for (size_t i = 0; i < count; ++i) {
        const float* p = points + (size_t)indices[i] * stride;
        if (p[axis] < split) {
            const uint32_t t = indices[i];
            indices[i] = indices[middle];
            indices[middle] = t;
            ++middle;
        }
    }
    return middle;
}

struct KdPending {
    size_t first, count;  // index range of the right subtree
    size_t parent;        // node whose right-child distance is set when the subtree starts
};

// vren/base/kd_tree.cpp:88-129 on the host: near child first, the far one when best > d * d.
void kd_search_host(const float* points, size_t stride, const vren_kd_tree_node* tree, size_t offset,
                    const float* s, vren_kd_tree_filter filter, void* user, uint32_t& best_point, float& best)
{
    const vren_kd_tree_node& node = tree[offset];
    const uint32_t axis = node.axis & 3u, value = node.value & kKdCountMask;
    if (axis == kKdLeafAxis) {
        for (uint32_t i = 0; i < value; ++i) {
            const uint32_t idx = tree[offset + i].index;
            if (filter && !filter(idx, user)) continue;
            const float* p = points + (size_t)idx * stride;
            const float dist = (s[0] - p[0]) * (s[0] - p[0]) + (s[1] - p[1]) * (s[1] - p[1]) + (s[2] - p[2]) * (s[2] - p[2]);
            if (dist < best) {
                best_point = idx;
                best = dist;
            }
        }
        return;
    }
    const float d = s[axis] - node.split;
    const size_t first = d <= 0.0f ? offset + 1 : offset + value;
    const size_t second = d <= 0.0f ? offset + value : offset + 1;
    kd_search_host(points, stride, tree, first, s, filter, user, best_point, best);
    if (best > d * d) kd_search_host(points, stride, tree, second, s, filter, user, best_point, best);
}

// ---- GPU batched search -------------------------------------------------------------------------
// One thread per sample; the reference's recursion with an explicit stack of (far child, d * d).  Node
// offsets and point indices are checked against the buffers, and a path deeper than the stack ends the
// sample's search with an error recorded (the caller sizes max_depth with vren_kd_tree_depth).
__global__ void __launch_bounds__(128) kd_search_kernel(const float* __restrict__ points, uint32_t stride,
                                                        uint32_t point_count, const uint32_t* __restrict__ tree,
                                                        uint32_t node_count, const float* __restrict__ samples,
                                                        uint32_t sample_stride, uint32_t sample_count,
                                                        const uint8_t* __restrict__ excluded,
                                                        uint32_t* __restrict__ best_points,
                                                        float* __restrict__ best_dist)
{
    uint32_t st_node[kKdMaxStack];
    float st_dd[kKdMaxStack];
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < sample_count; q += gridDim.x * blockDim.x) {
        const float s0 = samples[(size_t)q * sample_stride + 0], s1 = samples[(size_t)q * sample_stride + 1],
                    s2 = samples[(size_t)q * sample_stride + 2];
        float best = __int_as_float(0x7f800000);
        uint32_t best_point = 0xFFFFFFFFu;
        uint32_t sp = 0, cur = 0;
        bool ok = node_count > 0;
        while (ok) {
            // descend to a leaf run, deferring far children
            uint32_t w0 = __ldg(tree + 3 * (size_t)cur), axis = __ldg(tree + 3 * (size_t)cur + 1) & 3u;
            uint32_t value = __ldg(tree + 3 * (size_t)cur + 2) & kKdCountMask;
            while (axis != kKdLeafAxis) {
                const uint32_t dist = value;
                const float sa = axis == 0 ? s0 : (axis == 1 ? s1 : s2);
                const float d = fsub(sa, __uint_as_float(w0));
                const uint32_t near = d <= 0.0f ? cur + 1 : cur + dist;
                const uint32_t far = d <= 0.0f ? cur + dist : cur + 1;
                if (sp == kKdMaxStack || near >= node_count || far >= node_count) {
                    VREN_RECORD_ERROR(sp == kKdMaxStack ? VREN_ERR_CAPACITY : VREN_ERR_ARG);
                    ok = false;
                    break;
                }
                st_node[sp] = far;
                st_dd[sp] = fmul(d, d);
                ++sp;
                cur = near;
                w0 = __ldg(tree + 3 * (size_t)cur);
                axis = __ldg(tree + 3 * (size_t)cur + 1) & 3u;
                value = __ldg(tree + 3 * (size_t)cur + 2) & kKdCountMask;
            }
            if (!ok) break;
            const uint32_t run = value;
            if (cur + run > node_count) {
                VREN_RECORD_ERROR(VREN_ERR_ARG);
                break;
            }
            for (uint32_t i = 0; i < run; ++i) {
                const uint32_t idx = i == 0 ? w0 : __ldg(tree + 3 * ((size_t)cur + i));
                if (idx >= point_count) {
                    VREN_RECORD_ERROR(VREN_ERR_ARG);
                    continue;
                }
                if (excluded && excluded[idx]) continue;
                const float* p = points + (size_t)idx * stride;
                const float dx = fsub(s0, __ldg(p)), dy = fsub(s1, __ldg(p + 1)), dz = fsub(s2, __ldg(p + 2));
                const float dd = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
                if (dd < best) {
                    best = dd;
                    best_point = idx;
                }
            }
            // resume at the deepest deferred far child that can still hold a closer point
            bool resumed = false;
            while (sp > 0) {
                --sp;
                if (best > st_dd[sp]) {
                    cur = st_node[sp];
                    resumed = true;
                    break;
                }
            }
            if (!resumed) break;
        }
        best_points[q] = best_point;
        best_dist[q] = best;
    }
}

}  // namespace
}  // namespace vren_gb300

using namespace vren_gb300;

extern "C" size_t vren_kd_tree_build(const float* points, size_t point_stride, uint32_t* indices, size_t count,
                                     vren_kd_tree_node* kd_tree, size_t node_offset, size_t max_leaf_point_count)
{
    if (!points || !indices || !kd_tree || count == 0 || max_leaf_point_count == 0) return node_offset;
    std::vector<KdPending> pending;
    size_t first = 0, n = count, offset = node_offset;
    for (;;) {
        bool leaf = n <= max_leaf_point_count;
        uint32_t axis = 0;
        float split = 0.0f;
        size_t middle = 0;
        if (!leaf) {
            middle = kd_split(points, point_stride, indices + first, n, axis, split);
            leaf = middle == 0 || middle == n;
        }
        if (leaf) {
            kd_write_leaves(kd_tree, offset, indices + first, n);
            offset += n;
            if (pending.empty()) return offset;
            const KdPending r = pending.back();
            pending.pop_back();
            kd_tree[r.parent].value = (uint32_t)(offset - r.parent) & kKdCountMask;
            first = r.first;
            n = r.count;
            continue;
        }
        kd_tree[offset].split = split;
        kd_tree[offset].axis = axis;
        kd_tree[offset].value = 0;
        pending.push_back({first + middle, n - middle, offset});
        n = middle;
        ++offset;
    }
}

extern "C" uint32_t vren_kd_tree_depth(const vren_kd_tree_node* kd_tree, size_t node_offset)
{
    // inner nodes on the longest root-to-leaf path (the search's stack bound)
    if (!kd_tree) return 0;
    std::vector<std::pair<size_t, uint32_t>> stack = {{node_offset, 0u}};
    uint32_t depth = 0;
    while (!stack.empty()) {
        const auto [o, dpt] = stack.back();
        stack.pop_back();
        const uint32_t axis = kd_tree[o].axis & 3u, value = kd_tree[o].value & kKdCountMask;
        if (axis == kKdLeafAxis) {
            depth = dpt > depth ? dpt : depth;
            continue;
        }
        stack.push_back({o + 1, dpt + 1});
        stack.push_back({o + value, dpt + 1});
    }
    return depth;
}

extern "C" void vren_kd_tree_search(const float* points, size_t point_stride, const uint32_t* indices, size_t count,
                                    const vren_kd_tree_node* kd_tree, size_t node_offset, const float* sample,
                                    vren_kd_tree_filter filter, void* filter_user, uint32_t* best_point,
                                    float* best_distance_squared)
{
    (void)indices;
    if (!points || !kd_tree || !sample || !best_point || !best_distance_squared || count == 0) return;
    kd_search_host(points, point_stride, kd_tree, node_offset, sample, filter, filter_user, *best_point,
                   *best_distance_squared);
}

extern "C" int vren_kd_tree_search_batch(vren_stream_t s, const float* points, uint32_t point_stride,
                                         uint32_t point_count, const vren_kd_tree_node* kd_tree, uint32_t node_count,
                                         uint32_t max_depth, const float* samples, uint32_t sample_stride,
                                         uint32_t sample_count, const uint8_t* excluded, uint32_t* best_points,
                                         float* best_distances_squared)
{
    if (sample_count == 0) return VREN_OK;
    if (!points || !kd_tree || !samples || !best_points || !best_distances_squared) return VREN_ERR_ARG;
    if (point_stride < 3 || sample_stride < 3 || node_count == 0 || point_count == 0) return VREN_ERR_ARG;
    if (((uintptr_t)kd_tree) & 3u) return VREN_ERR_ARG;
    if (max_depth > kKdMaxStack) return VREN_ERR_CAPACITY;
    const uint32_t grid = min((sample_count + 127) / 128, (uint32_t)kNumSMsHint * 16);
    launch_kernel(kd_search_kernel, grid, 128, 0, as_stream(s), points, point_stride, point_count,
                  reinterpret_cast<const uint32_t*>(kd_tree), node_count, samples, sample_stride, sample_count, excluded,
                  best_points, best_distances_squared);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

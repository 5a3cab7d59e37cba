// Exercises the C++ mirror of vren's call surface (include/vren_gb300.hpp) the way the reference's
// tests call vren::radix_sort, vren::blelloch_scan, vren::reduce and vren::build_bvh
// (vren_test/vren_test/primitives/*.cpp).  Prints "api ok" and exits 0 on success.
#include "vren_gb300.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <numeric>
#include <vector>

#define EXPECT(cond)                                                        \
    do {                                                                    \
        if (!(cond)) {                                                      \
            std::fprintf(stderr, "check failed: %s (line %d)\n", #cond, __LINE__); \
            return 1;                                                       \
        }                                                                   \
    } while (0)

template <typename T>
static void upload(vren::device_buffer const& b, std::vector<T> const& v)
{
    cudaMemcpy(b.m_ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}

template <typename T>
static std::vector<T> download(vren::device_buffer const& b, size_t n)
{
    std::vector<T> v(n);
    cudaMemcpy(v.data(), b.m_ptr, n * sizeof(T), cudaMemcpyDeviceToHost);
    return v;
}

int main()
{
    vren::resource_container rc;
    cudaStream_t stream;
    cudaStreamCreate(&stream);

    // vren_test/primitives/radix_sort.cpp:68-132: reversed iota, 1024 keys
    {
        vren::radix_sort rs;
        const uint32_t n = 1024;
        std::vector<uint32_t> keys(n);
        std::iota(keys.begin(), keys.end(), 0u);
        std::reverse(keys.begin(), keys.end());
        vren::owned_buffer buf(n * 4);
        upload(buf, keys);
        auto s1 = rs.create_scratch_buffer_1(n);
        auto s2 = rs.create_scratch_buffer_2(n);
        rs(stream, rc, buf, n, s1, s2);
        cudaStreamSynchronize(stream);
        auto out = download<uint32_t>(buf, n);
        for (uint32_t i = 0; i < n; ++i) EXPECT(out[i] == i);
        bool threw = false;
        try {
            rs(stream, rc, buf, 1000, s1, s2);
        } catch (std::invalid_argument const&) {
            threw = true;
        }
        EXPECT(threw);
    }
    // vren_test/primitives/blelloch_scan.cpp:166-176: all ones
    {
        vren::blelloch_scan scan;
        const uint32_t n = 1 << 19;
        vren::owned_buffer buf(n * 4);
        upload(buf, std::vector<uint32_t>(n, 1u));
        scan(stream, rc, buf, n, 0, 1);
        cudaStreamSynchronize(stream);
        auto out = download<uint32_t>(buf, n);
        for (uint32_t i = 0; i < n; ++i) EXPECT(out[i] == i);
    }
    // vren_test/primitives/reduce.cpp:284-291: all-ones add, whole tree in place
    {
        vren::reduce<vren::uint_tag, vren::ReduceOperationAdd> red;
        const uint32_t n = 10000, P = vren::calc_reduce_output_buffer_length(n);
        std::vector<uint32_t> v(P, 0u);
        std::fill(v.begin(), v.begin() + n, 1u);
        vren::owned_buffer buf(P * 4);
        upload(buf, v);
        red(stream, rc, buf, n, 0, 1);
        cudaStreamSynchronize(stream);
        auto out = download<uint32_t>(buf, P);
        EXPECT(out[P - 1] == n);
        EXPECT(out[1] == 2 && out[3] == 4 && out[1023] == 1024);
    }
    // vren_test/primitives/build_bvh.cpp:223-254 helpers and a build of 1000 leaves
    {
        EXPECT(vren::calc_bvh_padded_leaf_count(2193819) == 33554432u);
        EXPECT(vren::calc_bvh_root_index(129) == 32u * 32u + 32u);
        const uint32_t leaves = 1000, P = vren::calc_bvh_padded_leaf_count(leaves);
        std::vector<vren::bvh_node> nodes(vren::calc_bvh_buffer_length(P));
        for (uint32_t i = 0; i < P; ++i) {
            auto& nd = nodes[i];
            for (int a = 0; a < 3; ++a) {
                nd.min[a] = (float)i;
                nd.max[a] = (float)i + 1.0f;
            }
            nd.next = i < leaves ? VREN_BVH_LEAF_NODE : VREN_BVH_INVALID_NODE;
        }
        vren::owned_buffer buf(nodes.size() * sizeof(vren::bvh_node));
        upload(buf, nodes);
        vren::build_bvh()(stream, rc, buf, P);
        cudaStreamSynchronize(stream);
        auto out = download<vren::bvh_node>(buf, nodes.size());
        const auto& root = out[vren::calc_bvh_root_index(P)];
        // P = 1024: leaves [0, 1024), 32 parents at [1024, 1056), root 1056 whose first child is 1024
        EXPECT(root.min[0] == 0.0f && root.max[0] == (float)leaves && root.next == P);
    }
    // point_light_bouncer.cpp:17-57: one light moving freely, one reflecting off the +x face
    {
        std::vector<float> pos = {0.0f, 0.0f, 0.0f, 1.0f, 0.75f, 0.0f, 0.0f, 1.0f};
        std::vector<float> dir = {1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f};
        vren::owned_buffer pb(pos.size() * sizeof(float)), db(dir.size() * sizeof(float));
        upload(pb, pos);
        upload(db, dir);
        const float lo[3] = {-1.0f, -1.0f, -1.0f}, hi[3] = {1.0f, 1.0f, 1.0f};
        vren_demo::point_light_bouncer().bounce(0, stream, rc, pb, db, 2, lo, hi, 1.0f, 0.5f);
        cudaStreamSynchronize(stream);
        auto p = download<float>(pb, 8);
        auto d = download<float>(db, 8);
        EXPECT(p[0] == 0.5f && p[1] == 0.0f && d[0] == 1.0f);
        EXPECT(p[4] > 0.7499f && p[4] < 0.7501f && d[4] == -1.0f);
    }
    // depth_buffer_pyramid.cpp:213-305: a 5x3 depth buffer -> levels 5x3, 2x1, 1x1
    {
        std::vector<float> depth = {0.1f, 0.9f, 0.2f, 0.3f, 0.95f,  //
                                    0.4f, -1.f, 0.5f, 0.8f, 0.99f,  //
                                    0.7f, 0.6f, 0.2f, 0.1f, 0.98f};
        vren::owned_buffer db(depth.size() * sizeof(float));
        upload(db, depth);
        vren::depth_buffer_pyramid pyramid(5, 3);
        EXPECT(pyramid.get_level_count() == 3 && pyramid.get_image_width(1) == 2 && pyramid.get_image_height(1) == 1);
        vren::depth_buffer_reductor().copy_and_reduce(stream, rc, db, pyramid);
        cudaStreamSynchronize(stream);
        std::vector<float> l1(2), l2(1);
        cudaMemcpy(l1.data(), pyramid.level(1), 2 * sizeof(float), cudaMemcpyDeviceToHost);
        cudaMemcpy(l2.data(), pyramid.level(2), sizeof(float), cudaMemcpyDeviceToHost);
        // the last column and row of the odd level are never read
        EXPECT(l1[0] == 0.9f && l1[1] == 0.8f && l2[0] == 0.9f);
    }
    // vren_test/kd_tree.cpp:29-112 in small: k-d search equals the linear search, with a filter too
    {
        std::vector<float> points(3 * 5000);
        uint32_t r = 12345u;
        for (auto& p : points) {
            r = r * 1664525u + 1013904223u;
            p = (float)(r >> 8) / (float)(1u << 24) * 100.0f;
        }
        std::vector<uint32_t> indices(5000);
        std::iota(indices.begin(), indices.end(), 0u);
        std::vector<vren::kd_tree_node> tree(2 * 5000);
        const size_t nodes = vren::kd_tree_build(points.data(), 3, indices.data(), indices.size(), tree.data(), 0, 8);
        EXPECT(nodes > 0 && nodes <= tree.size());
        for (int q = 0; q < 20; ++q) {
            const float s[3] = {points[3 * q] + 0.5f, points[3 * q + 1] - 0.25f, points[3 * q + 2]};
            for (int filtered = 0; filtered < 2; ++filtered) {
                auto keep = [&](uint32_t p) { return filtered == 0 || p % 3 != 0; };
                uint32_t best = UINT32_MAX, lin = UINT32_MAX;
                float bd = INFINITY, ld = INFINITY;
                vren::kd_tree_search(points.data(), 3, indices.data(), indices.size(), tree.data(), 0, s,
                                     filtered ? vren::kd_tree_search_filter_t(keep) : vren::k_kd_tree_default_search_filter,
                                     best, bd);
                for (uint32_t i = 0; i < 5000; ++i) {
                    if (!keep(i)) continue;
                    const float* p = &points[3 * i];
                    const float d = (s[0] - p[0]) * (s[0] - p[0]) + (s[1] - p[1]) * (s[1] - p[1]) + (s[2] - p[2]) * (s[2] - p[2]);
                    if (d < ld) {
                        ld = d;
                        lin = i;
                    }
                }
                EXPECT(best == lin && bd == ld);
            }
        }
    }
    EXPECT(vren_device_error(1) == 0);
    cudaStreamDestroy(stream);
    std::printf("api ok\n");
    return 0;
}

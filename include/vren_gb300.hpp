// vren_gb300.hpp — C++20 mirror of loryruta/vren's primitive and clustered-shading call surface,
// over the C ABI of vren_gb300.h.
//
// The reference's functors take (VkCommandBuffer, vren::resource_container&, vk_utils::buffer const&,
// lengths, byte offsets, ...).  Here the command buffer becomes a cudaStream_t, the Vulkan buffer a
// vren::device_buffer (device pointer + size), and resource_container is kept as an empty type so
// call sites keep their shape (nothing needs to be kept alive until a fence: the GPU work holds no
// descriptor sets).  Errors follow the reference: precondition failures throw
// std::invalid_argument (vren/primitives/radix_sort.cpp:158-161), other failures std::runtime_error (VREN_CHECK,
// vk_helpers/misc.cpp:22-37).
//
// Header-only; link against libvren_gb300.so and the CUDA runtime.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "vren_gb300.h"

namespace vren {

struct device_buffer {
    void* m_ptr = nullptr;
    size_t m_size = 0;

    template <typename T = void>
    T* at(size_t byte_offset = 0) const
    {
        return reinterpret_cast<T*>(static_cast<char*>(m_ptr) + byte_offset);
    }
};

struct resource_container {};

inline void check(int status, const char* what)
{
    if (status == VREN_OK) return;
    if (status == VREN_ERR_ARG) throw std::invalid_argument(std::string(what) + ": invalid argument");
    throw std::runtime_error(std::string(what) + ": " + vren_status_string(status));
}

// Owned device allocation (the reference's vk_utils::alloc_device_only_buffer).
class owned_buffer : public device_buffer {
public:
    owned_buffer() = default;
    explicit owned_buffer(size_t size, bool zero = true)
    {
        if (size && cudaMalloc(&m_ptr, size) != cudaSuccess) throw std::runtime_error("cudaMalloc failed");
        m_size = size;
        if (size && zero && cudaMemset(m_ptr, 0, size) != cudaSuccess) throw std::runtime_error("cudaMemset failed");
    }
    owned_buffer(owned_buffer&& o) noexcept { *this = static_cast<owned_buffer&&>(o); }
    owned_buffer& operator=(owned_buffer&& o) noexcept
    {
        if (this != &o) {
            release();
            m_ptr = o.m_ptr;
            m_size = o.m_size;
            o.m_ptr = nullptr;
            o.m_size = 0;
        }
        return *this;
    }
    owned_buffer(const owned_buffer&) = delete;
    owned_buffer& operator=(const owned_buffer&) = delete;
    ~owned_buffer() { release(); }

    void grow(size_t size)
    {
        if (size > m_size) *this = owned_buffer(size);
    }

private:
    void release()
    {
        if (m_ptr) cudaFree(m_ptr);
        m_ptr = nullptr;
        m_size = 0;
    }
};

inline uint32_t round_to_next_power_of_2(uint32_t v) { return vren_round_to_next_power_of_2(v); }
inline uint32_t round_to_next_power_of(uint32_t n, uint32_t base) { return vren_round_to_next_power_of(n, base); }
inline uint32_t divide_and_ceil(uint32_t v, uint32_t d) { return vren_divide_and_ceil(v, d); }

// ------------------------------------------------------------------------------------------------
// vren::reduce<T, Op> (vren/vren/primitives/reduce.hpp:8-49)
// ------------------------------------------------------------------------------------------------
enum reduce_operation { ReduceOperationAdd = VREN_REDUCE_ADD, ReduceOperationMin = VREN_REDUCE_MIN, ReduceOperationMax = VREN_REDUCE_MAX };

struct vec4_tag {};  // stands for glm::vec4
struct uint_tag {};  // stands for glm::uint

template <typename T, reduce_operation Op>
class reduce {
public:
    inline static const uint32_t k_workgroup_size = 1024;

    void operator()(cudaStream_t stream, resource_container&, device_buffer const& input_buffer,
                    uint32_t input_buffer_length, size_t input_buffer_offset, device_buffer const& output_buffer,
                    size_t output_buffer_offset, uint32_t blocks_num)
    {
        if constexpr (std::is_same_v<T, uint_tag>)
            check(vren_reduce_tree_u32(stream, Op, input_buffer.at<uint32_t>(input_buffer_offset), input_buffer_length,
                                       output_buffer.at<uint32_t>(output_buffer_offset), blocks_num),
                  "reduce");
        else
            check(vren_reduce_tree_vec4(stream, Op, input_buffer.at<float>(input_buffer_offset), input_buffer_length,
                                        output_buffer.at<float>(output_buffer_offset), blocks_num),
                  "reduce");
    }

    void operator()(cudaStream_t stream, resource_container& rc, device_buffer const& buffer, uint32_t length,
                    size_t offset, uint32_t blocks_num)
    {
        (*this)(stream, rc, buffer, length, offset, buffer, offset, blocks_num);
    }
};

inline uint32_t calc_reduce_output_buffer_length(uint32_t count) { return vren_calc_reduce_output_buffer_length(count); }

// ------------------------------------------------------------------------------------------------
// vren::blelloch_scan (vren/vren/primitives/blelloch_scan.hpp:9-49).  Owns the look-back scratch,
// grown on first use for a length (allocate with reserve() before capturing into a graph).
// ------------------------------------------------------------------------------------------------
class blelloch_scan {
public:
    inline static const uint32_t k_workgroup_size = 1024;

    void reserve(uint32_t length, uint32_t blocks_num = 1)
    {
        m_scratch.grow(vren_exclusive_scan_scratch_bytes(length, blocks_num));
    }

    void downsweep(cudaStream_t stream, resource_container&, device_buffer const& buffer, uint32_t length,
                   uint32_t offset, uint32_t blocks_num, bool clear_last)
    {
        check(vren_scan_downsweep_u32(stream, buffer.at<uint32_t>(offset), length, blocks_num, clear_last ? 1 : 0),
              "blelloch_scan::downsweep");
    }

    void operator()(cudaStream_t stream, resource_container&, device_buffer const& buffer, uint32_t length,
                    uint32_t offset, uint32_t blocks_num)
    {
        reserve(length, blocks_num);
        check(vren_exclusive_scan_u32(stream, buffer.at<uint32_t>(offset), length, blocks_num, m_scratch.m_ptr),
              "blelloch_scan");
    }

private:
    owned_buffer m_scratch;
};

// ------------------------------------------------------------------------------------------------
// vren::radix_sort (vren/vren/primitives/radix_sort.hpp:9-53)
// ------------------------------------------------------------------------------------------------
class radix_sort {
public:
    inline static const uint32_t k_workgroup_size = 1024;
    inline static constexpr uint32_t k_radix_bits = 8;

    owned_buffer create_scratch_buffer_1(uint32_t length) const
    {
        return owned_buffer(vren_radix_sort_scratch1_bytes(length, k_radix_bits));
    }
    owned_buffer create_scratch_buffer_2(uint32_t length) const { return owned_buffer((size_t)length * 4, false); }

    void operator()(cudaStream_t stream, resource_container&, device_buffer const& buffer, uint32_t length,
                    device_buffer const& scratch_buffer_1, device_buffer const& scratch_buffer_2)
    {
        if (!(length >= k_workgroup_size && (length & (length - 1)) == 0))
            throw std::invalid_argument("Length must be higher than 1024 and a power of 2");
        check(vren_radix_sort_u32(stream, buffer.at<uint32_t>(), length, scratch_buffer_1.m_ptr,
                                  scratch_buffer_2.at<uint32_t>()),
              "radix_sort");
    }

    // Key/value overload (any length): values follow their keys, ties keep their order.
    void operator()(cudaStream_t stream, resource_container&, device_buffer const& keys, device_buffer const& values,
                    uint32_t length, device_buffer const& scratch_buffer_1, device_buffer const& scratch_keys,
                    device_buffer const& scratch_values)
    {
        check(vren_radix_sort_u32_ex(stream, keys.at<uint32_t>(), values.at<uint32_t>(), length, k_radix_bits,
                                     scratch_buffer_1.m_ptr, scratch_keys.at<uint32_t>(), scratch_values.at<uint32_t>()),
              "radix_sort");
    }
};

// ------------------------------------------------------------------------------------------------
// vren::bucket_sort (vren/vren/primitives/bucket_sort.hpp:9-45)
// ------------------------------------------------------------------------------------------------
class bucket_sort {
public:
    inline static const uint32_t k_key_size = 1 << 16;
    inline static const uint32_t k_key_mask = k_key_size - 1;

    explicit bucket_sort(uint32_t key_bits = 16) : m_key_bits(key_bits) {}

    size_t get_required_output_buffer_size(uint32_t length) const
    {
        return vren_bucket_sort_output_bytes(length, m_key_bits);
    }

    void operator()(cudaStream_t stream, resource_container&, device_buffer const& input_buffer,
                    uint32_t input_buffer_length, size_t input_buffer_offset, device_buffer const& output_buffer,
                    size_t output_buffer_offset)
    {
        m_scratch.grow(vren_bucket_sort_scratch_bytes(input_buffer_length, m_key_bits));
        check(vren_bucket_sort_u32x2(stream, input_buffer.at<uint32_t>(input_buffer_offset), input_buffer_length,
                                     output_buffer.at(output_buffer_offset), m_key_bits, m_scratch.m_ptr),
              "bucket_sort");
    }

private:
    uint32_t m_key_bits;
    owned_buffer m_scratch;
};

// ------------------------------------------------------------------------------------------------
// vren::build_bvh (vren/vren/primitives/build_bvh.hpp:8-57)
// ------------------------------------------------------------------------------------------------
using bvh_node = vren_bvh_node;

inline uint32_t calc_bvh_padded_leaf_count(uint32_t n) { return vren_calc_bvh_padded_leaf_count(n); }
inline uint32_t calc_bvh_buffer_length(uint32_t n) { return vren_calc_bvh_buffer_length(n); }
inline size_t calc_bvh_buffer_size(uint32_t n) { return vren_calc_bvh_buffer_size(n); }
inline uint32_t calc_bvh_root_index(uint32_t n) { return vren_calc_bvh_root_index(n); }
inline uint32_t calc_bvh_level_count(uint32_t n) { return vren_calc_bvh_level_count(n); }

class build_bvh {
public:
    inline static const uint32_t k_workgroup_size = 1024;

    static size_t get_required_buffer_size(uint32_t leaf_count) { return calc_bvh_buffer_size(leaf_count); }

    void operator()(cudaStream_t stream, resource_container&, device_buffer const& buffer, uint32_t leaf_count)
    {
        check(vren_build_bvh(stream, buffer.at<vren_bvh_node>(), leaf_count), "build_bvh");
    }
};

// ------------------------------------------------------------------------------------------------
// vren::clustered_shading (vren/vren/pipeline/clustered_shading.hpp:13-141) — per-stage functors.
// The camera becomes a device frame block (vren_cs_frame) prepared once per frame by frame_params.
// ------------------------------------------------------------------------------------------------
using camera = vren_camera;

class frame_params {
public:
    frame_params() : m_device(sizeof(vren_cs_frame)) {}

    void set(cudaStream_t stream, camera const& cam, uint32_t width, uint32_t height,
             uint32_t slicing = VREN_CS_SLICING_REF, int offscreen = VREN_CS_OFFSCREEN_WRAP)
    {
        vren_cs_view v;
        vren_cs_view_from_camera(&cam, slicing, &v);
        check(vren_cs_frame_build(&v, width, height, offscreen, &m_host), "frame_params");
        check(vren_cs_frame_upload(stream, &m_host, m_device.at<vren_cs_frame>()), "frame_params");
    }
    const vren_cs_frame* device() const { return m_device.at<vren_cs_frame>(); }
    const vren_cs_frame& host() const { return m_host; }

private:
    vren_cs_frame m_host{};
    owned_buffer m_device;
};

namespace clustered_shading {

class construct_point_light_bvh {
public:
    explicit construct_point_light_bvh(uint32_t morton_bits = 15) : m_morton_bits(morton_bits) {}

    static size_t get_required_bvh_buffer_size(uint32_t light_count) { return calc_bvh_buffer_size(light_count); }
    static size_t get_required_point_light_index_buffer_size(uint32_t light_count) { return (size_t)light_count * 8; }

    void operator()(cudaStream_t stream, resource_container&, device_buffer const& light_positions,
                    device_buffer const& point_lights, uint32_t light_count, device_buffer const& view_space_positions,
                    frame_params const& frame, device_buffer const& bvh_buffer,
                    device_buffer const& point_light_index_buffer, device_buffer const* leaf_spheres = nullptr)
    {
        m_scratch.grow(vren_cs_light_bvh_scratch_bytes(light_count, m_morton_bits));
        check(vren_cs_construct_light_bvh(stream, light_positions.at<float>(), point_lights.at<float>(), light_count,
                                          frame.device(), m_morton_bits, view_space_positions.at<float>(),
                                          bvh_buffer.at<vren_bvh_node>(), point_light_index_buffer.at<uint32_t>(),
                                          leaf_spheres ? leaf_spheres->at<float>() : nullptr, m_scratch.m_ptr),
              "construct_point_light_bvh");
    }

private:
    uint32_t m_morton_bits;
    owned_buffer m_scratch;
};

class find_unique_cluster_list {
public:
    void operator()(cudaStream_t stream, resource_container&, uint32_t width, uint32_t height, frame_params const& frame,
                    device_buffer const& depth, device_buffer const& normals, device_buffer const& cluster_key_buffer,
                    device_buffer const& key_count_buffer, device_buffer const& cluster_reference_buffer)
    {
        m_scratch.grow(vren_cs_unique_clusters_scratch_bytes(width, height));
        check(vren_cs_find_unique_clusters(stream, depth.at<float>(), normals.at<float>(), width, height, frame.device(),
                                           cluster_key_buffer.at<uint32_t>(), (uint32_t)(cluster_key_buffer.m_size / 4),
                                           key_count_buffer.at<uint32_t>(), cluster_reference_buffer.at<uint32_t>(),
                                           m_scratch.m_ptr),
              "find_unique_cluster_list");
    }

private:
    owned_buffer m_scratch;
};

class assign_lights {
public:
    void operator()(cudaStream_t stream, resource_container&, frame_params const& frame,
                    device_buffer const& cluster_key_buffer, device_buffer const& key_count_buffer,
                    device_buffer const& light_bvh_buffer, uint32_t light_count, device_buffer const& light_index_buffer,
                    device_buffer const& assigned_light_indices_buffer, device_buffer const& assigned_light_counts_buffer,
                    device_buffer const& assigned_light_offsets_buffer, device_buffer const& view_space_positions,
                    device_buffer const* leaf_spheres = nullptr, device_buffer const* total = nullptr)
    {
        const uint32_t cap = (uint32_t)(cluster_key_buffer.m_size / 4);
        m_scratch.grow(vren_cs_assign_lights_scratch_bytes(cap));
        check(vren_cs_assign_lights(stream, cluster_key_buffer.at<uint32_t>(), key_count_buffer.at<uint32_t>(), cap,
                                    frame.device(), light_bvh_buffer.at<vren_bvh_node>(), light_count,
                                    light_index_buffer.at<uint32_t>(), view_space_positions.at<float>(),
                                    leaf_spheres ? leaf_spheres->at<float>() : nullptr,
                                    assigned_light_counts_buffer.at<uint32_t>(),
                                    assigned_light_offsets_buffer.at<uint32_t>(),
                                    assigned_light_indices_buffer.at<uint32_t>(),
                                    (uint32_t)(assigned_light_indices_buffer.m_size / 4),
                                    total ? total->at<uint32_t>() : nullptr, m_scratch.m_ptr),
              "assign_lights");
    }

private:
    owned_buffer m_scratch;
};

}  // namespace clustered_shading

// ------------------------------------------------------------------------------------------------
// vren::kd_tree_* (base/kd_tree.hpp): the reference's host build and search, same node array.
// ------------------------------------------------------------------------------------------------
using kd_tree_node = vren_kd_tree_node;
using kd_tree_search_filter_t = std::function<bool(uint32_t point)>;
inline const kd_tree_search_filter_t k_kd_tree_default_search_filter = [](uint32_t) -> bool { return true; };

inline size_t kd_tree_build(float const* points, size_t point_stride, uint32_t* indices, size_t count,
                            kd_tree_node* kd_tree, size_t node_offset, size_t max_leaf_point_count)
{
    return vren_kd_tree_build(points, point_stride, indices, count, kd_tree, node_offset, max_leaf_point_count);
}

inline void kd_tree_search(float const* points, size_t point_stride, uint32_t const* indices, size_t count,
                           kd_tree_node* kd_tree, size_t node_offset, float const* sample,
                           kd_tree_search_filter_t const& filter_predicate, uint32_t& best_point,
                           float& best_distance_squared)
{
    auto trampoline = [](uint32_t point, void* user) -> int {
        return (*static_cast<kd_tree_search_filter_t const*>(user))(point) ? 1 : 0;
    };
    vren_kd_tree_search(points, point_stride, indices, count, kd_tree, node_offset, sample, trampoline,
                        const_cast<kd_tree_search_filter_t*>(&filter_predicate), &best_point, &best_distance_squared);
}

// ------------------------------------------------------------------------------------------------
// vren::depth_buffer_pyramid / vren::depth_buffer_reductor (pipeline/depth_buffer_pyramid.hpp):
// all levels in one device buffer, level l at level_offset(l) floats, row pitch = its width.
// ------------------------------------------------------------------------------------------------
class depth_buffer_pyramid {
public:
    static const uint32_t k_max_depth_buffer_pyramid_level_count = 16;

    depth_buffer_pyramid(uint32_t width, uint32_t height) :
        m_base_width(width),
        m_base_height(height),
        m_level_count(vren_depth_pyramid_level_count(width, height))
    {
        if (m_level_count == 0) throw std::invalid_argument("depth_buffer_pyramid: unsupported size");
        m_image = owned_buffer(vren_depth_pyramid_level_offset(width, height, m_level_count) * sizeof(float), false);
    }

    uint32_t get_image_width(uint32_t level) const { return (m_base_width >> level) ? (m_base_width >> level) : 1u; }
    uint32_t get_image_height(uint32_t level) const { return (m_base_height >> level) ? (m_base_height >> level) : 1u; }
    uint32_t get_level_count() const { return m_level_count; }
    size_t level_offset(uint32_t level) const { return vren_depth_pyramid_level_offset(m_base_width, m_base_height, level); }
    float* level(uint32_t level) const { return m_image.at<float>(level_offset(level) * sizeof(float)); }
    device_buffer const& image() const { return m_image; }

private:
    friend class depth_buffer_reductor;
    uint32_t m_base_width, m_base_height, m_level_count;
    owned_buffer m_image;
};

class depth_buffer_reductor {
public:
    static const uint32_t k_workgroup_size_x = 32;
    static const uint32_t k_workgroup_size_y = 32;

    // depth_buffer: base_width x base_height floats, row-major (the depth attachment's texels).
    void copy_and_reduce(cudaStream_t stream, resource_container&, device_buffer const& depth_buffer,
                         depth_buffer_pyramid const& pyramid)
    {
        m_scratch.grow(vren_depth_pyramid_scratch_bytes(pyramid.m_base_width, pyramid.m_base_height));
        check(vren_depth_pyramid_copy_and_reduce(stream, depth_buffer.at<float>(), pyramid.m_base_width,
                                                 pyramid.m_base_height, pyramid.m_image.at<float>(), m_scratch.m_ptr),
              "depth_buffer_reductor::copy_and_reduce");
    }

private:
    owned_buffer m_scratch;
};

// ------------------------------------------------------------------------------------------------
// vren::cluster_and_shade (clustered_shading.hpp:147-182): owns its buffers.
// ------------------------------------------------------------------------------------------------
class cluster_and_shade {
public:
    cluster_and_shade(uint32_t max_width, uint32_t max_height, uint32_t max_lights, uint32_t max_assignments)
    {
        check(vren_cs_create(&m_handle, max_width, max_height, max_lights, max_assignments), "cluster_and_shade");
    }
    ~cluster_and_shade() { vren_cs_destroy(m_handle); }
    cluster_and_shade(const cluster_and_shade&) = delete;
    cluster_and_shade& operator=(const cluster_and_shade&) = delete;

    void set_options(vren_cs_options const& o) { check(vren_cs_set_options(m_handle, &o), "cluster_and_shade"); }

    // Light assignment for one frame (construct_point_light_bvh, find_unique_cluster_list, assign_lights).
    void cluster(cudaStream_t stream, camera const& cam, uint32_t width, uint32_t height, device_buffer const& depth,
                 device_buffer const& normals, device_buffer const& light_positions, device_buffer const& point_lights,
                 uint32_t light_count, uint32_t slicing = VREN_CS_SLICING_REF, int offscreen = VREN_CS_OFFSCREEN_WRAP)
    {
        vren_cs_view v;
        vren_cs_view_from_camera(&cam, slicing, &v);
        check(vren_cs_cluster(m_handle, stream, &v, width, height, offscreen, depth.at<float>(), normals.at<float>(),
                              light_positions.at<float>(), point_lights.at<float>(), light_count),
              "cluster_and_shade");
    }

    // cluster_and_shade::operator() (clustered_shading.cpp:924-1172): the light assignment of cluster(),
    // then shade over this context's light lists into `output` (f32x3 per pixel).  The G-buffer's
    // depth and normals (f32x3) are the clustering inputs too.
    void operator()(cudaStream_t stream, camera const& cam, uint32_t width, uint32_t height,
                    vren_cs_gbuffer const& gbuffer, device_buffer const& light_positions,
                    device_buffer const& point_lights, uint32_t light_count, device_buffer const& output,
                    float const* directional_lights = nullptr, uint32_t directional_count = 0,
                    int falloff = VREN_CS_FALLOFF_REF, int output_mode = VREN_CS_SHADE_COLOR,
                    uint32_t slicing = VREN_CS_SLICING_REF, int offscreen = VREN_CS_OFFSCREEN_WRAP)
    {
        vren_cs_view v;
        vren_cs_view_from_camera(&cam, slicing, &v);
        check(vren_cs_cluster_and_shade(m_handle, stream, &v, width, height, offscreen, &gbuffer,
                                        light_positions.at<float>(), point_lights.at<float>(), light_count,
                                        directional_lights, directional_count, falloff, output_mode,
                                        output.at<float>()),
              "cluster_and_shade");
    }

    vren_cs_outputs outputs() const
    {
        vren_cs_outputs o;
        check(vren_cs_get_outputs(m_handle, &o), "cluster_and_shade");
        return o;
    }

    vren_cluster_and_shade* handle() const { return m_handle; }

private:
    vren_cluster_and_shade* m_handle = nullptr;
};

}  // namespace vren

namespace vren_demo {

// vren_demo/vren_demo/clustered_shading_debug.cpp:6-200, headless: the views are written to device
// memory (RGBA float per pixel; 32 vren_debug_vertex per cluster) instead of a Vulkan image / draw buffer.
class show_clusters {
public:
    void operator()(cudaStream_t stream, int32_t mode, uint32_t width, uint32_t height, vren_cs_outputs const& outputs,
                    vren::device_buffer const& rgba_output)
    {
        m_scratch.grow(vren_cs_show_clusters_scratch_bytes(outputs.key_capacity));
        vren::check(vren_cs_show_clusters(stream, mode, width, height, outputs.cluster_refs, outputs.cluster_keys,
                                          outputs.key_count, outputs.key_capacity, outputs.counts, outputs.offsets,
                                          outputs.indices, outputs.index_capacity, rgba_output.at<float>(),
                                          m_scratch.m_ptr),
                    "show_clusters");
    }

private:
    vren::owned_buffer m_scratch;
};

inline void show_clusters_geometry(cudaStream_t stream, vren_cs_outputs const& outputs,
                                   vren::device_buffer const& vertices)
{
    vren::check(vren_cs_show_clusters_geometry(stream, outputs.frame, outputs.cluster_keys, outputs.key_count,
                                               outputs.key_capacity, vertices.at<vren_debug_vertex>()),
                "show_clusters_geometry");
}

// vren_demo/vren_demo/point_light_bouncer.cpp:17-57: moves each light speed * dt along its direction
// inside [aabb_min, aabb_max], reflecting off the faces; both buffers (vec4 per light) updated in place.
class point_light_bouncer {
public:
    void bounce(uint32_t /*frame_idx*/, cudaStream_t stream, vren::resource_container&,
                vren::device_buffer const& point_light_position_buffer,
                vren::device_buffer const& point_light_direction_buffer, uint32_t point_light_count,
                const float (&aabb_min)[3], const float (&aabb_max)[3], float speed, float dt)
    {
        vren::check(vren_bounce_point_lights(stream, point_light_position_buffer.at<float>(),
                                             point_light_direction_buffer.at<float>(), point_light_count, aabb_min,
                                             aabb_max, speed, dt),
                    "point_light_bouncer::bounce");
    }
};

}  // namespace vren_demo

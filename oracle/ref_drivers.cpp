// ref_drivers.cpp — runs the reference's shaders, rewritten into C++ by oracle/ref_shaders.py, on the
// CPU.  TEST INFRASTRUCTURE ONLY.  Each extern "C" function below plays the part of the reference's
// host code for one dispatch: it points the shader's buffers, samplers and images at the caller's
// arrays, sets its push constants, and calls the shader's main() for every invocation of the
// dispatch (gl_GlobalInvocationID, gl_WorkGroupID, ... set per invocation).  assign_lights.comp,
// whose main() uses subgroup ballots, runs as 32 host threads per cluster in lockstep.
//
// Built twice (VREN_REF_CANONICAL 0 / 1) from the two generated variants; the canonical variant's
// replaced expressions call the canon_* functions below, which read the host-built tables that
// ref_set_canonical installs.
#include <ucontext.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "glsl_subset.hpp"

namespace glsl {
struct Canonical {
    mat4 inv_proj, inv_view;
    const float* slice_near = nullptr;
    const float* slice_far = nullptr;
    uint max_slice = 0;
};
inline Canonical g_canon;
inline mat4 canon_inverse_projection() { return g_canon.inv_proj; }
inline mat4 canon_inverse_view() { return g_canon.inv_view; }
// the largest slice k <= max_slice whose near bound is <= z (0 if none)
inline uint canon_slice(float z)
{
    uint k = 0;
    for (uint i = 0; i <= g_canon.max_slice; ++i) {
        if (g_canon.slice_near[i] <= z) k = i;
        else break;
    }
    return k;
}
inline float canon_slice_near(uint k) { return g_canon.slice_near[k]; }
inline float canon_slice_far(uint k) { return g_canon.slice_far[k]; }
// integer texel (gid.x mod width, gid.y mod height)
inline vec4 canon_texel(const sampler2D& s)
{
    return texel(s, (int)(gl_GlobalInvocationID.x % (uint)s.w), (int)(gl_GlobalInvocationID.y % (uint)s.h));
}
inline uvec4 canon_utexel(const usampler2D& s)
{
    const uint x = gl_GlobalInvocationID.x % (uint)s.w, y = gl_GlobalInvocationID.y % (uint)s.h;
    return uvec4(s.data[(size_t)y * s.w + x], 0u, 0u, 1u);
}
}  // namespace glsl

#include VREN_REF_INC

using namespace glsl;

namespace {
template <class T> buffer<T> buf(const void* p, uint64_t n) { return buffer<T>{const_cast<T*>(static_cast<const T*>(p)), n}; }

// A 1-D dispatch of `count` invocations in work groups of `wg`.
template <class F> void dispatch_1d(uint64_t count, uint wg, F&& body)
{
    const uint64_t groups = (count + wg - 1) / wg;
    gl_NumWorkGroups = uvec3((uint)groups, 1u, 1u);
    gl_WorkGroupSize = uvec3(wg, 1u, 1u);
    for (uint64_t g = 0; g < groups; ++g)
        for (uint l = 0; l < wg; ++l) {
            gl_WorkGroupID = uvec3((uint)g, 0u, 0u);
            gl_LocalInvocationID = uvec3(l, 0u, 0u);
            gl_LocalInvocationIndex = l;
            gl_GlobalInvocationID = uvec3((uint)(g * wg + l), 0u, 0u);
            body();
        }
}

// A 2-D dispatch of groups_x x groups_y work groups of 32 x 32 invocations.
template <class F> void dispatch_2d(uint groups_x, uint groups_y, F&& body)
{
    gl_NumWorkGroups = uvec3(groups_x, groups_y, 1u);
    gl_WorkGroupSize = uvec3(32u, 32u, 1u);
    for (uint gy = 0; gy < groups_y; ++gy)
        for (uint gx = 0; gx < groups_x; ++gx)
            for (uint ly = 0; ly < 32; ++ly)
                for (uint lx = 0; lx < 32; ++lx) {
                    gl_WorkGroupID = uvec3(gx, gy, 0u);
                    gl_LocalInvocationID = uvec3(lx, ly, 0u);
                    gl_LocalInvocationIndex = ly * 32 + lx;
                    gl_GlobalInvocationID = uvec3(gx * 32 + lx, gy * 32 + ly, 0u);
                    body();
                }
}

vec3 v3(const float* p) { return vec3(p[0], p[1], p[2]); }

template <class PC> void set_assign_constants(PC& pc, uint32_t tiles_x, uint32_t tiles_y, float near_plane,
                                              float half_fov, const float* proj, uint32_t root, uint32_t levels)
{
    pc.num_tiles = uvec2(tiles_x, tiles_y);
    pc.camera_near = near_plane;
    pc.camera_half_fov = half_fov;
    pc.camera_proj = mat4_from(proj);
    pc.bvh_root_idx = root;
    pc.bvh_level_count = levels;
}

// One work group of assign_lights.comp: 32 invocations run as coroutines on the calling thread.  Each
// runs main() until its next subgroupBallot, where it stores its vote and yields; once all 32 have
// voted the mask is formed and each lane resumes with it, in lane order.  The shader's per-invocation
// globals (gl_SubgroupInvocationID, the thread_local g_level_overlaps) are swapped in and out at every
// switch, since the 32 coroutines share the thread.
struct Warp;
thread_local Warp* t_warp = nullptr;

struct Warp {
    static constexpr size_t kStack = 1 << 16;
    ucontext_t sched;
    ucontext_t lane_ctx[32];
    std::vector<char> stacks = std::vector<char>(32 * kStack);
    uint32_t overlaps[32][sizeof(sh_assign_write::g_level_overlaps) / sizeof(uint)];
    uint32_t votes[32] = {};
    uint32_t mask = 0, cur = 0, cluster = 0, groups = 0;
    bool done[32] = {};
    int write = 0;

    uint32_t* private_globals() const
    {
        return write ? sh_assign_write::g_level_overlaps : sh_assign_count::g_level_overlaps;
    }
    void enter_lane(uint32_t l)
    {
        cur = l;
        gl_SubgroupInvocationID = l;
        gl_LocalInvocationIndex = l;
        gl_LocalInvocationID = uvec3(l, 0u, 0u);
        gl_WorkGroupID = uvec3(cluster, 0u, 0u);
        gl_GlobalInvocationID = uvec3(cluster * 32 + l, 0u, 0u);
        gl_NumWorkGroups = uvec3(groups, 1u, 1u);
        std::memcpy(private_globals(), overlaps[l], sizeof(overlaps[l]));
    }
    void leave_lane(uint32_t l) { std::memcpy(overlaps[l], private_globals(), sizeof(overlaps[l])); }

    static uint ballot(bool b)
    {
        Warp& w = *t_warp;
        const uint32_t l = w.cur;
        w.votes[l] = b ? 1u : 0u;
        w.leave_lane(l);
        swapcontext(&w.lane_ctx[l], &w.sched);
        w.enter_lane(l);
        return w.mask;
    }
    static void entry()
    {
        Warp& w = *t_warp;
        if (w.write) sh_assign_write::shader_main();
        else sh_assign_count::shader_main();
        w.leave_lane(w.cur);
        w.done[w.cur] = true;  // returns to `sched` through uc_link
    }
    void run(uint32_t c, uint32_t U)
    {
        t_warp = this;
        g_ballot = &Warp::ballot;
        cluster = c;
        groups = U;
        for (uint32_t l = 0; l < 32; ++l) {
            getcontext(&lane_ctx[l]);
            lane_ctx[l].uc_stack.ss_sp = stacks.data() + l * kStack;
            lane_ctx[l].uc_stack.ss_size = kStack;
            lane_ctx[l].uc_link = &sched;
            makecontext(&lane_ctx[l], &Warp::entry, 0);
            std::memset(overlaps[l], 0, sizeof(overlaps[l]));
            done[l] = false;
        }
        for (;;) {
            for (uint32_t l = 0; l < 32; ++l) {
                enter_lane(l);
                swapcontext(&sched, &lane_ctx[l]);
            }
            uint32_t finished = 0;
            for (uint32_t l = 0; l < 32; ++l) finished += done[l] ? 1u : 0u;
            if (finished == 32) break;
            if (finished != 0) std::abort();  // a ballot outside uniform control flow
            mask = 0;
            for (uint32_t l = 0; l < 32; ++l) mask |= votes[l] << l;
        }
    }
};
}  // namespace

extern "C" {

int ref_is_canonical() { return VREN_REF_CANONICAL; }
uint64_t ref_oob_count(int clear)
{
    const uint64_t n = g_oob.load();
    if (clear) g_oob.store(0);
    return n;
}

void ref_set_canonical(const float* inv_proj, const float* inv_view, const float* slice_near, const float* slice_far,
                       uint32_t max_slice)
{
    g_canon.inv_proj = mat4_from(inv_proj);
    g_canon.inv_view = mat4_from(inv_view);
    g_canon.slice_near = slice_near;
    g_canon.slice_far = slice_far;
    g_canon.max_slice = max_slice;
}

// ---- clustered_shading.glsl ---------------------------------------------------------------------
void ref_normal_bin(const float* normals, uint64_t count, uint32_t* out)
{
    for (uint64_t i = 0; i < count; ++i) out[i] = sh_cs::clustered_shading_discretize_normal(v3(normals + 3 * i));
}

void ref_decode_cluster_key(const uint32_t* keys, uint64_t count, uint32_t* out /* 4 per key: i, j, k, normal */)
{
    for (uint64_t i = 0; i < count; ++i) {
        uvec3 ijk;
        uint nidx;
        sh_cs::clustered_shading_decode_cluster_key(keys[i], ijk, nidx);
        out[4 * i] = ijk.x;
        out[4 * i + 1] = ijk.y;
        out[4 * i + 2] = ijk.z;
        out[4 * i + 3] = nidx;
    }
}

// cluster box of each key: calc_cluster_aabb after decode_cluster_key, as assign_lights.comp:123-138
void ref_cluster_boxes(const uint32_t* keys, uint64_t count, uint32_t tiles_x, uint32_t tiles_y, float near_plane,
                       float half_fov, const float* proj, float* mn, float* mx)
{
    const mat4 P = mat4_from(proj);
    for (uint64_t i = 0; i < count; ++i) {
        uvec3 ijk;
        uint nidx;
        sh_cs::clustered_shading_decode_cluster_key(keys[i], ijk, nidx);
        vec4 a, b;
        sh_cs::clustered_shading_calc_cluster_aabb(ijk, uvec2(tiles_x, tiles_y), near_plane, half_fov, P, a, b);
        for (int c = 0; c < 4; ++c) {
            mn[4 * i + c] = a[c];
            mx[4 * i + c] = b[c];
        }
    }
}

// ---- assign_lights.comp's two box tests -----------------------------------------------------------
void ref_test_aabb_aabb(const float* v /* 12 per test: min1, max1, min2, max2 */, uint64_t count, uint8_t* out)
{
    for (uint64_t i = 0; i < count; ++i) {
        const float* t = v + 12 * i;
        out[i] = sh_assign_write::test_aabb_aabb(v3(t), v3(t + 3), v3(t + 6), v3(t + 9)) ? 1 : 0;
    }
}

void ref_test_sphere_aabb(const float* v /* 10 per test: centre, radius, min, max */, uint64_t count, uint8_t* out)
{
    for (uint64_t i = 0; i < count; ++i) {
        const float* t = v + 10 * i;
        out[i] = sh_assign_write::test_sphere_aabb(v3(t), t[3], v3(t + 4), v3(t + 7)) ? 1 : 0;
    }
}

// ---- construct_point_light_bvh's shaders ----------------------------------------------------------
void ref_view_space(const float* view, const float* positions, uint32_t L, float* out)
{
    using namespace sh_view;
    push_constants.camera_view = mat4_from(view);
    point_light_positions = buf<vec4>(positions, L);
    view_space_point_light_positions = buf<vec4>(out, L);
    dispatch_1d(L, 1024, [] { sh_view::shader_main(); });
}

void ref_morton(const float* view_pos, uint32_t L, const float* mn, const float* mx, uint32_t* codes /* 2 per light */)
{
    using namespace sh_morton;
    _min = vec4(mn[0], mn[1], mn[2], mn[3]);
    _max = vec4(mx[0], mx[1], mx[2], mx[3]);
    view_space_point_light_positions = buf<vec4>(view_pos, L);
    morton_codes = buf<uvec2>(codes, L);
    dispatch_1d(L, 1024, [] { sh_morton::shader_main(); });
}

// leaves of the light BVH from the sorted (code, light) pairs; bvh holds `padded` 32-byte nodes
void ref_leaves(const float* view_pos, const float* lights, const uint32_t* sorted_pairs, uint32_t L, uint32_t padded,
                void* bvh_out)
{
    using namespace sh_leaves;
    point_lights = buf<PointLight>(lights, L);
    view_space_point_light_positions = buf<vec4>(view_pos, L);
    morton_codes = buf<uvec2>(sorted_pairs, L);
    bvh = buf<BvhNode>(bvh_out, padded);
    dispatch_1d(padded, 1024, [] { sh_leaves::shader_main(); });
}

// ---- find_unique_clusters.comp: the cluster key of every invocation of the dispatch ---------------
// keys: (tiles_y * 32) rows of (tiles_x * 32) keys, one per invocation, the overhang included
void ref_pixel_keys(uint32_t W, uint32_t H, const float* depth, const float* normals, float near_plane,
                    float half_fov, const float* proj, uint32_t* keys)
{
    using namespace sh_unique;
    const uint32_t TX = (W + 31) / 32, TY = (H + 31) / 32;
    camera_near = near_plane;
    camera_half_fov_y = half_fov;
    camera_projection = mat4_from(proj);
    u_depth_buffer = sampler2D{depth, (int)W, (int)H, 1};
    gbuffer_normals = sampler2D{normals, (int)W, (int)H, 3};
    dispatch_2d(TX, TY, [&] {
        keys[(size_t)gl_GlobalInvocationID.y * (TX * 32) + gl_GlobalInvocationID.x] = sh_unique::shader_key();
    });
}

// ---- assign_lights.comp: count (write = 0) or write (write = 1) dispatch, one work group per key -----
void ref_assign_lights(int write, const uint32_t* keys, uint32_t U, uint32_t tiles_x, uint32_t tiles_y,
                       float near_plane, float half_fov, const float* proj, const void* bvh, uint64_t bvh_nodes,
                       uint32_t root, uint32_t levels, const uint32_t* light_index, uint64_t light_index_len,
                       const float* view_pos, uint32_t L, uint32_t* counts, const uint32_t* offsets,
                       uint32_t* indices, uint64_t index_cap)
{
    if (write) {
        using namespace sh_assign_write;
        set_assign_constants(push_constants, tiles_x, tiles_y, near_plane, half_fov, proj, root, levels);
        cluster_keys = buf<uint>(keys, U);
        sh_assign_write::bvh = buf<BvhNode>(bvh, bvh_nodes);
        light_indices = buf<uvec2>(light_index, light_index_len);
        assigned_light_indices = buf<uint>(indices, index_cap);
        assigned_light_counts = buf<uint>(counts, U);
        assigned_light_offsets = buf<uint>(offsets, U);
        view_space_point_light_positions = buf<vec4>(view_pos, L);
    } else {
        using namespace sh_assign_count;
        set_assign_constants(push_constants, tiles_x, tiles_y, near_plane, half_fov, proj, root, levels);
        cluster_keys = buf<uint>(keys, U);
        sh_assign_count::bvh = buf<BvhNode>(bvh, bvh_nodes);
        light_indices = buf<uvec2>(light_index, light_index_len);
        assigned_light_counts = buf<uint>(counts, U);
        assigned_light_offsets = buf<uint>(offsets, U);
        view_space_point_light_positions = buf<vec4>(view_pos, L);
        for (uint32_t c = 0; c < U; ++c) counts[c] = 0;  // the reference clears the counts first
    }
    // Work groups are independent (each writes its own count or its own list range), so they are
    // spread over host threads; inside one, the 32 invocations run as a Warp of coroutines.
    const unsigned nthreads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nthreads; ++t)
        pool.emplace_back([=] {
            Warp w;
            w.write = write;
            for (uint32_t c = t; c < U; c += nthreads) w.run(c, U);
        });
    for (auto& t : pool) t.join();
}

// ---- shade.comp ------------------------------------------------------------------------------------
// The G-buffer is given per pixel (albedo rgb, roughness, metallic); the shader reads it through its
// material model: the material of pixel p is material p (its material-index texture holds p) with
// base colour factor (albedo, 1), metallic and roughness factors, and texture 0 for both maps, a 1x1
// white texture, so albedo = 1 * albedo, metallic = 1 * metallic, roughness = 1 * roughness.
void ref_shade(uint32_t W, uint32_t H, const float* depth, const float* normals, const float* albedo, const float* rough,
               const float* metal, const uint32_t* refs, const uint32_t* counts, const uint32_t* offsets,
               const uint32_t* indices, uint32_t U, uint64_t total, const float* light_positions, const float* lights,
               uint32_t L, const float* directional, uint32_t n_directional, const float* eye, float far_plane,
               const float* view, const float* proj, float* out_rgba)
{
    using namespace sh_shade;
    static const float white[4] = {1.0f, 1.0f, 1.0f, 1.0f};
    static sampler2D white_tex{white, 1, 1, 4};
    std::vector<Material> mats((size_t)W * H);
    std::vector<uint> mat_idx((size_t)W * H);
    std::vector<float> texcoords((size_t)W * H * 2, 0.0f);
    for (size_t p = 0; p < (size_t)W * H; ++p) {
        mats[p].base_color_texture_idx = 0;
        mats[p].metallic_roughness_texture_idx = 0;
        mats[p].metallic_factor = metal[p];
        mats[p].roughness_factor = rough[p];
        mats[p].base_color_factor = vec4(albedo[3 * p], albedo[3 * p + 1], albedo[3 * p + 2], 1.0f);
        mat_idx[p] = (uint)p;
    }
    camera_position = v3(eye);
    camera_far_plane = far_plane;
    camera_view = mat4_from(view);
    camera_projection = mat4_from(proj);
    u_depth_buffer = sampler2D{depth, (int)W, (int)H, 1};
    u_gbuffer_normals = sampler2D{normals, (int)W, (int)H, 3};
    u_gbuffer_texcoords = sampler2D{texcoords.data(), (int)W, (int)H, 2};
    u_gbuffer_material_indices = usampler2D{mat_idx.data(), (int)W, (int)H, 1};
    u_cluster_references = uimage2D{const_cast<uint*>(refs), (int)W, (int)H, 1};
    assigned_light_indices = buf<uint>(indices, total);
    assigned_light_counts = buf<uint>(counts, U);
    assigned_light_offsets = buf<uint>(offsets, U);
    textures = buffer<sampler2D>{&white_tex, 1};
    point_light_positions = buf<vec4>(light_positions, L);
    point_lights = buf<PointLight>(lights, L);
    directional_lights = buf<DirectionalLight>(directional, n_directional);
    materials = buffer<Material>{mats.data(), mats.size()};
    u_output = image2D{out_rgba, (int)W, (int)H, 4};
    dispatch_2d((W + 31) / 32, (H + 31) / 32, [] { sh_shade::shader_main(); });
}

// ---- vren_demo's bouncer ---------------------------------------------------------------------------
void ref_bounce(float* positions, float* directions, uint32_t L, const float* mn, const float* mx, float speed, float dt)
{
    using namespace sh_bounce;
    point_light_positions = buf<vec4>(positions, L);
    point_lights_directions = buf<vec4>(directions, L);
    aabb_min = v3(mn);
    aabb_max = v3(mx);
    sh_bounce::speed = speed;
    sh_bounce::dt = dt;
    dispatch_1d(L, 1024, [] { sh_bounce::shader_main(); });
}

// ---- depth-buffer pyramid: the copy (unnormalised nearest sampler) and one reduce dispatch ----------
void ref_depth_copy(const float* depth, uint32_t W, uint32_t H, float* level0)
{
    using namespace sh_depth_copy;
    // the reference's depth sampler: NEAREST, unnormalised coordinates, CLAMP_TO_BORDER
    // (depth_buffer_pyramid.cpp:197-211)
    depth_buffer = sampler2D{depth, (int)W, (int)H, 1, true};
    depth_buffer_pyramid_base = image2D{level0, (int)W, (int)H, 1};
    dispatch_2d((W + 31) / 32, (H + 31) / 32, [] { sh_depth_copy::shader_main(); });
}

void ref_depth_reduce(const float* from, uint32_t fw, uint32_t fh, float* to, uint32_t tw, uint32_t th)
{
    using namespace sh_depth_reduce;
    from_image = image2D{const_cast<float*>(from), (int)fw, (int)fh, 1};
    to_image = image2D{to, (int)tw, (int)th, 1};
    dispatch_2d((tw + 31) / 32, (th + 31) / 32, [] { sh_depth_reduce::shader_main(); });
}

// ---- vren_demo's show_clusters ---------------------------------------------------------------------
void ref_show_clusters(int view_mode, uint32_t W, uint32_t H, uint32_t tiles_x, uint32_t tiles_y, const uint32_t* refs,
                       const uint32_t* keys, uint32_t U, const uint32_t* counts, const uint32_t* offsets,
                       const uint32_t* indices, uint64_t total, float* out_rgba)
{
    using namespace sh_show;
    mode = view_mode;
    num_tiles = uvec2(tiles_x, tiles_y);
    u_cluster_references = uimage2D{const_cast<uint*>(refs), (int)W, (int)H, 1};
    cluster_keys = buf<uint>(keys, U);
    assigned_light_counts = buf<uint>(counts, counts ? U : 0);
    assigned_light_offsets = buf<uint>(offsets, offsets ? U : 0);
    assigned_light_indices = buf<uint>(indices, total);
    u_output = image2D{out_rgba, (int)W, (int)H, 4};
    dispatch_2d((W + 31) / 32, (H + 31) / 32, [] { sh_show::shader_main(); });
}

}  // extern "C"

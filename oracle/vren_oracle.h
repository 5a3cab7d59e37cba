/*
 * vren_oracle.h — CPU oracle for the vren hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's algorithms (loryruta/vren), used by the tests, by
 * the smoke check and by the benchmark's CPU-baseline leg as the oracle — never by the product
 * path.  Every function cites the reference file:line it restates.
 *
 * Pinning.  The primitives (reduce, scan, down-sweep, radix sort, bucket sort, BVH build and
 * the BVH size helpers) are pinned against the reference's own known-answer tests
 * (vren_test/vren_test/primitives/*.cpp), restated as golden fixtures under tests/golden/.
 * The clustered-shading stages have no test, no CPU code and no golden vectors in the reference
 * (their shaders use GLSL built-ins compiled by a Vulkan driver that cannot run here), so
 * their parity is UNPINNED: this oracle restates the shaders under canonical decisions (a fixed
 * order where the reference's is unspecified, exactly rounded float steps, slice bounds from a
 * host table) and the CUDA kernels are checked against it.
 *
 * Float rules shared with the CUDA kernels: IEEE single precision, round to nearest, no FMA
 * contraction (built with -ffp-contract=off), division and sqrt correctly rounded, float->uint
 * conversions saturating (NaN and negatives -> 0).
 */
#ifndef VREN_ORACLE_H_
#define VREN_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_ADD = 0, ORACLE_MIN = 1, ORACLE_MAX = 2 };

/* ---- size helpers (vren/vren/base/base.hpp:32-79, vren/vren/primitives/build_bvh.cpp:101-136),
 *      restated with the reference's own double-precision log/pow formulas ---- */
uint32_t oracle_round_to_next_power_of_2(uint32_t v);
uint32_t oracle_round_to_next_power_of(uint32_t n, uint32_t base);
uint32_t oracle_divide_and_ceil(uint32_t value, uint32_t divider);
uint32_t oracle_calc_bvh_padded_leaf_count(uint32_t leaf_count);
uint32_t oracle_calc_bvh_buffer_length(uint32_t leaf_count);
uint32_t oracle_calc_bvh_root_index(uint32_t leaf_count);
uint32_t oracle_calc_bvh_level_count(uint32_t leaf_count);

/* ---- reduce (vren_test/vren_test/primitives/reduce.cpp:72-98 tree order, :141-196 fill;
 *      operand order of vren/resources/shaders/reduce.comp:76) ---- */
void oracle_reduce_tree_u32(int op, const uint32_t* in, uint32_t n, uint32_t* out /* P */);
void oracle_reduce_tree_vec4(int op, const float* in, uint32_t n, float* out /* 4P */);
uint32_t oracle_reduce_u32(int op, const uint32_t* in, uint64_t n);
float oracle_reduce_f32(int op, const float* in, uint64_t n); /* min/max in IEEE total order */

/* ---- scan (vren_test/vren_test/primitives/blelloch_scan.cpp:70-73 std::exclusive_scan) and the
 *      reference's down-sweep dispatch sequence (vren/vren/primitives/blelloch_scan.cpp:57-139,
 *      vren/resources/shaders/blelloch_scan_downsweep.comp:33-125) ---- */
void oracle_exclusive_scan_u32(uint32_t* data, uint64_t n);
void oracle_downsweep_u32(uint32_t* data, uint32_t n, int clear_last);

/* ---- sorts: stable LSD sort (radix_sort.cpp test:265 std::sort, made stable for pairs);
 *      bucket sort by masked key (bucket_sort.cpp test:449-452, stable) ---- */
void oracle_stable_sort_u32(uint32_t* keys, uint32_t* values /* may be NULL */, uint64_t n);
void oracle_bucket_sort_u32x2(const uint32_t* in, uint32_t n, uint32_t key_bits, uint32_t* out_pairs,
                              uint32_t* out_ends);

/* ---- BVH (vren/resources/shaders/build_bvh.comp:32-55; test traversal
 *      vren_test/vren_test/primitives/build_bvh.cpp:25-78) ---- */
typedef struct oracle_bvh_node {
    float min[3];
    uint32_t next;
    float max[3];
    uint32_t pad;
} oracle_bvh_node;
void oracle_build_bvh(oracle_bvh_node* bvh, uint32_t padded_leaf_count);
/* Point query: writes the leaf indices whose AABB contains p (DFS order), returns their count. */
uint32_t oracle_bvh_point_query(const oracle_bvh_node* bvh, uint32_t root_index, const float p[3],
                                uint32_t* out, uint32_t cap);

/* ---- clustered shading (see the .c file for the shader lines restated) ---- */
#define ORACLE_SLICES 1024
enum { ORACLE_SLICING_REF = 0, ORACLE_SLICING_FIXED32 = 1 };
enum { ORACLE_WRAP = 0, ORACLE_SKIP = 1 };

typedef struct oracle_cs_view {
    float view[16];      /* world -> view, column-major m[c*4+r] */
    float inv_proj[16];  /* inverse projection, column-major */
    float inv_view[16];  /* view -> world */
    float eye[3];
    float near_plane, far_plane, half_fov_y;
    uint32_t slicing;
    uint32_t reserved;
} oracle_cs_view;

/* Slice tables: near[k], far[k] for k in [0, 1024). */
void oracle_cs_slice_table(const oracle_cs_view* v, uint32_t tiles_y, float* near_out, float* far_out);

void oracle_cs_light_bvh(const float* positions, const float* lights, uint32_t L, const oracle_cs_view* v,
                         uint32_t morton_bits, float* view_pos /* vec4[L] */, oracle_bvh_node* bvh,
                         uint32_t* light_index /* uvec2[L] */);

/* The restatement's per-element steps, compared one by one with the reference's shaders run on the
 * CPU (oracle/_ref): view positions, their vec4 min / max and the unsorted (code, light) pairs; the
 * normal bin of each normal; the key of every invocation of the unique-cluster dispatch
 * ((TY*32) rows of TX*32, overhang included, WRAP texels); the view-space box of each key (3 floats
 * per corner); the two overlap tests (12 floats per AABB test: min1, max1, min2, max2; 10 per sphere
 * test: centre, radius, min, max). */
void oracle_cs_light_codes(const float* positions, uint32_t L, const oracle_cs_view* v, uint32_t morton_bits,
                           float* view_pos, float* mn, float* mx, uint32_t* codes);
void oracle_cs_normal_bins(const float* normals, uint64_t count, uint32_t* out);
void oracle_cs_pixel_keys(const float* depth, const float* normals, uint32_t W, uint32_t H, const oracle_cs_view* v,
                          uint32_t* keys);
void oracle_cs_cluster_boxes(const uint32_t* keys, uint64_t count, uint32_t W, uint32_t H, const oracle_cs_view* v,
                             float* mn, float* mx);
void oracle_cs_test_aabb_aabb(const float* t, uint64_t count, uint8_t* out);
void oracle_cs_test_sphere_aabb(const float* t, uint64_t count, uint8_t* out);

/* Returns the number of unique cluster keys U (keys[0..U) written), refs[W*H]. */
uint32_t oracle_cs_find_unique_clusters(const float* depth, const float* normals, uint32_t W, uint32_t H,
                                        const oracle_cs_view* v, int policy, uint32_t* keys, uint32_t key_cap,
                                        uint32_t* refs, int threads);

/* Returns the total number of assignments (indices[0..total) written, or the total needed if it
 * exceeds index_cap, in which case nothing beyond index_cap is written). */
uint64_t oracle_cs_assign_lights(const uint32_t* keys, uint32_t U, uint32_t W, uint32_t H, const oracle_cs_view* v,
                                 const oracle_bvh_node* bvh, uint32_t L, const uint32_t* light_index,
                                 const float* view_pos, uint32_t* counts, uint32_t* offsets, uint32_t* indices,
                                 uint64_t index_cap, int threads);

/* ---- Karras binary radix tree over the sorted light leaves (extension) ---- */
#define ORACLE_LBVH_LEAF 0x80000000u
typedef struct {
    float min[3];
    uint32_t left;   /* internal node index, or leaf position | ORACLE_LBVH_LEAF */
    float max[3];
    uint32_t right;
} oracle_lbvh_node;

/* n - 1 internal nodes (root = 0) over the n sorted leaves: light_index = uvec2(code, light)[n] in
 * sorted order, boxes[i] = the box of leaf i (e.g. level 0 of the 32-ary BVH). */
void oracle_lbvh_build(const uint32_t* light_index, const oracle_bvh_node* boxes, uint32_t n,
                       oracle_lbvh_node* nodes);
/* assign_lights by the Karras tree built over `boxes`: lights whose box and sphere (from `leaves`,
 * the 32-ary level 0) overlap the cluster box, in the reference's list order.  Same return
 * convention as oracle_cs_assign_lights. */
uint64_t oracle_cs_assign_lights_lbvh(const uint32_t* keys, uint32_t U, uint32_t W, uint32_t H,
                                      const oracle_cs_view* v, const oracle_lbvh_node* nodes,
                                      const oracle_bvh_node* boxes, const oracle_bvh_node* leaves, uint32_t L,
                                      const uint32_t* light_index, const float* view_pos, uint32_t* counts,
                                      uint32_t* offsets, uint32_t* indices, uint64_t index_cap, int threads);

/* Point-light bouncer (in place; vec4 positions and directions; aabb_min/max: 3 floats). */
void oracle_bounce_point_lights(float* positions, float* directions, uint32_t L, const float* aabb_min,
                                const float* aabb_max, float speed, float dt);

/* Depth-buffer pyramid: level count and all levels (level 0 = the depth copy), stored back to back. */
uint32_t oracle_depth_pyramid_level_count(uint32_t width, uint32_t height);
void oracle_depth_pyramid(const float* depth, uint32_t width, uint32_t height, float* out);

/* Cluster debug views: RGBA float per pixel (mode 0..5, other values red); 32 debug vertices
 * (x, y, z as float bits, colour) per cluster. */
void oracle_cs_show_clusters(int mode, uint32_t W, uint32_t H, const uint32_t* refs, const uint32_t* keys, uint32_t U,
                             const uint32_t* counts, const uint32_t* offsets, const uint32_t* indices, float* out);
void oracle_cs_show_clusters_geometry(const oracle_cs_view* v, uint32_t W, uint32_t H, const uint32_t* keys,
                                      uint32_t U, uint32_t* out);

/* k-d tree: build (returns the node count), batched recursive search, linear search. */
typedef struct oracle_kd_node {
    uint32_t word0; /* split (float bits) or point index */
    uint32_t axis;
    uint32_t value;
} oracle_kd_node;
size_t oracle_kd_tree_build(const float* points, size_t stride, uint32_t* indices, size_t count, oracle_kd_node* tree,
                            size_t max_leaf);
void oracle_kd_tree_search(const float* points, size_t stride, const oracle_kd_node* tree, const float* samples,
                           size_t sample_stride, uint32_t sample_count, const uint8_t* excluded, uint32_t* best_points,
                           float* best_dist);
void oracle_linear_nn_search(const float* points, size_t stride, const uint32_t* indices, size_t count,
                             const float* samples, size_t sample_stride, uint32_t sample_count, uint32_t* best_points,
                             float* best_dist);

/* ---- shading in FP64 (vren_oracle_shade.cpp): forward, forward-mode gradient, per-light loss ---- */
void oracle_cs_shade_f64(const oracle_cs_view* v, uint32_t W, uint32_t H, const float* depth, const float* normals,
                         const float* albedo, const float* rough, const float* metal, const uint32_t* refs,
                         const uint32_t* counts, const uint32_t* offsets, const uint32_t* indices, const float* lpos,
                         const float* lights, uint32_t L, int falloff, int mode, double* out, uint8_t* shaded,
                         int threads);
void oracle_cs_shade_grad_f64(const oracle_cs_view* v, uint32_t W, uint32_t H, const float* depth,
                              const float* normals, const float* albedo, const float* rough, const float* metal,
                              const uint32_t* refs, const uint32_t* counts, const uint32_t* offsets,
                              const uint32_t* indices, const float* lpos, const float* lights, uint32_t L, int falloff,
                              const float* grad, double* g7, int threads);
double oracle_cs_shade_light_loss_f64(const oracle_cs_view* v, uint32_t W, uint32_t H, const float* depth,
                                      const float* normals, const float* albedo, const float* rough, const float* metal,
                                      const uint32_t* refs, const uint32_t* counts, const uint32_t* offsets,
                                      const uint32_t* indices, uint32_t l, const double* theta, int falloff,
                                      const float* grad);
void oracle_cs_shade_grad_lights_f64(const oracle_cs_view* v, uint32_t W, uint32_t H, const float* depth,
                                     const float* normals, const float* albedo, const float* rough,
                                     const float* metal, const uint32_t* refs, const uint32_t* counts,
                                     const uint32_t* offsets, const uint32_t* indices, const float* lpos,
                                     const float* lights, uint32_t L, int falloff, const float* grad,
                                     const uint32_t* sel, uint32_t nsel, double h, double* g7, double* fd7,
                                     uint64_t* pair_counts, int threads);

#ifdef __cplusplus
}
#endif

#endif /* VREN_ORACLE_H_ */

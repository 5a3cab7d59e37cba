/*
 * vren_gb300.h — C ABI of the GB300-native (sm_103a) implementation of vren's
 * parallel primitives and clustered-shading light assignment.
 *
 * Every entry point takes plain device pointers and sizes; there are no Vulkan
 * or torch types in any signature.  A `vren_stream_t` is a `cudaStream_t`
 * (NULL = the legacy default stream).  All calls are asynchronous and
 * stream-ordered: they enqueue work and return a status describing argument
 * validation and launch success only.  Failures detected on the device (a
 * bounded wait that ran out, a capacity overflow) are recorded in a per-device
 * error word that `vren_device_error` reads.
 *
 * Scratch memory is owned by the caller; its size comes from the matching
 * `*_scratch_bytes` query.  No entry point allocates device memory, except
 * the context constructors (`vren_cs_create`, `vren_cs_batch_create`) which
 * own an arena, as the reference's `vren::cluster_and_shade` owns its buffers.
 * Two calls that share a scratch buffer must not overlap on the device.
 *
 * Reference interfaces replaced (paths inside loryruta/vren):
 *   vren::reduce<T,Op>          vren/vren/primitives/reduce.hpp:15-49
 *   vren::blelloch_scan         vren/vren/primitives/blelloch_scan.hpp:9-49
 *   vren::radix_sort            vren/vren/primitives/radix_sort.hpp:9-53
 *   vren::bucket_sort           vren/vren/primitives/bucket_sort.hpp:9-45
 *   vren::build_bvh, calc_bvh_* vren/vren/primitives/build_bvh.hpp:8-57
 */
#ifndef VREN_GB300_H_
#define VREN_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void* vren_stream_t;

/* ------------------------------------------------------------------------------------------------
 * Status codes.  The reference signals misuse with assert / std::invalid_argument
 * (vren/primitives/radix_sort.cpp:158-161) and Vulkan failures with VREN_CHECK -> std::runtime_error
 * (vk_helpers/misc.cpp:8-37); capacity overflows are unchecked there (config.hpp:23-24).
 * ------------------------------------------------------------------------------------------------ */
enum {
    VREN_OK = 0,
    VREN_ERR_ARG = 1,       /* invalid argument (null pointer, unsupported length, ...) */
    VREN_ERR_CAPACITY = 2,  /* an output did not fit in the capacity the caller gave */
    VREN_ERR_TIMEOUT = 3,   /* a bounded device-side wait ran out */
    VREN_ERR_CUDA = 4,      /* a CUDA runtime call failed */
    VREN_ERR_STATE = 5      /* object used in the wrong state */
};

const char* vren_status_string(int status);

/* Waits for the device, then returns the device error word (a VREN_ERR_* code, 0 if
 * none) recorded by kernels of this library since the last clear.  `clear` != 0 resets
 * it.  Synchronizes the current device. */
int vren_device_error(int clear);

/* Test hook: the number of polling rounds a device-side wait makes before it gives up
 * and records VREN_ERR_TIMEOUT.  `rounds` = 0 restores the default.  Returns the
 * previous value. */
uint32_t vren_set_wait_limit(uint32_t rounds);

/* Test hook (no counterpart in the reference): on the current device, the exclusive scans stop
 * publishing the look-back status of tile `tile_plus_one - 1` (every tile of every scan call with
 * that index), so the look-back waits of the tiles after it run out after the wait limit and record
 * VREN_ERR_TIMEOUT; the call still returns and the kernels end.  0 restores normal operation.  Call
 * it with no scan in flight (it copies to device memory synchronously).  After a timeout the scan's
 * scratch must be zero-filled again before its next use. */
int vren_test_withhold_scan_status(uint32_t tile_plus_one);

/* Test hook (no counterpart in the reference): on the current device, the bucket sort's column scan
 * (the one-scatter form, up to 10 key bits) stops publishing the look-back words of its row block
 * `block_plus_one - 1`, so the blocks after it wait until the wait limit and record
 * VREN_ERR_TIMEOUT; the call still returns and its kernels end (that call's output is not sorted).
 * 0 restores normal operation.  Call it with no bucket sort in flight.  The next call needs no
 * action: the sort resets its look-back words itself. */
int vren_test_withhold_bucket_scan_status(uint32_t block_plus_one);

/* Kernel variant knobs, read when work is enqueued (no counterpart in the reference; the autotuner
 * and benchmarks set them).  Every variant gives identical results.
 *   VREN_TUNE_SCAN_SLICES  128-element slices per warp in a scan tile: 4 (4096/tile) or 8 (8192/tile)
 *   VREN_TUNE_SPIN_POLLS   look-back polls before a waiting thread starts to back off with nanosleep
 *   VREN_TUNE_RADIX_RANK   digit ranking in a sort pass: 0 = one ballot per digit bit,
 *                          1 = match.any + shared-memory atomic per peer group,
 *                          2 = match.any + counter update by the group's first lane
 *   VREN_TUNE_RADIX_ITEMS  keys per thread in a sort pass: 0 = 15/16 (3840/4096 per tile), 1 = 23/24
 *   VREN_TUNE_SCAN_STAGED  scan form: 0 = automatic (the persistent form from 2^20 elements when
 *                          every tile starts 16-byte aligned, else tiles in registers), 1 = always
 *                          one CTA per tile in registers, 2 = one CTA per tile staged in shared
 *                          memory by bulk copies, 3 = persistent grid with a producer warp streaming
 *                          tiles by bulk copies (2 and 3 whenever the alignment allows)
 *   VREN_TUNE_REDUCE_FORM  scalar reduce form: 0 = automatic (= 1), 1 = grid-stride loop of uint4
 *                          loads, 2..5 = streaming through shared-memory stages filled by bulk copies
 *                          (16 KB x 6 contiguous, 16 KB x 6 interleaved, 32 KB x 6, 8 KB x 12)
 *   VREN_TUNE_LIGHT_BVH_CLUSTER  light BVH of 2049..32768 lights (15-bit codes): 1 = one kernel on a
 *                          16-CTA thread-block cluster when the device can hold one (default),
 *                          0 = the multi-kernel path
 *   VREN_TUNE_ASSIGN_FUSED assign_lights: 0 = count kernel, exclusive scan, write kernel (default);
 *                          1 = one kernel (count, look-back over the cluster counts, write); 2 = a
 *                          count kernel that also writes the offsets (its CTAs own ranges of
 *                          clusters and resolve the counts before their range by look-back), then
 *                          the write kernel
 *   VREN_TUNE_RADIX_PERSISTENT  sort passes over keys or pairs whose input starts 16-byte aligned:
 *                          1 = persistent grid whose producer warp streams tiles into shared memory
 *                          by bulk copies and publishes their digit counts on arrival, 0 = one CTA
 *                          per tile (ballot ranking, 15/16 keys per thread only)
 *   VREN_TUNE_FUC_FUSED    find_unique_cluster_list: 0 = tiles, then a fix-up whose CTAs sum their
 *                          own tile offsets (two kernels, up to 16384 tiles; the default), 1 = tiles,
 *                          tile-count scan and fix-up (three kernels), 2 = in the context's device
 *                          frames one kernel (tiles taken by ticket, offsets by look-back over the
 *                          tile counts)
 *   VREN_TUNE_BUCKET_FORM  bucket sort of up to 10 key bits: 0 = one scatter pass (per-tile bucket
 *                          histograms, a column scan of the tiles' count matrix, then one stable
 *                          scatter; the default), 1 = stable radix passes of at most 8 bits, then
 *                          the end offsets read back from the sorted elements
 *   VREN_TUNE_HOST_ZERO_COPY vren_cs_cluster_host: 0 = the G-buffer copied up in bands, each band's
 *                          tiles processed on arrival; 1 = the unique-cluster kernel (one-kernel
 *                          form) reads depth and normals straight from the page-locked host buffers
 *                          and writes the references to cluster_refs_out as it goes (used when the
 *                          device can address those buffers, else the banded copies run)
 *   VREN_TUNE_SHADE_PACKED vren_cs_shade and vren_cs_shade_backward: 1 = two lights per step in
 *                          packed f32x2 arithmetic (the same operations per light, a different
 *                          rounding of a few contracted products; the default), 0 = one light per
 *                          step */
enum { VREN_TUNE_SCAN_SLICES = 0, VREN_TUNE_SPIN_POLLS = 1, VREN_TUNE_RADIX_RANK = 2, VREN_TUNE_RADIX_ITEMS = 3,
       VREN_TUNE_SCAN_STAGED = 4, VREN_TUNE_REDUCE_FORM = 5, VREN_TUNE_LIGHT_BVH_CLUSTER = 6,
       VREN_TUNE_ASSIGN_FUSED = 7, VREN_TUNE_RADIX_PERSISTENT = 8, VREN_TUNE_FUC_FUSED = 9, VREN_TUNE_BUCKET_FORM = 10,
       VREN_TUNE_HOST_ZERO_COPY = 11, VREN_TUNE_SHADE_PACKED = 12, VREN_TUNE_COUNT = 13 };
int vren_tuning_set(int knob, int value);
int vren_tuning_get(int knob);

/* ------------------------------------------------------------------------------------------------
 * Size helpers (vren/vren/base/base.hpp:32-79, integer restatements)
 * ------------------------------------------------------------------------------------------------ */
uint32_t vren_round_to_next_power_of_2(uint32_t v);     /* base.hpp:37-47; maps 0 to 0 */
uint32_t vren_round_to_next_power_of(uint32_t n, uint32_t base); /* base.hpp:69-74 */
uint32_t vren_divide_and_ceil(uint32_t value, uint32_t divider); /* base.hpp:76-79 */

/* ------------------------------------------------------------------------------------------------
 * Reduce — vren::reduce<T,Op> (reduce.hpp:15-49, vren/primitives/reduce.cpp:32-140, reduce.comp:50-86)
 *
 * The drop-in form writes the whole Blelloch up-sweep tree: with P = next power of two
 * of n, out[i] = Op over in[i-2^t+1 .. i] where t = min(trailing ones of i, log2 P),
 * elements at n..P-1 being the identity of Op (add 0, uint min ~0u, uint max 0,
 * vec4 min 1e35, vec4 max -1e35; VRen.cmake:70-75).  out[P-1] is the total.
 * `blocks` independent segments: segment b reads in[b*n ..] and writes out[b*P ..].
 * `in` may equal `out` (the in-place form, reduce.hpp:39-46).  Float addition follows the
 * same pairwise tree, so results are bit-identical to the reference's tree order.
 * ------------------------------------------------------------------------------------------------ */
enum { VREN_REDUCE_ADD = 0, VREN_REDUCE_MIN = 1, VREN_REDUCE_MAX = 2 };

uint32_t vren_calc_reduce_output_buffer_length(uint32_t count);          /* vren/primitives/reduce.cpp:137-140 */
int vren_reduce_tree_u32(vren_stream_t s, int op, const uint32_t* in, uint32_t n,
                         uint32_t* out, uint32_t blocks);
int vren_reduce_tree_vec4(vren_stream_t s, int op, const float* in /* vec4[n] */, uint32_t n,
                          float* out /* vec4[P] */, uint32_t blocks);

/* Scalar reductions (a new, single-pass form used by the benchmark sweep).  The u32 sum
 * wraps modulo 2^32; min/max are exact in any order.  `out` is one element in device
 * memory.  n = 0 writes the identity. */
size_t vren_reduce_scratch_bytes(uint32_t n);
int vren_reduce_u32(vren_stream_t s, int op, const uint32_t* in, uint32_t n, uint32_t* out,
                    void* scratch);
int vren_reduce_f32(vren_stream_t s, int op, const float* in, uint32_t n, float* out,
                    void* scratch);

/* ------------------------------------------------------------------------------------------------
 * Exclusive scan — vren::blelloch_scan (blelloch_scan.hpp:9-49, vren/primitives/blelloch_scan.cpp:57-166)
 *
 * In-place exclusive prefix sum of uint32 (mod 2^32) over `blocks` independent segments
 * of length n.  The reference requires n to be a power of two (vren/primitives/blelloch_scan.cpp:67);
 * this implementation accepts any n (a power of two gives the reference's result).
 * Single pass with decoupled look-back.
 * ------------------------------------------------------------------------------------------------ */
size_t vren_exclusive_scan_scratch_bytes(uint32_t n, uint32_t blocks);
int vren_exclusive_scan_u32(vren_stream_t s, uint32_t* data, uint32_t n, uint32_t blocks,
                            void* scratch);

/* Same result as vren_exclusive_scan_u32, for callers that cannot provide scratch memory (an
 * engine allocator that owns all device memory, a plugin without access to an allocator, a frame
 * loop that must not call cudaMalloc): no counterpart in the reference.  Allocates nothing; the
 * look-back scratch is a fixed 32 KiB device array inside the library, so n * blocks must not
 * exceed 2^24 elements (VREN_ERR_CAPACITY otherwise).  Calls share that array: calls that overlap
 * on the GPU race and must be serialised by the caller.  The first call on a device resolves the
 * array's address and should come before any stream capture. */
int vren_exclusive_scan_u32_noalloc(vren_stream_t s, uint32_t* data, uint32_t n, uint32_t blocks);

/* The reference's public down-sweep (vren/primitives/blelloch_scan.cpp:57-139) applied to a buffer that
 * holds an up-sweep tree: n must be a power of two.  For n >= 1024 the root value is
 * kept unless `clear_last`; for n < 1024 the reference's single work-group pass always
 * propagates zero into the root, and so does this one. */
int vren_scan_downsweep_u32(vren_stream_t s, uint32_t* data, uint32_t n, uint32_t blocks,
                            int clear_last);

/* ------------------------------------------------------------------------------------------------
 * Radix sort — vren::radix_sort (radix_sort.hpp:9-53, vren/primitives/radix_sort.cpp:149-338)
 *
 * Stable ascending LSD sort of uint32 keys, in place, onesweep (one histogram kernel
 * then one kernel per digit with decoupled look-back).  scratch1 is this
 * implementation's histogram/status region (size from vren_radix_sort_scratch1_bytes),
 * scratch2 holds n keys (the reference's create_scratch_buffer_2, vren/primitives/radix_sort.cpp:138-147).
 *
 * vren_radix_sort_u32 is the drop-in: it keeps the reference's precondition (n >= 1024
 * and a power of two, else VREN_ERR_ARG — vren/primitives/radix_sort.cpp:158-161).  The _ex form sorts
 * any n, optionally carries a uint32 value per key (scratch_values holds n values), and
 * takes the digit width (4, 6 or 8 bits).
 * ------------------------------------------------------------------------------------------------ */
size_t vren_radix_sort_scratch1_bytes(uint32_t n, uint32_t digit_bits);
int vren_radix_sort_u32(vren_stream_t s, uint32_t* keys, uint32_t n, void* scratch1,
                        uint32_t* scratch2);
int vren_radix_sort_u32_ex(vren_stream_t s, uint32_t* keys, uint32_t* values, uint32_t n,
                           uint32_t digit_bits, void* scratch1, uint32_t* scratch_keys,
                           uint32_t* scratch_values);

/* ------------------------------------------------------------------------------------------------
 * Bucket sort — vren::bucket_sort (bucket_sort.hpp:9-45, vren/primitives/bucket_sort.cpp:72-161)
 *
 * Groups uvec2(key, value) elements by (key & (2^key_bits - 1)).  The reference uses
 * key_bits = 16 and global atomics (so its order within a bucket is unspecified); this
 * one is stable, which is one of the reference's possible outputs.  `out` holds
 * vren_bucket_sort_output_bytes(n, key_bits): the n sorted elements, then at byte offset
 * round_up(8n, 256) the 2^key_bits bucket END offsets (inclusive prefix of the counts),
 * which is what the reference leaves in its counter region after the call
 * (vren/primitives/bucket_sort.cpp:116-121, 134-142, bucket_sort_write.comp:32).
 * ------------------------------------------------------------------------------------------------ */
size_t vren_bucket_sort_output_bytes(uint32_t n, uint32_t key_bits);
size_t vren_bucket_sort_scratch_bytes(uint32_t n, uint32_t key_bits);
int vren_bucket_sort_u32x2(vren_stream_t s, const uint32_t* in /* uvec2[n] */, uint32_t n,
                           void* out, uint32_t key_bits, void* scratch);

/* ------------------------------------------------------------------------------------------------
 * BVH — vren::build_bvh (build_bvh.hpp:8-57, vren/primitives/build_bvh.cpp:38-136, build_bvh.comp:32-55)
 *
 * 32-ary bottom-up tree stored level after level: leaves [0, P), then P/32 parents, ...,
 * the root last.  A parent's next = index of its first child, or VREN_BVH_INVALID_NODE
 * when all 32 children are invalid; its AABB is the min/max over its valid children
 * (+inf/-inf when none).  `pad` of parents is written 0.
 * ------------------------------------------------------------------------------------------------ */
#define VREN_BVH_LEAF_NODE 0xFFFFFFFFu
#define VREN_BVH_INVALID_NODE 0xFFFFFFFEu

typedef struct vren_bvh_node {
    float min[3];
    uint32_t next;
    float max[3];
    uint32_t pad;
} vren_bvh_node;

uint32_t vren_calc_bvh_padded_leaf_count(uint32_t leaf_count);  /* vren/primitives/build_bvh.cpp:101-104 */
uint32_t vren_calc_bvh_buffer_length(uint32_t leaf_count);      /* vren/primitives/build_bvh.cpp:106-118 */
size_t vren_calc_bvh_buffer_size(uint32_t leaf_count);          /* vren/primitives/build_bvh.cpp:120-124 */
uint32_t vren_calc_bvh_root_index(uint32_t leaf_count);         /* vren/primitives/build_bvh.cpp:126-130 */
uint32_t vren_calc_bvh_level_count(uint32_t leaf_count);        /* vren/primitives/build_bvh.cpp:132-136 */
int vren_build_bvh(vren_stream_t s, vren_bvh_node* bvh, uint32_t padded_leaf_count);

/* Karras binary radix tree (extension beside the reference's 32-ary BuildBVH; T. Karras, "Maximizing
 * Parallelism in the Construction of BVHs, Octrees, and k-d Trees", HPG 2012).  Built over n leaves
 * already sorted by key: `sorted_pairs` = uvec2(key, payload)[n] in ascending key order (e.g. the
 * light index of vren_cs_construct_light_bvh, keys = 15- or 30-bit Morton codes); equal keys are
 * ordered by leaf position.  Node 0 is the root of the n - 1 internal nodes; a child index with
 * VREN_LBVH_LEAF set names leaf position (index & ~VREN_LBVH_LEAF).  Leaf i's box is
 * boxes[i >> box_shift] (box_shift 0: one box per leaf; 5 with boxes = level 1 of a 32-ary BVH: the
 * box of the leaf's 32-leaf group), or an infinite box when boxes is NULL; internal boxes are unions
 * in IEEE total order, so the tree is deterministic.  Scratch: vren_lbvh_scratch_bytes(n), no
 * initialisation needed.  n <= 2^24; n < 2 writes nothing. */
#define VREN_LBVH_LEAF 0x80000000u
typedef struct vren_lbvh_node {
    float min[3];
    uint32_t left;
    float max[3];
    uint32_t right;
} vren_lbvh_node;
size_t vren_lbvh_scratch_bytes(uint32_t leaf_count);
int vren_build_lbvh(vren_stream_t s, const uint32_t* sorted_pairs, uint32_t leaf_count, const vren_bvh_node* boxes,
                    uint32_t box_shift, vren_lbvh_node* nodes, void* scratch);


/* ------------------------------------------------------------------------------------------------
 * Clustered shading — vren::clustered_shading::{construct_point_light_bvh, find_unique_cluster_list,
 * assign_lights, shade} (vren/vren/pipeline/clustered_shading.hpp:13-141) and
 * vren::cluster_and_shade (clustered_shading.hpp:147-182, clustered_shading.cpp:817-1172).
 *
 * Data layouts (device memory, as in the reference):
 *   light positions  vec4[L], world space, w ignored        (light.hpp:27, light.cpp:11-21)
 *   point lights     {vec3 color; float intensity}[L]       (gpu_repr.hpp:61-64); intensity is
 *                    the light radius
 *   view positions   vec4[L]: view * vec4(p.xyz, 1)          (point_light_position_to_view_space.comp:30)
 *   light index      uvec2[L]: (morton code, light index), sorted by code, ties by light index
 *   BVH              vren_bvh_node[vren_calc_bvh_buffer_length(L)]
 *   depth            f32[W*H] NDC depth in [0, 1], row-major   (the reference's D32 depth buffer)
 *   normals          f32x3[W*H], or the reference's G-buffer format RGBA16F (half x4 per pixel,
 *                    gbuffer.cpp:7-12; w ignored), chosen by the frame's normal_format
 *   cluster keys     u32[U]: i | j << 8 | k << 16 | normal << 26 (find_unique_clusters.comp:72-76)
 *   cluster refs     u32[W*H]: index of the pixel's key in the key list
 *   counts/offsets   u32[U]; indices u32[sum(counts)]        (assign_lights.comp:57-70)
 *
 * Canonical semantics where the reference is nondeterministic or implementation-defined (the main
 * ones): key lists are ordered by tile (row-major) then ascending key; texels are
 * fetched at integer coordinates (x mod W, y mod H) like the reference's REPEAT sampler, or
 * skipped; depth slices come from a boundary table built on the host; light ties sort by index;
 * invalid BVH nodes are never traversed or assigned; float arithmetic follows a fixed order of
 * correctly rounded single-precision operations.
 * ------------------------------------------------------------------------------------------------ */
#define VREN_CS_SLICES 1024
enum { VREN_CS_SLICING_REF = 0, VREN_CS_SLICING_FIXED32 = 1 };
enum { VREN_CS_OFFSCREEN_WRAP = 0, VREN_CS_OFFSCREEN_SKIP = 1 };
/* Normal buffer formats: f32x3 per pixel, or the reference's G-buffer RGBA16F (half x4 per pixel,
 * converted exactly to float, so the keys equal those of the f32x3 normals holding the same values). */
enum { VREN_CS_NORMALS_F32X3 = 0, VREN_CS_NORMALS_RGBA16F = 1 };

/* vren::camera (vren/vren/camera.hpp:14-33) */
typedef struct vren_camera {
    float position[3];
    float yaw, pitch;
    float fov_y, aspect_ratio, near_plane, far_plane;
} vren_camera;

/* Camera-derived matrices, column-major m[c*4 + r] like glm. */
typedef struct vren_cs_view {
    float view[16];      /* world -> view (camera.cpp:32-38) */
    float inv_proj[16];  /* inverse of the projection (camera.cpp:40-50) */
    float inv_view[16];  /* view -> world */
    float eye[3];        /* camera position in world space */
    float near_plane, far_plane, half_fov_y;
    uint32_t slicing;    /* VREN_CS_SLICING_* */
    uint32_t reserved;
} vren_cs_view;

/* Per-frame parameter block that the kernels read from device memory (8448 bytes).
 * slice_near[k] / slice_far[k] are the view-space depth bounds of slice k:
 *   REF:     near * a^k and near * a^(k+1), a = 1 + 2 tan(fov_y/2) / tiles_y (find_unique_clusters.comp:65,
 *            clustered_shading.glsl:99-101), a^k by repeated double multiplication, rounded to float;
 *   FIXED32: near * (far/near)^(k/32) for k <= 32, +inf beyond (max_slice = 31).
 * A pixel at view depth z falls in the largest slice k <= max_slice with slice_near[k] <= z (0 if none). */
typedef struct vren_cs_frame {
    vren_cs_view view;
    uint32_t width, height, tiles_x, tiles_y;
    uint32_t max_slice;
    uint32_t offscreen;      /* VREN_CS_OFFSCREEN_* */
    uint32_t normal_format;  /* VREN_CS_NORMALS_* (vren_cs_frame_build sets F32X3) */
    uint32_t reserved;
    float slice_near[VREN_CS_SLICES];
    float slice_far[VREN_CS_SLICES];
} vren_cs_frame;

/* Host: matrices of a vren::camera (computed in double, rounded to float). */
void vren_cs_view_from_camera(const vren_camera* camera, uint32_t slicing, vren_cs_view* out);
/* Host: fills a frame block (slice tables included). */
int vren_cs_frame_build(const vren_cs_view* view, uint32_t width, uint32_t height, int offscreen,
                        vren_cs_frame* out);
/* Stream-ordered copy of a host frame block into device memory (a kernel launch carrying the block
 * by value, so it can be captured in a CUDA graph). */
int vren_cs_frame_upload(vren_stream_t s, const vren_cs_frame* host_frame, vren_cs_frame* device_frame);

/* construct_point_light_bvh (clustered_shading.cpp:60-346): view transform, min/max, 15-bit Morton
 * codes (discretize_point_light_positions.comp:30-39; morton_bits = 30 selects 10 bits per axis),
 * stable sort by code, leaves = AABB(view position +- intensity) (init_light_array_bvh.comp:42-65),
 * BuildBVH.  `leaf_spheres` (optional, vec4[padded leaf count]) receives, per leaf, the light's view
 * position and the radius the traversal tests, (max.x - min.x) / 2 (assign_lights.comp:214); invalid
 * leaves get radius -1.  light_count = 0 writes nothing. */
size_t vren_cs_light_bvh_scratch_bytes(uint32_t light_count, uint32_t morton_bits);
int vren_cs_construct_light_bvh(vren_stream_t s, const float* light_positions, const float* point_lights,
                                uint32_t light_count, const vren_cs_frame* frame, uint32_t morton_bits,
                                float* view_positions, vren_bvh_node* bvh, uint32_t* light_index,
                                float* leaf_spheres, void* scratch);

/* Point-light bouncer (vren_demo: bounce_point_lights.comp:33-73, point_light_bouncer.cpp:17-57), the
 * per-frame producer of the positions construct_point_light_bvh reads.  In place, per light: the
 * position (vec4, w written 1) is clamped into [aabb_min, aabb_max], then moves speed * dt along the
 * direction (vec4, w written 0), reflecting the direction components of the faces it reaches, at
 * most 32 bounces.  Every operation rounded on its own, IEEE division, GLSL min/max.  Both arrays
 * 16-byte aligned; aabb_min / aabb_max are 3 host floats. */
int vren_bounce_point_lights(vren_stream_t s, float* light_positions, float* light_directions, uint32_t light_count,
                             const float* aabb_min, const float* aabb_max, float speed, float dt);

/* ---- depth-buffer pyramid (vren/vren/pipeline/depth_buffer_pyramid.hpp) ---------------------------
 * Level count floor(log2(max(width, height))) + 1 (depth_buffer_pyramid.cpp:18), level l is
 * max(width >> l, 1) x max(height >> l, 1) texels (:48-54).  Levels are stored back to back in one
 * float buffer, each row-major with a row pitch of its width, starting at
 * vren_depth_pyramid_level_offset(width, height, l) floats (multiples of 64); level == level count
 * gives the buffer length in floats.  Sides of 1..65535 texels (16 levels at most); 0 otherwise. */
uint32_t vren_depth_pyramid_level_count(uint32_t width, uint32_t height);
size_t vren_depth_pyramid_level_offset(uint32_t width, uint32_t height, uint32_t level);
size_t vren_depth_pyramid_scratch_bytes(uint32_t width, uint32_t height);

/* depth_buffer_reductor::copy_and_reduce (depth_buffer_pyramid.cpp:212-303; depth_buffer_copy.comp,
 * depth_buffer_reduce.comp): level 0 = an exact copy of the row-major width x height depth buffer;
 * each texel above = GLSL max folded from 0 over the 2x2 texels of the level below that lie inside it
 * (NaN never enters, so texels above level 0 are +0 or positive).  One launch.  Both pointers 4-byte
 * aligned (16-byte aligned with width % 4 == 0 takes 128-bit accesses); scratch sized by
 * vren_depth_pyramid_scratch_bytes, zero-filled before first use, left reusable. */
int vren_depth_pyramid_copy_and_reduce(vren_stream_t s, const float* depth_buffer, uint32_t width, uint32_t height,
                                       float* pyramid, void* scratch);

/* find_unique_cluster_list (clustered_shading.cpp:363-448, find_unique_clusters.comp:46-120).
 * key_count receives the number of keys written (the reference's dispatch_params.x); a list longer
 * than key_capacity is truncated and VREN_ERR_CAPACITY recorded.  tiles_x*tiles_y*1024 keys always fit.
 * The scratch holds every tile's sorted keys, key count and offset (about 4 KiB per tile; no
 * initialisation needed); calls sharing a scratch must not overlap. */
size_t vren_cs_unique_clusters_scratch_bytes(uint32_t width, uint32_t height);
int vren_cs_find_unique_clusters(vren_stream_t s, const float* depth, const float* normals, uint32_t width,
                                 uint32_t height, const vren_cs_frame* frame, uint32_t* cluster_keys,
                                 uint32_t key_capacity, uint32_t* key_count, uint32_t* cluster_refs,
                                 void* scratch);

/* assign_lights (clustered_shading.cpp:473-690, assign_lights.comp:121-240): per cluster, the lights
 * whose sphere overlaps the cluster box, in the reference's order (BVH leaf groups in ascending
 * order, lanes of a group in descending order).  counts/offsets have key_capacity entries, the
 * first *key_count of which are written; `total` (optional) receives the number of assignments;
 * indices beyond index_capacity are dropped and VREN_ERR_CAPACITY recorded.  `leaf_spheres` is
 * optional (from vren_cs_construct_light_bvh); without it the leaf data are read from the BVH,
 * the light index and the view positions as the reference does.  Count kernel, exclusive scan and
 * write kernel (clusters with no light skip the second traversal); VREN_TUNE_ASSIGN_FUSED selects
 * one kernel in which a warp per cluster counts, resolves its first index by decoupled look-back over
 * the preceding clusters' counts, then writes.  The scratch (vren_cs_assign_lights_scratch_bytes)
 * must be zero-filled before its first use (and again after VREN_ERR_TIMEOUT); calls sharing it must
 * not overlap. */
size_t vren_cs_assign_lights_scratch_bytes(uint32_t key_capacity);
int vren_cs_assign_lights(vren_stream_t s, const uint32_t* cluster_keys, const uint32_t* key_count,
                          uint32_t key_capacity, const vren_cs_frame* frame, const vren_bvh_node* bvh,
                          uint32_t light_count, const uint32_t* light_index, const float* view_positions,
                          const float* leaf_spheres, uint32_t* counts, uint32_t* offsets, uint32_t* indices,
                          uint32_t index_capacity, uint32_t* total, void* scratch);

/* assign_lights through a Karras tree (extension): the same counts, offsets and index lists as
 * vren_cs_assign_lights on the same light BVH, when `nodes` was built by vren_build_lbvh over the
 * group boxes (boxes = the BVH's level 1, box_shift = 5; boxes = NULL for at most 32 lights).  The
 * reference's traversal tests the boxes of a light's ancestors and then its sphere; its box test is
 * monotone in box inclusion, so a light is assigned exactly when its 32-leaf group box and its sphere
 * overlap the cluster box, which is what this traversal tests, one cluster per thread, writing each
 * group's lights in the reference's order (groups ascending, lanes descending).  `bvh` supplies the
 * leaf boxes (and with `leaf_spheres` NULL, the radii); the other arguments are vren_cs_assign_lights'. */
int vren_cs_assign_lights_lbvh(vren_stream_t s, const uint32_t* cluster_keys, const uint32_t* key_count,
                               uint32_t key_capacity, const vren_cs_frame* frame, const vren_lbvh_node* nodes,
                               const vren_bvh_node* bvh, uint32_t light_count, const uint32_t* light_index,
                               const float* view_positions, const float* leaf_spheres, uint32_t* counts,
                               uint32_t* offsets, uint32_t* indices, uint32_t index_capacity, uint32_t* total,
                               void* scratch);

/* shade (clustered_shading.cpp:696-811, shade.comp:69-141, pbr.glsl:6-112): per on-screen pixel
 * whose view depth is below far - 0.001, Cook-Torrance/GGX over the lights of its cluster plus the
 * directional lights (the reference's constants: PI = 3.14, NDF with a = roughness, Smith with
 * k = roughness); VREN_CS_SHADE_COLOR adds 0.03 * albedo and applies pow(1/2.2) like the
 * reference, VREN_CS_SHADE_RADIANCE writes the point-light sum only (the quantity the adjoint
 * differentiates).  Falloff: VREN_CS_FALLOFF_REF = 1 - min(d/r, 1)^1.5 (pbr.glsl:89);
 * VREN_CS_FALLOFF_WINDOWED_INV_SQ = saturate(1 - (d/r)^4)^2 / (d^2 + 1) (Karis 2013).
 * Pixels that are not shaded are left untouched (the reference does not store them). */
enum { VREN_CS_FALLOFF_REF = 0, VREN_CS_FALLOFF_WINDOWED_INV_SQ = 1 };
enum { VREN_CS_SHADE_COLOR = 0, VREN_CS_SHADE_RADIANCE = 1 };

typedef struct vren_cs_gbuffer {
    const float* depth;     /* f32[W*H], NDC depth */
    const float* normals;   /* f32x3[W*H], world space */
    const float* albedo;    /* f32x3[W*H] */
    const float* roughness; /* f32[W*H] */
    const float* metallic;  /* f32[W*H] */
} vren_cs_gbuffer;

/* index_capacity: the entries `indices` holds (the assignment's index capacity).  After an assignment
 * that ran out of index capacity (VREN_ERR_CAPACITY), counts and offsets describe lists that reach
 * past it: the shading kernels cut every list there instead of reading beyond the buffer (and record
 * VREN_ERR_CAPACITY again).  Must be non-zero when lights are shaded. */
typedef struct vren_cs_light_lists {
    const uint32_t* cluster_refs; /* u32[W*H] */
    const uint32_t* counts;       /* per cluster */
    const uint32_t* offsets;      /* per cluster */
    const uint32_t* indices;      /* light indices */
    uint32_t index_capacity;      /* entries of indices */
    uint32_t reserved;
} vren_cs_light_lists;

/* directional_lights: {float direction[3], pad, color[3], pad}[count] (gpu_repr.hpp:66-70) */
int vren_cs_shade(vren_stream_t s, const vren_cs_frame* frame, uint32_t width, uint32_t height,
                  const vren_cs_gbuffer* gbuffer, const vren_cs_light_lists* lists, const float* light_positions,
                  const float* point_lights, uint32_t light_count, const float* directional_lights,
                  uint32_t directional_count, int falloff, int output_mode, float* out_rgb /* f32x3[W*H] */);

/* Adjoint of VREN_CS_SHADE_RADIANCE (no counterpart in the reference): given the upstream gradient
 * G (f32x3[W*H]) of a scalar loss with respect to the radiance image, writes dLoss/d(light
 * position) (f32x3[L]), dLoss/d(light colour) (f32x3[L]) and dLoss/d(light radius) (f32[L]), the
 * light-to-cluster assignment being held fixed.  Per-light terms are recomputed, nothing per
 * (pixel, light) pair is stored: one CTA per 32x32 tile sums each of its (cluster, light) slots
 * over the tile's pixels in a fixed order, the slots are grouped by light with the stable bucket
 * sort, and each light's slots are summed in slot order — the result is deterministic.
 * `assignments` is the number of assigned (cluster, light) pairs (the `total` output of
 * vren_cs_assign_lights, read on the host); light_count <= 65536. */
size_t vren_cs_shade_backward_scratch_bytes(uint32_t light_count, uint32_t assignments);
int vren_cs_shade_backward(vren_stream_t s, const vren_cs_frame* frame, uint32_t width, uint32_t height,
                           const vren_cs_gbuffer* gbuffer, const vren_cs_light_lists* lists, uint32_t assignments,
                           const float* light_positions, const float* point_lights, uint32_t light_count,
                           int falloff, const float* grad_radiance, float* grad_positions, float* grad_colors,
                           float* grad_radii, void* scratch);

/* vren::cluster_and_shade: owns its buffers (an arena sized at creation) and runs the stages above
 * for one frame.  With a non-default stream the sequence is captured once into a CUDA graph per
 * frame shape and replayed. */
typedef struct vren_cluster_and_shade vren_cluster_and_shade;

/* ---- k-d tree (vren/vren/base/kd_tree.hpp) --------------------------------------------------------
 * vren::kd_tree_node: 12 bytes (the reference's 2-bit axis field and the union of 30-bit fields after
 * it occupy separate words).  axis 0..2 = inner node splitting at `split`, right child `value` nodes
 * after it, left child next; axis 3 = leaf holding point `index`, the first leaf of a run has
 * value = run length, the others 0x3FFFFFFF. */
typedef struct vren_kd_tree_node {
    union {
        float split;
        uint32_t index;
    };
    uint32_t axis;
    uint32_t value;
} vren_kd_tree_node;

/* Returns nonzero to accept `point` (the reference's kd_tree_search_filter_t). */
typedef int (*vren_kd_tree_filter)(uint32_t point, void* user);

/* kd_tree_build (vren/base/kd_tree.cpp:5-78), on the host: same node array as the reference (pre-order, Welford
 * mean split on the axis its variance test picks, in-place swap partition of `indices`).  Returns the
 * offset after the last node written (the node count for node_offset = 0; at most 2 * count).  A node
 * whose split separates nothing (where the reference asserts) becomes one leaf run of all its points. */
size_t vren_kd_tree_build(const float* points, size_t point_stride, uint32_t* indices, size_t count,
                          vren_kd_tree_node* kd_tree, size_t node_offset, size_t max_leaf_point_count);
/* Inner nodes on the longest root-to-leaf path (host). */
uint32_t vren_kd_tree_depth(const vren_kd_tree_node* kd_tree, size_t node_offset);
/* kd_tree_search (vren/base/kd_tree.cpp:80-129), on the host: best_point / best_distance_squared are in-out (start
 * them at UINT32_MAX / +inf); filter NULL accepts every point. */
void vren_kd_tree_search(const float* points, size_t point_stride, const uint32_t* indices, size_t count,
                         const vren_kd_tree_node* kd_tree, size_t node_offset, const float* sample,
                         vren_kd_tree_filter filter, void* filter_user, uint32_t* best_point,
                         float* best_distance_squared);
/* The same search for many samples on the GPU (device pointers; one thread per sample), same visit
 * order and so the same results, ties included, as the host search started at UINT32_MAX / +inf.
 * excluded (optional, one byte per point, nonzero = filtered out) stands for the filter.  max_depth
 * (vren_kd_tree_depth) above 128 returns VREN_ERR_CAPACITY. */
int vren_kd_tree_search_batch(vren_stream_t s, const float* points, uint32_t point_stride, uint32_t point_count,
                              const vren_kd_tree_node* kd_tree, uint32_t node_count, uint32_t max_depth,
                              const float* samples, uint32_t sample_stride, uint32_t sample_count,
                              const uint8_t* excluded, uint32_t* best_points, float* best_distances_squared);

/* ---- headless cluster debug views (vren_demo/vren_demo/clustered_shading_debug.cpp:6-200) ---------- */
#define VREN_SHOW_CLUSTERS_KEY 0
#define VREN_SHOW_CLUSTERS_IJK 1
#define VREN_SHOW_CLUSTERS_NORMAL 2
#define VREN_SHOW_CLUSTERS_LIGHT_COUNTS 3
#define VREN_SHOW_CLUSTERS_LIGHT_OFFSETS 4
#define VREN_SHOW_CLUSTERS_LIGHT_INDICES 5

/* vren::debug_renderer_vertex (vren/vren/pipeline/debug_renderer.hpp:25-31): 16 bytes. */
typedef struct vren_debug_vertex {
    float position[3];
    uint32_t color; /* 0xRRGGBB */
} vren_debug_vertex;

/* show_clusters (show_clusters.comp:68-125): rgba (float4 per pixel, row-major width x height,
 * 16-byte aligned) = the colour of each pixel's cluster for `mode` (VREN_SHOW_CLUSTERS_*; any other
 * value draws red, as the shader does); tiles = ceil(size / 32) as in clustered_shading_debug.cpp:68-71.
 * A reference >= min(*key_count, max_clusters) is drawn magenta (the shader reads out of bounds).
 * counts/offsets are needed by the light modes, indices by LIGHT_INDICES; index_capacity = the
 * entries `indices` holds (lists reaching past it, after an assignment that ran out of capacity, are
 * cut there and VREN_ERR_CAPACITY recorded).  scratch: 16-byte aligned,
 * vren_cs_show_clusters_scratch_bytes(max_clusters). */
size_t vren_cs_show_clusters_scratch_bytes(uint32_t max_clusters);
int vren_cs_show_clusters(vren_stream_t s, int mode, uint32_t width, uint32_t height, const uint32_t* cluster_refs,
                          const uint32_t* cluster_keys, const uint32_t* key_count, uint32_t max_clusters,
                          const uint32_t* counts, const uint32_t* offsets, const uint32_t* indices,
                          uint32_t index_capacity, float* rgba, void* scratch);
/* show_clusters_geometry (show_clusters_geometry.comp:55-110, debug.glsl): for each of the first
 * min(*key_count, max_clusters) clusters, 32 vertices at vertices[32 c]: its view-space box as 12 lines
 * (white; black for keys without a normal bin) and an arrow of length 0.01 along its normal bin (green
 * shaft, red head; zero length without a bin).  The box is the one the light assignment tests. */
int vren_cs_show_clusters_geometry(vren_stream_t s, const vren_cs_frame* frame, const uint32_t* cluster_keys,
                                   const uint32_t* key_count, uint32_t max_clusters, vren_debug_vertex* vertices);

typedef struct vren_cs_outputs {
    const float* view_positions;
    const vren_bvh_node* bvh;
    const uint32_t* light_index;
    const float* leaf_spheres;
    const uint32_t* cluster_keys;
    const uint32_t* key_count;
    const uint32_t* cluster_refs;
    const uint32_t* counts;
    const uint32_t* offsets;
    const uint32_t* indices;
    const uint32_t* total;
    const vren_cs_frame* frame;
    uint32_t key_capacity;
    uint32_t index_capacity;
} vren_cs_outputs;

typedef struct vren_cs_options {
    uint32_t morton_bits;     /* 15 (reference) or 30 */
    uint32_t use_graph;       /* capture/replay a CUDA graph on non-default streams */
    uint32_t sort_digit_bits; /* 4, 6 or 8: digit width of the light sort */
    uint32_t assign_warps;    /* warps per CTA of the traversal kernels (1..32) */
    uint32_t normal_format;   /* VREN_CS_NORMALS_* of the normals passed to vren_cs_cluster(_host) */
} vren_cs_options;

int vren_cs_create(vren_cluster_and_shade** out, uint32_t max_width, uint32_t max_height, uint32_t max_lights,
                   uint32_t max_assignments);
void vren_cs_destroy(vren_cluster_and_shade* cs);
int vren_cs_set_options(vren_cluster_and_shade* cs, const vren_cs_options* options);
/* Runs construct_point_light_bvh, find_unique_cluster_list and assign_lights for one frame. */
int vren_cs_cluster(vren_cluster_and_shade* cs, vren_stream_t s, const vren_cs_view* view, uint32_t width,
                    uint32_t height, int offscreen, const float* depth, const float* normals,
                    const float* light_positions, const float* point_lights, uint32_t light_count);
int vren_cs_get_outputs(const vren_cluster_and_shade* cs, vren_cs_outputs* out);
/* cluster_and_shade::operator() (clustered_shading.cpp:924-1172): the three clustering stages of
 * vren_cs_cluster, then shade over the context's own light lists (the reference's m_shade call,
 * clustered_shading.cpp:1153-1168), in one CUDA graph of the context per frame shape (replayed on a
 * non-default stream when use_graph is set).  gbuffer->depth and gbuffer->normals are also the
 * clustering inputs, so the context's normal format must be VREN_CS_NORMALS_F32X3 (else
 * VREN_ERR_ARG).  Shading as vren_cs_shade: out_rgb is f32x3[W*H], pixels that are not shaded are
 * left untouched.  The clustering outputs are those of vren_cs_cluster on the same inputs. */
int vren_cs_cluster_and_shade(vren_cluster_and_shade* cs, vren_stream_t s, const vren_cs_view* view,
                              uint32_t width, uint32_t height, int offscreen, const vren_cs_gbuffer* gbuffer,
                              const float* light_positions, const float* point_lights, uint32_t light_count,
                              const float* directional_lights, uint32_t directional_count, int falloff,
                              int output_mode, float* out_rgb);
/* vren_cs_cluster for a frame held in page-locked host memory (no counterpart in the reference, whose
 * G-buffer is rendered on the GPU).  The lights are uploaded and their BVH built on a second stream
 * of the context while the depth and normals upload; when cluster_refs_out (page-locked, W*H) is
 * given, the references are downloaded while the light lists are assigned; when lists_out
 * (page-locked) is given, the device writes [U, total, keys[U], counts[U], offsets[U], indices[total]]
 * into it, cut at lists_capacity words (VREN_ERR_CAPACITY recorded).  The depth and normals upload in
 * bands of tile rows, each band's tiles starting as soon as it arrives.  The outputs are the same as
 * vren_cs_cluster's on the same data.  The first call allocates the context's input buffers and must
 * not be made during stream capture. */
int vren_cs_cluster_host(vren_cluster_and_shade* cs, vren_stream_t s, const vren_cs_view* view, uint32_t width,
                         uint32_t height, int offscreen, const float* depth, const float* normals,
                         const float* light_positions, const float* point_lights, uint32_t light_count,
                         uint32_t* cluster_refs_out, uint32_t* lists_out, uint64_t lists_capacity);

/* ------------------------------------------------------------------------------------------------
 * Batched cluster assignment (no counterpart in the reference, which runs one frame per
 * cluster_and_shade call).  Many independent frames - each with its own camera, resolution,
 * G-buffer and light set - go through one fixed kernel sequence (light view transform, Morton
 * codes, one stable sort of all frames' lights keyed by (frame, code), leaves and BVH levels,
 * unique clusters over all frames' tiles, traversal count, one scan, traversal write), replayed as
 * one CUDA graph.  Every frame's outputs are bit-identical to vren_cs_cluster on the same inputs
 * with the same morton bits (15 only; the 30-bit extension is per-frame only).
 * ------------------------------------------------------------------------------------------------ */
typedef struct vren_cs_batch vren_cs_batch;

typedef struct vren_cs_batch_frame {
    vren_cs_view view;
    uint32_t width, height;       /* <= 8192 each */
    uint32_t light_count;         /* <= 2^20 */
    int32_t offscreen;            /* VREN_CS_OFFSCREEN_* */
    uint32_t normal_format;       /* VREN_CS_NORMALS_* */
    uint32_t reserved;
    const float* depth;           /* device: float[W*H] NDC depth */
    const float* normals;         /* device: float[3*W*H] or half[4*W*H] (normal_format) */
    const float* light_positions; /* device: vec4[L], 16-byte aligned (null when L == 0) */
    const float* point_lights;    /* device: {rgb, radius}[L], 16-byte aligned */
} vren_cs_batch_frame;

typedef struct vren_cs_batch_options {
    uint32_t sort_digit_bits; /* 4, 6 or 8: digit width of the combined light sort */
    uint32_t radix_items;     /* radix tile variant (VREN_TUNE_RADIX_ITEMS) */
    uint32_t scan_slices;     /* scan tile variant (VREN_TUNE_SCAN_SLICES): 4 or 8 */
    uint32_t assign_warps;    /* warps per CTA of the traversal kernels (1..8) */
    uint32_t use_graph;       /* capture/replay one CUDA graph per batch shape (non-default streams) */
} vren_cs_batch_options;

int vren_cs_batch_create(vren_cs_batch** out);
void vren_cs_batch_destroy(vren_cs_batch* b);
/* Sizes the batch's device arena for these frames (allocates; call outside stream capture).
 * max_assignments bounds the light-index entries of all frames together. */
int vren_cs_batch_reserve(vren_cs_batch* b, const vren_cs_batch_frame* frames, uint32_t count,
                          uint64_t max_assignments);
int vren_cs_batch_set_options(vren_cs_batch* b, const vren_cs_batch_options* options);
int vren_cs_batch_get_options(const vren_cs_batch* b, vren_cs_batch_options* options);
/* Enqueues the batch on stream s (VREN_ERR_CAPACITY when it exceeds the reserved arena).  The
 * radix and scan tile variants of the options are applied to this batch's launches only.  Runs of
 * one batch object may be enqueued on different streams: when the frames' parameters change, the new
 * ones are uploaded after the previous upload has been read and the previous run (on whatever
 * stream) has ended.  The outputs of a run are overwritten by the next run of the same object. */
int vren_cs_batch_run(vren_cs_batch* b, vren_stream_t s, const vren_cs_batch_frame* frames, uint32_t count);
/* Times candidate option sets on these frames (digit bits x radix tile x scan tile x traversal
 * warps), keeps the fastest, and caches it per shape bucket (frame count, log2 of the total pixels
 * and of the total lights): a bucket seen before returns its cached choice without measuring.
 * Synchronizes s.  The chosen options are applied to the batch and written to *chosen. */
int vren_cs_batch_autotune(vren_cs_batch* b, vren_stream_t s, const vren_cs_batch_frame* frames, uint32_t count,
                           uint32_t reps, vren_cs_batch_options* chosen);
/* Device pointers of frame f's outputs from the last run (synchronizes s to read the per-frame
 * bases; offsets are frame-local and indices points at the frame's first index). */
int vren_cs_batch_frame_outputs(vren_cs_batch* b, vren_stream_t s, uint32_t f, vren_cs_outputs* out);

#ifdef __cplusplus
}
#endif

#endif /* VREN_GB300_H_ */

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
 * (radix_sort.cpp:212-215) and Vulkan failures with VREN_CHECK -> std::runtime_error
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

/* ------------------------------------------------------------------------------------------------
 * Size helpers (vren/vren/base/base.hpp:281-328, integer restatements)
 * ------------------------------------------------------------------------------------------------ */
uint32_t vren_round_to_next_power_of_2(uint32_t v);     /* base.hpp:286-296, 0 -> 0 */
uint32_t vren_round_to_next_power_of(uint32_t n, uint32_t base); /* base.hpp:318-323 */
uint32_t vren_divide_and_ceil(uint32_t value, uint32_t divider); /* base.hpp:325-328 */

/* ------------------------------------------------------------------------------------------------
 * Reduce — vren::reduce<T,Op> (reduce.hpp:15-49, reduce.cpp:82-190, reduce.comp:50-86)
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

uint32_t vren_calc_reduce_output_buffer_length(uint32_t count);          /* reduce.cpp:187-190 */
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
 * Exclusive scan — vren::blelloch_scan (blelloch_scan.hpp:9-49, blelloch_scan.cpp:107-216)
 *
 * In-place exclusive prefix sum of uint32 (mod 2^32) over `blocks` independent segments
 * of length n.  The reference requires n to be a power of two (blelloch_scan.cpp:117);
 * this implementation accepts any n (a power of two gives the reference's result).
 * Single pass with decoupled look-back.
 * ------------------------------------------------------------------------------------------------ */
size_t vren_exclusive_scan_scratch_bytes(uint32_t n, uint32_t blocks);
int vren_exclusive_scan_u32(vren_stream_t s, uint32_t* data, uint32_t n, uint32_t blocks,
                            void* scratch);

/* The reference's public down-sweep (blelloch_scan.cpp:107-189) applied to a buffer that
 * holds an up-sweep tree: n must be a power of two.  For n >= 1024 the root value is
 * kept unless `clear_last`; for n < 1024 the reference's single work-group pass always
 * propagates zero into the root, and so does this one. */
int vren_scan_downsweep_u32(vren_stream_t s, uint32_t* data, uint32_t n, uint32_t blocks,
                            int clear_last);

/* ------------------------------------------------------------------------------------------------
 * Radix sort — vren::radix_sort (radix_sort.hpp:9-53, radix_sort.cpp:178-392)
 *
 * Stable ascending LSD sort of uint32 keys, in place, onesweep (one histogram kernel
 * then one kernel per digit with decoupled look-back).  scratch1 is this
 * implementation's histogram/status region (size from vren_radix_sort_scratch1_bytes),
 * scratch2 holds n keys (the reference's create_scratch_buffer_2, radix_sort.cpp:192-201).
 *
 * vren_radix_sort_u32 is the drop-in: it keeps the reference's precondition (n >= 1024
 * and a power of two, else VREN_ERR_ARG — radix_sort.cpp:212-215).  The _ex form sorts
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
 * Bucket sort — vren::bucket_sort (bucket_sort.hpp:9-45, bucket_sort.cpp:114-208)
 *
 * Groups uvec2(key, value) elements by (key & (2^key_bits - 1)).  The reference uses
 * key_bits = 16 and global atomics (so its order within a bucket is unspecified); this
 * one is stable, which is one of the reference's possible outputs.  `out` holds
 * vren_bucket_sort_output_bytes(n, key_bits): the n sorted elements, then at byte offset
 * round_up(8n, 256) the 2^key_bits bucket END offsets (inclusive prefix of the counts),
 * which is what the reference leaves in its counter region after the call
 * (bucket_sort.cpp:114-117, 133, bucket_sort_write.comp:32).
 * ------------------------------------------------------------------------------------------------ */
size_t vren_bucket_sort_output_bytes(uint32_t n, uint32_t key_bits);
size_t vren_bucket_sort_scratch_bytes(uint32_t n, uint32_t key_bits);
int vren_bucket_sort_u32x2(vren_stream_t s, const uint32_t* in /* uvec2[n] */, uint32_t n,
                           void* out, uint32_t key_bits, void* scratch);

/* ------------------------------------------------------------------------------------------------
 * BVH — vren::build_bvh (build_bvh.hpp:8-57, build_bvh.cpp:95-193, build_bvh.comp:32-55)
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

uint32_t vren_calc_bvh_padded_leaf_count(uint32_t leaf_count);  /* build_bvh.cpp:158-161 */
uint32_t vren_calc_bvh_buffer_length(uint32_t leaf_count);      /* build_bvh.cpp:163-175 */
size_t vren_calc_bvh_buffer_size(uint32_t leaf_count);          /* build_bvh.cpp:177-181 */
uint32_t vren_calc_bvh_root_index(uint32_t leaf_count);         /* build_bvh.cpp:183-187 */
uint32_t vren_calc_bvh_level_count(uint32_t leaf_count);        /* build_bvh.cpp:189-193 */
int vren_build_bvh(vren_stream_t s, vren_bvh_node* bvh, uint32_t padded_leaf_count);

#ifdef __cplusplus
}
#endif

#endif /* VREN_GB300_H_ */

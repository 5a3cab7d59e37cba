// Host-side entry points shared between translation units of the library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/vren_gb300.h"

namespace vren_gb300 {

// Current value of a VREN_TUNE_* knob (capi.cu).
int tuning(int knob);

// Exclusive scan of min(*n_dev, n_cap) elements (n_cap when n_dev is null), in -> out (may alias);
// the total is written to *total_out when given.  Scratch: scan_scratch_bytes(n_cap), zero-filled
// before first use.
size_t scan_scratch_bytes(uint32_t n_cap);
int scan_exclusive_u32(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t n_cap, const uint32_t* n_dev,
                       uint32_t* total_out, void* scratch);

// Stable sort of uvec2 elements by (x & (2^key_bits - 1)), in -> out, through tmp (n elements).
size_t sort_uvec2_scratch_bytes(uint32_t n, uint32_t key_bits, uint32_t digit_bits);
int sort_uvec2(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t* tmp, uint32_t n, uint32_t key_bits,
               uint32_t digit_bits, void* scratch);

// Builds the BVH levels above `count` nodes that start at src_off (count a power of 32).
int build_bvh_levels(cudaStream_t st, vren_bvh_node* bvh, uint32_t src_off, uint32_t count);

}  // namespace vren_gb300

// C ABI support: status strings, device error word, wait limit and the integer size helpers of
// vren/vren/base/base.hpp:32-79.
#include "common.cuh"

#include <cmath>

namespace vren_gb300 {
uint32_t g_wait_limit = kDefaultWaitLimit;
}

using namespace vren_gb300;

// One error word per translation unit (see VREN_DEFINE_ERROR_WORD).
extern "C" int vren_internal_error_reduce(int clear);
extern "C" int vren_internal_error_scan(int clear);
extern "C" int vren_internal_error_radix(int clear);
extern "C" int vren_internal_error_bvh(int clear);
extern "C" int vren_internal_error_cs(int clear);
extern "C" int vren_internal_error_shade(int clear);
extern "C" int vren_internal_error_batch(int clear);
extern "C" int vren_internal_error_lbvh(int clear);
extern "C" int vren_internal_error_lights(int clear);
extern "C" int vren_internal_error_cluster_debug(int clear);
extern "C" int vren_internal_error_kd_tree(int clear);

extern "C" const char* vren_status_string(int status)
{
    switch (status) {
    case VREN_OK: return "ok";
    case VREN_ERR_ARG: return "invalid argument";
    case VREN_ERR_CAPACITY: return "capacity exceeded";
    case VREN_ERR_TIMEOUT: return "device wait timed out";
    case VREN_ERR_CUDA: return "CUDA runtime error";
    case VREN_ERR_STATE: return "invalid state";
    default: return "unknown status";
    }
}

extern "C" int vren_device_error(int clear)
{
    if (cudaDeviceSynchronize() != cudaSuccess) return VREN_ERR_CUDA;
    int (*const words[])(int) = {vren_internal_error_reduce, vren_internal_error_scan, vren_internal_error_radix,
                                 vren_internal_error_bvh, vren_internal_error_cs, vren_internal_error_shade,
                                 vren_internal_error_batch, vren_internal_error_lbvh,
                                 vren_internal_error_lights, vren_internal_error_cluster_debug,
                                 vren_internal_error_kd_tree};
    int first = 0;
    for (auto w : words) {
        int e = w(clear);
        if (e != 0 && first == 0) first = e;
    }
    return first;
}

namespace vren_gb300 {
// Kernel variant knobs (tile sizes, ranking method, polling policy), set by the autotuner or the
// caller; every launcher reads its knob when it enqueues work.
thread_local int g_pdl = 0;

static int g_tuning[VREN_TUNE_COUNT] = {
    /* VREN_TUNE_SCAN_SLICES */ 8,
    /* VREN_TUNE_SPIN_POLLS */ 64,
    /* VREN_TUNE_RADIX_RANK */ 0,
    /* VREN_TUNE_RADIX_ITEMS */ 0,
    /* VREN_TUNE_SCAN_STAGED */ 0,
    /* VREN_TUNE_REDUCE_FORM */ 0,
    /* VREN_TUNE_LIGHT_BVH_CLUSTER */ 1,
    /* VREN_TUNE_ASSIGN_FUSED */ 0,
    /* VREN_TUNE_RADIX_PERSISTENT */ 0,
    /* VREN_TUNE_FUC_FUSED */ 0,
    /* VREN_TUNE_BUCKET_FORM */ 0,
    /* VREN_TUNE_HOST_ZERO_COPY */ 0,
    /* VREN_TUNE_SHADE_PACKED */ 1,
};
int tuning(int knob) { return (knob >= 0 && knob < VREN_TUNE_COUNT) ? g_tuning[knob] : 0; }
}  // namespace vren_gb300

extern "C" int vren_tuning_set(int knob, int value)
{
    if (knob < 0 || knob >= VREN_TUNE_COUNT) return VREN_ERR_ARG;
    switch (knob) {
    case VREN_TUNE_SCAN_SLICES:
        if (value != 4 && value != 8) return VREN_ERR_ARG;
        break;
    case VREN_TUNE_SPIN_POLLS:
        if (value < 0 || value > (1 << 20)) return VREN_ERR_ARG;
        break;
    case VREN_TUNE_RADIX_RANK:
        if (value < 0 || value > 2) return VREN_ERR_ARG;
        break;
    case VREN_TUNE_RADIX_ITEMS:
        if (value != 0 && value != 1) return VREN_ERR_ARG;
        break;
    case VREN_TUNE_SCAN_STAGED:
        if (value < 0 || value > 3) return VREN_ERR_ARG;
        break;
    case VREN_TUNE_REDUCE_FORM:
        if (value < 0 || value > 5) return VREN_ERR_ARG;
        break;
    case VREN_TUNE_LIGHT_BVH_CLUSTER:
    case VREN_TUNE_FUC_FUSED:
    case VREN_TUNE_ASSIGN_FUSED:
        if (value < 0 || value > 2) return VREN_ERR_ARG;
        break;
    case VREN_TUNE_RADIX_PERSISTENT:
    case VREN_TUNE_BUCKET_FORM:
    case VREN_TUNE_HOST_ZERO_COPY:
    case VREN_TUNE_SHADE_PACKED:
        if (value != 0 && value != 1) return VREN_ERR_ARG;
        break;
    default: break;
    }
    g_tuning[knob] = value;
    return VREN_OK;
}

extern "C" int vren_tuning_get(int knob) { return tuning(knob); }

extern "C" uint32_t vren_set_wait_limit(uint32_t rounds)
{
    uint32_t prev = g_wait_limit;
    g_wait_limit = rounds ? rounds : kDefaultWaitLimit;
    return prev;
}

extern "C" uint32_t vren_round_to_next_power_of_2(uint32_t v)
{
    // Same bit trick as the reference: 0 maps to 0, values above 2^31 wrap to 0.
    v--;
    v |= v >> 1;
    v |= v >> 2;
    v |= v >> 4;
    v |= v >> 8;
    v |= v >> 16;
    v++;
    return v;
}

extern "C" uint32_t vren_round_to_next_power_of(uint32_t n, uint32_t base)
{
    // Smallest power of `base` that is >= n (the reference's ceil(log(n)/log(base)) in double,
    // restated with integers).  n = 0 gives 0 (the reference's pow(base, -inf)).
    if (base < 2) return 0;
    if (n == 0) return 0;
    uint64_t p = 1;
    while (p < n) p *= base;
    return p > 0xFFFFFFFFull ? 0u : (uint32_t)p;
}

extern "C" uint32_t vren_divide_and_ceil(uint32_t value, uint32_t divider)
{
    if (divider == 0) return 0;
    return (uint32_t)(((uint64_t)value + divider - 1) / divider);
}

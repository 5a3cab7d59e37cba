// Shared device/host helpers for the vren_gb300 kernels (sm_103a).
//
// Every translation unit of the library includes this header.  It provides:
//  - the per-TU device error word and the bounded-wait helper used by every
//    kernel that polls memory written by another CTA (decoupled look-back);
//  - acquire/release global-memory accessors written as inline PTX;
//  - correctly rounded float helpers for the paths that must be bit-identical
//    to the CPU oracle (no FMA contraction, no approximate division);
//  - launch/validation macros for the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vren_gb300.h"

namespace vren_gb300 {

constexpr int kNumSMsHint = 152;

// Host-side polling limit (number of rounds a device wait makes before giving up).
// One round is one load plus a __nanosleep of up to ~1 us, so the default bounds a
// stuck wait to roughly two seconds.
extern uint32_t g_wait_limit;
constexpr uint32_t kDefaultWaitLimit = 1u << 21;

inline cudaStream_t as_stream(vren_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

// ------------------------------------------------------------------------------------------------
// Programmatic dependent launch.  Inside the per-frame and batched clustering sequences every kernel
// is launched with programmatic stream serialisation, so the next kernel's launch overlaps this one.
// Each such kernel starts with pdl_enter(): griddepcontrol.wait blocks until the preceding grid has
// completed and its memory is visible (so nothing is read or written early), then
// launch_dependents lets the following grid be scheduled.  Launched without the attribute, both
// instructions do nothing.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ void pdl_enter()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Non-zero while a clustering sequence is being enqueued on this host thread (capi.cu).
extern thread_local int g_pdl;

struct PdlScope {
    int prev;
    explicit PdlScope(int on) : prev(g_pdl) { g_pdl = on; }
    ~PdlScope() { g_pdl = prev; }
};

// kernel<<<grid, block, smem, st>>>(args...), with programmatic stream serialisation when g_pdl is set.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_kernel(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                 Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    if (g_pdl) {
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

// ------------------------------------------------------------------------------------------------
// Device error word.  Each translation unit owns one (no relocatable device code is used);
// VREN_DEFINE_ERROR_WORD(tag) defines it and a host accessor vren_internal_error_<tag>().
// ------------------------------------------------------------------------------------------------
#define VREN_DEFINE_ERROR_WORD(tag)                                                      \
    static __device__ unsigned int g_vren_error_word;                                     \
    extern "C" int vren_internal_error_##tag(int clear)                                   \
    {                                                                                     \
        unsigned int v = 0;                                                               \
        if (cudaMemcpyFromSymbol(&v, g_vren_error_word, sizeof(v)) != cudaSuccess)        \
            return VREN_ERR_CUDA;                                                         \
        if (clear && v != 0) {                                                            \
            unsigned int z = 0;                                                           \
            if (cudaMemcpyToSymbol(g_vren_error_word, &z, sizeof(z)) != cudaSuccess)      \
                return VREN_ERR_CUDA;                                                     \
        }                                                                                 \
        return (int)v;                                                                    \
    }

// Record a device-side failure (first error wins).
#define VREN_RECORD_ERROR(code) atomicCAS(&g_vren_error_word, 0u, (unsigned int)(code))

// ------------------------------------------------------------------------------------------------
// Memory-model helpers (PTX ISA: ld.acquire / st.release at gpu scope)
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void st_relaxed_u32(uint32_t* p, uint32_t v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Look-back status words carry their whole payload (flag and value) in one naturally aligned
// word, so single-copy atomicity is all the protocol needs: relaxed gpu-scope accesses, no fences.
__device__ __forceinline__ uint64_t ld_relaxed_u64(const uint64_t* p)
{
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed_u64(uint64_t* p, uint64_t v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint32_t lanemask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint32_t lane_id()
{
    uint32_t l;
    asm("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}

// ------------------------------------------------------------------------------------------------
// Look-back status words: [flag:2 | value:30].  flag 0 = not yet published,
// 1 = tile aggregate only, 2 = inclusive prefix.  Values are element counts < 2^30.
// ------------------------------------------------------------------------------------------------
constexpr uint32_t kFlagShift = 30;
constexpr uint32_t kFlagAggregate = 1u << kFlagShift;
constexpr uint32_t kFlagPrefix = 2u << kFlagShift;
constexpr uint32_t kValueMask = (1u << kFlagShift) - 1u;

// Spin until *p carries a flag; returns the word, or a prefix-flagged 0 after the wait
// limit (and records VREN_ERR_TIMEOUT through the caller-provided error recorder).
// The first `spin` polls re-read immediately; later ones back off with __nanosleep (32 ns doubling
// to 512 ns).  `limit` bounds the total number of polls.
template <typename OnTimeout>
__device__ __forceinline__ uint32_t wait_for_flag(const uint32_t* p, uint32_t limit, uint32_t spin, OnTimeout on_timeout)
{
    uint32_t ns = 32;
    for (uint32_t round = 0;; ++round) {
        uint32_t v = ld_relaxed_u32(p);
        if (v & (3u << kFlagShift)) return v;
        if (round >= limit) {
            on_timeout();
            return kFlagPrefix;
        }
        if (round >= spin) {
            __nanosleep(ns);
            if (ns < 512) ns <<= 1;
        }
    }
}

// ------------------------------------------------------------------------------------------------
// Correctly rounded float helpers (never contracted into FMA).
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

// uint(floor(x)) with saturating semantics, written out so that it does not depend on
// the conversion instruction: NaN and negative values give 0, values >= 2^32 give
// 0xFFFFFFFF.  The oracle states the same function.
__device__ __forceinline__ uint32_t floor_to_u32(float x)
{
    float f = floorf(x);
    if (!(f >= 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}

}  // namespace vren_gb300

#define VREN_CUDA_TRY(expr)                                       \
    do {                                                          \
        cudaError_t _e = (expr);                                  \
        if (_e != cudaSuccess) return VREN_ERR_CUDA;              \
    } while (0)

#define VREN_LAUNCH_CHECK()                                       \
    do {                                                          \
        cudaError_t _e = cudaGetLastError();                      \
        if (_e != cudaSuccess) return VREN_ERR_CUDA;              \
    } while (0)

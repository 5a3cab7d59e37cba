// Reduce — drop-in tree form and scalar form.
//
// Drop-in semantics (vren::reduce<T,Op>, vren/vren/primitives/reduce.cpp:32-128 and
// vren/resources/shaders/reduce.comp:50-86): the output holds the Blelloch up-sweep tree
// of the input padded with the operation's identity to P = next power of two.  The
// reference walks the levels ten at a time with one dispatch each, reading strided
// elements into a 1024-wide shared-memory tree.  Here one pass covers 2 + log2(THREADS)
// levels: two in registers (4 consecutive items per thread), five by warp shuffles and
// the rest through shared memory, with vectorised loads/stores on the first pass.  The
// combine order at every node is op(right, left), the reference's
// VREN_OPERATION(s_data[b], s_data[a]) (reduce.comp:76), so float sums follow the same
// pairwise tree and are bit-identical.
//
// Scalar form: a single pass, block partials in scratch and a last-block-done combine (no
// spinning, integer/total-order ops, exact in any order): a grid-stride loop of uint4 loads, four
// in flight per thread.  Streaming forms that pull the input through shared-memory stages filled
// by bulk copies (cp.async.bulk) are selectable; they measured slower on GB300.
#include "common.cuh"
#include "internal.h"
#include "tma.cuh"

#include <cfloat>

namespace vren_gb300 {

VREN_DEFINE_ERROR_WORD(reduce)

// ------------------------------------------------------------------------------------------------
// Operations.  min/max follow GLSL's definitions min(x,y) = y < x ? y : x and
// max(x,y) = x < y ? y : x with x = right operand, y = left operand.
// ------------------------------------------------------------------------------------------------
template <int OP> struct U32Op;
template <> struct U32Op<VREN_REDUCE_ADD> {
    static __device__ __forceinline__ uint32_t identity() { return 0u; }
    static __device__ __forceinline__ uint32_t apply(uint32_t r, uint32_t l) { return r + l; }
};
template <> struct U32Op<VREN_REDUCE_MIN> {
    static __device__ __forceinline__ uint32_t identity() { return 0xFFFFFFFFu; }
    static __device__ __forceinline__ uint32_t apply(uint32_t r, uint32_t l) { return l < r ? l : r; }
};
template <> struct U32Op<VREN_REDUCE_MAX> {
    static __device__ __forceinline__ uint32_t identity() { return 0u; }
    static __device__ __forceinline__ uint32_t apply(uint32_t r, uint32_t l) { return r < l ? l : r; }
};

__device__ __forceinline__ float glsl_min(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float glsl_max(float x, float y) { return x < y ? y : x; }

template <int OP> struct Vec4Op;
template <> struct Vec4Op<VREN_REDUCE_ADD> {
    static __device__ __forceinline__ float4 identity() { return make_float4(0.f, 0.f, 0.f, 0.f); }
    static __device__ __forceinline__ float4 apply(float4 r, float4 l)
    {
        return make_float4(__fadd_rn(r.x, l.x), __fadd_rn(r.y, l.y), __fadd_rn(r.z, l.z), __fadd_rn(r.w, l.w));
    }
};
template <> struct Vec4Op<VREN_REDUCE_MIN> {
    static __device__ __forceinline__ float4 identity() { return make_float4(1e35f, 1e35f, 1e35f, 1e35f); }
    static __device__ __forceinline__ float4 apply(float4 r, float4 l)
    {
        return make_float4(glsl_min(r.x, l.x), glsl_min(r.y, l.y), glsl_min(r.z, l.z), glsl_min(r.w, l.w));
    }
};
template <> struct Vec4Op<VREN_REDUCE_MAX> {
    static __device__ __forceinline__ float4 identity() { return make_float4(-1e35f, -1e35f, -1e35f, -1e35f); }
    static __device__ __forceinline__ float4 apply(float4 r, float4 l)
    {
        return make_float4(glsl_max(r.x, l.x), glsl_max(r.y, l.y), glsl_max(r.z, l.z), glsl_max(r.w, l.w));
    }
};

template <typename T> __device__ __forceinline__ T shfl_up(T v, int d);
template <> __device__ __forceinline__ uint32_t shfl_up<uint32_t>(uint32_t v, int d) { return __shfl_up_sync(0xFFFFFFFFu, v, d); }
template <> __device__ __forceinline__ float4 shfl_up<float4>(float4 v, int d)
{
    return make_float4(__shfl_up_sync(0xFFFFFFFFu, v.x, d), __shfl_up_sync(0xFFFFFFFFu, v.y, d),
                       __shfl_up_sync(0xFFFFFFFFu, v.z, d), __shfl_up_sync(0xFFFFFFFFu, v.w, d));
}

// ------------------------------------------------------------------------------------------------
// One up-sweep pass.  Elements of this pass are e_j = buf[(j+1)*2^base - 1] for j < count
// (on the first pass e_j = in[j] for j < n_valid, identity beyond).  Each CTA owns 4*THREADS
// consecutive j and builds levels base .. base + 2 + log2(THREADS) - 1 of the tree over them.
// ------------------------------------------------------------------------------------------------
template <typename T, typename Op, int THREADS>
__global__ void __launch_bounds__(THREADS) reduce_tree_pass_kernel(
    const T* __restrict__ in, T* __restrict__ out, uint32_t in_seg_stride, uint32_t out_seg_stride,
    uint32_t n_valid, uint32_t count, uint32_t base, int first_pass)
{
    constexpr int WARPS = THREADS / 32;
    __shared__ T s_warp_root[WARPS];

    const uint32_t seg = blockIdx.y;
    const T* src = first_pass ? in + (size_t)seg * in_seg_stride : out + (size_t)seg * out_seg_stride;
    T* dst = out + (size_t)seg * out_seg_stride;

    const uint32_t tid = threadIdx.x;
    const uint32_t lane = tid & 31u, warp = tid >> 5;
    const uint32_t j0 = blockIdx.x * (4u * THREADS) + 4u * tid;  // first element of this thread
    const uint64_t stride = (uint64_t)1 << base;
    const uint32_t limit = first_pass ? n_valid : count;           // elements that exist in memory

    T v[4];
    if constexpr (sizeof(T) == 4) {
        // first pass over 16-byte aligned u32 input: the thread's four consecutive elements in one load
        if (base == 0 && j0 + 3u < limit && ((reinterpret_cast<uintptr_t>(src) & 15u) == 0)) {
            const uint4 q = *reinterpret_cast<const uint4*>(src + j0);
            v[0] = q.x;
            v[1] = q.y;
            v[2] = q.z;
            v[3] = q.w;
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                uint32_t j = j0 + k;
                v[k] = (j < limit) ? src[(size_t)((uint64_t)(j + 1) * stride - 1)] : Op::identity();
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            uint32_t j = j0 + k;
            v[k] = (j < limit) ? src[(size_t)((uint64_t)(j + 1) * stride - 1)] : Op::identity();
        }
    }
    // Elements 0 and 2 of the thread keep their value (they are not the end of a level-1 or higher
    // block); when this pass reads and writes the same positions, they need no store.
    const bool in_place = src == dst;

    // Levels 0 and 1 inside the thread.
    v[1] = Op::apply(v[1], v[0]);
    v[3] = Op::apply(v[3], v[2]);
    v[3] = Op::apply(v[3], v[1]);

    // Levels 2..6 across the warp: thread t (low s+1 bits all ones) combines with t - 2^s.
    T r = v[3];
#pragma unroll
    for (int s = 0; s < 5; ++s) {
        T left = shfl_up<T>(r, 1 << s);
        uint32_t mask = (2u << s) - 1u;
        if ((lane & mask) == mask) r = Op::apply(r, left);
    }
    v[3] = r;

    // Remaining levels across warps on the warp roots (lane 31).
    if (WARPS > 1) {
        if (lane == 31) s_warp_root[warp] = r;
        __syncthreads();
        if (warp == 0) {
            T w = (lane < WARPS) ? s_warp_root[lane] : Op::identity();
#pragma unroll
            for (int s = 0; (1 << s) < WARPS; ++s) {
                T left = shfl_up<T>(w, 1 << s);
                uint32_t mask = (2u << s) - 1u;
                if ((lane & mask) == mask) w = Op::apply(w, left);
            }
            if (lane < WARPS) s_warp_root[lane] = w;
        }
        __syncthreads();
        if (lane == 31) v[3] = s_warp_root[warp];
    }

#pragma unroll
    for (int k = 0; k < 4; ++k) {
        uint32_t j = j0 + k;
        if ((k & 1) == 0 && in_place && j < limit) continue;  // loaded from this position, unchanged
        if (j < count) dst[(size_t)((uint64_t)(j + 1) * stride - 1)] = v[k];
    }
}

template <typename T, typename Op, int THREADS>
static int reduce_tree_launch(cudaStream_t st, const T* in, uint32_t n, T* out, uint32_t blocks)
{
    constexpr uint32_t kLevels = 2 + (THREADS == 1024 ? 10 : THREADS == 256 ? 8 : 0);
    static_assert(THREADS == 1024 || THREADS == 256, "unsupported CTA size");
    const uint32_t P = vren_round_to_next_power_of_2(n);
    uint32_t levels = 0;
    while ((1ull << levels) < P) ++levels;
    if (levels == 0) levels = 1;  // reference: max(log2(P), 1) — a single element is copied
    for (uint32_t base = 0; base < levels; base += kLevels) {
        const uint32_t count = P >> base;
        const uint32_t per_cta = 4u * THREADS;
        dim3 grid((count + per_cta - 1) / per_cta, blocks);
        reduce_tree_pass_kernel<T, Op, THREADS><<<grid, THREADS, 0, st>>>(in, out, n, P, n, count, base, base == 0);
        VREN_LAUNCH_CHECK();
    }
    return VREN_OK;
}

// ------------------------------------------------------------------------------------------------
// Scalar reductions: u32 add/min/max, f32 min/max in IEEE total order.
// ------------------------------------------------------------------------------------------------
// Total-order key of a float: monotone map to uint32 (negative NaN < -inf < ... < -0 < +0 <
// ... < +inf < positive NaN).
__device__ __forceinline__ uint32_t f32_order_key(uint32_t bits)
{
    return (bits & 0x80000000u) ? ~bits : (bits | 0x80000000u);
}
__device__ __forceinline__ uint32_t f32_from_order_key(uint32_t key)
{
    return (key & 0x80000000u) ? (key & 0x7FFFFFFFu) : ~key;
}

constexpr int kScalarThreads = 512;
constexpr int kScalarVecPerThread = 4;  // uint4 loads in flight per thread per iteration

// Block combine of every thread's `acc`, the block partial into scratch[1 + block], and the final
// combine by the last block to finish (which also resets the ticket scratch[0]).
template <int OP, bool FLOAT_KEYS, int THREADS>
__device__ __forceinline__ void reduce_finish(uint32_t acc, uint32_t* __restrict__ out, uint32_t* __restrict__ scratch,
                                              uint32_t* s_warp, bool* s_last)
{
    using Op = U32Op<OP>;
    const uint32_t tid = threadIdx.x;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) acc = Op::apply(acc, __shfl_xor_sync(0xFFFFFFFFu, acc, d));
    if ((tid & 31) == 0) s_warp[tid >> 5] = acc;
    __syncthreads();
    if (tid < 32) {
        uint32_t w = tid < THREADS / 32 ? s_warp[tid] : Op::identity();
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) w = Op::apply(w, __shfl_xor_sync(0xFFFFFFFFu, w, d));
        if (tid == 0) {
            st_relaxed_u32(scratch + 1 + blockIdx.x, w);
            __threadfence();
            const uint32_t ticket = atomicAdd(scratch, 1u);
            *s_last = (ticket == gridDim.x - 1);
        }
    }
    __syncthreads();
    if (!*s_last) return;
    __threadfence();
    uint32_t total = Op::identity();
    for (uint32_t b = tid; b < gridDim.x; b += THREADS) total = Op::apply(total, ld_relaxed_u32(scratch + 1 + b));
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) total = Op::apply(total, __shfl_xor_sync(0xFFFFFFFFu, total, d));
    __syncthreads();
    if ((tid & 31) == 0) s_warp[tid >> 5] = total;
    __syncthreads();
    if (tid == 0) {
        uint32_t t = Op::identity();
        for (int w = 0; w < THREADS / 32; ++w) t = Op::apply(t, s_warp[w]);
        out[0] = FLOAT_KEYS ? f32_from_order_key(t) : t;
        scratch[0] = 0u;
    }
}

template <int OP, bool FLOAT_KEYS>
__global__ void __launch_bounds__(kScalarThreads) reduce_scalar_kernel(
    const uint32_t* __restrict__ in, uint32_t n, uint32_t* __restrict__ out, uint32_t* __restrict__ scratch)
{
    using Op = U32Op<OP>;
    __shared__ uint32_t s_warp[kScalarThreads / 32];
    __shared__ bool s_last;

    uint32_t acc = Op::identity();
    const uint32_t tid = threadIdx.x;
    const uint32_t nvec = n / 4;
    const uint4* in4 = reinterpret_cast<const uint4*>(in);
    const uint32_t grid_threads = gridDim.x * kScalarThreads;

    auto fold = [&](uint32_t x) {
        if (FLOAT_KEYS) x = f32_order_key(x);
        acc = Op::apply(acc, x);
    };

    // Main loop: kScalarVecPerThread independent uint4 loads per iteration.
    uint32_t i = blockIdx.x * kScalarThreads + tid;
    for (; i + (kScalarVecPerThread - 1) * grid_threads < nvec; i += kScalarVecPerThread * grid_threads) {
        uint4 q[kScalarVecPerThread];
#pragma unroll
        for (int k = 0; k < kScalarVecPerThread; ++k) q[k] = __ldcs(in4 + i + k * grid_threads);
#pragma unroll
        for (int k = 0; k < kScalarVecPerThread; ++k) {
            fold(q[k].x); fold(q[k].y); fold(q[k].z); fold(q[k].w);
        }
    }
    for (; i < nvec; i += grid_threads) {
        uint4 q = __ldcs(in4 + i);
        fold(q.x); fold(q.y); fold(q.z); fold(q.w);
    }
    // Tail (n not a multiple of 4), handled by block 0.
    if (blockIdx.x == 0 && tid < (n & 3u)) fold(in[nvec * 4 + tid]);

    reduce_finish<OP, FLOAT_KEYS, kScalarThreads>(acc, out, scratch, s_warp, &s_last);
}

// Streaming form: each CTA pulls its share of the input through a ring of `stages` shared-memory
// stages of `stage_vec` uint4, several in flight.  Warp 8 issues the bulk copies; each of the eight
// consumer warps folds its eighth of a stage and releases it on the stage's `empty` barrier (count
// 8), and the producer refills a stage once all eight have released it, so no CTA-wide barrier
// sits between stages.  A CTA's stages are either one contiguous run or every grid-th stage.
constexpr int kStreamConsumers = 256;
constexpr int kStreamThreads = kStreamConsumers + 32;
constexpr int kStreamMaxStages = 12;

struct StreamShape {
    uint32_t stage_vec;  // uint4 per stage (multiple of 256)
    uint32_t stages;     // ring depth (<= kStreamMaxStages)
    uint32_t per_sm;     // CTAs per SM the shape is sized for
    uint32_t interleave; // 1: CTA b takes stages b, b + grid, ...; 0: one contiguous run
};

template <int OP, bool FLOAT_KEYS>
__global__ void __launch_bounds__(kStreamThreads) reduce_stream_kernel(
    const uint32_t* __restrict__ in, uint32_t n, uint32_t* __restrict__ out, uint32_t* __restrict__ scratch,
    uint32_t wait_limit, StreamShape shape)
{
    using Op = U32Op<OP>;
    extern __shared__ __align__(128) uint4 s_stage[];
    __shared__ __align__(8) uint64_t s_full[kStreamMaxStages];
    __shared__ __align__(8) uint64_t s_empty[kStreamMaxStages];
    __shared__ uint32_t s_warp[kStreamThreads / 32];
    __shared__ bool s_last;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t V = shape.stage_vec, S = shape.stages;
    const uint32_t nvec = n / 4;
    const uint32_t stages_total = (nvec + V - 1) / V;
    uint32_t first, step, count;
    if (shape.interleave) {
        first = blockIdx.x;
        step = gridDim.x;
        count = first < stages_total ? (stages_total - first + step - 1) / step : 0u;
    } else {
        const uint32_t per = (stages_total + gridDim.x - 1) / gridDim.x;
        first = min(blockIdx.x * per, stages_total);
        step = 1;
        count = min(first + per, stages_total) - first;
    }
    const uint4* in4 = reinterpret_cast<const uint4*>(in);
    if (tid == 0) {
        for (uint32_t s = 0; s < S; ++s) {
            mbar_init(&s_full[s], 1u);
            mbar_init(&s_empty[s], kStreamConsumers / 32);
        }
        fence_barrier_init();
    }
    __syncthreads();

    uint32_t acc = Op::identity();
    auto fold = [&](uint32_t x) {
        if (FLOAT_KEYS) x = f32_order_key(x);
        acc = Op::apply(acc, x);
    };
    bool timed_out = false;
    if (warp == kStreamConsumers / 32) {
        if (lane == 0) {
            for (uint32_t k = 0; k < count; ++k) {
                const uint32_t s = k % S;
                if (k >= S && !mbar_wait(&s_empty[s], ((k - S) / S) & 1u, wait_limit)) {
                    timed_out = true;  // the consumers time out on `full` in turn
                    break;
                }
                const uint32_t v0 = (first + k * step) * V;
                const uint32_t nv = min(V, nvec - v0);
                mbar_arrive_expect_tx(&s_full[s], nv * 16u);
                bulk_load(s_stage + (size_t)s * V, in4 + v0, nv * 16u, &s_full[s]);
            }
        }
    } else {
        const uint32_t share = V / 8;  // uint4 per consumer warp per stage
        for (uint32_t k = 0; k < count; ++k) {
            const uint32_t s = k % S;
            if (!__all_sync(0xFFFFFFFFu, mbar_wait(&s_full[s], (k / S) & 1u, wait_limit))) {
                timed_out = true;
                break;
            }
            const uint32_t nv = min(V, nvec - (first + k * step) * V);
            const uint32_t base = warp * share;
            const uint4* st = s_stage + (size_t)s * V + base;
#pragma unroll 4
            for (uint32_t idx = lane; idx < share; idx += 32) {
                if (base + idx < nv) {
                    const uint4 q = st[idx];
                    fold(q.x); fold(q.y); fold(q.z); fold(q.w);
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&s_empty[s]);
        }
        if (blockIdx.x == 0 && tid < (n & 3u)) fold(in[nvec * 4 + tid]);
    }
    if (timed_out) VREN_RECORD_ERROR(VREN_ERR_TIMEOUT);
    __syncthreads();
    reduce_finish<OP, FLOAT_KEYS, kStreamThreads>(acc, out, scratch, s_warp, &s_last);
}

// Stream shapes selectable with VREN_TUNE_REDUCE_FORM (2..5).  Measured on GB300 (2^26 / 2^27
// elements): 60-65 us / 104-111 us against 52 us / 93 us for the grid-stride loop of uint4 loads,
// which is therefore the automatic choice at every size.
constexpr StreamShape kStreamShapes[4] = {
    {1024, 6, 2, 0},   // 16 KB x 6, two CTAs per SM, contiguous runs
    {1024, 6, 2, 1},   // the same, interleaved stages
    {2048, 6, 1, 1},   // 32 KB x 6, one CTA per SM, interleaved
    {512, 12, 2, 1},   // 8 KB x 12, two CTAs per SM, interleaved
};
constexpr uint32_t kStreamMaxGrid = 2 * kNumSMsHint;

static uint32_t stream_grid(uint32_t n, const StreamShape& sh)
{
    const uint32_t stages = (n / 4 + sh.stage_vec - 1) / sh.stage_vec;
    const uint32_t cap = sh.per_sm * kNumSMsHint;
    return stages < cap ? (stages ? stages : 1) : cap;
}

template <int OP, bool FLOAT_KEYS>
static int launch_stream(cudaStream_t st, const uint32_t* in, uint32_t n, uint32_t* out, uint32_t* sc,
                         const StreamShape& sh)
{
    static bool attr_set = false;  // per instantiation: the largest ring any shape uses
    if (!attr_set) {
        VREN_CUDA_TRY(cudaFuncSetAttribute(reduce_stream_kernel<OP, FLOAT_KEYS>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 192 * 1024));
        attr_set = true;
    }
    const size_t smem = (size_t)sh.stage_vec * sh.stages * sizeof(uint4);
    reduce_stream_kernel<OP, FLOAT_KEYS><<<stream_grid(n, sh), kStreamThreads, smem, st>>>(in, n, out, sc,
                                                                                         g_wait_limit, sh);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

static uint32_t scalar_grid(uint32_t n)
{
    uint32_t nvec = n / 4;
    uint32_t per_cta = kScalarThreads * kScalarVecPerThread;
    uint32_t g = (nvec + per_cta - 1) / per_cta;
    uint32_t cap = kNumSMsHint * 4;
    if (g > cap) g = cap;
    if (g == 0) g = 1;
    return g;
}

template <bool FLOAT_KEYS>
static int reduce_scalar_dispatch(cudaStream_t st, int op, const uint32_t* in, uint32_t n, uint32_t* out, void* scratch)
{
    uint32_t g = scalar_grid(n);
    uint32_t* sc = static_cast<uint32_t*>(scratch);
    const int form = tuning(VREN_TUNE_REDUCE_FORM);
    if (form >= 2 && n > 0) {
        const StreamShape& sh = kStreamShapes[form - 2];
        switch (op) {
        case VREN_REDUCE_ADD: return launch_stream<VREN_REDUCE_ADD, FLOAT_KEYS>(st, in, n, out, sc, sh);
        case VREN_REDUCE_MIN: return launch_stream<VREN_REDUCE_MIN, FLOAT_KEYS>(st, in, n, out, sc, sh);
        case VREN_REDUCE_MAX: return launch_stream<VREN_REDUCE_MAX, FLOAT_KEYS>(st, in, n, out, sc, sh);
        default: return VREN_ERR_ARG;
        }
    }
    switch (op) {
    case VREN_REDUCE_ADD: reduce_scalar_kernel<VREN_REDUCE_ADD, FLOAT_KEYS><<<g, kScalarThreads, 0, st>>>(in, n, out, sc); break;
    case VREN_REDUCE_MIN: reduce_scalar_kernel<VREN_REDUCE_MIN, FLOAT_KEYS><<<g, kScalarThreads, 0, st>>>(in, n, out, sc); break;
    case VREN_REDUCE_MAX: reduce_scalar_kernel<VREN_REDUCE_MAX, FLOAT_KEYS><<<g, kScalarThreads, 0, st>>>(in, n, out, sc); break;
    default: return VREN_ERR_ARG;
    }
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

}  // namespace vren_gb300

using namespace vren_gb300;

extern "C" uint32_t vren_calc_reduce_output_buffer_length(uint32_t count) { return vren_round_to_next_power_of_2(count); }

extern "C" int vren_reduce_tree_u32(vren_stream_t s, int op, const uint32_t* in, uint32_t n, uint32_t* out, uint32_t blocks)
{
    if (blocks == 0 || (n > 0 && (!in || !out)) || n > 0x80000000u) return VREN_ERR_ARG;
    if (n == 0) return VREN_OK;
    cudaStream_t st = as_stream(s);
    switch (op) {
    case VREN_REDUCE_ADD: return reduce_tree_launch<uint32_t, U32Op<VREN_REDUCE_ADD>, 1024>(st, in, n, out, blocks);
    case VREN_REDUCE_MIN: return reduce_tree_launch<uint32_t, U32Op<VREN_REDUCE_MIN>, 1024>(st, in, n, out, blocks);
    case VREN_REDUCE_MAX: return reduce_tree_launch<uint32_t, U32Op<VREN_REDUCE_MAX>, 1024>(st, in, n, out, blocks);
    default: return VREN_ERR_ARG;
    }
}

extern "C" int vren_reduce_tree_vec4(vren_stream_t s, int op, const float* in, uint32_t n, float* out, uint32_t blocks)
{
    if (blocks == 0 || (n > 0 && (!in || !out)) || n > 0x80000000u) return VREN_ERR_ARG;
    if (((uintptr_t)in & 15u) || ((uintptr_t)out & 15u)) return VREN_ERR_ARG;
    if (n == 0) return VREN_OK;
    cudaStream_t st = as_stream(s);
    const float4* i4 = reinterpret_cast<const float4*>(in);
    float4* o4 = reinterpret_cast<float4*>(out);
    switch (op) {
    case VREN_REDUCE_ADD: return reduce_tree_launch<float4, Vec4Op<VREN_REDUCE_ADD>, 256>(st, i4, n, o4, blocks);
    case VREN_REDUCE_MIN: return reduce_tree_launch<float4, Vec4Op<VREN_REDUCE_MIN>, 256>(st, i4, n, o4, blocks);
    case VREN_REDUCE_MAX: return reduce_tree_launch<float4, Vec4Op<VREN_REDUCE_MAX>, 256>(st, i4, n, o4, blocks);
    default: return VREN_ERR_ARG;
    }
}

extern "C" size_t vren_reduce_scratch_bytes(uint32_t n)
{
    // partials for the largest grid any form may use at this size
    const uint32_t g = scalar_grid(n) > kStreamMaxGrid ? scalar_grid(n) : kStreamMaxGrid;
    return (size_t)(1 + g) * sizeof(uint32_t);
}

extern "C" int vren_reduce_u32(vren_stream_t s, int op, const uint32_t* in, uint32_t n, uint32_t* out, void* scratch)
{
    if (!out || !scratch || (n > 0 && !in) || ((uintptr_t)in & 15u)) return VREN_ERR_ARG;
    return reduce_scalar_dispatch<false>(as_stream(s), op, in, n, out, scratch);
}

extern "C" int vren_reduce_f32(vren_stream_t s, int op, const float* in, uint32_t n, float* out, void* scratch)
{
    if (!out || !scratch || (n > 0 && !in) || ((uintptr_t)in & 15u)) return VREN_ERR_ARG;
    if (op != VREN_REDUCE_MIN && op != VREN_REDUCE_MAX) return VREN_ERR_ARG;
    return reduce_scalar_dispatch<true>(as_stream(s), op, reinterpret_cast<const uint32_t*>(in), n,
                                        reinterpret_cast<uint32_t*>(out), scratch);
}

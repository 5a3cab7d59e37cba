// Reduce — drop-in tree form and scalar form.
//
// Drop-in semantics (vren::reduce<T,Op>, vren/vren/primitives/reduce.cpp:82-178 and
// vren/resources/shaders/reduce.comp:50-86): the output holds the Blelloch up-sweep tree
// of the input padded with the operation's identity to P = next power of two.  The
// reference walks the levels ten at a time with one dispatch each, reading strided
// elements into a 1024-wide shared-memory tree.  Here one pass covers 2 + log2(THREADS)
// levels: two in registers (4 consecutive items per thread), five by warp shuffles and
// the rest through shared memory, with vectorised loads/stores on the first pass.  The
// combine order at every node is op(right, left), the reference's
// VREN_OPERATION(s_data[b], s_data[a]) (reduce.comp:266), so float sums follow the same
// pairwise tree and are bit-identical.
//
// Scalar form: a single pass over uint4-vectorised loads, block partials in scratch and a
// last-block-done combine (no spinning, integer/total-order ops, exact in any order).
#include "common.cuh"

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
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        uint32_t j = j0 + k;
        v[k] = (j < limit) ? src[(size_t)((uint64_t)(j + 1) * stride - 1)] : Op::identity();
    }

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

    // Block reduction.
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) acc = Op::apply(acc, __shfl_xor_sync(0xFFFFFFFFu, acc, d));
    if ((tid & 31) == 0) s_warp[tid >> 5] = acc;
    __syncthreads();
    if (tid < 32) {
        uint32_t w = tid < kScalarThreads / 32 ? s_warp[tid] : Op::identity();
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) w = Op::apply(w, __shfl_xor_sync(0xFFFFFFFFu, w, d));
        if (tid == 0) {
            // scratch[0] = ticket, scratch[1 + b] = partial of block b.
            st_relaxed_u32(scratch + 1 + blockIdx.x, w);
            __threadfence();
            uint32_t ticket = atomicAdd(scratch, 1u);
            s_last = (ticket == gridDim.x - 1);
        }
    }
    __syncthreads();
    if (!s_last) return;

    // Last block: combine the partials and reset the ticket for the next call.
    __threadfence();
    uint32_t total = Op::identity();
    for (uint32_t b = tid; b < gridDim.x; b += kScalarThreads) total = Op::apply(total, ld_relaxed_u32(scratch + 1 + b));
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) total = Op::apply(total, __shfl_xor_sync(0xFFFFFFFFu, total, d));
    __syncthreads();
    if ((tid & 31) == 0) s_warp[tid >> 5] = total;
    __syncthreads();
    if (tid == 0) {
        uint32_t t = Op::identity();
        for (int w = 0; w < kScalarThreads / 32; ++w) t = Op::apply(t, s_warp[w]);
        out[0] = FLOAT_KEYS ? f32_from_order_key(t) : t;
        scratch[0] = 0u;
    }
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
    return (size_t)(1 + scalar_grid(n)) * sizeof(uint32_t);
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

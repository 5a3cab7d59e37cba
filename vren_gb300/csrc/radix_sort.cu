// Onesweep LSD radix sort and stable bucket sort.
//
// Reference: vren::radix_sort (vren/vren/primitives/radix_sort.cpp:149-338) sorts uint32 keys with
// eight 4-bit passes, each made of a buffer fill, a per-work-group 16-bin count
// (radix_sort_local_count.comp), an up-sweep reduce of the counts, a 16-lane scan
// (radix_sort_global_offset.comp), a down-sweep and a reorder that issues 16 ballots per key and
// scatters uncoalesced (radix_sort_reorder.comp:55-113): ~48 commands per sort.
// vren::bucket_sort (vren/primitives/bucket_sort.cpp:102-160) counts with global atomics, scans 65536 counters and
// scatters with atomics, so its order inside a bucket is unspecified.
//
// Here: one histogram kernel reads the keys once and builds the digit histograms of every pass;
// then one kernel per digit pass ("onesweep", Adinets & Merrill 2022):
//   1. a CTA takes the next tile ticket (tiles start in order, so look-back always terminates);
//   2. each warp loads 32*ITEMS consecutive keys, striped, with coalesced loads;
//   3. stable in-warp ranks from DIGIT_BITS ballots per key (peers = lanes with an equal digit)
//      and per-warp digit counters in shared memory;
//   4. the tile's digit counts are published and each digit's global offset is resolved by
//      decoupled look-back over the preceding tiles (one thread per digit, bounded wait);
//   5. keys (and values) are staged in shared memory in digit order and written out so that
//      consecutive threads write consecutive addresses of the same digit run.
// Status words ([flag:2 | count:30]) alternate between two buffers: pass p reads buffer p&1 and
// clears the rows of buffer (p+1)&1 for its own tile, so no pass needs a separate memset.
#include "common.cuh"
#include "internal.h"

#include <type_traits>

namespace vren_gb300 {

VREN_DEFINE_ERROR_WORD(radix)

enum ElemMode { kKeys = 0, kPairs = 1, kUvec2 = 2 };

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kMaxPasses = 8;
constexpr int kMaxRadix = 256;

// Scratch layout in uint32 words.
constexpr uint32_t kTicketWords = 16;                      // [0, 8): pass tickets, [8]: histogram done ticket
constexpr uint32_t kHistOffset = kTicketWords;              // hist[pass][radix]
constexpr uint32_t kOffsOffset = kHistOffset + kMaxPasses * kMaxRadix;  // exclusive digit offsets
constexpr uint32_t kStatusOffset = kOffsOffset + kMaxPasses * kMaxRadix;
constexpr uint32_t kZeroWords = kOffsOffset;               // region cleared at the start of a sort

struct PassInfo {
    uint32_t shift[kMaxPasses];
    uint32_t width[kMaxPasses];
    uint32_t count;
};

template <int MODE> struct KeyOf;

__device__ __forceinline__ uint32_t digit_of(uint32_t key, uint32_t shift, uint32_t width)
{
    return (key >> shift) & ((1u << width) - 1u);
}

// ------------------------------------------------------------------------------------------------
// Histogram of all passes.  Also clears status buffer 0 (used by the first pass).
// ------------------------------------------------------------------------------------------------
template <int RADIX, int MODE>
__global__ void __launch_bounds__(kSortThreads) onesweep_hist_kernel(
    const uint32_t* keys, uint32_t n, PassInfo passes, uint32_t* __restrict__ scratch,
    uint32_t status_words)
{
    pdl_enter();
    __shared__ uint32_t s_hist[kMaxPasses * RADIX];
    const uint32_t tid = threadIdx.x;
    for (uint32_t i = tid; i < passes.count * RADIX; i += kSortThreads) s_hist[i] = 0u;
    __syncthreads();

    auto count_key = [&](uint32_t k) {
#pragma unroll
        for (int p = 0; p < kMaxPasses; ++p)
            if (p < (int)passes.count) atomicAdd(&s_hist[p * RADIX + digit_of(k, passes.shift[p], passes.width[p])], 1u);
    };

    const uint32_t grid_threads = gridDim.x * kSortThreads;
    if (MODE == kUvec2) {
        // Elements are (key, value) pairs; a uint4 holds two.
        const uint32_t npair = n / 2;
        const uint4* p4 = reinterpret_cast<const uint4*>(keys);
        for (uint32_t i = blockIdx.x * kSortThreads + tid; i < npair; i += grid_threads) {
            uint4 q = __ldg(p4 + i);
            count_key(q.x);
            count_key(q.z);
        }
        if ((n & 1u) && blockIdx.x == 0 && tid == 0) count_key(keys[2 * (n - 1)]);
    } else {
        const uint32_t nvec = n / 4;
        const uint4* p4 = reinterpret_cast<const uint4*>(keys);
        for (uint32_t i = blockIdx.x * kSortThreads + tid; i < nvec; i += grid_threads) {
            uint4 q = __ldg(p4 + i);
            count_key(q.x); count_key(q.y); count_key(q.z); count_key(q.w);
        }
        if (blockIdx.x == 0 && tid < (n & 3u)) count_key(keys[nvec * 4 + tid]);
    }
    __syncthreads();

    uint32_t* g_hist = scratch + kHistOffset;
    for (uint32_t i = tid; i < passes.count * RADIX; i += kSortThreads) {
        uint32_t v = s_hist[i];
        if (v) atomicAdd(&g_hist[(i / RADIX) * kMaxRadix + (i % RADIX)], v);
    }

    // Clear status buffer 0.
    uint32_t* status0 = scratch + kStatusOffset;
    for (uint32_t i = blockIdx.x * kSortThreads + tid; i < status_words; i += grid_threads) status0[i] = 0u;

    // Last CTA turns the histograms into exclusive digit offsets.
    __shared__ bool s_last;
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        s_last = (atomicAdd(scratch + 8, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // One block-wide exclusive scan per pass (RADIX <= 256 = threads), all loads in parallel.
    __shared__ uint32_t s_wsum[kSortThreads / 32];
    const uint32_t lane = tid & 31u, warp = tid >> 5;
    for (uint32_t p = 0; p < passes.count; ++p) {
        const uint32_t c = tid < (uint32_t)RADIX ? ld_relaxed_u32(g_hist + p * kMaxRadix + tid) : 0u;
        uint32_t incl = c;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        if (lane == 31) s_wsum[warp] = incl;
        __syncthreads();
        uint32_t before = 0;
        for (uint32_t w = 0; w < warp; ++w) before += s_wsum[w];
        if (tid < (uint32_t)RADIX) scratch[kOffsOffset + p * kMaxRadix + tid] = before + incl - c;
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------------------
// One digit pass.  RANK 0: peers from one ballot per digit bit; RANK 1: peers from match.any and one
// shared-memory atomic per peer group; RANK 2: peers from match.any, counters updated by the group's
// first lane as in RANK 0.  All give the same (stable) ranks.  Keys/values are staged in dynamic
// shared memory.  FULL tiles (all but the last) skip every per-item bounds test.
// ------------------------------------------------------------------------------------------------
template <int DIGIT_BITS, int ITEMS, int MODE, int RANK>
struct PassSmem {
    static constexpr int RADIX = 1 << DIGIT_BITS;
    uint32_t warp_hist[kSortWarps][RADIX];  // per-warp digit counts, then each warp's first staging slot
    int32_t delta[RADIX];
    uint32_t wsum[kSortWarps];
};

template <int DIGIT_BITS, int ITEMS, int MODE, int RANK, bool FULL>
__device__ __forceinline__ void onesweep_pass_body(
    const uint32_t* __restrict__ in_keys, const uint32_t* __restrict__ in_vals, uint32_t* __restrict__ out_keys,
    uint32_t* __restrict__ out_vals, uint32_t n, uint32_t pass, uint32_t shift, uint32_t width, uint32_t num_tiles,
    uint32_t* __restrict__ scratch, uint32_t wait_limit, uint32_t spin, uint32_t tile,
    PassSmem<DIGIT_BITS, ITEMS, MODE, RANK>& sm, uint4* s_stage)
{
    constexpr int RADIX = 1 << DIGIT_BITS;
    constexpr int TILE = kSortThreads * ITEMS;
    using Elem = typename std::conditional<MODE == kUvec2, uint2, uint32_t>::type;
    Elem* s_keys = reinterpret_cast<Elem*>(s_stage);
    uint2* s_pairs = reinterpret_cast<uint2*>(s_stage);  // MODE == kPairs: (key, value) as one 64-bit word
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;

    uint32_t* status = scratch + kStatusOffset + (size_t)(pass & 1u) * num_tiles * RADIX;
    uint32_t* status_next = scratch + kStatusOffset + (size_t)((pass + 1u) & 1u) * num_tiles * RADIX;
    for (uint32_t d = tid; d < RADIX; d += kSortThreads) status_next[(size_t)tile * RADIX + d] = 0u;

    // Striped load: item j of lane l is element warp_base + 32*j + l.
    const uint32_t warp_base = tile * TILE + warp * (32 * ITEMS);
    Elem key[ITEMS];
    uint32_t val[ITEMS];
    uint32_t pos[ITEMS];
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const uint32_t idx = warp_base + 32 * j + lane;
        key[j] = Elem{};
        val[j] = 0u;
        if (FULL || idx < n) {
            if (MODE == kUvec2) {
                (reinterpret_cast<uint2*>(&key[j]))[0] = __ldcs(reinterpret_cast<const uint2*>(in_keys) + idx);
            } else {
                (reinterpret_cast<uint32_t*>(&key[j]))[0] = __ldcs(in_keys + idx);
                if (MODE == kPairs) val[j] = __ldcs(in_vals + idx);
            }
        }
    }

    // Stable in-warp ranking, items in order.
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const uint32_t idx = warp_base + 32 * j + lane;
        const bool valid = FULL || idx < n;
        uint32_t k;
        if (MODE == kUvec2) k = (reinterpret_cast<uint2*>(&key[j]))->x;
        else k = *(reinterpret_cast<uint32_t*>(&key[j]));
        const uint32_t d = valid ? digit_of(k, shift, width) : 0u;
        if (RANK == 1) {
            // invalid lanes get a value no digit can take, so they form groups of one
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, valid ? d : (0x10000u + lane));
            const uint32_t leader = __ffs(peers) - 1;
            uint32_t base = 0;
            if (valid && lane == leader) base = atomicAdd(&sm.warp_hist[warp][d], (uint32_t)__popc(peers));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            pos[j] = valid ? (d | ((base + __popc(peers & lanemask_lt())) << 8)) : 0xFFFFFFFFu;
        } else {
            uint32_t peers;
            if (RANK == 2) {
                peers = __match_any_sync(0xFFFFFFFFu, valid ? d : (0x10000u + lane));
            } else {
                peers = FULL ? 0xFFFFFFFFu : __ballot_sync(0xFFFFFFFFu, valid);
#pragma unroll
                for (int b = 0; b < DIGIT_BITS; ++b) {
                    // keep the lanes whose bit b equals mine: m where my bit is 1, ~m where it is 0
                    const bool bit = (d >> b) & 1u;
                    const uint32_t m = __ballot_sync(0xFFFFFFFFu, bit);
                    peers &= bit ? m : ~m;
                }
            }
            const uint32_t below = peers & lanemask_lt();
            const uint32_t before = valid ? sm.warp_hist[warp][d] : 0u;
            __syncwarp();
            if (valid && below == 0) sm.warp_hist[warp][d] = before + __popc(peers);
            __syncwarp();
            pos[j] = valid ? (d | ((before + __popc(below)) << 8)) : 0xFFFFFFFFu;
        }
    }
    __syncthreads();

    // Thread d: warp prefixes of digit d, the tile's count, publish it.
    uint32_t count = 0;
    if (tid < (uint32_t)RADIX) {
        const uint32_t d = tid;
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) {  // digit d's count in the warps before w
            const uint32_t c = sm.warp_hist[w][d];
            sm.warp_hist[w][d] = count;
            count += c;
        }
        st_relaxed_u32(status + (size_t)tile * RADIX + d, (tile == 0 ? kFlagPrefix : kFlagAggregate) | count);
    }
    // Block-wide exclusive scan of the counts over digits (all warps), while the aggregates travel.
    uint32_t incl = count;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) sm.wsum[warp] = incl;
    __syncthreads();
    // Tile-local digit offsets, and the first look-back read for digit d issued now: its latency
    // overlaps the staging below, which needs only tile-local offsets.
    uint32_t excl = 0, lb_word = 0, goff = 0;
    if (tid < (uint32_t)RADIX) {
        const uint32_t d = tid;
        excl = incl - count;
        for (uint32_t w = 0; w < warp; ++w) excl += sm.wsum[w];
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) sm.warp_hist[w][d] += excl;  // first staging slot of (w, d)
        if (tile != 0) lb_word = ld_relaxed_u32(status + (size_t)(tile - 1) * RADIX + d);
        goff = ld_relaxed_u32(scratch + kOffsOffset + pass * kMaxRadix + d);
    }
    __syncthreads();

    // Stage in digit order.
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        if (FULL || pos[j] != 0xFFFFFFFFu) {
            const uint32_t d = pos[j] & 0xFFu;
            const uint32_t p = sm.warp_hist[warp][d] + (pos[j] >> 8);
            if (MODE == kPairs) s_pairs[p] = make_uint2(*reinterpret_cast<const uint32_t*>(&key[j]), val[j]);
            else s_keys[p] = key[j];
        }
    }

    // Decoupled look-back for digit d (thread d), starting from the word read before staging.
    if (tid < (uint32_t)RADIX) {
        const uint32_t d = tid;
        uint32_t prefix = 0;
        if (tile != 0) {
            // four predecessors per step: tile t is examined while t-1..t-3 are already being read
            int64_t t = (int64_t)tile - 1;
            uint32_t w[4];
            w[0] = lb_word;
            bool done = false;
            while (!done) {
#pragma unroll
                for (int i = 1; i < 4; ++i) w[i] = t - i >= 0 ? ld_relaxed_u32(status + (size_t)(t - i) * RADIX + d) : 0u;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    if (done || t - i < 0) continue;
                    uint32_t x = w[i];
                    if (!(x & (3u << kFlagShift)))
                        x = wait_for_flag(status + (size_t)(t - i) * RADIX + d, wait_limit, spin,
                                          [] { VREN_RECORD_ERROR(VREN_ERR_TIMEOUT); });
                    prefix += x & kValueMask;
                    if ((x & kFlagPrefix) || t - i == 0) done = true;
                }
                t -= 4;
                if (!done) w[0] = ld_relaxed_u32(status + (size_t)t * RADIX + d);
            }
            st_relaxed_u32(status + (size_t)tile * RADIX + d, kFlagPrefix | (prefix + count));
        }
        sm.delta[d] = (int32_t)(goff + prefix) - (int32_t)excl;
    }
    __syncthreads();

    // Write out: consecutive threads take consecutive staged elements.
    const uint32_t tile_valid = FULL ? (uint32_t)TILE : ((tile + 1) * TILE <= n ? TILE : n - tile * TILE);
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const uint32_t p = j * kSortThreads + tid;
        if (FULL || p < tile_valid) {
            uint32_t k, v = 0;
            Elem e{};
            if (MODE == kPairs) {
                const uint2 kv = s_pairs[p];
                k = kv.x;
                v = kv.y;
            } else {
                e = s_keys[p];
                if (MODE == kUvec2) k = (reinterpret_cast<const uint2*>(&e))->x;
                else k = *(reinterpret_cast<const uint32_t*>(&e));
            }
            const uint32_t d = digit_of(k, shift, width);
            const uint32_t dst = (uint32_t)((int32_t)p + sm.delta[d]);
            if (dst < n) {  // false only after a timed-out look-back (error recorded)
                if (MODE == kUvec2) {
                    reinterpret_cast<uint2*>(out_keys)[dst] = *(reinterpret_cast<const uint2*>(&e));
                } else {
                    out_keys[dst] = k;
                    if (MODE == kPairs) out_vals[dst] = v;
                }
            }
        }
    }
}

template <int DIGIT_BITS, int ITEMS, int MODE, int RANK>
__global__ void __launch_bounds__(kSortThreads, 4) onesweep_pass_kernel(
    const uint32_t* in_keys, const uint32_t* in_vals,
    uint32_t* __restrict__ out_keys, uint32_t* __restrict__ out_vals,
    uint32_t n, uint32_t pass, uint32_t shift, uint32_t width, uint32_t num_tiles,
    uint32_t* __restrict__ scratch, uint32_t wait_limit, uint32_t spin)
{
    pdl_enter();
    constexpr int TILE = kSortThreads * ITEMS;
    extern __shared__ uint4 s_stage[];
    __shared__ PassSmem<DIGIT_BITS, ITEMS, MODE, RANK> sm;
    __shared__ uint32_t s_tile;
    const uint32_t tid = threadIdx.x;
    if (tid == 0) s_tile = atomicAdd(scratch + pass, 1u);
    for (uint32_t i = tid; i < kSortWarps * (1u << DIGIT_BITS); i += kSortThreads) (&sm.warp_hist[0][0])[i] = 0u;
    __syncthreads();
    const uint32_t tile = s_tile;
    if ((uint64_t)(tile + 1) * TILE <= n)
        onesweep_pass_body<DIGIT_BITS, ITEMS, MODE, RANK, true>(in_keys, in_vals, out_keys, out_vals, n, pass, shift,
                                                                width, num_tiles, scratch, wait_limit, spin, tile, sm,
                                                                s_stage);
    else
        onesweep_pass_body<DIGIT_BITS, ITEMS, MODE, RANK, false>(in_keys, in_vals, out_keys, out_vals, n, pass, shift,
                                                                 width, num_tiles, scratch, wait_limit, spin, tile, sm,
                                                                 s_stage);
}

}  // namespace vren_gb300

#include "radix_persistent.cuh"

namespace vren_gb300 {

// ------------------------------------------------------------------------------------------------
// Bucket end offsets from the sorted output: end[b] = number of elements with bucket <= b.
// Thread i (i in [-1, n)) writes end[b] = i + 1 for every b in [bucket(i), bucket(i+1)).
// ------------------------------------------------------------------------------------------------
__global__ void bucket_end_offsets_kernel(const uint2* __restrict__ sorted, uint32_t n, uint32_t key_mask,
                                          uint32_t* __restrict__ ends)
{
    const uint32_t nb = key_mask + 1u;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - 1; i < (int64_t)n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t lo = (i < 0) ? 0u : (sorted[i].x & key_mask);
        const uint32_t hi = (i + 1 < (int64_t)n) ? (sorted[i + 1].x & key_mask) : nb;
        const uint32_t v = (uint32_t)(i + 1);
        for (uint32_t b = (i < 0 ? 0u : lo); b < hi; ++b) ends[b] = v;
    }
}

// ------------------------------------------------------------------------------------------------
// Bucket sort in one scatter pass, for up to 10 key bits (1024 buckets).
//
// The reference counts with global atomics, scans its 65536 counters and scatters with atomics
// (vren/primitives/bucket_sort.cpp:116-160, bucket_sort_count.comp:27-33, bucket_sort_write.comp:27-34).
// Here, over tiles of 4096 elements (one matrix row each):
//   1. bucket_tile_hist_kernel: one CTA per row reads it once and writes its 1024 bucket counts as one
//      row of a [rows][1024] matrix (4 KB per 32 KB of elements);
//   2. bucket_column_scan_kernel: each CTA takes a block of 256 rows x 32 columns (every warp load
//      one 128-byte line), turns it into exclusive prefixes over the rows in place, and gets the
//      rows above from the blocks above in its columns by decoupled look-back; the last CTA scans
//      the bucket totals into the start offsets (scratch) and the end offsets (the output's
//      counters region);
//   3. bucket_scatter_kernel: one CTA per row reads it again (keys first; values when staging, from
//      L2), ranks it stably in shared memory (1024 16-bit counters per warp), stages it in bucket
//      order and writes each element to start[bucket] + (the bucket's count in the elements before
//      its tile) + (its rank in the tile).
// Every row's place is known before the scatter starts, so no CTA waits on another (an earlier
// form resolved the tile prefixes by decoupled look-back over 1024 buckets; measured per CTA, that
// look-back was its longest phase).  The scatter takes the rows from the last one down: the
// histogram read the end of the input last, so that part is still in L2.  One tile per row keeps
// the CTAs that write the two halves of a bucket boundary's 32-byte sector running at the same
// time: with two or four tiles per row, written one after the other by one CTA, the DRAM traffic of
// the scatter grew by a third (sectors evicted half written).
// Traffic: the elements read twice and written once (24 B each), plus the matrix written, read and
// written by the scan and read by the scatter (16 KB per 4096 elements, 1/6 of the 96 KB; most of
// it stays in L2 between the three kernels).
// ------------------------------------------------------------------------------------------------
constexpr int kBucketBits = 10;
constexpr uint32_t kBucketRadix = 1u << kBucketBits;
constexpr int kBucketItems = 16;
constexpr uint32_t kBucketTile = kSortThreads * kBucketItems;   // 4096 elements
constexpr uint32_t kBucketRow = kBucketTile;                      // elements per matrix row (one tile)
constexpr int kBucketScanThreads = 256;
constexpr uint32_t kBucketScanCols = 32;                         // columns per scan CTA (128 B of a row)
constexpr uint32_t kBucketScanBlock = 256;                       // rows per scan CTA (32 per warp)
constexpr uint32_t kBucketScanGroups = kBucketRadix / kBucketScanCols;
// Scratch, in uint32 words: [0] scan CTA ticket, [1] finished scan CTAs, [16, 1040) bucket totals,
// [1040, 2064) bucket start offsets, then the count matrix [rows][1024] (16-byte aligned), then the
// scan's look-back words [row blocks][1024].
constexpr uint32_t kBkTotals = 16, kBkStarts = kBkTotals + kBucketRadix, kBkRows = kBkStarts + kBucketRadix;
__host__ __device__ inline uint32_t bucket_scan_blocks(uint32_t rows_n) { return (rows_n + kBucketScanBlock - 1) / kBucketScanBlock; }

__global__ void __launch_bounds__(kSortThreads) bucket_tile_hist_kernel(const uint2* in, uint32_t n,
                                                                       uint32_t key_bits,
                                                                       uint32_t* __restrict__ scratch)
{
    pdl_enter();
    __shared__ alignas(16) uint32_t s_hist[kBucketRadix];
    const uint32_t tid = threadIdx.x, row = blockIdx.x;
    reinterpret_cast<uint4*>(s_hist)[tid] = make_uint4(0u, 0u, 0u, 0u);
    if (row == 0 && tid < 2) scratch[tid] = 0u;  // the scan's CTA ticket and finished count
    {
        // the scan's look-back words start unpublished
        const uint32_t rows_n = gridDim.x;
        const uint32_t words = bucket_scan_blocks(rows_n) * kBucketRadix;
        uint32_t* status = scratch + kBkRows + (size_t)rows_n * kBucketRadix;
        for (uint32_t i = row * kSortThreads + tid; i < words; i += rows_n * kSortThreads) status[i] = 0u;
    }
    __syncthreads();
    const uint32_t mask = (1u << key_bits) - 1u;
    const uint32_t base = row * kBucketRow;
    if (base + kBucketRow <= n) {
        // chunks of 4096 uint4 (two elements each), sixteen per thread, each chunk's loads in flight
        constexpr int Q = kBucketRow >= 2u * 16u * kSortThreads ? 16 : (int)(kBucketRow / 2u / kSortThreads);
        constexpr uint32_t kChunk = 2u * Q * kSortThreads;
        static_assert(kBucketRow % kChunk == 0, "rows are whole chunks");
#pragma unroll 1
        for (uint32_t c = 0; c < kBucketRow; c += kChunk) {
            const uint4* p4 = reinterpret_cast<const uint4*>(in + base + c);
            uint4 q[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) q[k] = __ldg(p4 + tid + k * kSortThreads);
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                atomicAdd(&s_hist[q[k].x & mask], 1u);
                atomicAdd(&s_hist[q[k].z & mask], 1u);
            }
        }
    } else {
        for (uint32_t i = base + tid; i < n; i += kSortThreads) atomicAdd(&s_hist[__ldg(&in[i].x) & mask], 1u);
    }
    __syncthreads();
    reinterpret_cast<uint4*>(scratch + kBkRows + (size_t)row * kBucketRadix)[tid] =
        reinterpret_cast<const uint4*>(s_hist)[tid];
}

// Test hook (vren_test_withhold_bucket_scan_status): row block + 1 whose look-back words the column
// scan never publishes, so the blocks after it run out their bounded waits; 0 (the default)
// publishes every block.
__device__ uint32_t g_bucket_withheld_block = 0;

__global__ void __launch_bounds__(kBucketScanThreads) bucket_column_scan_kernel(uint32_t* scratch, uint32_t rows_n,
                                                                              uint32_t key_bits, uint32_t* ends,
                                                                              uint32_t wait_limit, uint32_t spin)
{
    // Let the scatter launch at once (it loads and ranks its tiles meanwhile and waits for this grid
    // before it reads the matrix), then wait for the histograms.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    constexpr uint32_t kWarps = kBucketScanThreads / 32u;
    constexpr uint32_t kRowsPerWarp = kBucketScanBlock / kWarps;
    __shared__ uint32_t s_wsum[kWarps][32];
    __shared__ uint32_t s_look[kWarps][32];
    __shared__ uint32_t s_unit;
    __shared__ bool s_last;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    // Units in the order the CTAs start, so a unit's predecessors in its column group have started.
    if (tid == 0) s_unit = atomicAdd(scratch, 1u);
    __syncthreads();
    const uint32_t unit = s_unit;
    const uint32_t blocks = bucket_scan_blocks(rows_n);
    const uint32_t rb = unit / kBucketScanGroups;
    const uint32_t col = (unit % kBucketScanGroups) * kBucketScanCols + lane;
    uint32_t* mat = scratch + kBkRows;
    uint32_t* status = mat + (size_t)rows_n * kBucketRadix;

    // Warp w: rows r0 .. r0+31 of the block, lane = column (each load one 128-byte line).
    const uint32_t r0 = rb * kBucketScanBlock + warp * kRowsPerWarp;
    uint32_t v[kRowsPerWarp];
#pragma unroll
    for (uint32_t i = 0; i < kRowsPerWarp; ++i)
        v[i] = r0 + i < rows_n ? mat[(size_t)(r0 + i) * kBucketRadix + col] : 0u;
    uint32_t run = 0;
#pragma unroll
    for (uint32_t i = 0; i < kRowsPerWarp; ++i) {
        const uint32_t x = v[i];
        v[i] = run;
        run += x;
    }
    s_wsum[warp][lane] = run;
    __syncthreads();
    uint32_t agg = 0, before = 0;
#pragma unroll
    for (uint32_t w = 0; w < kWarps; ++w) {
        const uint32_t x = s_wsum[w][lane];
        before += w < warp ? x : 0u;
        agg += x;
    }
    uint32_t* my_status = status + (size_t)rb * kBucketRadix + col;
    const bool publish = rb + 1u != *reinterpret_cast<volatile uint32_t*>(&g_bucket_withheld_block);
    if (warp == 0 && publish) st_relaxed_u32(my_status, (rb == 0 ? kFlagPrefix : kFlagAggregate) | agg);

    // Look-back over the blocks above in the same columns, eight blocks a round (warp w reads block
    // base - w); every warp folds the round's words the same way, so all hold the prefix.
    uint32_t excl = 0;
    if (rb != 0) {
        bool done = false;
        for (int64_t base = (int64_t)rb - 1;; base -= kWarps) {
            const int64_t p = base - (int64_t)warp;
            uint32_t word = kFlagPrefix;  // above the first block: a zero prefix
            if (p >= 0 && !done)
                word = wait_for_flag(status + (size_t)p * kBucketRadix + col, wait_limit, spin,
                                     [] { VREN_RECORD_ERROR(VREN_ERR_TIMEOUT); });
            s_look[warp][lane] = word;
            __syncthreads();
#pragma unroll
            for (uint32_t w = 0; w < kWarps; ++w) {
                const uint32_t x = s_look[w][lane];
                if (!done) {
                    excl += x & kValueMask;
                    done = (x & kFlagPrefix) != 0;
                }
            }
            if (__syncthreads_and(done)) break;  // also keeps s_look until every warp has read it
        }
        if (warp == 0 && publish) st_relaxed_u32(my_status, kFlagPrefix | (excl + agg));
    }
    if (warp == 0 && rb == blocks - 1) scratch[kBkTotals + col] = excl + agg;
    const uint32_t add = excl + before;
#pragma unroll
    for (uint32_t i = 0; i < kRowsPerWarp; ++i)
        if (r0 + i < rows_n) mat[(size_t)(r0 + i) * kBucketRadix + col] = v[i] + add;

    // The last CTA to finish turns the totals into the bucket start offsets (scratch) and end
    // offsets (the output's counters region), four buckets per thread.
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(scratch + 1, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const uint32_t b = 4u * tid;
    uint32_t t[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) t[k] = ld_relaxed_u32(scratch + kBkTotals + b + k);
    const uint32_t sum4 = t[0] + t[1] + t[2] + t[3];
    uint32_t incl = sum4;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= (uint32_t)d) incl += y;
    }
    if (lane == 31) s_wsum[0][warp] = incl;
    __syncthreads();
    for (uint32_t w = 0; w < warp; ++w) incl += s_wsum[0][w];
    uint32_t start = incl - sum4;
    const uint32_t mask = (1u << key_bits) - 1u;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        scratch[kBkStarts + b + k] = start;
        if (b + k <= mask) ends[b + k] = start + t[k];
        start += t[k];
    }
}

__device__ __forceinline__ uint4 ld_v4_after_wait(const uint32_t* p)
{
    uint4 v;
    asm volatile("ld.relaxed.gpu.global.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p) : "memory");
    return v;
}

struct alignas(16) BucketSmem {
    uint16_t warp_hist[kSortWarps][kBucketRadix];  // per-warp bucket counts, then each warp's first staging slot
    int32_t delta[kBucketRadix];  // the tile's place in each bucket - the bucket's staging start
    uint32_t wsum[kSortWarps];
};

// Tile `tile` (4096 elements, one matrix row); sm.warp_hist is zero on entry.  In the RAGGED last
// tile the slots past n take the key `mask`, the last bucket: ranked after every element of the
// tile (their indices are the highest), they land at or past the end of that bucket, which is n,
// and are not written.
template <int RANK, bool RAGGED>
__device__ __forceinline__ void bucket_scatter_body(const uint2* __restrict__ in, uint2* __restrict__ out, uint32_t n,
                                                    uint32_t key_bits, uint32_t tile,
                                                    const uint32_t* __restrict__ scratch, BucketSmem& sm,
                                                    uint2* s_stage)
{
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t mask = (1u << key_bits) - 1u;

    // Striped load of the keys: item j of lane l is element warp_base + 32*j + l.  The values are
    // read again when the tile is staged (the line is still in L2), so only keys stay in registers.
    const uint32_t warp_base = tile * kBucketTile + warp * (32u * kBucketItems);
    const uint32_t* keys = reinterpret_cast<const uint32_t*>(in);
    uint32_t k[kBucketItems];
    uint32_t pos[kBucketItems];
#pragma unroll
    for (int j = 0; j < kBucketItems; ++j) {
        const uint32_t idx = warp_base + 32u * j + lane;
        k[j] = (!RAGGED || idx < n) ? __ldg(keys + 2u * idx) : mask;
    }
    // RANK 1's per-warp bucket-name table (1 KB per warp), inside the staging area, which is free
    // until the tile is ranked.
    uint8_t* rep_tab = reinterpret_cast<uint8_t*>(s_stage) + warp * kBucketRadix;

    // Stable in-warp ranks, items in order: peers (lanes with my bucket) from one ballot per key bit
    // (RANK 0; bits at and above key_bits are zero in every lane, so all ten ballots serve any
    // key_bits), from a bucket name and five ballots (RANK 1) or from match.any (RANK 2).
#pragma unroll
    for (int j = 0; j < kBucketItems; ++j) {
        const uint32_t d = k[j] & mask;
        uint32_t peers;
        if (RANK == 2) {
            peers = __match_any_sync(0xFFFFFFFFu, d);
        } else if (RANK == 1) {
            // Every lane writes its id into its bucket's slot of a per-warp table; the lanes of one
            // bucket then read back the same id (whichever write landed), a 5-bit name for the bucket
            // within the warp, and five ballots on that name find the peers.
            rep_tab[d] = (uint8_t)lane;
            __syncwarp();
            const uint32_t r = rep_tab[d];
            peers = 0xFFFFFFFFu;
#pragma unroll
            for (int b = 0; b < 5; ++b) {
                const bool bit = (r >> b) & 1u;
                const uint32_t m = __ballot_sync(0xFFFFFFFFu, bit);
                peers &= bit ? m : ~m;
            }
        } else {
            peers = 0xFFFFFFFFu;
#pragma unroll
            for (int b = 0; b < kBucketBits; ++b) {
                const bool bit = (d >> b) & 1u;
                const uint32_t m = __ballot_sync(0xFFFFFFFFu, bit);
                peers &= bit ? m : ~m;
            }
        }
        const uint32_t below = peers & lanemask_lt();
        const uint32_t before = sm.warp_hist[warp][d];
        __syncwarp();
        if (below == 0) sm.warp_hist[warp][d] = (uint16_t)(before + __popc(peers));
        __syncwarp();
        pos[j] = d | ((before + __popc(below)) << kBucketBits);
    }
    __syncthreads();

    // Thread t owns buckets 4t..4t+3: warp prefixes, the tile's counts and tile-local offsets.
    uint32_t cnt[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
        uint2* row = reinterpret_cast<uint2*>(sm.warp_hist[w]) + tid;  // four uint16 counters
        const uint2 x = *row;
        *row = make_uint2(cnt[0] | (cnt[1] << 16), cnt[2] | (cnt[3] << 16));
        cnt[0] += x.x & 0xFFFFu; cnt[1] += x.x >> 16; cnt[2] += x.y & 0xFFFFu; cnt[3] += x.y >> 16;
    }
    const uint32_t sum4 = cnt[0] + cnt[1] + cnt[2] + cnt[3];
    uint32_t incl = sum4;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) sm.wsum[warp] = incl;
    __syncthreads();
    uint32_t excl0 = incl - sum4;
    for (uint32_t w = 0; w < warp; ++w) excl0 += sm.wsum[w];
    const uint32_t excl1 = excl0 + cnt[0], excl2 = excl1 + cnt[1], excl3 = excl2 + cnt[2];
    const uint32_t e01 = excl0 | (excl1 << 16), e23 = excl2 | (excl3 << 16);
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
        uint2* row = reinterpret_cast<uint2*>(sm.warp_hist[w]) + tid;
        const uint2 x = *row;  // per-lane sums stay below 2^16 (at most 4096)
        *row = make_uint2(x.x + e01, x.y + e23);
    }
    __syncthreads();

    // Stage in bucket order (the value read again, from L2).
#pragma unroll
    for (int j = 0; j < kBucketItems; ++j) {
        const uint32_t d = pos[j] & (kBucketRadix - 1u);
        const uint32_t idx = warp_base + 32u * j + lane;
        const uint32_t v = (!RAGGED || idx < n) ? __ldg(keys + 2u * idx + 1u) : 0u;
        s_stage[sm.warp_hist[warp][d] + (pos[j] >> kBucketBits)] = make_uint2(k[j], v);
    }
    {
        // The tile's place in each bucket: start + the bucket's count in the tiles before (the column
        // scan's output, which this grid may only read once that kernel has completed), less the
        // bucket's staging start (warp 0's first slot, which is the tile-local exclusive offset).
        // (inline-assembly loads, so the compiler cannot move them above the wait, as it may move
        // loads through a const __restrict__ pointer)
        asm volatile("griddepcontrol.wait;" ::: "memory");
        const uint4 col = ld_v4_after_wait(scratch + kBkRows + (size_t)tile * kBucketRadix + 4u * tid);
        const uint4 start = ld_v4_after_wait(scratch + kBkStarts + 4u * tid);
        const uint2 w0 = reinterpret_cast<const uint2*>(sm.warp_hist[0])[tid];
        reinterpret_cast<int4*>(sm.delta)[tid] = make_int4((int32_t)(start.x + col.x) - (int32_t)(w0.x & 0xFFFFu),
                                                           (int32_t)(start.y + col.y) - (int32_t)(w0.x >> 16),
                                                           (int32_t)(start.z + col.z) - (int32_t)(w0.y & 0xFFFFu),
                                                           (int32_t)(start.w + col.w) - (int32_t)(w0.y >> 16));
    }
    __syncthreads();

    // Write out: consecutive threads take consecutive staged elements.
#pragma unroll
    for (int j = 0; j < kBucketItems; ++j) {
        const uint32_t p = j * kSortThreads + tid;
        const uint2 v = s_stage[p];
        const uint32_t dst = (uint32_t)((int32_t)p + sm.delta[v.x & mask]);
        if (dst < n) out[dst] = v;
    }
}

// Launched as a programmatic dependent of the column scan: each CTA loads and ranks its tile while
// the scan may still be running, and waits for it (griddepcontrol.wait) only before reading the
// scan's output.
template <int RANK>
__global__ void __launch_bounds__(kSortThreads, 4) bucket_scatter_kernel(const uint2* __restrict__ in,
                                                                        uint2* __restrict__ out, uint32_t n,
                                                                        uint32_t key_bits, uint32_t num_rows,
                                                                        const uint32_t* __restrict__ scratch)
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    extern __shared__ uint4 s_dyn[];
    __shared__ BucketSmem sm;
    const uint32_t tid = threadIdx.x;
    uint4* h4 = reinterpret_cast<uint4*>(&sm.warp_hist[0][0]);
    for (uint32_t i = tid; i < sizeof(sm.warp_hist) / 16u; i += kSortThreads) h4[i] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    const uint32_t tile = num_rows - 1u - blockIdx.x;
    uint2* s_stage = reinterpret_cast<uint2*>(s_dyn);
    if ((uint64_t)(tile + 1) * kBucketTile <= n)
        bucket_scatter_body<RANK, false>(in, out, n, key_bits, tile, scratch, sm, s_stage);
    else
        bucket_scatter_body<RANK, true>(in, out, n, key_bits, tile, scratch, sm, s_stage);
}

// ------------------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------------------
// Keys per thread: variant 0 = 15 (8-bit digits) / 16, variant 1 = 23 / 24 (bigger tiles).
template <int DB, int V> constexpr int items_for() { return V == 1 ? (DB >= 8 ? 23 : 24) : (DB >= 8 ? 15 : 16); }

static uint32_t tile_of(uint32_t digit_bits, int variant)
{
    const uint32_t items = variant == 1 ? (digit_bits >= 8 ? 23u : 24u) : (digit_bits >= 8 ? 15u : 16u);
    return kSortThreads * items;
}

// Scratch is sized for the smaller tile (more tiles), so every variant fits.
// Status rows per buffer: enough for the smallest tile of either pass form.
static uint32_t tiles_for(uint32_t n, uint32_t digit_bits)
{
    const uint32_t tile = tile_of(digit_bits, 0) < kPTile ? tile_of(digit_bits, 0) : kPTile;
    return (n + tile - 1) / tile;
}

static uint32_t radix_of(uint32_t digit_bits) { return 1u << digit_bits; }

static size_t scratch1_bytes(uint32_t n, uint32_t digit_bits)
{
    const uint64_t tiles = tiles_for(n, digit_bits);
    return (size_t)(kStatusOffset + 2ull * (tiles ? tiles : 1) * radix_of(digit_bits)) * sizeof(uint32_t);
}

static bool supported_bits(uint32_t db) { return db == 4 || db == 5 || db == 6 || db == 8; }

// Persistent pass grid: SMs x resident CTAs (shared memory opted in once per variant).
template <int DB, int MODE>
static int launch_persistent_pass(cudaStream_t st, const uint32_t* sk, const uint32_t* sv, uint32_t* ok, uint32_t* ov,
                                  uint32_t n, uint32_t p, uint32_t shift, uint32_t width, uint32_t tiles,
                                  uint32_t* scratch, uint32_t spin)
{
    constexpr size_t smem = persist_dyn_smem<DB, MODE>();
    auto kern = onesweep_persistent_kernel<DB, MODE>;
    static int grid = 0;  // per variant
    if (grid == 0) {
        VREN_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int dev = 0, sms = 0, per_sm = 0;
        VREN_CUDA_TRY(cudaGetDevice(&dev));
        VREN_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        VREN_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPThreads, smem));
        grid = sms * (per_sm > 0 ? per_sm : 1);
    }
    const uint32_t g = tiles < (uint32_t)grid ? tiles : (uint32_t)grid;
    VREN_CUDA_TRY(launch_kernel(kern, g, kPThreads, smem, st, sk, sv, ok, ov, n, p, shift, width, tiles, scratch,
                                g_wait_limit, spin));
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

template <int DB, int MODE, int V, int RANK>
static int launch_pass(cudaStream_t st, const uint32_t* sk, const uint32_t* sv, uint32_t* ok, uint32_t* ov, uint32_t n,
                       uint32_t p, uint32_t shift, uint32_t width, uint32_t tiles, uint32_t* scratch, uint32_t spin)
{
    constexpr int ITEMS = items_for<DB, V>();
    constexpr size_t elem = MODE == kUvec2 ? 8 : 4;
    constexpr size_t smem = (size_t)kSortThreads * ITEMS * (elem + (MODE == kPairs ? 4 : 0));
    auto kern = onesweep_pass_kernel<DB, ITEMS, MODE, RANK>;
    VREN_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    VREN_CUDA_TRY(launch_kernel(kern, tiles, kSortThreads, smem, st, sk, sv, ok, ov, n, p, shift, width, tiles, scratch,
                                g_wait_limit, spin));
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

template <int DB, int MODE>
static int run_passes(cudaStream_t st, const uint32_t* src_k, const uint32_t* src_v, uint32_t* dst_k, uint32_t* dst_v,
                      uint32_t* tmp_k, uint32_t* tmp_v, uint32_t n, const PassInfo& passes, uint32_t* scratch)
{
    constexpr int RADIX = 1 << DB;
    const int variant = tuning(VREN_TUNE_RADIX_ITEMS) == 1 ? 1 : 0;
    const int rank = tuning(VREN_TUNE_RADIX_RANK);
    const uint32_t spin = (uint32_t)tuning(VREN_TUNE_SPIN_POLLS);
    // One pass form for the whole sort (the two use different tile counts, hence status row strides):
    // the persistent one when every buffer a pass may read starts 16-byte aligned.
    const bool aligned = ((reinterpret_cast<uintptr_t>(src_k) | reinterpret_cast<uintptr_t>(src_v) |
                           reinterpret_cast<uintptr_t>(dst_k) | reinterpret_cast<uintptr_t>(dst_v) |
                           reinterpret_cast<uintptr_t>(tmp_k) | reinterpret_cast<uintptr_t>(tmp_v)) & 15u) == 0;
    const bool persistent = MODE != kUvec2 && variant == 0 && rank == 0 &&
                            tuning(VREN_TUNE_RADIX_PERSISTENT) != 0 && aligned;
    const uint32_t tile_n = persistent ? kPTile : tile_of(DB, variant);
    const uint32_t tiles = (n + tile_n - 1) / tile_n;
    const uint32_t status_tiles = tiles_for(n, DB);  // rows per status buffer (scratch layout)

    VREN_CUDA_TRY(cudaMemsetAsync(scratch, 0, kZeroWords * sizeof(uint32_t), st));
    uint32_t hist_grid = (n / 4 + kSortThreads - 1) / kSortThreads;
    if (hist_grid > (uint32_t)kNumSMsHint * 4) hist_grid = kNumSMsHint * 4;
    if (hist_grid == 0) hist_grid = 1;
    launch_kernel(onesweep_hist_kernel<RADIX, MODE>, hist_grid, kSortThreads, 0, st, src_k, n, passes, scratch, tiles * RADIX);
    VREN_LAUNCH_CHECK();

    const uint32_t P = passes.count;
    for (uint32_t p = 0; p < P; ++p) {
        // dst of pass p: the final buffer when (P-1-p) is even, else the temporary.
        const bool to_final = ((P - 1 - p) % 2) == 0;
        uint32_t* ok = to_final ? dst_k : tmp_k;
        uint32_t* ov = to_final ? dst_v : tmp_v;
        int rc;
#define VREN_PASS(V, R) launch_pass<DB, MODE, V, R>(st, src_k, src_v, ok, ov, n, p, passes.shift[p], passes.width[p], tiles, scratch, spin)
        if (persistent)
            rc = launch_persistent_pass<DB, MODE == kUvec2 ? kKeys : MODE>(st, src_k, src_v, ok, ov, n, p,
                                                                          passes.shift[p], passes.width[p], tiles,
                                                                          scratch, spin);
        else if (variant == 1) rc = rank == 1 ? VREN_PASS(1, 1) : rank == 2 ? VREN_PASS(1, 2) : VREN_PASS(1, 0);
        else rc = rank == 1 ? VREN_PASS(0, 1) : rank == 2 ? VREN_PASS(0, 2) : VREN_PASS(0, 0);
#undef VREN_PASS
        if (rc != VREN_OK) return rc;
        src_k = ok;
        src_v = ov;
    }
    (void)status_tiles;
    return VREN_OK;
}

template <int MODE>
static int radix_dispatch(cudaStream_t st, uint32_t db, const uint32_t* src_k, const uint32_t* src_v, uint32_t* dst_k,
                          uint32_t* dst_v, uint32_t* tmp_k, uint32_t* tmp_v, uint32_t n, const PassInfo& passes,
                          uint32_t* scratch)
{
    switch (db) {
    case 4: return run_passes<4, MODE>(st, src_k, src_v, dst_k, dst_v, tmp_k, tmp_v, n, passes, scratch);
    case 5: return run_passes<5, MODE>(st, src_k, src_v, dst_k, dst_v, tmp_k, tmp_v, n, passes, scratch);
    case 6: return run_passes<6, MODE>(st, src_k, src_v, dst_k, dst_v, tmp_k, tmp_v, n, passes, scratch);
    case 8: return run_passes<8, MODE>(st, src_k, src_v, dst_k, dst_v, tmp_k, tmp_v, n, passes, scratch);
    default: return VREN_ERR_ARG;
    }
}

static PassInfo make_passes(uint32_t key_bits, uint32_t digit_bits)
{
    PassInfo pi{};
    pi.count = (key_bits + digit_bits - 1) / digit_bits;
    // Spread the bits evenly: widths differ by at most one, none exceeds digit_bits.
    uint32_t shift = 0;
    for (uint32_t p = 0; p < pi.count; ++p) {
        uint32_t remaining = key_bits - shift;
        uint32_t left = pi.count - p;
        uint32_t w = (remaining + left - 1) / left;
        pi.shift[p] = shift;
        pi.width[p] = w;
        shift += w;
    }
    return pi;
}

}  // namespace vren_gb300

using namespace vren_gb300;

extern "C" size_t vren_radix_sort_scratch1_bytes(uint32_t n, uint32_t digit_bits)
{
    if (!supported_bits(digit_bits)) return 0;
    return scratch1_bytes(n, digit_bits);
}

// Once a pass has more tiles than one wave of resident CTAs, each pass launches while the one
// before ends and waits for it in-kernel (measured: 2^22 pairs 0.181 -> 0.167 ms, 2^26 1.83 ->
// 1.81 ms).  With fewer tiles the next pass's CTAs would all wait resident and start at once,
// which measured slower (2^20 pairs: 0.085 -> 0.094 ms), so those sorts keep the caller's setting.
static int passes_pdl(uint32_t n, uint32_t digit_bits)
{
    return n / tile_of(digit_bits, tuning(VREN_TUNE_RADIX_ITEMS) == 1 ? 1 : 0) > 4u * kNumSMsHint ? 1 : g_pdl;
}

extern "C" int vren_radix_sort_u32_ex(vren_stream_t s, uint32_t* keys, uint32_t* values, uint32_t n, uint32_t digit_bits,
                                      void* scratch1, uint32_t* scratch_keys, uint32_t* scratch_values)
{
    if (!supported_bits(digit_bits) || !scratch1 || (n > 0 && (!keys || !scratch_keys))) return VREN_ERR_ARG;
    if (values && !scratch_values) return VREN_ERR_ARG;
    if (n >= (1u << 30)) return VREN_ERR_ARG;
    if (((uintptr_t)keys & 15u) || ((uintptr_t)scratch1 & 15u)) return VREN_ERR_ARG;
    if (n <= 1) return VREN_OK;
    cudaStream_t st = as_stream(s);
    const PdlScope pdl(passes_pdl(n, digit_bits));
    PassInfo passes = make_passes(32, digit_bits);
    uint32_t* sc = static_cast<uint32_t*>(scratch1);
    const uint32_t* src_k = keys;
    const uint32_t* src_v = values;
    if (passes.count % 2 == 1) {
        // With an odd pass count the first pass would run in place: start from a copy.
        VREN_CUDA_TRY(cudaMemcpyAsync(scratch_keys, keys, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
        if (values) VREN_CUDA_TRY(cudaMemcpyAsync(scratch_values, values, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
        src_k = scratch_keys;
        src_v = scratch_values;
    }
    if (values)
        return radix_dispatch<kPairs>(st, digit_bits, src_k, src_v, keys, values, scratch_keys, scratch_values, n, passes, sc);
    return radix_dispatch<kKeys>(st, digit_bits, src_k, nullptr, keys, nullptr, scratch_keys, nullptr, n, passes, sc);
}

extern "C" int vren_radix_sort_u32(vren_stream_t s, uint32_t* keys, uint32_t n, void* scratch1, uint32_t* scratch2)
{
    // vren/primitives/radix_sort.cpp:158-161: "Length must be higher than 1024 and a power of 2"
    if (!(n >= 1024 && (n & (n - 1)) == 0)) return VREN_ERR_ARG;
    return vren_radix_sort_u32_ex(s, keys, nullptr, n, 8, scratch1, scratch2, nullptr);
}

static uint32_t bucket_digit_bits(uint32_t key_bits)
{
    const uint32_t passes = (key_bits + 7) / 8;
    const uint32_t w = (key_bits + passes - 1) / passes;
    return w <= 4 ? 4 : w == 5 ? 5 : w == 6 ? 6 : 8;
}

extern "C" size_t vren_bucket_sort_output_bytes(uint32_t n, uint32_t key_bits)
{
    if (key_bits == 0 || key_bits > 16) return 0;
    const size_t pairs = ((size_t)n * 8 + 255) / 256 * 256;
    return pairs + ((size_t)1 << key_bits) * sizeof(uint32_t);
}

// The one-scatter form (up to 10 key bits): header, bucket totals and starts, and one 1024-word row
// of the count matrix per 4096-element tile.
static size_t bucket_onepass_scratch_bytes(uint32_t n)
{
    uint64_t rows = ((uint64_t)n + kBucketRow - 1) / kBucketRow;
    if (rows == 0) rows = 1;
    return (size_t)(kBkRows + (rows + bucket_scan_blocks((uint32_t)rows)) * kBucketRadix) * sizeof(uint32_t);
}

// The radix-pass form: digit-pass scratch, then a ping-pong element buffer.
static size_t bucket_passes_scratch_bytes(uint32_t n, uint32_t key_bits)
{
    const size_t status = scratch1_bytes(n, bucket_digit_bits(key_bits));
    const size_t tmp = ((size_t)n * 8 + 255) / 256 * 256;
    return ((status + 255) / 256 * 256) + tmp;
}

extern "C" size_t vren_bucket_sort_scratch_bytes(uint32_t n, uint32_t key_bits)
{
    if (key_bits == 0 || key_bits > 16) return 0;
    const size_t passes = bucket_passes_scratch_bytes(n, key_bits);
    if (key_bits > (uint32_t)kBucketBits) return passes;
    // Either form may run (VREN_TUNE_BUCKET_FORM), so the scratch fits both.
    const size_t one = bucket_onepass_scratch_bytes(n);
    return one > passes ? one : passes;
}

static int bucket_sort_onepass(cudaStream_t st, const uint2* in, uint32_t n, uint2* out, uint32_t* ends,
                               uint32_t key_bits, uint32_t* scratch)
{
    if (n == 0) {
        VREN_CUDA_TRY(cudaMemsetAsync(ends, 0, sizeof(uint32_t) << key_bits, st));
        return VREN_OK;
    }
    const uint32_t rows = (n + kBucketRow - 1) / kBucketRow;
    VREN_CUDA_TRY(launch_kernel(bucket_tile_hist_kernel, rows, kSortThreads, 0, st, in, n, key_bits, scratch));
    VREN_LAUNCH_CHECK();
    PdlScope pdl(1);  // the scan and the scatter start early and wait for their predecessor in-kernel
    const uint32_t scan_ctas = bucket_scan_blocks(rows) * kBucketScanGroups;
    VREN_CUDA_TRY(launch_kernel(bucket_column_scan_kernel, scan_ctas, kBucketScanThreads, 0, st, scratch, rows, key_bits,
                                ends, g_wait_limit, (uint32_t)tuning(VREN_TUNE_SPIN_POLLS)));
    VREN_LAUNCH_CHECK();
    constexpr size_t smem = (size_t)kBucketTile * sizeof(uint2);
    const int rank = tuning(VREN_TUNE_RADIX_RANK);
    auto kern = rank == 0 ? bucket_scatter_kernel<0> : rank == 1 ? bucket_scatter_kernel<1> : bucket_scatter_kernel<2>;
    static bool opted[3] = {false, false, false};
    if (!opted[rank]) {
        VREN_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        opted[rank] = true;
    }
    VREN_CUDA_TRY(launch_kernel(kern, rows, kSortThreads, smem, st, in, out, n, key_bits, rows,
                                static_cast<const uint32_t*>(scratch)));
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

extern "C" int vren_test_withhold_bucket_scan_status(uint32_t block_plus_one)
{
    return cudaMemcpyToSymbol(g_bucket_withheld_block, &block_plus_one, sizeof(block_plus_one)) == cudaSuccess
               ? VREN_OK
               : VREN_ERR_CUDA;
}

extern "C" int vren_bucket_sort_u32x2(vren_stream_t s, const uint32_t* in, uint32_t n, void* out, uint32_t key_bits,
                                      void* scratch)
{
    if (key_bits == 0 || key_bits > 16 || !out || !scratch || (n > 0 && !in)) return VREN_ERR_ARG;
    if (n >= (1u << 30)) return VREN_ERR_ARG;
    if (((uintptr_t)in & 15u) || ((uintptr_t)out & 255u) || ((uintptr_t)scratch & 255u)) return VREN_ERR_ARG;
    cudaStream_t st = as_stream(s);
    uint32_t* out_pairs = static_cast<uint32_t*>(out);
    uint32_t* ends = reinterpret_cast<uint32_t*>(static_cast<char*>(out) + ((size_t)n * 8 + 255) / 256 * 256);
    uint32_t* sc = static_cast<uint32_t*>(scratch);
    if (key_bits <= (uint32_t)kBucketBits && tuning(VREN_TUNE_BUCKET_FORM) == 0)
        return bucket_sort_onepass(st, reinterpret_cast<const uint2*>(in), n, reinterpret_cast<uint2*>(out_pairs), ends,
                                   key_bits, sc);
    const uint32_t db = bucket_digit_bits(key_bits);
    uint32_t* tmp = reinterpret_cast<uint32_t*>(static_cast<char*>(scratch) + (scratch1_bytes(n, db) + 255) / 256 * 256);
    if (n > 0) {
        const PdlScope pdl(passes_pdl(n, db));
        PassInfo passes = make_passes(key_bits, db);
        int rc = radix_dispatch<kUvec2>(st, db, in, nullptr, out_pairs, nullptr, tmp, nullptr, n, passes, sc);
        if (rc != VREN_OK) return rc;
    }
    const uint32_t key_mask = (1u << key_bits) - 1u;
    uint32_t grid = (n + 1 + 255) / 256;
    if (grid > 4096) grid = 4096;
    bucket_end_offsets_kernel<<<grid, 256, 0, st>>>(reinterpret_cast<const uint2*>(out_pairs), n, key_mask, ends);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

namespace vren_gb300 {
size_t sort_uvec2_scratch_bytes(uint32_t n, uint32_t key_bits, uint32_t digit_bits)
{
    (void)key_bits;
    return supported_bits(digit_bits) ? scratch1_bytes(n, digit_bits) : 0;
}

int sort_uvec2(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t* tmp, uint32_t n, uint32_t key_bits,
               uint32_t digit_bits, void* scratch)
{
    if (n == 0) return VREN_OK;
    if (!supported_bits(digit_bits) || key_bits == 0 || key_bits > 32) return VREN_ERR_ARG;
    PassInfo passes = make_passes(key_bits, digit_bits);
    if (passes.count > (uint32_t)kMaxPasses) return VREN_ERR_ARG;
    return radix_dispatch<kUvec2>(st, digit_bits, in, nullptr, out, nullptr, tmp, nullptr, n, passes,
                                  static_cast<uint32_t*>(scratch));
}
}  // namespace vren_gb300

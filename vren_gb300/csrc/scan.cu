// Exclusive scan (vren::blelloch_scan, vren/vren/primitives/blelloch_scan.cpp:141-166) and the
// reference's public down-sweep (vren/primitives/blelloch_scan.cpp:57-139, blelloch_scan_downsweep.comp:33-125).
//
// The reference runs an up-sweep (reduce) and then log2(n)-10 global down-sweep dispatches plus
// one shared-memory dispatch, all with strided access.  Here the scan is one kernel and one pass
// over the data (8 bytes of HBM traffic per element): each 8192- (or 4096-) element tile is
// reduced, its aggregate published, its exclusive prefix resolved by decoupled look-back over the
// preceding tiles of its segment, and its exclusive sums written.  Three forms of the kernel:
//  - one CTA per tile, the tile in registers (uint4 loads and stores): small inputs, device-side
//    lengths, unaligned segments;
//  - one CTA per tile staged in shared memory by bulk copies (selectable);
//  - a persistent grid whose producer warp streams tiles into shared memory by bulk copies and
//    publishes their aggregates on arrival while eight consumer warps resolve and store earlier
//    tiles: the default from 2^20 aligned elements.
//
// Scratch layout (uint32 words): [0..1] one 64-bit word [epoch:32 | ticket:32], [2] completion
// counter of the persistent form, [3] unused,
// then one 64-bit status word per tile: [epoch:30 | flag:2 | value:32].  Every CTA takes its tile
// and the call's epoch with one 64-bit atomic add; the CTA that takes the last ticket stores
// [epoch + 1 | 0] right away (every other CTA of the launch has its ticket by then).  Status words
// from an earlier call carry an older epoch and read as "not published", so the scratch needs no
// clearing between calls.  The scratch must be zero-filled before its first use (and again after
// VREN_ERR_TIMEOUT).
#include <mutex>

#include "common.cuh"
#include "internal.h"
#include "lookback.cuh"
#include "tma.cuh"

namespace vren_gb300 {

VREN_DEFINE_ERROR_WORD(scan)

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;  // 4096
constexpr uint32_t kScanHeaderWords = 4;

// Test hook (vren_test_withhold_scan_status): tile + 1 of the one tile whose look-back status the
// scan never publishes, so that its successors' bounded waits run out and record VREN_ERR_TIMEOUT;
// 0 (the default) publishes every tile.  Only lane 0 of the publishing warp reads it, once per tile.
__device__ uint32_t g_scan_withheld_tile = 0;

__device__ __forceinline__ void publish_status(uint64_t* status, uint32_t tile, uint64_t word)
{
    if (tile + 1u != *reinterpret_cast<volatile uint32_t*>(&g_scan_withheld_tile)) st_relaxed_u64(status + tile, word);
}

// Takes this CTA's tile and the call's epoch (thread 0 only); the taker of the last ticket opens the
// next call's epoch.
__device__ __forceinline__ uint32_t take_tile(uint32_t* scratch, uint32_t total_tiles, uint32_t& epoch)
{
    return take_ticket(scratch, total_tiles, epoch);
}

// One CTA = one 4096-element tile; warp w owns 512 contiguous elements as four 128-element slices,
// lane l holding elements 4l..4l+3 of each slice, so every load and store instruction of a warp
// covers 512 contiguous bytes.
//
// `in` may equal `data` (in place).  When n_dev is given the element count is min(*n_dev, n)
// (a single segment whose length is only known on the device); tiles past it do nothing.
// When total_out is given the segment-0 total is written there.
template <int SLICES>
__global__ void __launch_bounds__(kScanThreads, 4) exclusive_scan_kernel(
    const uint32_t* in, uint32_t* data, uint32_t n, uint32_t tiles_per_seg, uint32_t total_tiles,
    uint32_t* __restrict__ scratch, uint32_t wait_limit, uint32_t spin, const uint32_t* n_dev,
    uint32_t* __restrict__ total_out)
{
    pdl_enter();
    constexpr int kSlices = SLICES;
    constexpr uint32_t kTile = SLICES * 128u * (kScanThreads / 32);
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_epoch;
    __shared__ uint32_t s_warp_sum[kScanThreads / 32];
    __shared__ uint32_t s_prefix;

    uint64_t* status = reinterpret_cast<uint64_t*>(scratch + kScanHeaderWords);
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;

    if (tid == 0) {
        uint32_t e;
        s_tile = take_tile(scratch, total_tiles, e);
        s_epoch = e;
    }
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t epoch = s_epoch;
    const uint32_t seg = tile / tiles_per_seg;
    const uint32_t tile_in_seg = tile - seg * tiles_per_seg;
    const size_t seg_off = (size_t)seg * n;
    if (n_dev) {
        const uint32_t m = *n_dev;
        n = m < n ? m : n;
    }
    const uint32_t tiles_eff = (n + kTile - 1) / kTile;
    if (tile_in_seg >= tiles_eff) {
        if (total_out && tiles_eff == 0 && tile == 0 && tid == 0) *total_out = 0u;
        return;
    }
    {
    const uint32_t* seg_in = in + seg_off;
    uint32_t* seg_data = data + seg_off;
    const uint32_t warp_base = tile_in_seg * kTile + warp * (kSlices * 128u);
    const bool full = (tile_in_seg + 1) * kTile <= n;
    const bool aligned = ((reinterpret_cast<uintptr_t>(seg_data) & 15u) == 0) &&
                         ((reinterpret_cast<uintptr_t>(seg_in) & 15u) == 0);
    const bool vec = full && aligned;

    uint32_t v[kSlices][4];
#pragma unroll
    for (int k = 0; k < kSlices; ++k) {
        const uint32_t b = warp_base + k * 128 + lane * 4;
        if (vec) {
            const uint4 q = *reinterpret_cast<const uint4*>(seg_in + b);
            v[k][0] = q.x; v[k][1] = q.y; v[k][2] = q.z; v[k][3] = q.w;
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) v[k][j] = (b + j < n) ? seg_in[b + j] : 0u;
        }
    }

    // Per slice: lane-local exclusive scan of 4 items, warp scan of the lane sums.
    uint32_t lane_off[kSlices];
    uint32_t warp_run = 0;
#pragma unroll
    for (int k = 0; k < kSlices; ++k) {
        uint32_t s = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t x = v[k][j];
            v[k][j] = s;
            s += x;
        }
        uint32_t incl = s;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        lane_off[k] = warp_run + incl - s;
        warp_run += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    if (lane == 0) s_warp_sum[warp] = warp_run;
    __syncthreads();
    uint32_t warp_prefix = 0, tile_sum = 0;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; ++w) {
        const uint32_t ws = s_warp_sum[w];
        if (w < (int)warp) warp_prefix += ws;
        tile_sum += ws;
    }

    if (warp == 0) {
        uint32_t prefix = 0;
        if (tile_in_seg == 0) {
            if (lane == 0) publish_status(status, tile, make_status(epoch, 2u, tile_sum));
        } else {
            if (lane == 0) publish_status(status, tile, make_status(epoch, 1u, tile_sum));
            bool timed_out = false;
            prefix = warp_lookback(status, tile, tile - tile_in_seg, epoch, lane, wait_limit, spin, timed_out);
            if (__any_sync(0xFFFFFFFFu, timed_out) && lane == 0) VREN_RECORD_ERROR(VREN_ERR_TIMEOUT);
            if (lane == 0) publish_status(status, tile, make_status(epoch, 2u, prefix + tile_sum));
        }
        if (lane == 0) {
            s_prefix = prefix;
            if (total_out && seg == 0 && tile_in_seg == tiles_eff - 1) *total_out = prefix + tile_sum;
        }
    }
    __syncthreads();
    const uint32_t base_off = s_prefix + warp_prefix;

#pragma unroll
    for (int k = 0; k < kSlices; ++k) {
        const uint32_t b = warp_base + k * 128 + lane * 4;
        const uint32_t o = base_off + lane_off[k];
        if (vec) {
            *reinterpret_cast<uint4*>(seg_data + b) = make_uint4(v[k][0] + o, v[k][1] + o, v[k][2] + o, v[k][3] + o);
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (b + j < n) seg_data[b + j] = v[k][j] + o;
        }
    }
    }
}

// ------------------------------------------------------------------------------------------------
// Shared-memory staged form of the same scan, for tiles that start on 16-byte boundaries.  Thread 0
// takes the ticket and brings the whole tile into shared memory with one bulk copy (cp.async.bulk,
// completion on an mbarrier); the CTA scans it in place in two passes over shared memory (lane sums,
// then the sums written back), holding a few registers per thread instead of the whole tile, so up to
// seven 32 KB tiles are resident per SM; thread 0 writes the tile back with one bulk store.  The last
// (partial) tile of a segment is read and written with plain loads and stores.
// ------------------------------------------------------------------------------------------------
template <int SLICES>
__global__ void __launch_bounds__(kScanThreads, 6) exclusive_scan_staged_kernel(
    const uint32_t* in, uint32_t* data, uint32_t n, uint32_t tiles_per_seg, uint32_t total_tiles,
    uint32_t* __restrict__ scratch, uint32_t wait_limit, uint32_t spin)
{
    pdl_enter();
    constexpr uint32_t kTile = SLICES * 128u * (kScanThreads / 32);
    constexpr uint32_t kTileBytes = kTile * 4u;
    extern __shared__ __align__(128) uint4 s_buf[];  // one tile
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_epoch;
    __shared__ uint32_t s_warp_sum[kScanThreads / 32];
    __shared__ uint32_t s_prefix;

    uint64_t* status = reinterpret_cast<uint64_t*>(scratch + kScanHeaderWords);
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) {
        uint32_t e;
        const uint32_t t = take_tile(scratch, total_tiles, e);
        s_tile = t;
        s_epoch = e;
        const uint32_t seg = t / tiles_per_seg, ts = t - seg * tiles_per_seg;
        if ((uint64_t)(ts + 1) * kTile <= n) {
            mbar_init(&s_bar, 1u);
            fence_barrier_init();
            mbar_arrive_expect_tx(&s_bar, kTileBytes);
            bulk_load(s_buf, in + (size_t)seg * n + (size_t)ts * kTile, kTileBytes, &s_bar);
        }
    }
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t epoch = s_epoch;
    const uint32_t seg = tile / tiles_per_seg;
    const uint32_t tile_in_seg = tile - seg * tiles_per_seg;
    const uint32_t* seg_in = in + (size_t)seg * n;
    uint32_t* seg_data = data + (size_t)seg * n;
    const bool full = (uint64_t)(tile_in_seg + 1) * kTile <= n;
    const uint32_t warp_base = tile_in_seg * kTile + warp * (SLICES * 128u);
    uint4* ws = s_buf + warp * (SLICES * 32u);  // this warp's slices; lane l holds uint4 l of each

    bool timed_out = false;
    if (full) {
        if (!mbar_wait(&s_bar, 0u, wait_limit)) timed_out = true;
    } else {
#pragma unroll
        for (int q = 0; q < SLICES; ++q) {
            const uint32_t b = warp_base + q * 128 + lane * 4;
            uint4 x;
            x.x = b + 0 < n ? seg_in[b + 0] : 0u;
            x.y = b + 1 < n ? seg_in[b + 1] : 0u;
            x.z = b + 2 < n ? seg_in[b + 2] : 0u;
            x.w = b + 3 < n ? seg_in[b + 3] : 0u;
            ws[q * 32 + lane] = x;
        }
    }

    // Pass 1: lane sums of each slice, warp scans of them.
    uint32_t lane_off[SLICES];
    uint32_t warp_run = 0;
#pragma unroll
    for (int q = 0; q < SLICES; ++q) {
        const uint4 x = ws[q * 32 + lane];
        const uint32_t sum = (x.x + x.y) + (x.z + x.w);
        uint32_t incl = sum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        lane_off[q] = warp_run + incl - sum;
        warp_run += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    if (lane == 0) s_warp_sum[warp] = warp_run;
    __syncthreads();
    uint32_t warp_prefix = 0, tile_sum = 0;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; ++w) {
        const uint32_t x = s_warp_sum[w];
        if (w < (int)warp) warp_prefix += x;
        tile_sum += x;
    }
    if (warp == 0) {
        uint32_t prefix = 0;
        if (tile_in_seg == 0) {
            if (lane == 0) publish_status(status, tile, make_status(epoch, 2u, tile_sum));
        } else {
            if (lane == 0) publish_status(status, tile, make_status(epoch, 1u, tile_sum));
            bool lb_timeout = false;
            prefix = warp_lookback(status, tile, tile - tile_in_seg, epoch, lane, wait_limit, spin, lb_timeout);
            if (lb_timeout) timed_out = true;
            if (lane == 0) publish_status(status, tile, make_status(epoch, 2u, prefix + tile_sum));
        }
        if (lane == 0) s_prefix = prefix;
    }
    if (__any_sync(0xFFFFFFFFu, timed_out) && lane == 0) VREN_RECORD_ERROR(VREN_ERR_TIMEOUT);
    __syncthreads();

    // Pass 2: exclusive sums written back in place.
    const uint32_t base_off = s_prefix + warp_prefix;
#pragma unroll
    for (int q = 0; q < SLICES; ++q) {
        uint4 x = ws[q * 32 + lane];
        uint32_t o = base_off + lane_off[q];
        const uint32_t a = x.x, b = x.y, c = x.z;
        x.x = o;
        x.y = (o += a);
        x.z = (o += b);
        x.w = o + c;
        if (full) {
            ws[q * 32 + lane] = x;
        } else {
            const uint32_t e = warp_base + q * 128 + lane * 4;
            if (e + 0 < n) seg_data[e + 0] = x.x;
            if (e + 1 < n) seg_data[e + 1] = x.y;
            if (e + 2 < n) seg_data[e + 2] = x.z;
            if (e + 3 < n) seg_data[e + 3] = x.w;
        }
    }
    if (full) {
        fence_smem_to_async();  // the writes above are read by the bulk store
        __syncthreads();
        if (tid == 0) bulk_store(seg_data + (size_t)tile_in_seg * kTile, s_buf, kTileBytes);
    }
}

// ------------------------------------------------------------------------------------------------
// Persistent, warp-specialised form (large aligned inputs).  A grid of (SMs x resident CTAs) of nine
// warps; each CTA cycles STAGES shared-memory tile buffers.
//  - Warp 8 (producer): takes tickets from the same counter, starts one bulk copy per tile
//    (cp.async.bulk, completion on the stage's `full` barrier), and as soon as a tile has landed sums
//    it and publishes the tile's aggregate, then signals `ready`.  It refills a stage when the
//    consumers release it (`empty`).  Aggregates therefore depend only on data arrival, never on a
//    look-back, so no chain of look-backs forms across CTAs.
//  - Warps 0-7 (consumers): take the ready tiles in order, resolve the exclusive prefix by
//    decoupled look-back (warp 0), write the sums back into the stage and store it with one bulk
//    copy, then release the stage.
// Forward progress: every CTA's tickets increase in the order they are taken and are consumed in
// that order, and each taken ticket's aggregate is published once its data lands, so the smallest
// unfinished tile always has every predecessor's aggregate or prefix available.
// Ticket word: [epoch | ticket] as in the other forms; tickets past the end are taken here, so the
// last CTA to finish (completion counter, word 2) opens the next epoch.
// ------------------------------------------------------------------------------------------------
constexpr uint32_t kNoTile = 0xFFFFFFFFu;
constexpr uint32_t kPersistThreads = kScanThreads + 32;

template <int SLICES, int STAGES>
__global__ void __launch_bounds__(kPersistThreads) exclusive_scan_persistent_kernel(
    const uint32_t* in, uint32_t* data, uint32_t n, uint32_t tiles_per_seg, uint32_t total_tiles,
    uint32_t* __restrict__ scratch, uint32_t wait_limit, uint32_t spin)
{
    pdl_enter();
    constexpr uint32_t kTile = SLICES * 128u * (kScanThreads / 32);
    constexpr uint32_t kTileBytes = kTile * 4u;
    constexpr uint32_t kTileVec = kTile / 4u;
    constexpr uint32_t kProducerWarp = kScanThreads / 32;
    extern __shared__ __align__(128) uint4 s_buf[];  // STAGES tiles
    __shared__ __align__(8) uint64_t s_full[STAGES];
    __shared__ __align__(8) uint64_t s_ready[STAGES];
    __shared__ __align__(8) uint64_t s_empty[STAGES];
    __shared__ uint32_t s_ticket[STAGES];
    __shared__ uint32_t s_agg[STAGES];
    __shared__ uint32_t s_epoch;
    __shared__ uint32_t s_warp_sum[kScanThreads / 32];
    __shared__ uint32_t s_prefix;

    uint64_t* status = reinterpret_cast<uint64_t*>(scratch + kScanHeaderWords);
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&s_full[s], 1u);
            mbar_init(&s_ready[s], 1u);
            mbar_init(&s_empty[s], 1u);
        }
        fence_barrier_init();
    }
    __syncthreads();
    bool timed_out = false;

    if (warp == kProducerWarp) {
        uint32_t filled = 0, j = 0;
        bool exhausted = false;
        // Takes the next ticket into stage (filled % STAGES) and starts its copy (lane 0).  Every fill
        // completes one phase of the stage's `full` barrier, with or without a copy.
        auto fill = [&]() {
            const uint32_t s = filled % STAGES;
            uint32_t t = kNoTile;
            if (lane == 0) {
                const unsigned long long w = atomicAdd(reinterpret_cast<unsigned long long*>(scratch), 1ull);
                if (filled == 0) s_epoch = (uint32_t)(w >> 32) & 0x3FFFFFFFu;
                t = (uint32_t)w < total_tiles ? (uint32_t)w : kNoTile;
                s_ticket[s] = t;
                bool copy = false;
                if (t != kNoTile) {
                    const uint32_t seg = t / tiles_per_seg, ts = t - seg * tiles_per_seg;
                    if ((uint64_t)(ts + 1) * kTile <= n) {
                        mbar_arrive_expect_tx(&s_full[s], kTileBytes);
                        bulk_load(s_buf + (size_t)s * kTileVec, in + (size_t)seg * n + (size_t)ts * kTile,
                                  kTileBytes, &s_full[s]);
                        copy = true;
                    }
                }
                if (!copy) mbar_arrive(&s_full[s]);
            }
            __syncwarp();
            t = __shfl_sync(0xFFFFFFFFu, t, 0);
            ++filled;
            if (t == kNoTile) exhausted = true;
        };
        for (int i = 0; i < STAGES && !exhausted; ++i) fill();
        const uint32_t epoch = s_epoch;  // written by lane 0 in the first fill (ordered by __syncwarp)

        while (true) {
            if (j < filled) {
                // Aggregate the oldest filled tile as soon as it lands.
                const uint32_t s = j % STAGES;
                if (!__all_sync(0xFFFFFFFFu, mbar_wait(&s_full[s], (j / STAGES) & 1u, wait_limit))) timed_out = true;
                const uint32_t t = s_ticket[s];
                if (t == kNoTile) {
                    if (lane == 0) mbar_arrive(&s_ready[s]);
                    break;
                }
                const uint32_t seg = t / tiles_per_seg, ts = t - seg * tiles_per_seg;
                uint4* buf = s_buf + (size_t)s * kTileVec;
                uint32_t sum = 0;
                if ((uint64_t)(ts + 1) * kTile <= n) {
#pragma unroll 8
                    for (uint32_t i = lane; i < kTileVec; i += 32) {
                        const uint4 x = buf[i];
                        sum += (x.x + x.y) + (x.z + x.w);
                    }
                } else {
                    const uint32_t* src = in + (size_t)seg * n;
                    for (uint32_t i = lane; i < kTileVec; i += 32) {
                        const uint32_t e = ts * kTile + 4u * i;
                        uint4 x;
                        x.x = e + 0 < n ? src[e + 0] : 0u;
                        x.y = e + 1 < n ? src[e + 1] : 0u;
                        x.z = e + 2 < n ? src[e + 2] : 0u;
                        x.w = e + 3 < n ? src[e + 3] : 0u;
                        buf[i] = x;
                        sum += (x.x + x.y) + (x.z + x.w);
                    }
                }
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) sum += __shfl_xor_sync(0xFFFFFFFFu, sum, d);
                if (lane == 0) {
                    s_agg[s] = sum;
                    publish_status(status, t, make_status(epoch, ts == 0 ? 2u : 1u, sum));
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(&s_ready[s]);  // releases the stage's data, ticket and sum
                ++j;
            }
            if (!exhausted) {
                // Refill the stage whose previous use the consumers have released; block only when
                // every filled tile is already aggregated.
                const uint32_t u = filled - STAGES;
                const uint32_t s = u % STAGES, parity = (u / STAGES) & 1u;
                bool freed;
                if (j < filled) {
                    freed = mbar_test(&s_empty[s], parity);
                } else {
                    freed = __all_sync(0xFFFFFFFFu, mbar_wait(&s_empty[s], parity, wait_limit));
                    if (!freed) {
                        timed_out = true;
                        break;  // the consumers time out on `ready` in turn
                    }
                }
                freed = __shfl_sync(0xFFFFFFFFu, freed ? 1u : 0u, 0) != 0;
                if (freed) fill();
            } else if (j >= filled) {
                break;
            }
        }
        // Copies still in flight (only after a timeout) land before the CTA exits.
        for (; j < filled; ++j) mbar_wait(&s_full[j % STAGES], (j / STAGES) & 1u, wait_limit);
    } else {
        for (uint32_t k = 0;; ++k) {
            const uint32_t s = k % STAGES;
            const uint32_t parity = (k / STAGES) & 1u;
            bool ok = mbar_wait(&s_ready[s], parity, wait_limit);
            ok = ok && mbar_wait(&s_full[s], parity, wait_limit);
            if (!named_sync_and(1, kScanThreads, ok)) {  // uniform over the eight consumer warps
                timed_out = true;
                break;
            }
            const uint32_t tile = s_ticket[s];
            if (tile == kNoTile) break;
            const uint32_t epoch = s_epoch;
            const uint32_t tile_sum = s_agg[s];
            const uint32_t seg = tile / tiles_per_seg;
            const uint32_t tile_in_seg = tile - seg * tiles_per_seg;
            uint32_t* seg_data = data + (size_t)seg * n;
            const bool full = (uint64_t)(tile_in_seg + 1) * kTile <= n;
            const uint32_t warp_base = tile_in_seg * kTile + warp * (SLICES * 128u);
            uint4* ws = s_buf + (size_t)s * kTileVec + warp * (SLICES * 32u);

            uint32_t lane_off[SLICES];
            uint32_t warp_run = 0;
#pragma unroll
            for (int q = 0; q < SLICES; ++q) {
                const uint4 x = ws[q * 32 + lane];
                const uint32_t sum = (x.x + x.y) + (x.z + x.w);
                uint32_t incl = sum;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
                    if (lane >= (uint32_t)d) incl += y;
                }
                lane_off[q] = warp_run + incl - sum;
                warp_run += __shfl_sync(0xFFFFFFFFu, incl, 31);
            }
            if (lane == 0) s_warp_sum[warp] = warp_run;
            named_sync(1, kScanThreads);
            uint32_t warp_prefix = 0;
#pragma unroll
            for (int w = 0; w < kScanThreads / 32; ++w)
                if (w < (int)warp) warp_prefix += s_warp_sum[w];
            if (warp == 0) {
                uint32_t prefix = 0;
                if (tile_in_seg != 0) {
                    bool lb_timeout = false;
                    prefix = warp_lookback(status, tile, tile - tile_in_seg, epoch, lane, wait_limit, spin,
                                           lb_timeout);
                    if (lb_timeout) timed_out = true;
                    if (lane == 0) publish_status(status, tile, make_status(epoch, 2u, prefix + tile_sum));
                }
                if (lane == 0) s_prefix = prefix;
            }
            named_sync(1, kScanThreads);
            const uint32_t base_off = s_prefix + warp_prefix;
#pragma unroll
            for (int q = 0; q < SLICES; ++q) {
                uint4 x = ws[q * 32 + lane];
                uint32_t o = base_off + lane_off[q];
                const uint32_t a = x.x, b = x.y, c = x.z;
                x.x = o;
                x.y = (o += a);
                x.z = (o += b);
                x.w = o + c;
                if (full) {
                    ws[q * 32 + lane] = x;
                } else {
                    const uint32_t e = warp_base + q * 128 + lane * 4;
                    if (e + 0 < n) seg_data[e + 0] = x.x;
                    if (e + 1 < n) seg_data[e + 1] = x.y;
                    if (e + 2 < n) seg_data[e + 2] = x.z;
                    if (e + 3 < n) seg_data[e + 3] = x.w;
                }
            }
            if (full) fence_smem_to_async();
            named_sync(1, kScanThreads);
            if (tid == 0) {
                if (full) bulk_store(seg_data + (size_t)tile_in_seg * kTile, s_buf + (size_t)s * kTileVec, kTileBytes);
                mbar_arrive(&s_empty[s]);
            }
        }
    }
    if (__any_sync(0xFFFFFFFFu, timed_out) && lane == 0) VREN_RECORD_ERROR(VREN_ERR_TIMEOUT);

    // The last CTA to finish opens the next call's epoch (tickets past the end were taken above).
    __syncthreads();
    if (tid == 0) {
        const uint32_t done = atomicAdd(scratch + 2, 1u);
        if (done == gridDim.x - 1) {
            st_relaxed_u64(reinterpret_cast<uint64_t*>(scratch), (uint64_t)(s_epoch + 1u) << 32);
            scratch[2] = 0u;
        }
    }
}

// ------------------------------------------------------------------------------------------------
// Down-sweep on an up-sweep tree (the reference's global levels blelloch_scan_downsweep.comp:33-53
// and its shared-memory pass :56-125).  Levels d >= 12 only touch positions that are the last
// element of a 4096-element chunk, and they form a down-sweep over the array of chunk roots.
// So the host recurses: the chunk roots (stride 4096) are down-swept first, which leaves each
// chunk root holding the value arriving from above; then one CTA per chunk runs the 12 in-chunk
// levels in shared memory.  The top-most array sets its root to zero unless the root is kept.
// ------------------------------------------------------------------------------------------------
constexpr int kDownThreads = 1024;
constexpr uint32_t kDownChunkLog2 = 12;
constexpr uint32_t kDownChunk = 1u << kDownChunkLog2;

// Elements of this level: e_j = seg[(j+1)*stride - 1], chunks of C = 2^chunk_log2 elements.
__global__ void __launch_bounds__(kDownThreads) downsweep_chunk_kernel(
    uint32_t* __restrict__ data, uint32_t seg_len, uint64_t stride, uint32_t chunk_log2, int top, int keep_root)
{
    __shared__ uint32_t s[kDownChunk];
    const uint32_t C = 1u << chunk_log2;
    uint32_t* seg = data + (size_t)blockIdx.y * seg_len;
    const uint64_t chunk_base = (uint64_t)blockIdx.x * C;
    const uint32_t tid = threadIdx.x;

    for (uint32_t i = tid; i < C; i += kDownThreads) s[i] = seg[(size_t)((chunk_base + i + 1) * stride - 1)];
    __syncthreads();
    if (top && tid == 0 && !keep_root) s[C - 1] = 0u;
    __syncthreads();
    for (int d = (int)chunk_log2 - 1; d >= 0; --d) {
        const uint32_t half = 1u << d;
        const uint32_t pairs = C >> (d + 1);
        for (uint32_t k = tid; k < pairs; k += kDownThreads) {
            const uint32_t a = k * (half << 1) + half - 1;
            const uint32_t b = a + half;
            const uint32_t t = s[b];
            s[b] = s[a] + t;
            s[a] = t;
        }
        __syncthreads();
    }
    for (uint32_t i = tid; i < C; i += kDownThreads) seg[(size_t)((chunk_base + i + 1) * stride - 1)] = s[i];
}

static int downsweep_level(cudaStream_t st, uint32_t* data, uint32_t seg_len, uint32_t blocks, uint64_t stride,
                           uint32_t log2m, int keep_root)
{
    if (log2m <= kDownChunkLog2) {
        downsweep_chunk_kernel<<<dim3(1, blocks), kDownThreads, 0, st>>>(data, seg_len, stride, log2m, 1, keep_root);
        VREN_LAUNCH_CHECK();
        return VREN_OK;
    }
    int rc = downsweep_level(st, data, seg_len, blocks, stride << kDownChunkLog2, log2m - kDownChunkLog2, keep_root);
    if (rc != VREN_OK) return rc;
    dim3 grid(1u << (log2m - kDownChunkLog2), blocks);
    downsweep_chunk_kernel<<<grid, kDownThreads, 0, st>>>(data, seg_len, stride, kDownChunkLog2, 0, keep_root);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

// Persistent grid for one variant: SMs x resident CTAs (shared memory opted in once per device).
template <int SLICES, int STAGES>
static int launch_persistent(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t n, uint32_t tiles_per_seg,
                             uint32_t total, uint32_t* sc, uint32_t spin)
{
    constexpr size_t kSmem = (size_t)STAGES * SLICES * 1024u * sizeof(uint32_t);
    static std::mutex mu;
    static int cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return VREN_ERR_CUDA;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (cached[dev] == 0) {
            auto kernel = exclusive_scan_persistent_kernel<SLICES, STAGES>;
            VREN_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem));
            int sms = 0, per_sm = 0;
            VREN_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            VREN_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPersistThreads, kSmem));
            cached[dev] = sms * (per_sm > 0 ? per_sm : 1);
        }
    }
    uint32_t grid = (uint32_t)cached[dev];
    if (grid > total) grid = total;
    launch_kernel(exclusive_scan_persistent_kernel<SLICES, STAGES>, grid, kPersistThreads, kSmem, st, in, out, n,
                  tiles_per_seg, total, sc, g_wait_limit, spin);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

// Dispatches the tile size chosen by VREN_TUNE_SCAN_SLICES (scratch is always sized for 4096-element
// tiles, the smaller one, so either variant fits) and the form (VREN_TUNE_SCAN_STAGED): automatic
// = the persistent warp-specialised grid from 2^20 elements when every tile starts 16-byte aligned
// (measured: 70% of HBM at 2^26 against 48% for tiles in registers), else tiles in registers.
static int scan_launch(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t n, uint32_t blocks, void* scratch,
                       const uint32_t* n_dev, uint32_t* total_out)
{
    const int slices = tuning(VREN_TUNE_SCAN_SLICES) == 8 ? 8 : 4;
    const uint32_t tile = (uint32_t)slices * 1024u;
    const uint32_t tiles_per_seg = (n + tile - 1) / tile;
    const uint64_t total = (uint64_t)(tiles_per_seg ? tiles_per_seg : 1) * blocks;
    if (total > 0x7FFFFFFFull) return VREN_ERR_ARG;
    const uint32_t spin = (uint32_t)tuning(VREN_TUNE_SPIN_POLLS);
    uint32_t* sc = static_cast<uint32_t*>(scratch);
    const int mode = tuning(VREN_TUNE_SCAN_STAGED);
    const bool aligned = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u) == 0 &&
                         (blocks == 1 || (n & 3u) == 0);
    const bool eligible = !n_dev && !total_out && aligned;
    const bool large = (uint64_t)n * blocks >= (1u << 20);
    if (eligible && (mode == 3 || (mode == 0 && large))) {
        if (slices == 8) return launch_persistent<8, 3>(st, in, out, n, tiles_per_seg, (uint32_t)total, sc, spin);
        return launch_persistent<4, 4>(st, in, out, n, tiles_per_seg, (uint32_t)total, sc, spin);
    }
    if (eligible && mode == 2) {
        if (slices == 8)
            launch_kernel(exclusive_scan_staged_kernel<8>, (uint32_t)total, kScanThreads, 8192u * 4u, st, in, out, n,
                          tiles_per_seg, (uint32_t)total, sc, g_wait_limit, spin);
        else
            launch_kernel(exclusive_scan_staged_kernel<4>, (uint32_t)total, kScanThreads, 4096u * 4u, st, in, out, n,
                          tiles_per_seg, (uint32_t)total, sc, g_wait_limit, spin);
        VREN_LAUNCH_CHECK();
        return VREN_OK;
    }
    if (slices == 8)
        launch_kernel(exclusive_scan_kernel<8>, (uint32_t)total, kScanThreads, 0, st, 
            in, out, n, tiles_per_seg ? tiles_per_seg : 1, (uint32_t)total, sc, g_wait_limit, spin, n_dev, total_out);
    else
        launch_kernel(exclusive_scan_kernel<4>, (uint32_t)total, kScanThreads, 0, st, 
            in, out, n, tiles_per_seg ? tiles_per_seg : 1, (uint32_t)total, sc, g_wait_limit, spin, n_dev, total_out);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

}  // namespace vren_gb300

using namespace vren_gb300;

extern "C" size_t vren_exclusive_scan_scratch_bytes(uint32_t n, uint32_t blocks)
{
    uint64_t tiles = (uint64_t)((n + kScanTile - 1) / kScanTile) * (blocks ? blocks : 1);
    return (size_t)(kScanHeaderWords * sizeof(uint32_t) + tiles * sizeof(uint64_t));
}

extern "C" int vren_test_withhold_scan_status(uint32_t tile_plus_one)
{
    return cudaMemcpyToSymbol(g_scan_withheld_tile, &tile_plus_one, sizeof(tile_plus_one)) == cudaSuccess
               ? VREN_OK
               : VREN_ERR_CUDA;
}

extern "C" int vren_exclusive_scan_u32(vren_stream_t s, uint32_t* data, uint32_t n, uint32_t blocks, void* scratch)
{
    if (blocks == 0 || !scratch || (n > 0 && !data)) return VREN_ERR_ARG;
    if (n == 0) return VREN_OK;
    if (n > (1u << 31)) return VREN_ERR_ARG;
    return scan_launch(as_stream(s), data, data, n, blocks, scratch, nullptr, nullptr);
}

namespace vren_gb300 {
size_t scan_scratch_bytes(uint32_t n_cap) { return vren_exclusive_scan_scratch_bytes(n_cap, 1); }

int scan_exclusive_u32(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t n_cap, const uint32_t* n_dev,
                       uint32_t* total_out, void* scratch)
{
    return scan_launch(st, in, out, n_cap, 1, scratch, n_dev, total_out);
}
}  // namespace vren_gb300

extern "C" int vren_scan_downsweep_u32(vren_stream_t s, uint32_t* data, uint32_t n, uint32_t blocks, int clear_last)
{
    if (blocks == 0 || blocks > 65535 || !data || n == 0 || (n & (n - 1))) return VREN_ERR_ARG;
    uint32_t log2n = 0;
    while ((1u << log2n) < n) ++log2n;
    // n < 1024 is a single reference work-group: its zero padding always reaches the root.
    const int keep_root = (n >= 1024 && !clear_last) ? 1 : 0;
    return downsweep_level(as_stream(s), data, n, blocks, 1, log2n, keep_root);
}

// ================================================================================================
// Exclusive scan without any allocation by the caller.
//
// Some callers cannot hand the library a scratch buffer: code that runs inside an engine whose
// allocator owns all device memory and forbids extra allocations, plugins loaded into a host
// application that exposes no allocator, or frame loops that must not call cudaMalloc because it
// can synchronise the device.  For them this variant keeps the look-back scratch in a fixed
// device array that is part of the library image: every GPU that loads the library holds it
// (32 KiB + 16 B) until the process exits.  The largest input is therefore bounded:
// n * blocks <= kNoAllocMaxElements (2^24 elements); larger inputs are rejected with
// VREN_ERR_CAPACITY before anything is enqueued.
//
// All calls share the array and it keeps the last call's contents, so each call first clears the
// part it uses (tickets, epoch, one status word per tile) with cudaMemsetAsync on the caller's
// stream.  Two calls that overlap on the GPU (other streams, other host threads) race on the array
// and must be serialised by the caller.  The first call on a device (and in each CUDA context on it)
// looks the array's device address up (cudaGetSymbolAddress, with that device current) and caches
// it under the (device, current context) pair: a context created after a cudaDeviceReset, or a
// driver context other than the primary one, loads the library image again and gets its own copy
// of the array, which is looked up afresh.  Make the first call in a context before capturing a
// stream into a CUDA graph.
// ================================================================================================
#include <cuda.h>  // CUcontext and the cuCtxGetCurrent prototype (resolved at run time below)
#include <mutex>

namespace vren_gb300 {
constexpr uint32_t kNoAllocMaxElements = 1u << 24;
constexpr uint32_t kNoAllocMaxTiles = kNoAllocMaxElements / kScanTile;  // 4096
constexpr uint32_t kNoAllocWords = kScanHeaderWords + 2u * kNoAllocMaxTiles;

static __device__ __align__(256) uint32_t g_noalloc_scan_scratch[kNoAllocWords];

struct NoAllocEntry {
    int dev;
    CUcontext ctx;
    void* ptr;
};
constexpr int kNoAllocMaxEntries = 64;
static std::mutex g_noalloc_mutex;
static NoAllocEntry g_noalloc_cache[kNoAllocMaxEntries];
static int g_noalloc_entries = 0;

// The calling thread's current driver context (the runtime's primary context after cudaGetDevice has
// made one current); cuCtxGetCurrent is taken from the driver through the runtime, so the library
// does not link libcuda itself.
static int current_context(CUcontext* ctx)
{
    using GetCurrent = CUresult (*)(CUcontext*);
    static GetCurrent fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<GetCurrent>(p);
    }();
    *ctx = nullptr;
    if (!fn) return VREN_ERR_CUDA;
    return fn(ctx) == CUDA_SUCCESS ? VREN_OK : VREN_ERR_CUDA;  // null when no context is current yet
}

// Device address of g_noalloc_scan_scratch in the current device's current context (looked up once
// per device and context).
static int noalloc_scratch(uint32_t** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return VREN_ERR_CUDA;
    CUcontext ctx = nullptr;
    if (current_context(&ctx) != VREN_OK) return VREN_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    for (int i = 0; ctx && i < g_noalloc_entries; ++i)
        if (g_noalloc_cache[i].dev == dev && g_noalloc_cache[i].ctx == ctx) {
            *out = static_cast<uint32_t*>(g_noalloc_cache[i].ptr);
            return VREN_OK;
        }
    // the lookup makes the device's primary context current when no context is yet
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scan_scratch) != cudaSuccess || p == nullptr) return VREN_ERR_CUDA;
    if (!ctx && (current_context(&ctx) != VREN_OK || !ctx)) return VREN_ERR_CUDA;
    // a context handle can be reused after its context is destroyed: a stale entry for this device is
    // replaced; otherwise the oldest entry makes room
    int slot = -1;
    for (int i = 0; i < g_noalloc_entries; ++i)
        if (g_noalloc_cache[i].dev == dev) slot = i;
    if (slot < 0) slot = g_noalloc_entries < kNoAllocMaxEntries ? g_noalloc_entries++ : 0;
    g_noalloc_cache[slot] = {dev, ctx, p};
    *out = static_cast<uint32_t*>(p);
    return VREN_OK;
}
}  // namespace vren_gb300

extern "C" int vren_exclusive_scan_u32_noalloc(vren_stream_t s, uint32_t* data, uint32_t n, uint32_t blocks)
{
    if (blocks == 0 || (n > 0 && !data)) return VREN_ERR_ARG;
    if (n == 0) return VREN_OK;
    if ((uint64_t)n * blocks > kNoAllocMaxElements) return VREN_ERR_CAPACITY;
    const uint32_t tiles_per_seg = (n + kScanTile - 1) / kScanTile;
    const uint32_t total = tiles_per_seg * blocks;
    if (total > kNoAllocMaxTiles) return VREN_ERR_CAPACITY;
    uint32_t* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc != VREN_OK) return rc;
    cudaStream_t st = as_stream(s);
    VREN_CUDA_TRY(cudaMemsetAsync(scratch, 0, (kScanHeaderWords + 2u * total) * sizeof(uint32_t), st));
    launch_kernel(exclusive_scan_kernel<4>, total, kScanThreads, 0, st, data, data, n, tiles_per_seg, total, scratch, g_wait_limit,
                                                             (uint32_t)tuning(VREN_TUNE_SPIN_POLLS), nullptr, nullptr);
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}

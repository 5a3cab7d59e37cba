// Persistent onesweep pass for keys or key/value pairs whose arrays start 16-byte aligned.
//
// The one-tile-per-CTA pass (onesweep_pass_kernel) has loads in flight only at the start of a CTA and
// stores only at its end.  Here a grid of (SMs x 2) CTAs loops over tiles:
//  - warp 8 takes the tickets, brings each tile's keys (and values) into one of two shared-memory
//    stages with bulk copies (cp.async.bulk, completion on the stage's `full` barrier), and as soon
//    as a tile has landed counts its digits in shared memory and publishes the counts as the tile's
//    aggregates, then signals `ready`;
//  - warps 0-7 rank the ready tile from shared memory (ballots, per-warp digit counters), resolve
//    every digit's global offset by decoupled look-back, stage the elements in digit order, release
//    the input stage (`empty`) and write out, while the next tile is already landing.
// A tile's aggregates depend only on its data arriving, never on a look-back, and every CTA takes
// its tickets in increasing order and processes them in that order, so the smallest unfinished tile
// always sees every predecessor's aggregate (no chain of look-backs across CTAs).
// The status words and their alternating buffers are those of the one-tile pass.
#pragma once

#include "tma.cuh"

namespace vren_gb300 {

constexpr int kPStages = 2;
constexpr int kPConsumerWarps = 16;                    // consumers per CTA (two CTAs per SM)
constexpr int kPItems = 6;                             // keys per consumer thread
constexpr int kPConsumers = kPConsumerWarps * 32;
constexpr int kPThreads = kPConsumers + 32;            // + the producer/histogram warp
constexpr uint32_t kPTile = (uint32_t)kPConsumers * kPItems;  // 3072 keys
constexpr uint32_t kPNone = 0xFFFFFFFFu;

template <int DB>
struct PersistSmem {
    static constexpr int RADIX = 1 << DB;
    uint64_t full[kPStages];
    uint64_t ready[kPStages];
    uint64_t empty[kPStages];
    uint32_t ticket[kPStages];
    uint32_t hist[kPStages][RADIX];
    uint32_t warp_hist[kPConsumerWarps][RADIX];
    int32_t delta[RADIX];
    uint32_t wsum[kPConsumerWarps];
};

template <int DB, int MODE>
constexpr size_t persist_dyn_smem()
{
    return kPStages * (size_t)kPTile * 4 * (MODE == kPairs ? 2 : 1) + (size_t)kPTile * (MODE == kPairs ? 8 : 4);
}

// Producer/histogram warp (all 32 lanes; lane 0 takes tickets and issues the copies).
template <int DB, int MODE, int TILE>
__device__ __forceinline__ void persist_producer(const uint32_t* __restrict__ in_keys,
                                                 const uint32_t* __restrict__ in_vals, uint32_t n, uint32_t shift,
                                                 uint32_t width, uint32_t num_tiles, uint32_t* ticket_ctr,
                                                 uint32_t* status, uint32_t* status_next, uint32_t* stage_k,
                                                 uint32_t* stage_v, PersistSmem<DB>& sm, uint32_t wait_limit,
                                                 bool& timed_out)
{
    constexpr int RADIX = 1 << DB;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t filled = 0, j = 0;
    bool exhausted = false;
    // Takes the next ticket into stage (filled % kPStages) and starts its copies.  Every fill completes
    // one phase of the stage's `full` barrier, with or without copies.
    auto fill = [&]() {
        const uint32_t s = filled % kPStages;
        uint32_t t = kPNone;
        if (lane == 0) {
            const uint32_t x = atomicAdd(ticket_ctr, 1u);
            t = x < num_tiles ? x : kPNone;
            sm.ticket[s] = t;
            uint32_t bytes = 0;
            if (t != kPNone) {
                const uint32_t valid = (uint64_t)(t + 1) * TILE <= n ? (uint32_t)TILE : n - t * (uint32_t)TILE;
                bytes = (valid * 4u) & ~15u;  // the last few elements of a partial tile are read by the warp
            }
            if (bytes) {
                mbar_arrive_expect_tx(&sm.full[s], MODE == kPairs ? 2u * bytes : bytes);
                bulk_load(stage_k + (size_t)s * TILE, in_keys + (size_t)t * TILE, bytes, &sm.full[s]);
                if (MODE == kPairs)
                    bulk_load(stage_v + (size_t)s * TILE, in_vals + (size_t)t * TILE, bytes, &sm.full[s]);
            } else {
                mbar_arrive(&sm.full[s]);
            }
        }
        __syncwarp();
        t = __shfl_sync(0xFFFFFFFFu, t, 0);
        ++filled;
        if (t == kPNone) exhausted = true;
    };
    for (int i = 0; i < kPStages && !exhausted; ++i) fill();

    while (true) {
        if (j < filled) {
            const uint32_t s = j % kPStages;
            if (!__all_sync(0xFFFFFFFFu, mbar_wait(&sm.full[s], (j / kPStages) & 1u, wait_limit))) timed_out = true;
            const uint32_t t = sm.ticket[s];
            if (t == kPNone) {
                if (lane == 0) mbar_arrive(&sm.ready[s]);
                break;
            }
            const uint32_t valid = (uint64_t)(t + 1) * TILE <= n ? (uint32_t)TILE : n - t * (uint32_t)TILE;
            uint32_t* sk = stage_k + (size_t)s * TILE;
            // elements past the copied 16-byte multiple (partial tile only)
            for (uint32_t i = (valid & ~3u) + lane; i < valid; i += 32) {
                sk[i] = in_keys[(size_t)t * TILE + i];
                if (MODE == kPairs) stage_v[(size_t)s * TILE + i] = in_vals[(size_t)t * TILE + i];
            }
            for (uint32_t d = lane; d < (uint32_t)RADIX; d += 32) {
                sm.hist[s][d] = 0u;
                status_next[(size_t)t * RADIX + d] = 0u;  // the next pass's row of this tile
            }
            __syncwarp();
            for (uint32_t i = lane; i < valid; i += 32) atomicAdd(&sm.hist[s][digit_of(sk[i], shift, width)], 1u);
            __syncwarp();
            for (uint32_t d = lane; d < (uint32_t)RADIX; d += 32)
                st_relaxed_u32(status + (size_t)t * RADIX + d, (t == 0 ? kFlagPrefix : kFlagAggregate) | sm.hist[s][d]);
            __syncwarp();
            if (lane == 0) mbar_arrive(&sm.ready[s]);  // releases the stage's data (incl. the tail) and ticket
            ++j;
        }
        if (!exhausted) {
            // refill the stage whose previous use the consumers have released; block only when every
            // filled tile is already counted
            const uint32_t u = filled - kPStages;
            const uint32_t s = u % kPStages, parity = (u / kPStages) & 1u;
            bool freed;
            if (j < filled) {
                freed = mbar_test(&sm.empty[s], parity);
            } else {
                freed = __all_sync(0xFFFFFFFFu, mbar_wait(&sm.empty[s], parity, wait_limit));
                if (!freed) {
                    timed_out = true;
                    break;
                }
            }
            freed = __shfl_sync(0xFFFFFFFFu, freed ? 1u : 0u, 0) != 0;
            if (freed) fill();
        } else if (j >= filled) {
            break;
        }
    }
    // copies still in flight (only after a timeout) land before the CTA exits
    for (; j < filled; ++j) mbar_wait(&sm.full[j % kPStages], (j / kPStages) & 1u, wait_limit);
}

template <int DB, int MODE>
__global__ void __launch_bounds__(kPThreads, 2) onesweep_persistent_kernel(
    const uint32_t* in_keys, const uint32_t* in_vals, uint32_t* __restrict__ out_keys,
    uint32_t* __restrict__ out_vals, uint32_t n, uint32_t pass, uint32_t shift, uint32_t width, uint32_t num_tiles,
    uint32_t* __restrict__ scratch, uint32_t wait_limit, uint32_t spin)
{
    pdl_enter();
    constexpr int RADIX = 1 << DB;
    constexpr int ITEMS = kPItems;
    constexpr int TILE = (int)kPTile;
    extern __shared__ __align__(128) uint4 s_dyn4[];
    uint32_t* stage_k = reinterpret_cast<uint32_t*>(s_dyn4);           // [kPStages][TILE]
    uint32_t* stage_v = stage_k + kPStages * TILE;                       // [kPStages][TILE] (pairs)
    uint32_t* staging = stage_v + (MODE == kPairs ? kPStages * TILE : 0);  // [TILE] keys or (key, value) pairs
    uint2* staging2 = reinterpret_cast<uint2*>(staging);
    __shared__ PersistSmem<DB> sm;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    uint32_t* status = scratch + kStatusOffset + (size_t)(pass & 1u) * num_tiles * RADIX;
    uint32_t* status_next = scratch + kStatusOffset + (size_t)((pass + 1u) & 1u) * num_tiles * RADIX;
    if (tid == 0) {
        for (int s = 0; s < kPStages; ++s) {
            mbar_init(&sm.full[s], 1u);
            mbar_init(&sm.ready[s], 1u);
            mbar_init(&sm.empty[s], 1u);
        }
        fence_barrier_init();
    }
    __syncthreads();
    bool timed_out = false;

    if (warp == kPConsumerWarps) {
        persist_producer<DB, MODE, TILE>(in_keys, in_vals, n, shift, width, num_tiles, scratch + pass, status,
                                         status_next, stage_k, stage_v, sm, wait_limit, timed_out);
    } else {
        for (uint32_t u = 0;; ++u) {
            const uint32_t s = u % kPStages, parity = (u / kPStages) & 1u;
            bool ok = mbar_wait(&sm.ready[s], parity, wait_limit);
            ok = ok && mbar_wait(&sm.full[s], parity, wait_limit);
            // zero the per-warp counters while waiting is settled (the previous tile is done with them)
            for (uint32_t i = tid; i < (uint32_t)(kPConsumerWarps * RADIX); i += kPConsumers) (&sm.warp_hist[0][0])[i] = 0u;
            if (!named_sync_and(1, kPConsumers, ok)) {  // uniform over the consumer warps
                timed_out = true;
                break;
            }
            const uint32_t tile = sm.ticket[s];
            if (tile == kPNone) break;
            const uint32_t valid = (uint64_t)(tile + 1) * TILE <= n ? (uint32_t)TILE : n - tile * (uint32_t)TILE;
            const uint32_t* sk = stage_k + (size_t)s * TILE;
            const uint32_t* sv = stage_v + (size_t)s * TILE;

            // stable in-warp ranking, striped items (item j of lane l = element 32 ITEMS warp + 32 j + l)
            const uint32_t wbase = warp * (32u * ITEMS);
            uint32_t pos[ITEMS];
#pragma unroll
            for (int j = 0; j < ITEMS; ++j) {
                const uint32_t idx = wbase + 32u * j + lane;
                const bool v = idx < valid;
                const uint32_t d = v ? digit_of(sk[idx], shift, width) : 0u;
                uint32_t peers = __ballot_sync(0xFFFFFFFFu, v);
#pragma unroll
                for (int b = 0; b < DB; ++b) {
                    const uint32_t m = __ballot_sync(0xFFFFFFFFu, (d >> b) & 1u);
                    const uint32_t mine = (uint32_t)((int32_t)(d << (31 - b)) >> 31);
                    peers &= ~(m ^ mine);
                }
                const uint32_t below = peers & lanemask_lt();
                const uint32_t before = v ? sm.warp_hist[warp][d] : 0u;
                __syncwarp();
                if (v && below == 0) sm.warp_hist[warp][d] = before + __popc(peers);
                __syncwarp();
                pos[j] = v ? (d | ((before + __popc(below)) << 8)) : 0xFFFFFFFFu;
            }
            named_sync(1, kPConsumers);

            // thread d: warp prefixes of digit d and the tile's count; exclusive scan over digits
            uint32_t count = 0;
            if (tid < (uint32_t)RADIX) {
#pragma unroll
                for (int w = 0; w < kPConsumerWarps; ++w) {
                    const uint32_t c = sm.warp_hist[w][tid];
                    sm.warp_hist[w][tid] = count;
                    count += c;
                }
            }
            uint32_t incl = count;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= (uint32_t)o) incl += y;
            }
            if (lane == 31) sm.wsum[warp] = incl;
            named_sync(1, kPConsumers);
            uint32_t excl = 0, lb_word = 0, goff = 0;
            if (tid < (uint32_t)RADIX) {
                excl = incl - count;
                for (uint32_t w = 0; w < warp; ++w) excl += sm.wsum[w];
#pragma unroll
                for (int w = 0; w < kPConsumerWarps; ++w) sm.warp_hist[w][tid] += excl;  // first staging slot of (w, d)
                if (tile != 0) lb_word = ld_relaxed_u32(status + (size_t)(tile - 1) * RADIX + tid);
                goff = ld_relaxed_u32(scratch + kOffsOffset + pass * kMaxRadix + tid);
            }
            named_sync(1, kPConsumers);

            // stage in digit order (keys and values read again from the input stage)
#pragma unroll
            for (int j = 0; j < ITEMS; ++j) {
                if (pos[j] != 0xFFFFFFFFu) {
                    const uint32_t idx = wbase + 32u * j + lane;
                    const uint32_t p = sm.warp_hist[warp][pos[j] & 0xFFu] + (pos[j] >> 8);
                    if (MODE == kPairs) staging2[p] = make_uint2(sk[idx], sv[idx]);
                    else staging[p] = sk[idx];
                }
            }

            // decoupled look-back for digit d (thread d), four predecessors per round trip
            if (tid < (uint32_t)RADIX) {
                const uint32_t d = tid;
                uint32_t prefix = 0;
                if (tile != 0) {
                    int64_t t = (int64_t)tile - 1;
                    uint32_t w[4];
                    w[0] = lb_word;
                    bool done = false;
                    while (!done) {
#pragma unroll
                        for (int i = 1; i < 4; ++i)
                            w[i] = t - i >= 0 ? ld_relaxed_u32(status + (size_t)(t - i) * RADIX + d) : 0u;
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
            named_sync(1, kPConsumers);  // staging and deltas complete; the input stage is free
            if (tid == 0) mbar_arrive(&sm.empty[s]);

            // write out: consecutive threads take consecutive staged elements
#pragma unroll
            for (int j = 0; j < ITEMS; ++j) {
                const uint32_t p = j * kPConsumers + tid;
                if (p < valid) {
                    uint32_t k, v = 0;
                    if (MODE == kPairs) {
                        const uint2 kv = staging2[p];
                        k = kv.x;
                        v = kv.y;
                    } else {
                        k = staging[p];
                    }
                    const uint32_t dst = (uint32_t)((int32_t)p + sm.delta[digit_of(k, shift, width)]);
                    if (dst < n) {  // false only after a timed-out look-back (error recorded)
                        out_keys[dst] = k;
                        if (MODE == kPairs) out_vals[dst] = v;
                    }
                }
            }
            named_sync(1, kPConsumers);  // the staging buffer and the deltas may be reused
        }
    }
    if (__any_sync(0xFFFFFFFFu, timed_out) && lane == 0) VREN_RECORD_ERROR(VREN_ERR_TIMEOUT);
}

}  // namespace vren_gb300

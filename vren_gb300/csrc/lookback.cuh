// Decoupled look-back over 64-bit status words [epoch:30 | flag:2 | value:32] (flag 1 = aggregate of
// the unit, 2 = inclusive prefix), shared by the single-pass scan and the fused light assignment.
// Status words carry the call's epoch, so words left by an earlier call read as "not published".
#pragma once

#include "common.cuh"

namespace vren_gb300 {

__device__ __forceinline__ uint64_t make_status(uint32_t epoch, uint32_t flag, uint32_t value)
{
    return ((uint64_t)((epoch << 2) | flag) << 32) | value;
}

// Takes the calling CTA's unit (a ticket) and the call's epoch from the 64-bit word
// [epoch:32 | ticket:32] at `header`, one thread per CTA: units are taken in the order the CTAs start,
// so a unit's predecessors have all started when it looks back.  The taker of the last ticket opens
// the next call's epoch with ticket 0 (every other CTA of the launch has its ticket by then).
__device__ __forceinline__ uint32_t take_ticket(uint32_t* header, uint32_t total_units, uint32_t& epoch)
{
    unsigned long long* word = reinterpret_cast<unsigned long long*>(header);
    const unsigned long long w = atomicAdd(word, 1ull);
    const uint32_t unit = (uint32_t)w;
    epoch = (uint32_t)(w >> 32);
    if (unit == total_units - 1) st_relaxed_u64(reinterpret_cast<uint64_t*>(header), (uint64_t)(epoch + 1u) << 32);
    epoch &= 0x3FFFFFFFu;
    return unit;
}

// Warp-wide decoupled look-back over status[seg_first .. tile-1]: lane i examines tile - 1 - i
// (then 32 further back, ...) and the warp sums aggregates up to the nearest inclusive prefix.
// Returns the exclusive prefix of `tile` in every lane.
__device__ __forceinline__ uint32_t warp_lookback(const uint64_t* status, uint32_t tile, uint32_t seg_first,
                                                  uint32_t epoch, uint32_t lane, uint32_t wait_limit, uint32_t spin,
                                                  bool& timed_out)
{
    uint32_t prefix = 0;
    int64_t pos = (int64_t)tile - 1;
    while (true) {
        const int64_t idx = pos - lane;
        uint32_t flag = 2u, val = 0u;  // lanes before the segment start act as a zero prefix
        if (idx >= (int64_t)seg_first) {
            uint32_t ns = 32;
            for (uint32_t round = 0;; ++round) {
                const uint64_t w = ld_relaxed_u64(status + idx);
                const uint32_t hi = (uint32_t)(w >> 32);
                if ((hi >> 2) == epoch && (hi & 3u) != 0) {
                    flag = hi & 3u;
                    val = (uint32_t)w;
                    break;
                }
                if (round >= wait_limit) {
                    timed_out = true;
                    break;
                }
                if (round >= spin) {
                    __nanosleep(ns);
                    if (ns < 512) ns <<= 1;
                }
            }
        }
        const uint32_t prefix_mask = __ballot_sync(0xFFFFFFFFu, flag == 2u);
        const uint32_t stop = prefix_mask ? (uint32_t)(__ffs(prefix_mask) - 1) : 31u;
        uint32_t contrib = (lane <= stop) ? val : 0u;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) contrib += __shfl_xor_sync(0xFFFFFFFFu, contrib, d);
        prefix += contrib;
        if (prefix_mask) break;
        pos -= 32;
    }
    return prefix;
}

}  // namespace vren_gb300

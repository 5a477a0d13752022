// fgc_scan.cuh -- block-wide scans and a single-pass, order-preserving global
// allocation (decoupled look-back, Merrill & Garland 2016).
//
// A kernel that emits a variable number of records per input element calls
// ordered_alloc(): every thread gets the exclusive prefix of all counts of
// earlier elements, so records land in submission order with one pass over
// the input. Logical block indices come from an atomic ticket so every
// predecessor of a block has already started; each wait on a predecessor is
// bounded (kSpinLimit polls unless the host sets a smaller limit) and
// reports ST_LOOKBACK_TIMEOUT instead of hanging.
#pragma once

#include "fgc_device.cuh"

namespace fgc {

constexpr uint64_t kFlagAgg = 1ull << 62;
constexpr uint64_t kFlagPre = 2ull << 62;
constexpr uint64_t kValMask = (1ull << 62) - 1;

struct Lookback {
    unsigned long long* tiles;  // one word per logical block, zeroed before launch
    unsigned int* ticket;       // zeroed before launch
    unsigned int* status;       // device status word
    unsigned long long* total;  // receives the grand total (written by the last block)
    uint32_t spin_limit = kSpinLimit;   // polls of an unpublished predecessor before giving up
    uint32_t withhold = 0xFFFFFFFFu;    // test hook: this logical block never publishes
};

template <int BLOCK>
__device__ __forceinline__ uint32_t block_ticket(const Lookback& L, uint32_t* s_tile) {
    if (threadIdx.x == 0) *s_tile = atomicAdd(L.ticket, 1u);
    __syncthreads();
    return *s_tile;
}

// Inclusive warp scan of a 64-bit value.
__device__ __forceinline__ uint64_t warp_inclusive_scan(uint64_t v) {
    const unsigned lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= (unsigned)o) v += t;
    }
    return v;
}

// Block exclusive scan; returns the thread's exclusive prefix and writes the
// block aggregate to *agg. s_warp must hold BLOCK/32 + 1 words.
template <int BLOCK>
__device__ __forceinline__ uint64_t block_exclusive_scan(uint64_t v, uint64_t* s_warp, uint64_t* agg) {
    constexpr int NW = BLOCK / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t inc = warp_inclusive_scan(v);
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint64_t w = (lane < NW) ? s_warp[lane] : 0;
        uint64_t wi = warp_inclusive_scan(w);
        if (lane < NW) s_warp[lane] = wi - w;
        if (lane == NW - 1) s_warp[NW] = wi;
    }
    __syncthreads();
    uint64_t r = s_warp[warp] + inc - v;
    *agg = s_warp[NW];
    __syncthreads();
    return r;
}

// Publish this block's aggregate, look back over predecessors and return the
// block's exclusive prefix (warp 0 computes; all threads receive it). The
// look-back reads a window of 32 predecessors per round, one per lane: the
// nearest one holding an inclusive prefix ends the walk, and a window whose
// relevant part still has an unpublished tile is read again.
template <int BLOCK>
__device__ __forceinline__ uint64_t lookback_prefix(const Lookback& L, uint32_t tile, uint64_t agg,
                                                    uint64_t* s_prefix) {
    if (threadIdx.x < 32) {
        const uint32_t lane = threadIdx.x;
        uint64_t excl = 0;
        const bool publish = tile != L.withhold;
        if (tile == 0) {
            if (lane == 0 && publish) atomicExch(&L.tiles[0], (unsigned long long)(kFlagPre | (agg & kValMask)));
        } else {
            if (lane == 0 && publish) atomicExch(&L.tiles[tile], (unsigned long long)(kFlagAgg | (agg & kValMask)));
            int64_t hi = (int64_t)tile - 1;  // the window is tiles hi, hi-1, ..., hi-31 (lane order)
            uint32_t spins = 0;
            for (;;) {
                const int64_t j = hi - (int64_t)lane;
                // before tile 0: an inclusive prefix of 0
                const uint64_t s = j >= 0 ? *(volatile unsigned long long*)&L.tiles[j] : kFlagPre;
                const uint64_t flag = s & ~kValMask;
                const uint32_t pre = __ballot_sync(0xffffffffu, flag == kFlagPre);
                const uint32_t unset = __ballot_sync(0xffffffffu, flag == 0);
                // lanes up to the nearest inclusive prefix (all 32 when there is none)
                const uint32_t upto = pre ? ((pre & (0u - pre)) << 1) - 1u : 0xffffffffu;
                if (unset & upto) {
                    if (++spins > L.spin_limit) {
                        if (lane == 0) atomicOr(L.status, ST_LOOKBACK_TIMEOUT);
                        break;
                    }
                    __nanosleep(32);
                    continue;
                }
                uint64_t v = ((upto >> lane) & 1u) ? (s & kValMask) : 0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                excl += v;
                if (pre) break;
                hi -= 32;
            }
            if (lane == 0 && publish)
                atomicExch(&L.tiles[tile], (unsigned long long)(kFlagPre | ((excl + agg) & kValMask)));
        }
        if (lane == 0) {
            if (tile == gridDim.x - 1 && L.total) *L.total = excl + agg;
            *s_prefix = excl;
        }
    }
    __syncthreads();
    uint64_t r = *s_prefix;
    __syncthreads();
    return r;
}

// One call per thread per launch: exclusive global offset of this thread's
// count in (logical block, thread) order.
template <int BLOCK>
struct OrderedAllocSmem {
    uint64_t warp[BLOCK / 32 + 1];
    uint64_t prefix;
};

template <int BLOCK>
__device__ __forceinline__ uint64_t ordered_alloc(const Lookback& L, uint32_t tile, uint64_t count,
                                                  OrderedAllocSmem<BLOCK>& sm) {
    uint64_t agg;
    uint64_t local = block_exclusive_scan<BLOCK>(count, sm.warp, &agg);
    uint64_t base = lookback_prefix<BLOCK>(L, tile, agg, &sm.prefix);
    return base + local;
}

// ordered_alloc of `count` that also scans a second per-thread value in the
// same pass: the two sums share one 64-bit scan (count in the high half,
// other in the low half; a block's sums of either stay below 2^32).
template <int BLOCK>
__device__ __forceinline__ uint64_t ordered_alloc_pair(const Lookback& L, uint32_t tile, uint32_t count, uint32_t other,
                                                       OrderedAllocSmem<BLOCK>& sm, uint32_t& other_excl,
                                                       uint32_t& other_total) {
    uint64_t agg;
    const uint64_t local = block_exclusive_scan<BLOCK>(((uint64_t)count << 32) | other, sm.warp, &agg);
    other_excl = (uint32_t)local;
    other_total = (uint32_t)agg;
    const uint64_t base = lookback_prefix<BLOCK>(L, tile, agg >> 32, &sm.prefix);
    return base + (local >> 32);
}

// Ordered allocation of two counts at once: every thread gets the global
// exclusive prefix of both (a in [0, 2^31) per block and overall, b likewise).
// They travel packed as a << 31 | b through one block scan and one look-back
// (L.total must be null); `total` receives the packed inclusive sum of the
// block, which for the last block is the grand total.
constexpr uint64_t kLow31 = (1ull << 31) - 1;
template <int BLOCK>
__device__ __forceinline__ void ordered_alloc2(const Lookback& L, uint32_t tile, uint32_t a, uint32_t b,
                                               OrderedAllocSmem<BLOCK>& sm, uint64_t& a_excl, uint64_t& b_excl,
                                               uint64_t& total) {
    uint64_t agg;
    const uint64_t local = block_exclusive_scan<BLOCK>(((uint64_t)a << 31) | b, sm.warp, &agg);
    const uint64_t base = lookback_prefix<BLOCK>(L, tile, agg, &sm.prefix);
    a_excl = (base >> 31) + (local >> 31);
    b_excl = (base & kLow31) + (local & kLow31);
    total = base + agg;
}

}  // namespace fgc

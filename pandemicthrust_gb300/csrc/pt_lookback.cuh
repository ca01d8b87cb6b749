// pt_lookback.cuh - block-level scans and the single-pass decoupled look-back shared
// by the kernels of one simulation and of a batch of simulations.
//
// Waits between thread blocks are bounded: after kSpinLimit polls a block records an
// error and carries on, so a fault in the ordering logic surfaces as PT_ERR_TIMEOUT on
// the host instead of a hang.
#pragma once
#include <cstdint>

namespace ptk {

constexpr long long kSpinLimit = 1ll << 22;

// ------------------------------------------------------------------ look-back
// Tile status word: bits 63..34 epoch, 33..32 flag (1 aggregate, 2 inclusive
// prefix), 31..0 value.  The epoch makes words of earlier launches stale without a
// memset: the last block to finish a launch increments it and resets the tickets.
struct LookBack {
    unsigned long long *tiles;
    int *ctl;   // ctl[0] ticket, ctl[1] finished, ctl[2] epoch
    int *error;
};

__device__ __forceinline__ unsigned long long lb_word(unsigned epoch, unsigned flag, unsigned value)
{
    return ((unsigned long long)epoch << 34) | ((unsigned long long)flag << 32) | value;
}

// Called by all 32 lanes of one warp.  Publishes the tile aggregate, then walks back
// 32 predecessors per step (one word per lane) to the nearest inclusive prefix,
// publishes the tile's inclusive prefix and returns the exclusive one on every lane.
// A tile that starts a segment (segment_start) publishes its aggregate as its
// inclusive prefix: the scans of consecutive segments are independent.  After
// spin_limit polls without progress the wait records lb.error and gives up.
static __device__ unsigned lookback_publish_warp(const LookBack &lb, unsigned epoch, int tile, unsigned aggregate,
                                                 bool segment_start = false, long long spin_limit = kSpinLimit)
{
    volatile unsigned long long *t = lb.tiles;
    const int lane = threadIdx.x & 31;
    if (tile == 0 || segment_start) {
        if (lane == 0) t[tile] = lb_word(epoch, 2, aggregate);
        return 0;
    }
    if (lane == 0) t[tile] = lb_word(epoch, 1, aggregate);
    unsigned excl = 0;
    int top = tile - 1;  // the window covers tiles top, top-1, ..., top-31
    long long spins = 0;
    while (true) {
        const int j = top - lane;
        unsigned long long w = j >= 0 ? t[j] : lb_word(epoch, 2, 0);  // before tile 0: prefix 0
        const bool ready = (unsigned)(w >> 34) == (epoch & 0x3FFFFFFFu) && ((unsigned)(w >> 32) & 3u) != 0;
        const bool prefix = ready && ((unsigned)(w >> 32) & 3u) == 2;
        const unsigned rmask = __ballot_sync(0xffffffffu, ready);
        const unsigned pmask = __ballot_sync(0xffffffffu, prefix);
        // lanes up to (and including) the closest prefix must all be ready
        const int stop = pmask ? __ffs(pmask) - 1 : 31;
        const unsigned need = stop == 31 ? 0xffffffffu : ((2u << stop) - 1u);
        if ((rmask & need) == need) {
            unsigned v = (lane <= stop) ? (unsigned)w : 0u;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            excl += v;
            if (pmask) break;
            top -= 32;
            continue;
        }
        if (++spins > spin_limit) {
            if (lane == 0) atomicExch(lb.error, 1);
            break;
        }
        __nanosleep(64);
    }
    if (lane == 0) t[tile] = lb_word(epoch, 2, excl + aggregate);
    return excl;
}

// Start of a look-back launch: returns the tile index and epoch (broadcast).
__device__ __forceinline__ void lookback_begin(const LookBack &lb, int &tile, unsigned &epoch)
{
    __shared__ int s_tile;
    __shared__ unsigned s_epoch;
    if (threadIdx.x == 0) {
        s_tile = atomicAdd(&lb.ctl[0], 1);
        s_epoch = (unsigned)(*(volatile int *)&lb.ctl[2]) & 0x3FFFFFFFu;
    }
    __syncthreads();
    tile = s_tile;
    epoch = s_epoch;
}

// End of a look-back launch: the last block resets the ticket and bumps the epoch.
__device__ __forceinline__ void lookback_end(const LookBack &lb)
{
    if (threadIdx.x == 0) {
        __threadfence();
        int fin = atomicAdd(&lb.ctl[1], 1);
        if (fin == (int)gridDim.x - 1) {
            lb.ctl[0] = 0;
            lb.ctl[1] = 0;
            atomicAdd(&lb.ctl[2], 1);
            __threadfence();
        }
    }
}

// ------------------------------------------------------------------ block scan
template <int THREADS, typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T &total)
{
    static_assert(THREADS % 32 == 0, "");
    constexpr int W = THREADS / 32;
    __shared__ T s_warp[W];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = lane < W ? s_warp[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < W) s_warp[lane] = w;
    }
    __syncthreads();
    T warp_prefix = warp > 0 ? s_warp[warp - 1] : T(0);
    total = s_warp[W - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

__device__ __forceinline__ int warp_inclusive_scan(int v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    return v;
}

}  // namespace ptk

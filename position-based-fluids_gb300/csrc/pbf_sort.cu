// pbf_sort.cu — stable LSD radix sort of (cell key, particle index) pairs.
//
// The reference sorts with 6 passes of 5 bits over 2048 "virtual processors"
// (radixsort.cl:61-308, src/Simulation.cpp:456-536).  Its result is the
// stable sort of the keys (every key is below 2^30), and that order is the
// contract here: equal keys keep their input order.
//
// Here the keys are < gridBufSize, so only ceil(log2(gridBufSize) / 8)
// passes of 8-bit digits are run (3 at gridBufSize = 2^19).  Each pass is
//   upsweep   : per-tile 256-bin digit histogram -> hist[digit][tile]
//   scan      : per digit, an exclusive scan over the tiles (one block per
//               digit); the downsweep adds the exclusive scan of the digit
//               totals
//   downsweep : per-warp stable ranking with __match_any_sync and per-warp
//               digit counters in shared memory, then the scatter.
// A tile is 8 warps x kRounds rounds of 32 keys: 4096 keys (16 rounds) above
// 2^21 keys, 2048 (8 rounds) above 2^18 and 1024 (4 rounds) below, so that
// smaller sorts still spread over the SMs (at 2^20 keys, 512 tiles sort
// 12 % faster than 256).  Each warp owns consecutive keys taken round by
// round, so (warp, round, lane) order is input order.

#include <cuda_runtime.h>
#include <cstdint>

#include "pbf_internal.h"

namespace pbf {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kSmallSortKeys = 1 << 18;     // at most this many keys: 4-round tiles
constexpr int kMidSortKeys = 1 << 21;       // at most this many keys: 8-round tiles

template <int kRounds>
__global__ void __launch_bounds__(kThreads)
radix_upsweep_kernel(const uint32_t* __restrict__ keys, int n, int shift, int tiles, uint32_t* __restrict__ hist) {
    constexpr int kTile = kThreads * kRounds;
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * kTile;
#pragma unroll 4
    for (int r = 0; r < kRounds; ++r) {
        const size_t idx = base + (size_t)r * kThreads + threadIdx.x;
        if (idx < (size_t)n) atomicAdd(&h[(keys[idx] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Per-digit exclusive scan over the tiles: block d scans row d of
// hist[digit][tile] in place and writes the row's total to totals[d].
__global__ void __launch_bounds__(kThreads)
radix_scan_kernel(uint32_t* __restrict__ hist, int tiles, uint32_t* __restrict__ totals) {
    __shared__ uint32_t warpSums[kWarps];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t* row = hist + (size_t)blockIdx.x * tiles;
    uint32_t carry = 0;
    for (int base = 0; base < tiles; base += kThreads) {
        const int k = base + t;
        const uint32_t v = k < tiles ? row[k] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= d) incl += u;
        }
        if (lane == 31) warpSums[warp] = incl;
        __syncthreads();
        uint32_t before = 0, all = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t ws = warpSums[w];
            before += w < warp ? ws : 0u;
            all += ws;
        }
        if (k < tiles) row[k] = carry + before + incl - v;
        carry += all;
        __syncthreads();
    }
    if (t == 0) totals[blockIdx.x] = carry;
}

template <int kRounds>
__global__ void __launch_bounds__(kThreads)
radix_downsweep_kernel(const uint32_t* __restrict__ keysIn, const uint32_t* __restrict__ permIn,
                       uint32_t* __restrict__ keysOut, uint32_t* __restrict__ permOut, int n, int shift,
                       int tiles, const uint32_t* __restrict__ hist, const uint32_t* __restrict__ totals) {
    constexpr int kTile = kThreads * kRounds;
    constexpr int kWarpKeys = 32 * kRounds;
    __shared__ uint32_t warpCount[kWarps][256];
    __shared__ uint32_t digitBase[256];
    __shared__ uint32_t warpSums[kWarps];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) warpCount[w][t] = 0;
    {   // digitBase[d] = keys of all tiles with a smaller digit (exclusive scan of the totals)
        const uint32_t v = totals[t];
        uint32_t incl = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= d) incl += u;
        }
        if (lane == 31) warpSums[warp] = incl;
        __syncthreads();
        uint32_t before = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) before += w < warp ? warpSums[w] : 0u;
        digitBase[t] = before + incl - v;
    }
    __syncthreads();

    const size_t base = (size_t)blockIdx.x * kTile + (size_t)warp * kWarpKeys;
    const unsigned ltMask = (1u << lane) - 1u;
    uint32_t key[kRounds], rank[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        const size_t idx = base + (size_t)r * 32 + lane;
        const bool valid = idx < (size_t)n;
        const unsigned active = __ballot_sync(0xFFFFFFFFu, valid);
        uint32_t k = 0, rk = 0, peers = 0, prior = 0;
        if (valid) {
            k = keysIn[idx];
            const uint32_t d = (k >> shift) & 0xFFu;
            peers = __match_any_sync(active, d);
            prior = warpCount[warp][d];
            rk = prior + __popc(peers & ltMask);
        }
        __syncwarp();
        if (valid && (__ffs(peers) - 1) == lane) warpCount[warp][(k >> shift) & 0xFFu] = prior + __popc(peers);
        __syncwarp();
        key[r] = k;
        rank[r] = rk;
    }
    __syncthreads();
    {   // exclusive scan over warps for digit t
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t c = warpCount[w][t];
            warpCount[w][t] = run;
            run += c;
        }
        digitBase[t] += hist[(size_t)t * tiles + blockIdx.x];
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        const size_t idx = base + (size_t)r * 32 + lane;
        if (idx < (size_t)n) {
            const uint32_t d = (key[r] >> shift) & 0xFFu;
            const uint32_t dst = digitBase[d] + warpCount[warp][d] + rank[r];
            keysOut[dst] = key[r];
            permOut[dst] = permIn[idx];
        }
    }
}

}  // namespace

SortPlan make_sort_plan(int n, uint32_t gridBufSize) {
    SortPlan p;
    p.n = n;
    int bits = 0;
    while (bits < 32 && ((uint64_t)1 << bits) < (uint64_t)gridBufSize) ++bits;  // keys <= gridBufSize-1
    p.passes = (bits + 7) / 8;
    p.rounds = n <= kSmallSortKeys ? 4 : (n <= kMidSortKeys ? 8 : 16);
    const int tile = kThreads * p.rounds;
    p.tiles = (n + tile - 1) / tile;
    p.histWords = (size_t)256 * p.tiles + 256;  // per-tile histograms, then the 256 digit totals
    return p;
}

int radix_sort_launches(const SortPlan& plan) { return 3 * plan.passes; }

int launch_radix_sort(const SortPlan& plan, uint32_t* keys[2], uint32_t* perm[2], uint32_t* hist,
                      const float4*, const float4*, float4*, float4*, cudaStream_t s) {
    int cur = 0;
    uint32_t* totals = hist + (size_t)256 * plan.tiles;
    for (int pass = 0; pass < plan.passes; ++pass) {
        const int shift = 8 * pass;
        if (plan.rounds == 4)
            radix_upsweep_kernel<4><<<plan.tiles, kThreads, 0, s>>>(keys[cur], plan.n, shift, plan.tiles, hist);
        else if (plan.rounds == 8)
            radix_upsweep_kernel<8><<<plan.tiles, kThreads, 0, s>>>(keys[cur], plan.n, shift, plan.tiles, hist);
        else
            radix_upsweep_kernel<16><<<plan.tiles, kThreads, 0, s>>>(keys[cur], plan.n, shift, plan.tiles, hist);
        radix_scan_kernel<<<256, kThreads, 0, s>>>(hist, plan.tiles, totals);
        if (plan.rounds == 4)
            radix_downsweep_kernel<4><<<plan.tiles, kThreads, 0, s>>>(keys[cur], perm[cur], keys[cur ^ 1],
                                                                      perm[cur ^ 1], plan.n, shift, plan.tiles, hist,
                                                                      totals);
        else if (plan.rounds == 8)
            radix_downsweep_kernel<8><<<plan.tiles, kThreads, 0, s>>>(keys[cur], perm[cur], keys[cur ^ 1],
                                                                      perm[cur ^ 1], plan.n, shift, plan.tiles, hist,
                                                                      totals);
        else
            radix_downsweep_kernel<16><<<plan.tiles, kThreads, 0, s>>>(keys[cur], perm[cur], keys[cur ^ 1],
                                                                       perm[cur ^ 1], plan.n, shift, plan.tiles, hist,
                                                                       totals);
        cur ^= 1;
    }
    return cur;
}

}  // namespace pbf

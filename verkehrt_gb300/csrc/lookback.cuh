// Helpers of the one-tile-per-block lookback kernels (group numbering, radix passes): tickets,
// block sums, and the publish / look back / publish sequence over the records of tilepass.cuh.
#pragma once

#include "tilepass.cuh"

namespace vkc {

// Run by all 32 lanes of one warp: publishes the tile's aggregate, looks back, publishes the
// inclusive prefix, and returns the exclusive prefix in every lane.
template <int P, class R>
__device__ typename R::V lookback_publish(typename R::W *recs, int tile, typename R::V agg, typename R::V init,
                                          unsigned epoch, DevStatus *status) {
    const int lane = threadIdx.x & 31;
    if (lane == 0) R::store(rec_at<R>(recs, tile), R::make(epoch, 1u, agg));
    __syncwarp();
    const typename R::V pre = tile_lookback<P, R>(recs, tile, init, epoch, status);
    if (lane == 0) R::store(rec_at<R>(recs, tile), R::make(epoch, 2u, R::op(pre, agg)));
    return pre;
}

// Block-wide exclusive sum of one value per thread (blockDim.x a multiple of 32, at most 1024).
// Returns the exclusive prefix; *total gets the block sum.
template <class V> __device__ __forceinline__ V block_exclusive_sum(V v, V *total) {
    __shared__ V warp_tot[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    V x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        V y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        V t = lane < nw ? warp_tot[lane] : V(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            V y = __shfl_up_sync(FULL, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) warp_tot[lane] = t;  // inclusive over warps
    }
    __syncthreads();
    V before = w ? warp_tot[w - 1] : V(0);
    *total = warp_tot[nw - 1];
    __syncthreads();
    return before + x - v;
}

// Ticket and end-of-launch reset shared by the lookback kernels: tiles are handed out in
// launch order so that every tile a block waits on belongs to a block that already runs.
__device__ __forceinline__ int take_ticket(unsigned *counters) {
    __shared__ unsigned s_tile;
    if (threadIdx.x == 0) s_tile = atomicAdd(&counters[0], 1u);
    __syncthreads();
    return static_cast<int>(s_tile);
}

// Counts the block out; the last of `tiles` blocks resets the ticket counters for the next
// launch (every block took its ticket before it counts out).
__device__ __forceinline__ void release_ticket(unsigned *counters, int tiles) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned prev = atomicAdd(&counters[1], 1u);
        if (prev == static_cast<unsigned>(tiles) - 1) {
            counters[0] = 0;
            counters[1] = 0;
        }
    }
}

}  // namespace vkc

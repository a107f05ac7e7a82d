// Decoupled lookback over tiles (single-pass prefix across thread blocks), for compaction and
// scans. Flags live in the context's flag arena and carry the launch epoch; aggregate and
// inclusive values live in separate arrays so a published aggregate is never overwritten.
#pragma once

#include "kcommon.cuh"

namespace vkc {

template <class V> struct LookbackTiles {
    unsigned *flag;  // [tiles] epoch<<2 | 1 (aggregate) | 2 (inclusive)
    V *agg;          // [tiles]
    V *inc;          // [tiles]
};

// The exclusive prefix of `tile` under the associative `op` (prefix, then tile), run by one
// thread. `init` is the prefix before tile 0. Publishes the aggregate first and the inclusive
// value after. On a wait that runs out it records a timeout and returns what it has.
template <class V, class Op>
__device__ V lookback_exclusive(LookbackTiles<V> lb, int tile, V agg, V init, unsigned epoch,
                                Op op, DevStatus *status) {
    lb.agg[tile] = agg;
    __threadfence();
    st_release(&lb.flag[tile], (epoch << 2) | 1u);
    V excl{};
    bool have = false;  // excl holds the combination of the tiles walked so far
    int tp = tile - 1;
    for (; tp >= 0; --tp) {
        unsigned f, it = 0;
        while (((f = ld_acquire(&lb.flag[tp])) >> 2) != epoch) {
            if (++it > SPIN_LIMIT) {
                set_timeout(status);
                return init;
            }
            backoff(it);
        }
        if ((f & 3u) == 2u) {
            V p = lb.inc[tp];
            excl = have ? op(p, excl) : p;
            have = true;
            break;
        }
        V a = lb.agg[tp];
        excl = have ? op(a, excl) : a;
        have = true;
    }
    if (tp < 0) excl = have ? op(init, excl) : init;
    lb.inc[tile] = op(excl, agg);
    __threadfence();
    st_release(&lb.flag[tile], (epoch << 2) | 2u);
    return excl;
}

// Warp shuffles of lookback values.
__device__ __forceinline__ unsigned long long shfl_down_v(unsigned long long v, int o) {
    return __shfl_down_sync(FULL, v, o);
}
__device__ __forceinline__ unsigned long long __shfl_sync_v(unsigned long long v, int src) {
    return __shfl_sync(FULL, v, src);
}

// Warp-parallel decoupled lookback, run by all 32 lanes of one warp: publishes the tile's
// aggregate, then reads the flags of 32 predecessor tiles per step (lane i reads tile
// hi - i), combines every aggregate up to the closest inclusive value in one ordered warp
// reduction, and stops at that inclusive value (or at `init` before tile 0). Publishes the
// inclusive value and returns the exclusive prefix in every lane. `ident` is the identity of
// `op`. On a wait that runs out it records a timeout and returns `init`.
template <class V, class Op>
__device__ V warp_lookback(LookbackTiles<V> lb, int tile, V agg, V init, V ident, unsigned epoch, Op op,
                           DevStatus *status) {
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        lb.agg[tile] = agg;
        __threadfence();
        st_release(&lb.flag[tile], (epoch << 2) | 1u);
    }
    __syncwarp();
    V excl = ident;
    bool have = false;
    for (int hi = tile - 1;; hi -= 32) {
        int tp = hi - lane;
        unsigned f = 0;
        bool bad = false;
        if (tp >= 0) {
            unsigned it = 0;
            while (((f = ld_acquire(&lb.flag[tp])) >> 2) != epoch) {
                if (++it > SPIN_LIMIT) {
                    set_timeout(status);
                    bad = true;
                    break;
                }
                backoff(it);
            }
        }
        if (__any_sync(FULL, bad)) return init;
        bool incl = tp < 0 || (f & 3u) == 2u;
        unsigned m = __ballot_sync(FULL, incl);
        int k = m ? __ffs(m) - 1 : 32;
        V v = ident;
        if (lane < k) v = lb.agg[tp];
        else if (lane == k) v = tp >= 0 ? lb.inc[tp] : init;
        // Lane i holds tile hi - i, so the higher lane is the earlier tile.
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            V other = shfl_down_v(v, o);
            if (lane + o < 32) v = op(other, v);
        }
        V window = __shfl_sync_v(v, 0);
        excl = have ? op(window, excl) : window;
        have = true;
        if (k < 32) break;
    }
    if (lane == 0) {
        lb.inc[tile] = op(excl, agg);
        __threadfence();
        st_release(&lb.flag[tile], (epoch << 2) | 2u);
    }
    return excl;
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

// Returns true in every thread of the block that finishes last, after its fence, so that
// block may read what every other block wrote.
__device__ __forceinline__ bool release_ticket_last(unsigned *counters, int tiles) {
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned prev = atomicAdd(&counters[1], 1u);
        s_last = prev == static_cast<unsigned>(tiles) - 1;
        if (s_last) {
            counters[0] = 0;
            counters[1] = 0;
        }
    }
    __syncthreads();
    if (s_last) __threadfence();
    return s_last != 0;
}

__device__ __forceinline__ void release_ticket(unsigned *counters, int tiles) {
    release_ticket_last(counters, tiles);
}

}  // namespace vkc

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
// aggregate, then reads the flags of 32*P predecessor tiles per step (lane i reads tiles
// hi - P*i - j, j < P), combines every aggregate up to the closest inclusive value in one
// ordered warp reduction, and stops at that inclusive value (or at `init` before tile 0).
// Publishes the inclusive value and returns the exclusive prefix in every lane. `ident` is
// the identity of `op`. On a wait that runs out it records a timeout and returns `init`.
//
// A step costs two L2 round trips (the flags, then the values), and a tile waits for the
// tiles before it in launch order, so the window width is what bounds the tile rate.
template <int P, class V, class Op>
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
    for (int hi = tile - 1;; hi -= 32 * P) {
        unsigned f[P];
        bool bad = false;
#pragma unroll
        for (int j = 0; j < P; ++j) {
            const int tp = hi - P * lane - j;
            f[j] = 0;
            if (tp >= 0) {
                unsigned it = 0;
                while (((f[j] = ld_acquire(&lb.flag[tp])) >> 2) != epoch) {
                    if (++it > SPIN_LIMIT) {
                        set_timeout(status);
                        bad = true;
                        break;
                    }
                    backoff(it);
                }
            }
        }
        if (__any_sync(FULL, bad)) return init;
        // The lane's closest inclusive item, and the warp's.
        int jin = P;
#pragma unroll
        for (int j = P - 1; j >= 0; --j) {
            const int tp = hi - P * lane - j;
            if (tp < 0 || (f[j] & 3u) == 2u) jin = j;
        }
        const unsigned m = __ballot_sync(FULL, jin < P);
        const int kl = m ? __ffs(m) - 1 : 32;  // first lane holding an inclusive item
        // Lane value: its items from the earliest used one to the latest, in order.
        V v = ident;
        if (lane <= kl) {
            const int jmax = lane == kl ? jin : P - 1;
#pragma unroll
            for (int j = P - 1; j >= 0; --j) {
                if (j > jmax) continue;
                const int tp = hi - P * lane - j;
                V x;
                if (lane == kl && j == jin) x = tp >= 0 ? lb.inc[tp] : init;
                else x = lb.agg[tp];
                v = (j == jmax) ? x : op(v, x);
            }
        }
        // Lane i holds later tiles than lane i + 1.
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            V other = shfl_down_v(v, o);
            if (lane + o < 32) v = op(other, v);
        }
        V window = __shfl_sync_v(v, 0);
        excl = have ? op(window, excl) : window;
        have = true;
        if (kl < 32) break;
    }
    if (lane == 0) {
        lb.inc[tile] = op(excl, agg);
        __threadfence();
        st_release(&lb.flag[tile], (epoch << 2) | 2u);
    }
    return excl;
}

// Counts in one word: epoch (24 bits) | state (2 bits) | count (38 bits), so a lookback step
// is a single L2 round trip. Counts must stay below 2^38.
__device__ __forceinline__ unsigned long long packed_word(unsigned epoch, unsigned state, unsigned long long c) {
    return (static_cast<unsigned long long>(epoch & 0xffffffu) << 40) | (static_cast<unsigned long long>(state) << 38) | c;
}

// warp_lookback for additive counts in packed words: `words` holds one word per tile.
template <int P>
__device__ unsigned long long warp_lookback_count(unsigned long long *words, int tile, unsigned long long agg,
                                                  unsigned epoch, DevStatus *status) {
    const int lane = threadIdx.x & 31;
    const unsigned long long ep = epoch & 0xffffffu;
    if (lane == 0) st_release64(words + tile, packed_word(epoch, 1, agg));
    __syncwarp();
    unsigned long long excl = 0;
    for (int hi = tile - 1;; hi -= 32 * P) {
        unsigned long long w[P];
        bool bad = false;
#pragma unroll
        for (int j = 0; j < P; ++j) {
            const int tp = hi - P * lane - j;
            w[j] = packed_word(epoch, 2, 0);  // before tile 0: inclusive zero
            if (tp >= 0) {
                unsigned it = 0;
                while (((w[j] = ld_acquire64(words + tp)) >> 40) != ep) {
                    if (++it > SPIN_LIMIT) {
                        set_timeout(status);
                        bad = true;
                        break;
                    }
                    backoff(it);
                }
            }
        }
        if (__any_sync(FULL, bad)) return 0;
        int jin = P;
#pragma unroll
        for (int j = P - 1; j >= 0; --j)
            if (((w[j] >> 38) & 3u) == 2u) jin = j;
        const unsigned m = __ballot_sync(FULL, jin < P);
        const int kl = m ? __ffs(m) - 1 : 32;
        unsigned long long v = 0;
        if (lane <= kl) {
            const int jmax = lane == kl ? jin : P - 1;
#pragma unroll
            for (int j = 0; j < P; ++j)
                if (j <= jmax) v += w[j] & ((1ull << 38) - 1);
        }
        excl += warp_sum(v);
        if (kl < 32) break;
    }
    if (lane == 0) st_release64(words + tile, packed_word(epoch, 2, excl + agg));
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

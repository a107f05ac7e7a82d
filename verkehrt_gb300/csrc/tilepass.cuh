// Persistent single-pass driver for order-dependent passes over tiles (compaction, scans).
//
// A pass over an array whose output position depends on everything before it needs, per tile,
// the combination of all earlier tiles: the decoupled lookback. Done the textbook way (load a
// tile, wait for its prefix, write it) a block idles for the lookback's L2 round trips with no
// loads in flight, and on GB300 that idling, not HBM, set the rate. Here a block holds two
// tiles and works one tile ahead:
//
//   count(next)    stream the next tile from HBM and publish its aggregate (no waits)
//   lookback(cur)  its predecessors published their aggregates one tile-time ago, so the
//                  lookback is normally one round of polls
//   write(cur)     re-read the current tile, now in L2, and write its output
//
// The data between the two reads of a tile stays in L2: about two tiles per resident block,
// 40 MB over the whole GPU against 126 MB of L2. Tiles are handed out by an atomic ticket in
// launch order, and a block publishes the aggregate of a tile before it waits on anything, so
// every tile a block waits on belongs to a running block that publishes without waiting.
//
// Lookback records are packed words carrying the launch epoch, the state (1 aggregate,
// 2 inclusive prefix) and the value, written and polled with relaxed accesses: a record is
// read whole or seen as not ready, and no other data is ordered behind it.
#pragma once

#include "kcommon.cuh"

namespace vkc {

// Sleep between two polls of records that were not ready. Polling warps all read the few L2
// lines that hold the newest records; without a pause they slow the stores they wait for.
constexpr unsigned LB_POLL_NS = 200;

// Counts below 2^38 in one word: epoch (24 bits) | state (2 bits) | count (38 bits).
struct CountRec {
    using V = unsigned long long;
    using W = unsigned long long;
    __device__ static V ident() { return 0; }
    __device__ static V op(V a, V b) { return a + b; }
    __device__ static W make(unsigned ep, unsigned state, V v) {
        return (static_cast<unsigned long long>(ep & 0xffffffu) << 40) | (static_cast<unsigned long long>(state) << 38) | v;
    }
    __device__ static bool ready(W w, unsigned ep) { return (w >> 40) == (ep & 0xffffffu); }
    __device__ static unsigned state(W w) { return static_cast<unsigned>(w >> 38) & 3u; }
    __device__ static V value(W w) { return w & ((1ull << 38) - 1); }
    __device__ static W load(const W *p) { return ld_relaxed64(p); }
    __device__ static void store(W *p, W w) { st_relaxed64(p, w); }
    __device__ static V shfl_up(V v, int o) { return __shfl_up_sync(FULL, v, o); }
    __device__ static V shfl(V v, int src) { return __shfl_sync(FULL, v, src); }
    __device__ static V shfl_down(V v, int o) { return __shfl_down_sync(FULL, v, o); }
};

// The closest-first exclusive prefix of `tile`: run by all 32 lanes of one warp. Each step
// reads the records of the 32*P tiles before the window end at once (lane i takes tiles
// hi - P*i - j), polls again only those not yet published, combines every aggregate back to
// the closest inclusive prefix in one ordered warp reduction, and stops there (or at `init`
// before tile 0). Returns the prefix in every lane. On a wait that runs out it records a
// timeout and returns `init`.
template <int P, class R>
__device__ typename R::V tile_lookback(typename R::W *recs, int tile, typename R::V init, unsigned epoch,
                                       DevStatus *status) {
    using V = typename R::V;
    using W = typename R::W;
    const int lane = threadIdx.x & 31;
    V excl = R::ident();
    bool have = false;
    for (int hi = tile - 1;; hi -= 32 * P) {
        W w[P];
        bool got[P];
#pragma unroll
        for (int j = 0; j < P; ++j) {
            w[j] = W{};
            got[j] = hi - P * lane - j < 0;
        }
        bool bad = false;
        for (unsigned it = 0;;) {
#pragma unroll
            for (int j = 0; j < P; ++j)
                if (!got[j]) w[j] = R::load(recs + (hi - P * lane - j));
            bool all = true;
#pragma unroll
            for (int j = 0; j < P; ++j) {
                if (!got[j]) got[j] = R::ready(w[j], epoch);
                all = all && got[j];
            }
            if (all) break;
            if (++it > SPIN_LIMIT) {
                set_timeout(status);
                bad = true;
                break;
            }
            __nanosleep(LB_POLL_NS);
        }
        if (__any_sync(FULL, bad)) return init;
        // The lane's closest inclusive item (tiles before 0 count as the inclusive `init`).
        int jin = P;
#pragma unroll
        for (int j = P - 1; j >= 0; --j)
            if (hi - P * lane - j < 0 || R::state(w[j]) == 2u) jin = j;
        const unsigned m = __ballot_sync(FULL, jin < P);
        const int kl = m ? __ffs(m) - 1 : 32;  // first lane holding an inclusive item
        // Lane value: its items from the earliest one used to the latest, in order.
        V v = R::ident();
        if (lane <= kl) {
            const int jmax = lane == kl ? jin : P - 1;
#pragma unroll
            for (int j = P - 1; j >= 0; --j) {
                if (j > jmax) continue;
                const int tp = hi - P * lane - j;
                const V x = tp < 0 ? init : R::value(w[j]);
                v = j == jmax ? x : R::op(v, x);
            }
        }
        // Lane i holds later tiles than lane i + 1: fold from lane 31 down to lane 0.
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const V other = R::shfl_down(v, o);
            if (lane + o < 32) v = R::op(other, v);
        }
        const V window = R::shfl(v, 0);
        excl = have ? R::op(window, excl) : window;
        have = true;
        if (kl < 32) break;
    }
    return excl;
}

// Ordered inclusive scan of one value per lane under R::op (lane 0 first).
template <class R> __device__ __forceinline__ typename R::V warp_inclusive(typename R::V v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const typename R::V y = R::shfl_up(v, o);
        if (lane >= o) v = R::op(y, v);
    }
    return v;
}

// The driver. `Pass` supplies
//   THREADS                      block size (a multiple of 32, at most 1024)
//   R                            the record type above
//   V count(int tile)            run by every warp on its slice of the tile; the slice
//                                aggregate in every lane (no block synchronisation inside)
//   void write(int tile, V pre)  run by every warp on its slice, given the combination of
//                                everything before the slice
//   void last_tile(V inclusive)  run by one thread with the inclusive prefix of the last tile
// and the launch hands out `tiles` tiles. Returns true in every thread of the block that
// finishes last (after a fence: it may read what every block wrote); that block has reset the
// ticket counters for the next launch.
template <int P, class Pass>
__device__ bool tile_pass(Pass &p, typename Pass::R::W *recs, int tiles, unsigned epoch, unsigned *counters,
                          DevStatus *status, typename Pass::R::V init) {
    using R = typename Pass::R;
    using V = typename R::V;
    constexpr int WARPS = Pass::THREADS / 32;
    static_assert(WARPS <= 32, "one warp combines the warps of a tile");
    __shared__ V s_agg[2][WARPS];  // slice aggregates of the two held tiles, then slice prefixes
    __shared__ V s_prefix;
    __shared__ int s_tile[2];
    __shared__ int s_last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;

    // Lane 0 of warp 0: the tile aggregate from the slice aggregates of `slot`, published.
    auto publish_agg = [&](int tile, int slot) {
        V a = warp_inclusive<R>(lane < WARPS ? s_agg[slot][lane] : R::ident());
        a = R::shfl(a, WARPS - 1);
        if (lane == 0) R::store(recs + tile, R::make(epoch, 1u, a));
    };

    if (threadIdx.x == 0) s_tile[0] = static_cast<int>(atomicAdd(&counters[0], 1u));
    __syncthreads();
    int cur = s_tile[0], slot = 0;
    if (cur < tiles) {
        const V a = p.count(cur);
        if (lane == 0) s_agg[0][w] = a;
        __syncthreads();
        if (w == 0) publish_agg(cur, 0);
    }
    while (cur < tiles) {
        if (threadIdx.x == 0) s_tile[slot ^ 1] = static_cast<int>(atomicAdd(&counters[0], 1u));
        __syncthreads();  // also: every warp is done with the previous write
        const int nxt = s_tile[slot ^ 1];
        if (nxt < tiles) {
            const V a = p.count(nxt);
            if (lane == 0) s_agg[slot ^ 1][w] = a;
        }
        __syncthreads();
        if (w == 0) {
            if (nxt < tiles) publish_agg(nxt, slot ^ 1);
            const V c = lane < WARPS ? s_agg[slot][lane] : R::ident();
            const V inc = warp_inclusive<R>(c);
            V ex = R::shfl_up(inc, 1);
            if (lane == 0) ex = R::ident();
            const V tile_agg = R::shfl(inc, WARPS - 1);
            const V pre = tile_lookback<P, R>(recs, cur, init, epoch, status);
            if (lane == 0) {
                const V all = R::op(pre, tile_agg);
                R::store(recs + cur, R::make(epoch, 2u, all));
                s_prefix = pre;
                if (cur == tiles - 1) p.last_tile(all);
            }
            if (lane < WARPS) s_agg[slot][lane] = ex;
        }
        __syncthreads();
        p.write(cur, R::op(s_prefix, s_agg[slot][w]));
        cur = nxt;
        slot ^= 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&counters[1], 1u);
        s_last = prev == gridDim.x - 1;
        if (s_last) {
            counters[0] = 0;
            counters[1] = 0;
        }
    }
    __syncthreads();
    if (s_last) __threadfence();
    return s_last != 0;
}

// Blocks of a persistent tile pass: as many as can be resident at once (at most one per tile).
template <class K> int tile_pass_grid(vkc_ctx *ctx, K kernel, int threads, size_t smem, int tiles) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    const long long g = static_cast<long long>(per_sm) * ctx->sms;
    return static_cast<int>(g < tiles ? g : tiles);
}

}  // namespace vkc

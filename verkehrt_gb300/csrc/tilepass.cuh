// Persistent single-pass driver for order-dependent passes over tiles (compaction, scans).
//
// A pass over an array whose output position depends on everything before it needs, per tile,
// the combination of all earlier tiles: the decoupled lookback. Done the textbook way (load a
// tile, wait for its prefix, write it) a block idles for the lookback's L2 round trips with no
// loads in flight. Here each block is warp-specialised around a ring of tiles in shared memory:
//
//   producer warp   takes tickets (one ahead) and streams tiles from HBM into free slots of
//                   the ring with TMA bulk copies (cp.async.bulk, completion on an mbarrier)
//   compute warps   count(next)   aggregate of the next tile, one per warp slice
//                   stage(cur)    everything of the current tile's output that needs no
//                                 prefix, in shared memory
//                   flush(cur)    write the output, given the prefix, and free the slot
//   lookback warp   looks back for the current tile while the compute warps work on (the
//                   aggregates are published by the compute warps right after each count) and
//                   publishes its inclusive prefix
//
// The data moves once, by TMA, which also keeps the SM's load/store pipeline free for the
// lookback's polls and stores (with the tiles loaded through that pipeline, those waited
// behind the loads for microseconds). The roles meet at named barriers and the slots'
// mbarriers, so the compute warps wait only for data or for a lookback slower than a count and
// a stage. Several blocks share an SM so that their lookbacks overlap. Tiles are handed out by
// an atomic ticket in launch order, and a tile's aggregate is published after a count that
// waits on nothing but its own copy, so every tile a lookback waits on belongs to a running
// block that publishes it.
//
// Lookback records are packed words carrying the launch epoch, the state (1 aggregate,
// 2 inclusive prefix) and the value, written and polled with relaxed accesses: a record is
// read whole or seen as not ready, and no other data is ordered behind it. Records sit 128
// bytes apart: every block polls the newest records, and packed together they would fall on
// a few L2 slices.
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

// Bytes between two consecutive tiles' records.
constexpr int REC_STRIDE = 128;

template <class R> __device__ __forceinline__ typename R::W *rec_at(typename R::W *recs, int tile) {
    return recs + static_cast<int64_t>(tile) * (REC_STRIDE / sizeof(typename R::W));
}

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
        const unsigned limit = wait_limit(status);
        // The test hook lookback_never_ready polls for another epoch, which no block writes.
        const unsigned want = never_ready(status) ? epoch % 0xffffffu + 1u : epoch;
        for (unsigned it = 0;;) {
#pragma unroll
            for (int j = 0; j < P; ++j)
                if (!got[j]) w[j] = R::load(rec_at<R>(recs, hi - P * lane - j));
            bool all = true;
#pragma unroll
            for (int j = 0; j < P; ++j) {
                if (!got[j]) got[j] = R::ready(w[j], want);
                all = all && got[j];
            }
            if (all) break;
            if (++it > limit) {
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

// Named barriers with immediate ids (so a block reserves only the ids it names).
template <int ID, int THREADS> __device__ __forceinline__ void named_arrive() {
    asm volatile("bar.arrive %0, %1;" ::"n"(ID), "n"(THREADS) : "memory");
}
template <int ID, int THREADS> __device__ __forceinline__ void named_sync() {
    asm volatile("bar.sync %0, %1;" ::"n"(ID), "n"(THREADS) : "memory");
}
// Id BASE + i for a runtime i < N (N <= 8).
template <int BASE, int N, int THREADS, int I = 0> __device__ __forceinline__ void named_arrive_i(int i) {
    if constexpr (I < N) {
        if (i == I) named_arrive<BASE + I, THREADS>();
        else named_arrive_i<BASE, N, THREADS, I + 1>(i);
    }
}
template <int BASE, int N, int THREADS, int I = 0> __device__ __forceinline__ void named_sync_i(int i) {
    if constexpr (I < N) {
        if (i == I) named_sync<BASE + I, THREADS>();
        else named_sync_i<BASE, N, THREADS, I + 1>(i);
    }
}

// ------------------------------------------------------------------ TMA bulk copies

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// A 1-D bulk copy global -> shared (16-byte aligned ends, a multiple of 16 bytes), completing
// on `bar`.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// Orders this thread's shared-memory accesses before later bulk copies into the same bytes.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Waits for phase `parity` of `bar` to complete. On a wait that runs out it records a timeout
// and waits once more, as long again, for the copy to land before the block goes on.
__device__ __forceinline__ void mbar_wait(unsigned long long *bar, unsigned parity, DevStatus *status) {
    for (unsigned it = 0; !mbar_try_wait(bar, parity);) {
        if (++it > SPIN_LIMIT) {
            set_timeout(status);
            for (unsigned again = 0; !mbar_try_wait(bar, parity) && again < SPIN_LIMIT; ++again) {
            }
            return;
        }
    }
}

// ------------------------------------------------------------------ the pass kernel body

// Run by a block of Pass::THREADS compute threads plus two warps (producer, then lookback),
// with Pass::SLOTS * Pass::SLOT_BYTES of dynamic shared memory (16-byte aligned slots). Tile k
// of a block sits in slot k % SLOTS from its copy to its flush, so up to SLOTS - 2 copies are in
// flight while the compute warps count one tile and stage another. `Pass` supplies
//   THREADS, SLOTS, SLOT_BYTES   compute threads (a multiple of 32, at most 30 warps); slots
//                                (3 to 8); bytes of one slot
//   R                            the record type above
//   Staged                       what stage() hands to flush() (per warp)
//   unsigned bulk_bytes(int tile)   bytes the TMA copies for `tile` (0: the compute warps read
//                                it from global memory themselves, e.g. a ragged last tile)
//   void load(int tile, unsigned char *slot, unsigned long long *bar)
//                                issues those copies (one thread)
//   V count(int tile, unsigned char *slot)      per compute warp, on its slice: the slice
//                                aggregate in every lane (no block synchronisation inside)
//   Staged stage(int tile, unsigned char *slot) per compute warp, on its slice
//   void flush(int tile, V pre, const Staged &, unsigned char *slot)
//                                per compute warp: writes the slice given everything before it
//   void last_tile(V inclusive)  run by one thread with the inclusive prefix of the last tile
// and the launch hands out `tiles` tiles. Returns true in every thread of the block that
// finishes last (after a fence: it may read what every block wrote); that block has reset the
// ticket counters for the next launch.
template <int P, class Pass>
__device__ bool tile_pass(const Pass &p, typename Pass::R::W *recs, int tiles, unsigned epoch, unsigned *counters,
                          DevStatus *status, typename Pass::R::V init) {
    using R = typename Pass::R;
    using V = typename R::V;
    constexpr int WARPS = Pass::THREADS / 32;  // compute warps; then the producer and lookback warps
    constexpr int NB = Pass::THREADS + 32;     // threads at each named barrier: compute + one warp
    constexpr int S = Pass::SLOTS;
    static_assert(WARPS <= 30, "one warp combines the slices of a tile");
    static_assert(S >= 3 && S <= 8, "slots: one counted, one staged, at least one in flight");
    static_assert(Pass::SLOT_BYTES % 16 == 0, "slots hold whole 16-byte units");
    constexpr int BAR_AGG = 1, BAR_PRE = 3, BAR_CNT = 5, BAR_FREE = 6;  // 2, 2, 1 and S ids
    extern __shared__ __align__(128) unsigned char tp_smem[];
    __shared__ unsigned long long s_full[S];  // mbarriers: the slot's tile id is set, its copy landed
    __shared__ V s_agg[2][WARPS];             // slice aggregates (tile k in [k & 1])
    __shared__ V s_pre[2][WARPS];             // slice prefixes (everything before the slice)
    __shared__ int s_tile[S];                 // the tile in each slot (tile k in k % S), or `tiles`
    __shared__ int s_last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    auto slot_ptr = [&](int i) { return tp_smem + i * Pass::SLOT_BYTES; };

    if (threadIdx.x == 0) {
        for (int i = 0; i < S; ++i) mbar_init(&s_full[i], 1);
        mbar_fence_init();
    }
    __syncthreads();

    if (w == WARPS) {
        // Producer warp: the whole warp meets the barriers, lane 0 takes the tickets and issues
        // the copies. Tile k goes to slot k % S once tile k - S has left it; the ticket for each
        // load is taken one load ahead.
        int t = 0;
        if (lane == 0) t = static_cast<int>(atomicAdd(&counters[0], 1u));
        int k = 0;
        for (;; ++k) {
            const int slot = k % S;
            if (k >= S) named_sync_i<BAR_FREE, S, NB>(slot);
            t = __shfl_sync(FULL, t, 0);
            const bool real = t < tiles;
            if (lane == 0) {
                s_tile[slot] = real ? t : tiles;
                const unsigned bytes = real ? p.bulk_bytes(t) : 0u;
                mbar_expect_tx(&s_full[slot], bytes);  // also the arrival that publishes s_tile
                if (bytes) p.load(t, slot_ptr(slot), &s_full[slot]);
                if (real) t = static_cast<int>(atomicAdd(&counters[0], 1u));
            }
            if (!real) break;
        }
        // Tiles 0..k-1 were real; the releases of tiles k-S+1..k-1 are still to be matched.
        for (int j = k - S + 1 > 0 ? k - S + 1 : 0; j < k; ++j) named_sync_i<BAR_FREE, S, NB>(j % S);
    } else if (w == WARPS + 1) {
        // Lookback warp: the aggregates of tile k are in s_agg[k & 1] (and published) when it
        // starts on tile k, so each lookback overlaps the compute warps' stage, flush and next
        // count.
        named_sync_i<BAR_AGG, 2, NB>(0);
        int cur = s_tile[0];
        for (int k = 0; cur < tiles; ++k) {
            const V inc = warp_inclusive<R>(lane < WARPS ? s_agg[k & 1][lane] : R::ident());
            V ex = R::shfl_up(inc, 1);
            if (lane == 0) ex = R::ident();
            const V tile_agg = R::shfl(inc, WARPS - 1);
            const V pre = tile_lookback<P, R>(recs, cur, init, epoch, status);
            if (lane == 0) {
                const V all = R::op(pre, tile_agg);
                R::store(rec_at<R>(recs, cur), R::make(epoch, 2u, all));
                if (cur == tiles - 1) p.last_tile(all);
            }
            if (lane < WARPS) s_pre[k & 1][lane] = R::op(pre, ex);
            named_arrive_i<BAR_PRE, 2, NB>(k & 1);
            named_sync_i<BAR_AGG, 2, NB>((k + 1) & 1);
            cur = s_tile[(k + 1) % S];
        }
    } else {
        // Compute warps. After each count, warp 0 publishes the tile's aggregate.
        auto counted = [&](int tile, int k) {
            named_sync<BAR_CNT, Pass::THREADS>();
            if (w == 0 && tile < tiles) {
                V a = warp_inclusive<R>(lane < WARPS ? s_agg[k][lane] : R::ident());
                a = R::shfl(a, WARPS - 1);
                if (lane == 0) R::store(rec_at<R>(recs, tile), R::make(epoch, 1u, a));
            }
            named_arrive_i<BAR_AGG, 2, NB>(k);
        };
        unsigned phase = 0;  // parity of the next wait, per slot
        mbar_wait(&s_full[0], 0, status);
        phase ^= 1u;
        int cur = s_tile[0];
        if (cur < tiles) {
            const V a = p.count(cur, slot_ptr(0));
            if (lane == 0) s_agg[0][w] = a;
        }
        counted(cur, 0);
        for (int k = 0; cur < tiles; ++k) {
            const int sc = k % S, sn = (k + 1) % S;
            mbar_wait(&s_full[sn], (phase >> sn) & 1u, status);
            phase ^= 1u << sn;
            const int nxt = s_tile[sn];
            if (nxt < tiles) {
                const V a = p.count(nxt, slot_ptr(sn));
                if (lane == 0) s_agg[(k + 1) & 1][w] = a;
            }
            counted(nxt, (k + 1) & 1);
            const typename Pass::Staged st = p.stage(cur, slot_ptr(sc));
            named_sync_i<BAR_PRE, 2, NB>(k & 1);
            p.flush(cur, s_pre[k & 1][w], st, slot_ptr(sc));
            fence_proxy_async();
            named_arrive_i<BAR_FREE, S, NB>(sc);
            cur = nxt;
        }
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

// The context's flag arena as lookback records of `tiles` tiles (REC_STRIDE bytes each). Every
// kernel that indexes records with rec_at takes them from here.
template <class W> vkc_status rec_arena(vkc_ctx *ctx, int tiles, W **out) {
    unsigned *f = nullptr;
    const vkc_status st = flag_arena(ctx, static_cast<size_t>(tiles) * (REC_STRIDE / sizeof(unsigned)), &f);
    *out = reinterpret_cast<W *>(f);
    return st;
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

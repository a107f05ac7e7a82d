// group_id_i64 and group_id2_i64_i64: dense ids numbered by first occurrence
// (src/kernels/scalar/group.rs:207-301).
//
// The ids depend only on the order in which distinct keys first appear (group.rs:1-5), so any
// correct table gives the reference's output. Three kernels:
//  1. insert: open addressing with linear probing in a table of nextpow2(2n) slots (the
//     reference's maximum, group.rs:226-229). A slot is claimed by CAS on its state word
//     (empty -> writing -> ready), so pair keys become visible whole. Equal keys of one warp
//     elect one leader (warp match), and each key keeps the smallest row that holds it
//     (atomicMin, skipped when the stored row is already smaller). Each row records its slot.
//  2. number: a row is a first occurrence when its slot's smallest row is itself; a
//     decoupled-lookback compaction over rows gives each first occurrence its rank, which is
//     the group's id, stored in the slot.
//  3. out: every row reads its slot's id.
#include "lookback.cuh"
#include "reduce_common.h"

namespace vkc {

constexpr int GI_THREADS = 256;
constexpr int GI_ITEMS = 16;
constexpr int GI_TILE = GI_THREADS * GI_ITEMS;

struct GroupTable {
    unsigned long long *ka, *kb;
    unsigned *state;    // 0 empty, 1 being written, 2 ready
    unsigned *minrow;   // smallest row of the key
    unsigned *id;       // group id, after numbering
    unsigned long long mask;  // slots - 1
};

// group.rs:40-47 (mix) with a fixed odd multiplier; the ids do not depend on it.
__device__ __forceinline__ unsigned long long gmix(unsigned long long x) {
    return (x ^ (x >> 32)) * 0x9E3779B97F4A7C15ull;
}

template <bool PAIR>
__global__ void __launch_bounds__(GI_THREADS) gi_insert_kernel(const long long *__restrict__ a,
                                                               const long long *__restrict__ b, int64_t n,
                                                               GroupTable t, unsigned *__restrict__ slot_of,
                                                               DevStatus *st) {
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const unsigned lane = threadIdx.x & 31, lt = (1u << lane) - 1;
    // Whole warps iterate together so the warp match sees every active lane.
    for (int64_t base = static_cast<int64_t>(blockIdx.x) * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        int64_t i = base + lane;
        bool in = i < n;
        unsigned long long ka = in ? static_cast<unsigned long long>(__ldcs(a + i)) : 0ull;
        unsigned long long kb = (PAIR && in) ? static_cast<unsigned long long>(__ldcs(b + i)) : 0ull;
        unsigned active = __ballot_sync(FULL, in);
        unsigned peers = __match_any_sync(FULL, ka) & active;
        if (PAIR) peers &= __match_any_sync(FULL, kb);
        bool leader = in && (peers & lt) == 0;
        unsigned long long s = 0;
        if (leader) {
            unsigned long long h = PAIR ? gmix(gmix(ka) ^ kb) : gmix(ka);
            s = (h >> 32 ^ h) & t.mask;
            unsigned long long probes = 0;
            for (;;) {
                unsigned sv = ld_acquire(t.state + s);
                if (sv == 0) {
                    sv = atomicCAS(t.state + s, 0u, 1u);
                    if (sv == 0) {
                        t.ka[s] = ka;
                        if (PAIR) t.kb[s] = kb;
                        __threadfence();
                        st_release(t.state + s, 2u);
                        break;
                    }
                }
                if (sv == 1) {
                    unsigned it = 0;
                    while ((sv = ld_acquire(t.state + s)) == 1) {
                        if (++it > SPIN_LIMIT) {
                            set_timeout(st);
                            break;
                        }
                        backoff(it);
                    }
                }
                if (sv == 2 && t.ka[s] == ka && (!PAIR || t.kb[s] == kb)) break;
                s = (s + 1) & t.mask;
                // A table at most half full always has a free slot; the bound only guards.
                if (++probes > t.mask) {
                    set_timeout(st);
                    break;
                }
            }
            unsigned row = static_cast<unsigned>(i);
            if (t.minrow[s] > row) atomicMin(t.minrow + s, row);
        }
        int src = __ffs(peers) - 1;
        s = __shfl_sync(FULL, s, src < 0 ? lane : src);
        if (in) slot_of[i] = static_cast<unsigned>(s);
    }
}

// Numbers the first occurrences in row order (a compaction of the rows whose slot's smallest
// row is themselves) and stores each group's id in its slot.
__global__ void __launch_bounds__(GI_THREADS) gi_number_kernel(const unsigned *__restrict__ slot_of, int64_t n,
                                                               GroupTable t, int tiles, unsigned long long *words,
                                                               unsigned epoch, unsigned *counters,
                                                               DevStatus *st) {
    __shared__ unsigned long long s_prefix;
    const int tile = take_ticket(counters);
    const int64_t row0 = static_cast<int64_t>(tile) * GI_TILE + threadIdx.x * GI_ITEMS;
    unsigned sl[GI_ITEMS];
    unsigned keep = 0;
#pragma unroll
    for (int j = 0; j < GI_ITEMS; ++j) {
        int64_t r = row0 + j;
        sl[j] = r < n ? slot_of[r] : 0u;
        if (r < n && t.minrow[sl[j]] == static_cast<unsigned>(r)) keep |= 1u << j;
    }
    unsigned long long c = __popc(keep), tile_count;
    unsigned long long off = block_exclusive_sum<unsigned long long>(c, &tile_count);
    if (threadIdx.x < 32) {
        unsigned long long pre = lookback_publish<4, CountRec>(words, tile, tile_count, 0ull, epoch, st);
        if (threadIdx.x == 0) s_prefix = pre;
    }
    __syncthreads();
    unsigned r = static_cast<unsigned>(s_prefix + off);
#pragma unroll
    for (int j = 0; j < GI_ITEMS; ++j)
        if (keep & (1u << j)) t.id[sl[j]] = r++;
    release_ticket(counters, tiles);
}

__global__ void __launch_bounds__(256) gi_out_kernel(const unsigned *__restrict__ slot_of, int64_t n,
                                                     const unsigned *__restrict__ id, long long *__restrict__ out) {
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = static_cast<long long>(id[__ldcs(slot_of + i)]);
}

static vkc_status run_group(vkc_ctx *ctx, const vkc_array *xa, const vkc_array *xb, vkc_value *out) {
    vkc_status st;
    int64_t n = xa->len;
    if (n >= (int64_t(1) << 31))
        return fail(ctx, VKC_USAGE, "group_id of " + std::to_string(n) + " rows: at most 2^31 - 1 rows per call");
    vkc_array *o;
    if ((st = new_array(ctx, VKC_I64, n, false, &o))) return st;
    if (n == 0) {
        out->kind = VKC_VALUE_ARRAY;
        out->array = o;
        return VKC_OK;
    }
    uint64_t slots = 2;
    while (slots < static_cast<uint64_t>(2 * n)) slots <<= 1;
    // Table and per-row slots, from the device pool (group.rs:128-137 reports a failed
    // table allocation).
    vkc_array *tka = nullptr, *tkb = nullptr, *tst = nullptr, *tmin = nullptr, *tid = nullptr, *rows = nullptr;
    auto cleanup = [&]() {
        for (vkc_array *a : {tka, tkb, tst, tmin, tid, rows})
            if (a) vkc_array_release(a);
    };
    if (new_array(ctx, VKC_U64, static_cast<int64_t>(slots), false, &tka) ||
        (xb && new_array(ctx, VKC_U64, static_cast<int64_t>(slots), false, &tkb)) ||
        new_array(ctx, VKC_I32, static_cast<int64_t>(slots), true, &tst) ||
        new_array(ctx, VKC_I32, static_cast<int64_t>(slots), false, &tmin) ||
        new_array(ctx, VKC_I32, static_cast<int64_t>(slots), false, &tid) ||
        new_array(ctx, VKC_I32, n, false, &rows)) {
        cleanup();
        vkc_array_release(o);
        return fail(ctx, VKC_ALLOC, "cannot allocate a group_id table of " + std::to_string(slots) + " slots for " +
                                        std::to_string(n) + " rows");
    }
    VKC_CUDA(ctx, cudaMemsetAsync(tmin->data(), 0xff, slots * sizeof(unsigned), ctx->stream));
    GroupTable t{static_cast<unsigned long long *>(tka->data()), tkb ? static_cast<unsigned long long *>(tkb->data()) : nullptr,
                 static_cast<unsigned *>(tst->data()), static_cast<unsigned *>(tmin->data()),
                 static_cast<unsigned *>(tid->data()), slots - 1};
    auto *slot_of = static_cast<unsigned *>(rows->data());
    const auto *a = static_cast<const long long *>(xa->data());
    int grid = stream_grid(ctx, n, GI_THREADS, 8, 1024);
    if (xb)
        gi_insert_kernel<true><<<grid, GI_THREADS, 0, ctx->stream>>>(a, static_cast<const long long *>(xb->data()), n, t, slot_of, ctx->status);
    else
        gi_insert_kernel<false><<<grid, GI_THREADS, 0, ctx->stream>>>(a, nullptr, n, t, slot_of, ctx->status);
    if ((st = launched(ctx, "gi_insert"))) {
        cleanup();
        vkc_array_release(o);
        return st;
    }
    int tiles = static_cast<int>((n + GI_TILE - 1) / GI_TILE);
    unsigned long long *recs;
    if ((st = rec_arena(ctx, tiles, &recs))) {
        cleanup();
        vkc_array_release(o);
        return st;
    }
    gi_number_kernel<<<tiles, GI_THREADS, 0, ctx->stream>>>(slot_of, n, t, tiles, recs, next_epoch(ctx), ctx->counters,
                                                           ctx->status);
    if ((st = launched(ctx, "gi_number"))) {
        cleanup();
        vkc_array_release(o);
        return st;
    }
    gi_out_kernel<<<stream_grid(ctx, n, 256, 8, 2048), 256, 0, ctx->stream>>>(slot_of, n, t.id, static_cast<long long *>(o->data()));
    if ((st = launched(ctx, "gi_out"))) {
        cleanup();
        vkc_array_release(o);
        return st;
    }
    DevStatus ds;
    st = read_status(ctx, &ds);
    cleanup();
    if (st) {
        vkc_array_release(o);
        return st;
    }
    out->kind = VKC_VALUE_ARRAY;
    out->array = o;
    return VKC_OK;
}

// group.rs:260-277 (GroupId<i64>).
static vkc_status group_id_i64(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 1) return fail(ctx, VKC_RUNTIME, arity_error(1, nargs));
    if (!array_arg(ctx, args[0], VKC_I64, &st)) return st;
    return run_group(ctx, args[0].array, nullptr, out);
}

// group.rs:280-301 (GroupId2<i64, i64>).
static vkc_status group_id2_i64_i64(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
    if (!array_arg(ctx, args[0], VKC_I64, &st) || !array_arg(ctx, args[1], VKC_I64, &st)) return st;
    if (args[0].array->len != args[1].array->len)
        return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(args[0].array->len) + " vs " +
                                          std::to_string(args[1].array->len));
    return run_group(ctx, args[0].array, args[1].array, out);
}

void register_group(std::vector<KernelDef> &t) {
    // group.rs:305-340: cost = key widths + 8.
    KernelDef d{"group_id_i64", VKC_WHOLE, {InSpec{IN_ARRAY, VKC_I64}}, true, VKC_I64, 16};
    d.whole = group_id_i64;
    t.push_back(d);
    d = KernelDef{"group_id2_i64_i64", VKC_WHOLE, {InSpec{IN_ARRAY, VKC_I64}, InSpec{IN_ARRAY, VKC_I64}}, true,
                  VKC_I64, 24};
    d.whole = group_id2_i64_i64;
    t.push_back(d);
}

}  // namespace vkc

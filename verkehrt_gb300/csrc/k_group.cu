// group_id_i64 and group_id2_i64_i64: dense ids numbered by first occurrence
// (src/kernels/scalar/group.rs:207-301).
//
// The ids depend only on the order in which distinct keys first appear (group.rs:1-5), so any
// correct table gives the reference's output. Three kernels:
//  1. insert: open addressing with linear probing. A free slot holds the key EMPTY (the byte
//     0x80 repeated) and is claimed by a CAS on the key itself (a 128-bit CAS for key pairs),
//     so a probe that reads its key needs no further synchronisation. Slot 0 is never probed:
//     it belongs to the key EMPTY (or the pair (EMPTY, EMPTY)), whose rows go there directly.
//     Each slot keeps the smallest row that holds its key (atomicMin, skipped when the stored
//     row is already smaller), and each row records its slot. A thread probes four rows at once.
//  2. number: a row is a first occurrence when its slot's smallest row is itself; a
//     decoupled-lookback compaction over rows gives each first occurrence its rank, which is
//     the group's id, stored in the slot.
//  3. out: every row reads its slot's id.
// Table size: the reference's maximum is nextpow2(2n) slots (group.rs:226-229). When that is
// above 2^21 slots, the insert first runs on a 2^21-slot table, which stays in L2; it gives up
// (an overflow flag) once 2^20 distinct keys or a probe of 64 slots is reached, and only then
// is the full table filled. Inputs with few distinct keys never touch the large table.
#include "lookback.cuh"
#include "reduce_common.h"

namespace vkc {

constexpr int GI_THREADS = 256;
constexpr int GI_ITEMS = 16;
constexpr int GI_TILE = GI_THREADS * GI_ITEMS;
constexpr int GI_ROWS = 4;  // rows a thread probes at once
constexpr unsigned long long GI_EMPTY = 0x8080808080808080ull;
constexpr uint64_t GI_SMALL_SLOTS = uint64_t(1) << 21;
constexpr unsigned GI_SMALL_PROBES = 64;

struct GroupTable {
    unsigned long long *keys;  // one word per slot (two for key pairs); GI_EMPTY when free
    uint2 *meta;               // per slot: x = smallest row of the key, y = group id
    unsigned long long mask;   // slots - 1
};

// group.rs:40-47 (mix) with a fixed odd multiplier; the ids do not depend on it.
__device__ __forceinline__ unsigned long long gmix(unsigned long long x) {
    return (x ^ (x >> 32)) * 0x9E3779B97F4A7C15ull;
}

__device__ __forceinline__ unsigned long long gi_first(unsigned long long h, unsigned long long mask) {
    const unsigned long long s = (h >> 32 ^ h) & mask;
    return s ? s : 1ull;
}

__device__ __forceinline__ unsigned long long gi_next(unsigned long long s, unsigned long long mask) {
    s = (s + 1) & mask;
    return s ? s : 1ull;
}

__device__ __forceinline__ void ld_relaxed_pair(const unsigned long long *p, unsigned long long &a,
                                                unsigned long long &b) {
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
}

// 128-bit compare-and-swap of the pair at p (16-byte aligned): returns the old pair.
__device__ __forceinline__ void cas_pair(unsigned long long *p, unsigned long long ca, unsigned long long cb,
                                         unsigned long long na, unsigned long long nb, unsigned long long &oa,
                                         unsigned long long &ob) {
    asm volatile(
        "{\n\t.reg .b128 c, v, o;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 v, {%4, %5};\n\t"
        "atom.relaxed.gpu.global.cas.b128 o, [%6], c, v;\n\t"
        "mov.b128 {%0, %1}, o;\n\t}"
        : "=l"(oa), "=l"(ob)
        : "l"(ca), "l"(cb), "l"(na), "l"(nb), "l"(p)
        : "memory");
}

__device__ __forceinline__ unsigned ld_relaxed32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// SMALL: the attempt on the small table, which gives up through flags[1] (flags[0] counts the
// distinct keys inserted). Otherwise the table has room for every key and a probe longer than
// the table only records a timeout.
template <bool PAIR, bool SMALL>
__global__ void __launch_bounds__(GI_THREADS) gi_insert_kernel(const long long *__restrict__ a,
                                                               const long long *__restrict__ b, int64_t n,
                                                               GroupTable t, unsigned *__restrict__ slot_of,
                                                               unsigned *flags, DevStatus *st) {
    const int lane = threadIdx.x & 31;
    const int64_t step = static_cast<int64_t>(gridDim.x) * GI_THREADS * GI_ROWS;
    // The full table always has a free slot, so a probe ends within `mask` steps.
    const unsigned long long limit = SMALL ? GI_SMALL_PROBES : t.mask;
    const unsigned max_keys = static_cast<unsigned>((t.mask + 1) / 2);
    for (int64_t base = static_cast<int64_t>(blockIdx.x) * GI_THREADS * GI_ROWS; base < n; base += step) {
        if (SMALL) {
            unsigned ov = lane == 0 ? ld_relaxed32(flags + 1) : 0u;
            if (__shfl_sync(FULL, ov, 0)) return;  // the whole warp leaves together
        }
        unsigned long long ka[GI_ROWS], kb[GI_ROWS], s[GI_ROWS];
        unsigned pend = 0, in = 0, fresh = 0;
        bool gave_up = false;
#pragma unroll
        for (int j = 0; j < GI_ROWS; ++j) {
            const int64_t r = base + j * GI_THREADS + threadIdx.x;
            ka[j] = kb[j] = GI_EMPTY;
            s[j] = 0;
            if (r < n) {
                in |= 1u << j;
                ka[j] = static_cast<unsigned long long>(__ldcs(a + r));
                if (PAIR) kb[j] = static_cast<unsigned long long>(__ldcs(b + r));
                if (ka[j] != GI_EMPTY || (PAIR && kb[j] != GI_EMPTY)) {
                    s[j] = gi_first(PAIR ? gmix(gmix(ka[j]) ^ kb[j]) : gmix(ka[j]), t.mask);
                    pend |= 1u << j;
                }
            }
        }
        unsigned long long probes = 0;
        while (pend) {
            unsigned long long va[GI_ROWS], vb[GI_ROWS];
#pragma unroll
            for (int j = 0; j < GI_ROWS; ++j) {
                va[j] = vb[j] = 0;
                if (pend & (1u << j)) {
                    if (PAIR) ld_relaxed_pair(t.keys + 2 * s[j], va[j], vb[j]);
                    else va[j] = ld_relaxed64(t.keys + s[j]);
                }
            }
#pragma unroll
            for (int j = 0; j < GI_ROWS; ++j) {
                if (!(pend & (1u << j))) continue;
                bool done = false;
                if (!PAIR) {
                    if (va[j] == ka[j]) {
                        done = true;
                    } else if (va[j] == GI_EMPTY) {
                        const unsigned long long old = atomicCAS(t.keys + s[j], GI_EMPTY, ka[j]);
                        if (old == GI_EMPTY) ++fresh;
                        done = old == GI_EMPTY || old == ka[j];
                    }
                } else if (va[j] != GI_EMPTY && vb[j] != GI_EMPTY) {
                    // A slot is written once, from (EMPTY, EMPTY): a pair with no EMPTY half is whole.
                    done = va[j] == ka[j] && vb[j] == kb[j];
                } else {
                    unsigned long long oa, ob;
                    cas_pair(t.keys + 2 * s[j], GI_EMPTY, GI_EMPTY, ka[j], kb[j], oa, ob);
                    if (oa == GI_EMPTY && ob == GI_EMPTY) ++fresh;
                    done = (oa == GI_EMPTY && ob == GI_EMPTY) || (oa == ka[j] && ob == kb[j]);
                }
                if (done) pend &= ~(1u << j);
                else s[j] = gi_next(s[j], t.mask);
            }
            if (pend && ++probes > limit) {
                gave_up = true;
                break;
            }
        }
        if (gave_up) {
            if (SMALL) atomicExch(flags + 1, 1u);
            else set_timeout(st);
        }
        if (SMALL) {
            const unsigned c = __reduce_add_sync(FULL, fresh);
            if (lane == 0 && c && atomicAdd(flags, c) + c > max_keys) atomicExch(flags + 1, 1u);
        }
        if (gave_up) continue;
#pragma unroll
        for (int j = 0; j < GI_ROWS; ++j) {
            if (!(in & (1u << j))) continue;
            const unsigned row = static_cast<unsigned>(base + j * GI_THREADS + threadIdx.x);
            unsigned *m = &t.meta[s[j]].x;
            if (ld_relaxed32(m) > row) atomicMin(m, row);
            slot_of[row] = static_cast<unsigned>(s[j]);
        }
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
    if (row0 + GI_ITEMS <= n) {
        const uint4 *v = reinterpret_cast<const uint4 *>(slot_of + row0);
#pragma unroll
        for (int q = 0; q < GI_ITEMS / 4; ++q) {
            const uint4 w = __ldcs(v + q);
            sl[4 * q] = w.x;
            sl[4 * q + 1] = w.y;
            sl[4 * q + 2] = w.z;
            sl[4 * q + 3] = w.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < GI_ITEMS; ++j) sl[j] = row0 + j < n ? slot_of[row0 + j] : 0u;
    }
    unsigned keep = 0;
#pragma unroll
    for (int j = 0; j < GI_ITEMS; ++j) {
        const int64_t r = row0 + j;
        if (r < n && t.meta[sl[j]].x == static_cast<unsigned>(r)) keep |= 1u << j;
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
        if (keep & (1u << j)) t.meta[sl[j]].y = r++;
    release_ticket(counters, tiles);
}

// Four rows per thread: one 16-byte load of their slots, four id loads, two 16-byte stores.
__global__ void __launch_bounds__(256) gi_out_kernel(const unsigned *__restrict__ slot_of, int64_t n,
                                                     const uint2 *__restrict__ meta, long long *__restrict__ out) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x * 4;
    for (int64_t i = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) * 4; i < n; i += stride) {
        if (i + 4 <= n) {
            const uint4 sl = __ldcs(reinterpret_cast<const uint4 *>(slot_of + i));
            const longlong2 lo = make_longlong2(meta[sl.x].y, meta[sl.y].y);
            const longlong2 hi = make_longlong2(meta[sl.z].y, meta[sl.w].y);
            __stcs(reinterpret_cast<longlong2 *>(out + i), lo);
            __stcs(reinterpret_cast<longlong2 *>(out + i) + 1, hi);
        } else {
            for (int64_t r = i; r < n; ++r) out[r] = static_cast<long long>(meta[slot_of[r]].y);
        }
    }
}

struct GroupScratch {
    vkc_array *keys = nullptr, *meta = nullptr;
    void release() {
        if (keys) vkc_array_release(keys);
        if (meta) vkc_array_release(meta);
        keys = meta = nullptr;
    }
};

// A table of `slots` slots (slot 0 included), every slot free.
static vkc_status new_table(vkc_ctx *ctx, uint64_t slots, bool pair, GroupScratch *g, GroupTable *t) {
    const int64_t words = static_cast<int64_t>(pair ? 2 * slots : slots);
    if (new_array(ctx, VKC_U64, words, false, &g->keys) ||
        new_array(ctx, VKC_U64, static_cast<int64_t>(slots), false, &g->meta)) {
        g->release();
        return VKC_ALLOC;
    }
    VKC_CUDA(ctx, cudaMemsetAsync(g->keys->data(), 0x80, static_cast<size_t>(words) * 8, ctx->stream));
    VKC_CUDA(ctx, cudaMemsetAsync(g->meta->data(), 0xff, static_cast<size_t>(slots) * 8, ctx->stream));
    *t = GroupTable{static_cast<unsigned long long *>(g->keys->data()), static_cast<uint2 *>(g->meta->data()),
                    slots - 1};
    return VKC_OK;
}

template <bool PAIR>
static void launch_insert(vkc_ctx *ctx, bool small, const long long *a, const long long *b, int64_t n,
                          const GroupTable &t, unsigned *slot_of, unsigned *flags) {
    const int grid = stream_grid(ctx, n, GI_THREADS, 8, GI_THREADS * GI_ROWS);
    if (small)
        gi_insert_kernel<PAIR, true><<<grid, GI_THREADS, 0, ctx->stream>>>(a, b, n, t, slot_of, flags, ctx->status);
    else
        gi_insert_kernel<PAIR, false><<<grid, GI_THREADS, 0, ctx->stream>>>(a, b, n, t, slot_of, flags, ctx->status);
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
    GroupScratch small, full;
    vkc_array *rows = nullptr, *flag_arr = nullptr;
    auto cleanup = [&]() {
        small.release();
        full.release();
        if (rows) vkc_array_release(rows);
        if (flag_arr) vkc_array_release(flag_arr);
    };
    auto alloc_fail = [&]() {
        cleanup();
        vkc_array_release(o);
        // group.rs:128-137 reports a failed table allocation.
        return fail(ctx, VKC_ALLOC, "cannot allocate a group_id table of " + std::to_string(slots) + " slots for " +
                                        std::to_string(n) + " rows");
    };
    if (new_array(ctx, VKC_I32, n, false, &rows) || new_array(ctx, VKC_I32, 2, true, &flag_arr)) return alloc_fail();
    auto *slot_of = static_cast<unsigned *>(rows->data());
    auto *flags = static_cast<unsigned *>(flag_arr->data());
    const auto *a = static_cast<const long long *>(xa->data());
    const auto *b = xb ? static_cast<const long long *>(xb->data()) : nullptr;
    GroupTable t{};
    bool done = false;
    if (slots > GI_SMALL_SLOTS) {
        if (new_table(ctx, GI_SMALL_SLOTS, xb != nullptr, &small, &t)) return alloc_fail();
        if (xb) launch_insert<true>(ctx, true, a, b, n, t, slot_of, flags);
        else launch_insert<false>(ctx, true, a, b, n, t, slot_of, flags);
        if ((st = launched(ctx, "gi_insert"))) {
            cleanup();
            vkc_array_release(o);
            return st;
        }
        void *h;
        if ((st = pinned(ctx, 16, &h))) {
            cleanup();
            vkc_array_release(o);
            return st;
        }
        VKC_CUDA(ctx, cudaMemcpyAsync(h, flags, 8, cudaMemcpyDeviceToHost, ctx->stream));
        VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        done = static_cast<unsigned *>(h)[1] == 0;
        if (!done) small.release();
    }
    if (!done) {
        if (new_table(ctx, slots, xb != nullptr, &full, &t)) return alloc_fail();
        if (xb) launch_insert<true>(ctx, false, a, b, n, t, slot_of, flags);
        else launch_insert<false>(ctx, false, a, b, n, t, slot_of, flags);
        if ((st = launched(ctx, "gi_insert"))) {
            cleanup();
            vkc_array_release(o);
            return st;
        }
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
    gi_out_kernel<<<stream_grid(ctx, n, 256, 8, 1024), 256, 0, ctx->stream>>>(slot_of, n, t.meta,
                                                                               static_cast<long long *>(o->data()));
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

// Selections: filter_<cmp>_f64, compress_T and where (src/kernels/scalar/select.rs:81-104,
// src/kernels/scalar/fused.rs:225-236).
//
// One persistent pass (tilepass.cuh): each tile is copied into shared memory by TMA, its
// survivor count goes to the decoupled lookback, its survivors are compacted in place while
// the lookback runs, and then written out at the tile's offset. The output is the rows in
// input order, so it does not depend on the tiling (select.rs:36-57 writes the same rows).
#include "reduce_common.h"
#include "tilepass.cuh"

namespace vkc {

constexpr int SEL_THREADS = 512;                           // compute threads (+ 2 warps)
constexpr int SEL_TILE = 8192;                             // rows per tile
constexpr int SEL_SLICE = SEL_TILE / (SEL_THREADS / 32);   // rows per compute warp
constexpr int SEL_WINDOW = 4;                              // lookback: 32 * 4 tiles per step
constexpr int SEL_SLOTS = 3;                               // tile ring: 1 copy in flight
// (Filter tiles of 6144 rows in four slots, two copies in flight, were slower at 2^28: 0.56
// against 0.46 ms at 1% kept; a third more tiles meet the lookback rate.)
constexpr int SEL_BLOCKS = 1;                              // blocks per SM

enum SelKind { SEL_FILTER = 0, SEL_COMPRESS = 1, SEL_WHERE = 2 };

template <int W> struct Word;
template <> struct Word<8> { using T = unsigned long long; };
template <> struct Word<4> { using T = unsigned; };
template <> struct Word<1> { using T = unsigned char; };

struct SelArgs {
    const void *x;          // values (filter, compress)
    const unsigned char *m; // mask (compress, where)
    CmpRange r;             // filter predicate
    int64_t n;
    int64_t base;           // where: global row of row 0
    void *out;
    unsigned long long *total;  // survivor count of the launch
    bool aligned;           // values and mask start on 16-byte boundaries: whole tiles go by TMA
};

// Nonzero bytes of a 32-bit word.
__device__ __forceinline__ unsigned nonzero_bytes(unsigned v) {
    const unsigned t = ~(((v & 0x7f7f7f7fu) + 0x7f7f7f7fu) | v | 0x7f7f7f7fu);  // 0x80 per zero byte
    return 4u - __popc(t);
}

// A selection as a tile pass. A slot holds the tile's values (filter, compress) and mask
// (compress, where); the survivors are compacted into the values in place, or for `where`
// (8-byte row numbers from 1-byte mask rows) into an output area after the mask. A compute
// warp's slice is SEL_SLICE consecutive rows, read in steps of VV rows per lane (16 bytes of
// values, or of mask for `where`), ranked with ballots, and copied out with consecutive lanes
// on consecutive rows. A filter's count keeps its ballots in the slot, so the stage touches
// only the steps and rows that survive. A tile that is not whole, or not 16-byte aligned, is
// read from global memory instead of the slot.
template <int KIND, int W, bool POS = false> struct SelectPass {
    static constexpr int THREADS = SEL_THREADS;
    using R = CountRec;
    using V = unsigned long long;
    using T = typename Word<W>::T;
    using O = typename Word<KIND == SEL_WHERE ? 8 : W>::T;
    static constexpr int VAL_BYTES = KIND == SEL_WHERE ? 0 : W * SEL_TILE;
    static constexpr int MASK_BYTES = KIND == SEL_FILTER ? 0 : SEL_TILE;
    static constexpr int OUT_BYTES = KIND == SEL_WHERE ? 8 * SEL_TILE : 0;
    static constexpr int VK = KIND == SEL_FILTER ? 2 : 16;  // keys per lane per count step
    static constexpr int SK = SEL_SLICE / (32 * VK);
    static constexpr int BALLOT_BYTES = KIND == SEL_FILTER ? (SEL_THREADS / 32) * SK * 8 : 0;
    static constexpr int SLOT_BYTES = VAL_BYTES + MASK_BYTES + OUT_BYTES + BALLOT_BYTES;
    static constexpr int SLOTS = SEL_SLOTS;
    static constexpr int VV = KIND == SEL_WHERE ? 16 : 16 / W;  // rows per lane per stage step
    static constexpr int SV = SEL_SLICE / (32 * VV);
    static_assert(SK >= 1 && SV >= 1, "a slice holds whole steps");
    static_assert(KIND != SEL_FILTER || SK <= 32, "one lane stores each step's ballots");
    using Staged = unsigned;  // survivors compacted in the warp's slice

    SelArgs a;

    __device__ bool whole(int tile) const {
        return a.aligned && static_cast<int64_t>(tile + 1) * SEL_TILE <= a.n;
    }
    __device__ unsigned bulk_bytes(int tile) const { return whole(tile) ? VAL_BYTES + MASK_BYTES : 0u; }
    __device__ void load(int tile, unsigned char *slot, unsigned long long *bar) const {
        const int64_t r0 = static_cast<int64_t>(tile) * SEL_TILE;
        if (VAL_BYTES) bulk_load(slot, static_cast<const T *>(a.x) + r0, VAL_BYTES, bar);
        if (MASK_BYTES) bulk_load(slot + VAL_BYTES, a.m + r0, MASK_BYTES, bar);
    }
    __device__ bool keep_filter(unsigned long long v) const { return in_range_t<POS>(a.r, v); }

    // The slice's keys from `keys` (the slot, or global memory at the tile's first row).
    template <class K> __device__ unsigned count_keys(const K *keys, int64_t r0) const {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const int j = w * SEL_SLICE + lane * VK;  // row in the tile
        unsigned c = 0;
        if (KIND == SEL_FILTER) {
            ulonglong2 u[SK];
#pragma unroll
            for (int s = 0; s < SK; ++s) u[s] = *reinterpret_cast<const ulonglong2 *>(keys + j + s * 64);
#pragma unroll
            for (int s = 0; s < SK; ++s) c += keep_filter(u[s].x) + keep_filter(u[s].y);
        } else {
#pragma unroll
            for (int s = 0; s < SK; ++s) {
                const uint4 u = *reinterpret_cast<const uint4 *>(keys + j + s * 512);
                c += nonzero_bytes(u.x) + nonzero_bytes(u.y) + nonzero_bytes(u.z) + nonzero_bytes(u.w);
            }
        }
        return c;
    }

    // The filter's ballots of the warp's slice: step s, element e in [s].(x, y).
    __device__ uint2 *ballots(unsigned char *slot) const {
        return reinterpret_cast<uint2 *>(slot + VAL_BYTES + MASK_BYTES + OUT_BYTES) + (threadIdx.x >> 5) * SK;
    }

    __device__ V count(int tile, unsigned char *slot) const {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const int64_t r0 = static_cast<int64_t>(tile) * SEL_TILE;
        unsigned c = 0;
        if (KIND == SEL_FILTER && whole(tile)) {
            const auto *k = reinterpret_cast<const unsigned long long *>(slot) + w * SEL_SLICE + lane * 2;
            uint2 *mb = ballots(slot);
            ulonglong2 u[SK];
#pragma unroll
            for (int s = 0; s < SK; ++s) u[s] = *reinterpret_cast<const ulonglong2 *>(k + s * 64);
#pragma unroll
            for (int s = 0; s < SK; ++s) {
                const unsigned m0 = __ballot_sync(FULL, keep_filter(u[s].x));
                const unsigned m1 = __ballot_sync(FULL, keep_filter(u[s].y));
                if (lane == s) mb[s] = make_uint2(m0, m1);
                c += __popc(m0) + __popc(m1);
            }
            return c;
        }
        if (whole(tile)) {
            c = KIND == SEL_FILTER ? count_keys(reinterpret_cast<const unsigned long long *>(slot), r0)
                                   : count_keys(slot + VAL_BYTES, r0);
        } else {
            // Row by row from global memory.
            for (int i = lane; i < SEL_SLICE; i += 32) {
                const int64_t r = r0 + w * SEL_SLICE + i;
                if (r >= a.n) break;
                if (KIND == SEL_FILTER) c += keep_filter(static_cast<const unsigned long long *>(a.x)[r]);
                else c += a.m[r] != 0;
            }
        }
        return warp_sum(c);
    }

    __device__ unsigned stage(int tile, unsigned char *slot) const {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const unsigned lt = (1u << lane) - 1;
        const int64_t r0 = static_cast<int64_t>(tile) * SEL_TILE;
        const bool sm = whole(tile);
        if (KIND == SEL_FILTER && sm) {
            // From the count's ballots: steps with no survivor are skipped, and a lane reads
            // its two rows only when one survives.
            unsigned long long *st = reinterpret_cast<unsigned long long *>(slot) + w * SEL_SLICE;
            const uint2 *mb = ballots(slot);
            unsigned total = 0;
            __syncwarp();
#pragma unroll 4
            for (int s = 0; s < SK; ++s) {
                const uint2 m = mb[s];
                if ((m.x | m.y) == 0) continue;
                const unsigned b = ((m.x >> lane) & 1u) | (((m.y >> lane) & 1u) << 1);
                ulonglong2 u = make_ulonglong2(0, 0);
                if (b) u = *reinterpret_cast<const ulonglong2 *>(st + s * 64 + lane * 2);
                unsigned q = total + __popc(m.x & lt) + __popc(m.y & lt);
                __syncwarp();  // the step is read before any of it is overwritten
                if (b & 1u) st[q++] = u.x;
                if (b & 2u) st[q] = u.y;
                total += __popc(m.x) + __popc(m.y);
            }
            return total;
        }
        O *st = reinterpret_cast<O *>(slot + VAL_BYTES + MASK_BYTES) + w * SEL_SLICE;  // where
        if (KIND != SEL_WHERE) st = reinterpret_cast<O *>(slot) + w * SEL_SLICE;          // in place
        unsigned total = 0;
#pragma unroll 2
        for (int s = 0; s < SV; ++s) {
            const int j = w * SEL_SLICE + s * (32 * VV) + lane * VV;  // row in the tile
            const int64_t i0 = r0 + j;
            T v[KIND == SEL_WHERE ? 1 : VV];
            unsigned bits = 0;
            if (sm) {
                if (KIND != SEL_WHERE) {
                    const uint4 u = *reinterpret_cast<const uint4 *>(reinterpret_cast<const T *>(slot) + j);
                    const T *e = reinterpret_cast<const T *>(&u);
#pragma unroll
                    for (int k = 0; k < VV; ++k) v[k] = e[k];
                }
                if (KIND != SEL_FILTER) {
                    const unsigned char *m = slot + VAL_BYTES + j;
                    if (VV == 16) {
                        const uint4 u = *reinterpret_cast<const uint4 *>(m);
                        const unsigned wd[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                        for (int k = 0; k < 16; ++k)
                            if ((wd[k >> 2] >> (8 * (k & 3))) & 0xffu) bits |= 1u << k;
                    } else {
                        const unsigned wd = VV == 4 ? *reinterpret_cast<const unsigned *>(m)
                                                    : *reinterpret_cast<const unsigned short *>(m);
#pragma unroll
                        for (int k = 0; k < VV; ++k)
                            if ((wd >> (8 * k)) & 0xffu) bits |= 1u << k;
                    }
                }
            } else {
#pragma unroll
                for (int k = 0; k < VV; ++k) {
                    const bool in = i0 + k < a.n;
                    if (KIND != SEL_WHERE) v[k] = in ? static_cast<const T *>(a.x)[i0 + k] : T(0);
                    if (KIND != SEL_FILTER && in && a.m[i0 + k]) bits |= 1u << k;
                }
            }
            if (KIND == SEL_FILTER) {
#pragma unroll
                for (int k = 0; k < VV; ++k)
                    if ((sm || i0 + k < a.n) && keep_filter(static_cast<unsigned long long>(v[k]))) bits |= 1u << k;
            }
            // In-order ranks: the lanes before this one, element by element.
            unsigned before = 0, step_total = 0;
#pragma unroll
            for (int k = 0; k < VV; ++k) {
                const unsigned m = __ballot_sync(FULL, (bits >> k) & 1u);
                before += __popc(m & lt);
                step_total += __popc(m);
            }
            __syncwarp();  // the step is read before any of it is overwritten
            unsigned q = total + before;
#pragma unroll
            for (int k = 0; k < VV; ++k)
                if ((bits >> k) & 1u) {
                    if (KIND == SEL_WHERE) st[q] = static_cast<O>(a.base + i0 + k);
                    else st[q] = static_cast<O>(v[KIND == SEL_WHERE ? 0 : k]);
                    ++q;
                }
            total += step_total;
        }
        return total;
    }

    __device__ void flush(int, V pre, unsigned total, unsigned char *slot) const {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const O *st = KIND == SEL_WHERE ? reinterpret_cast<const O *>(slot + VAL_BYTES + MASK_BYTES) + w * SEL_SLICE
                                        : reinterpret_cast<const O *>(slot) + w * SEL_SLICE;
        __syncwarp();
        O *out = static_cast<O *>(a.out) + pre;
        unsigned i0 = 0;
        if (sizeof(O) == 8) {
            // Pairs of rows as aligned 16-byte stores, after a single row when the output does
            // not start on a 16-byte boundary.
            const unsigned mis = (reinterpret_cast<uintptr_t>(out) & 15) ? 1u : 0u;
            const unsigned head = mis < total ? mis : total;
            if (head && lane == 0) out[0] = st[0];
            const unsigned pairs = (total - head) >> 1;
            for (unsigned i = lane; i < pairs; i += 32) {
                ulonglong2 u;
                u.x = static_cast<unsigned long long>(st[head + 2 * i]);
                u.y = static_cast<unsigned long long>(st[head + 2 * i + 1]);
                *reinterpret_cast<ulonglong2 *>(out + head + 2 * i) = u;
            }
            i0 = head + 2 * pairs;
        }
        for (unsigned i = i0 + lane; i < total; i += 32) out[i] = st[i];
    }

    __device__ void last_tile(V inclusive) const { *a.total = inclusive; }
};

template <int KIND, int W, bool POS>
__global__ void __launch_bounds__(SEL_THREADS + 64, SEL_BLOCKS) select_kernel(SelArgs a, int tiles, unsigned long long *recs,
                                                                     unsigned epoch, unsigned *counters,
                                                                     DevStatus *status) {
    SelectPass<KIND, W, POS> p{a};
    tile_pass<SEL_WINDOW>(p, recs, tiles, epoch, counters, status, 0ull);
}

template <int KIND, int W>
static vkc_status run_select(vkc_ctx *ctx, SelArgs a, int64_t n, Builder *b) {
    if (n >= (int64_t(1) << 38)) return fail(ctx, VKC_USAGE, "selection of 2^38 rows or more");
    const int64_t tiles64 = (n + SEL_TILE - 1) / SEL_TILE;
    const int tiles = static_cast<int>(tiles64);
    void *p;
    unsigned long long *recs;
    vkc_status st;
    if ((st = scratch(ctx, 256, &p))) return st;
    if ((st = rec_arena(ctx, tiles, &recs))) return st;
    a.total = static_cast<unsigned long long *>(p);
    void *at;
    if ((st = b->reserve(n, &at))) return st;
    a.out = at;
    const unsigned epoch = next_epoch(ctx);
    a.aligned = (reinterpret_cast<uintptr_t>(a.x) & 15) == 0 && (reinterpret_cast<uintptr_t>(a.m) & 15) == 0;
    constexpr size_t smem = SEL_SLOTS * SelectPass<KIND, W>::SLOT_BYTES;
    static std::atomic<unsigned long long> configured{0};
    once_per_device(configured, ctx->device, [] {
        cudaFuncSetAttribute(select_kernel<KIND, W, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if constexpr (KIND == SEL_FILTER)
            cudaFuncSetAttribute(select_kernel<KIND, W, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    });
    bool launched_pos = false;
    if constexpr (KIND == SEL_FILTER) {
        if (pos_range(a.r)) {
            const int grid = tile_pass_grid(ctx, select_kernel<KIND, W, true>, SEL_THREADS + 64, smem, tiles);
            select_kernel<KIND, W, true><<<grid, SEL_THREADS + 64, smem, ctx->stream>>>(a, tiles, recs, epoch, ctx->counters, ctx->status);
            launched_pos = true;
        }
    }
    if (!launched_pos) {
        const int grid = tile_pass_grid(ctx, select_kernel<KIND, W, false>, SEL_THREADS + 64, smem, tiles);
        select_kernel<KIND, W, false><<<grid, SEL_THREADS + 64, smem, ctx->stream>>>(a, tiles, recs, epoch, ctx->counters, ctx->status);
    }
    if ((st = launched(ctx, "select"))) return st;
    DevStatus ds;
    if ((st = read_status(ctx, &ds))) return st;
    void *h;
    if ((st = pinned(ctx, 8, &h))) return st;
    VKC_CUDA(ctx, cudaMemcpyAsync(h, a.total, 8, cudaMemcpyDeviceToHost, ctx->stream));
    VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const unsigned long long k = *static_cast<unsigned long long *>(h);
    // The count can only be at most the rows reserved; anything else is a broken launch.
    if (k > static_cast<unsigned long long>(n))
        return fail(ctx, VKC_DEVICE, "selection returned " + std::to_string(k) + " rows for " +
                                         std::to_string(n) + " input rows");
    b->len += static_cast<int64_t>(k);
    return VKC_OK;
}

// fused.rs:214-223 (filter_args) and :225-236.
template <int C> static vkc_status filter_f64(vkc_ctx *ctx, const Arg *args, int nargs, int64_t, Builder *b) {
    vkc_status st;
    if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
    if (!rows_arg(ctx, args[0], VKC_F64, &st) || !splat_arg(ctx, args[1], VKC_F64, &st)) return st;
    int64_t n = args[0].len();
    if (n == 0) return VKC_OK;
    SelArgs a{};
    a.x = args[0].a->data();
    a.r = cmp_range(C, args[1].f64());
    a.n = n;
    return run_select<SEL_FILTER, 8>(ctx, a, n, b);
}

// select.rs:163-186 (compress_args): kinds, then equal row counts.
template <vkc_type T> static vkc_status compress(vkc_ctx *ctx, const Arg *args, int nargs, int64_t, Builder *b) {
    vkc_status st;
    if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
    if (!rows_arg(ctx, args[0], T, &st) || !rows_arg(ctx, args[1], VKC_BOOL, &st)) return st;
    int64_t n = args[0].len();
    if (n != args[1].len())
        return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(n) + " values vs " +
                                          std::to_string(args[1].len()) + " mask rows");
    if (n == 0) return VKC_OK;
    SelArgs a{};
    a.x = args[0].a->data();
    a.m = static_cast<const unsigned char *>(args[1].a->data());
    a.n = n;
    switch (type_width(T)) {
    case 8: return run_select<SEL_COMPRESS, 8>(ctx, a, n, b);
    case 4: return run_select<SEL_COMPRESS, 4>(ctx, a, n, b);
    default: return run_select<SEL_COMPRESS, 1>(ctx, a, n, b);
    }
}

// select.rs:98-125 (where_append, check_row_indices): global rows base + i.
static vkc_status where_sel(vkc_ctx *ctx, const Arg *args, int nargs, int64_t base, Builder *b) {
    vkc_status st;
    if (nargs != 1) return fail(ctx, VKC_RUNTIME, arity_error(1, nargs));
    if (!rows_arg(ctx, args[0], VKC_BOOL, &st)) return st;
    int64_t n = args[0].len();
    if (base < 0 || n > INT64_MAX - base) return fail(ctx, VKC_RUNTIME, "row index fits in i64");
    if (n == 0) return VKC_OK;
    SelArgs a{};
    a.m = static_cast<const unsigned char *>(args[0].a->data());
    a.n = n;
    a.base = base;
    return run_select<SEL_WHERE, 1>(ctx, a, n, b);
}

void register_select(std::vector<KernelDef> &t) {
    static const char *names[6] = {"eq", "ne", "lt", "le", "gt", "ge"};
    SelectFn filters[6] = {filter_f64<0>, filter_f64<1>, filter_f64<2>,
                           filter_f64<3>, filter_f64<4>, filter_f64<5>};
    InSpec xa{IN_ARRAY, VKC_F64}, xs{IN_SCALAR, VKC_F64};
    for (int c = 0; c < 6; ++c) {
        // fused.rs:307-318: cost 2 widths.
        KernelDef d{std::string("filter_") + names[c] + "_f64", VKC_SELECTION, {xa, xs}, true, VKC_F64, 16};
        d.sel = filters[c];
        t.push_back(d);
    }
    struct C { vkc_type t; SelectFn f; };
    const C comp[] = {{VKC_F64, compress<VKC_F64>}, {VKC_F32, compress<VKC_F32>},
                      {VKC_I64, compress<VKC_I64>}, {VKC_U64, compress<VKC_U64>},
                      {VKC_I32, compress<VKC_I32>}, {VKC_U8, compress<VKC_U8>},
                      {VKC_BOOL, compress<VKC_BOOL>}};
    for (const C &c : comp) {
        // select.rs:190-210: cost 2 widths + 1.
        KernelDef d{std::string("compress_") + type_name(c.t), VKC_SELECTION,
                    {InSpec{IN_ARRAY, c.t}, InSpec{IN_ARRAY, VKC_BOOL}}, true, c.t,
                    static_cast<uint64_t>(2 * type_width(c.t) + 1)};
        d.sel = c.f;
        t.push_back(d);
    }
    KernelDef d{"where", VKC_SELECTION, {InSpec{IN_ARRAY, VKC_BOOL}}, true, VKC_I64, 9};
    d.sel = where_sel;
    t.push_back(d);
}

}  // namespace vkc

// Selections: filter_<cmp>_f64, compress_T and where (src/kernels/scalar/select.rs:81-104,
// src/kernels/scalar/fused.rs:225-236).
//
// One pass: each 8192-row tile computes its keep flags, the tile's survivor count goes through
// a decoupled lookback for the tile's output offset, and the survivors are compacted in shared
// memory and written out contiguously. The output is the rows in input order, so it does not
// depend on the tiling (select.rs:36-57 writes the same rows).
#include "lookback.cuh"
#include "reduce_common.h"

namespace vkc {

constexpr int SEL_THREADS = 512;
constexpr int SEL_ITEMS = 16;
constexpr int SEL_TILE = SEL_THREADS * SEL_ITEMS;

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
};

// Per thread, ITEMS items in ROWS rows of the warp's 512-item slice: in row r the warp reads
// 32 * VEC consecutive items, VEC per lane (one 16-byte load), so every load is coalesced and
// item order is (row, lane, element).
template <int W> struct SelShape {
    static constexpr int VEC = 16 / W;
    static constexpr int ROWS = SEL_ITEMS / VEC;
};

template <int KIND, int W, bool ALIGNED>
__global__ void __launch_bounds__(SEL_THREADS) select_kernel(SelArgs a, int tiles, unsigned long long *words,
                                                             unsigned epoch, unsigned *counters,
                                                             DevStatus *status) {
    using T = typename Word<W>::T;
    using O = typename Word<KIND == SEL_WHERE ? 8 : W>::T;
    constexpr int VEC = SelShape<W>::VEC, ROWS = SelShape<W>::ROWS;
    constexpr int SLICE = 32 * SEL_ITEMS;  // rows of one warp
    // Each warp compacts its survivors into its own slice of shared memory row by row, so no
    // row value waits in registers while the block waits for its offset.
    extern __shared__ __align__(16) unsigned char sel_smem[];
    __shared__ unsigned s_warp[SEL_THREADS / 32];
    __shared__ unsigned long long s_prefix, s_count;
    const int tile = take_ticket(counters);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    O *s_out = reinterpret_cast<O *>(sel_smem) + w * SLICE;
    const unsigned lt = (1u << lane) - 1;
    const int64_t wbase = static_cast<int64_t>(tile) * SEL_TILE + static_cast<int64_t>(w) * SLICE;

    // Every row's load is issued before any is used: the loads of a thread are all in flight.
    T vv[ROWS][VEC];
    if (KIND != SEL_WHERE) {
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            const int64_t i0 = wbase + r * (32 * VEC) + lane * VEC;
            if (ALIGNED && i0 + VEC <= a.n) {
                uint4 u = __ldcs(reinterpret_cast<const uint4 *>(static_cast<const T *>(a.x) + i0));
                const T *e = reinterpret_cast<const T *>(&u);
#pragma unroll
                for (int k = 0; k < VEC; ++k) vv[r][k] = e[k];
            } else {
#pragma unroll
                for (int k = 0; k < VEC; ++k) vv[r][k] = i0 + k < a.n ? static_cast<const T *>(a.x)[i0 + k] : T(0);
            }
        }
    }
    unsigned total = 0;
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
        const int64_t i0 = wbase + r * (32 * VEC) + lane * VEC;
        T v[VEC];
#pragma unroll
        for (int k = 0; k < VEC; ++k) v[k] = KIND != SEL_WHERE ? vv[r][k] : T(0);
        unsigned bits = 0;
        if (KIND == SEL_FILTER) {
#pragma unroll
            for (int k = 0; k < VEC; ++k)
                if (i0 + k < a.n && in_range(a.r, static_cast<unsigned long long>(v[k]))) bits |= 1u << k;
        } else if (ALIGNED && VEC == 16 && i0 + 16 <= a.n) {
            uint4 u = __ldcs(reinterpret_cast<const uint4 *>(a.m + i0));
            unsigned wd[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int k = 0; k < 16; ++k)
                if ((wd[k >> 2] >> (8 * (k & 3))) & 0xffu) bits |= 1u << k;
        } else {
#pragma unroll
            for (int k = 0; k < VEC; ++k)
                if (i0 + k < a.n && a.m[i0 + k]) bits |= 1u << k;
        }
        // In-order ranks: the lanes before this one, element by element.
        unsigned before = 0, row_total = 0;
#pragma unroll
        for (int k = 0; k < VEC; ++k) {
            unsigned m = __ballot_sync(FULL, (bits >> k) & 1u);
            before += __popc(m & lt);
            row_total += __popc(m);
        }
        unsigned p = total + before;
#pragma unroll
        for (int k = 0; k < VEC; ++k)
            if ((bits >> k) & 1u) {
                s_out[p] = KIND == SEL_WHERE ? static_cast<O>(a.base + i0 + k) : static_cast<O>(v[k]);
                ++p;
            }
        total += row_total;
    }
    if (lane == 0) s_warp[w] = total;
    __syncthreads();
    if (w == 0) {
        unsigned c = lane < SEL_THREADS / 32 ? s_warp[lane] : 0u, x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        const unsigned long long tile_count = __shfl_sync(FULL, x, SEL_THREADS / 32 - 1);
        unsigned long long pre = warp_lookback_count<4>(words, tile, tile_count, epoch, status);
        if (lane < SEL_THREADS / 32) s_warp[lane] = x - c;  // exclusive over warps
        if (lane == 0) {
            s_prefix = pre;
            s_count = tile_count;
            if (tile == tiles - 1) *a.total = pre + tile_count;
        }
    }
    __syncthreads();
    // Each warp writes its slice's survivors after those of the warps before it.
    O *out = static_cast<O *>(a.out) + s_prefix + s_warp[w];
    for (unsigned i = lane; i < total; i += 32) out[i] = s_out[i];
    release_ticket(counters, tiles);
}

template <int KIND, int W>
static vkc_status run_select(vkc_ctx *ctx, SelArgs a, int64_t n, Builder *b) {
    int64_t tiles64 = (n + SEL_TILE - 1) / SEL_TILE;
    int tiles = static_cast<int>(tiles64);
    void *p;
    unsigned *flags;
    vkc_status st;
    if ((st = scratch(ctx, 256, &p))) return st;
    if ((st = flag_arena(ctx, 2 * static_cast<size_t>(tiles), &flags))) return st;
    auto *words = reinterpret_cast<unsigned long long *>(flags);
    a.total = static_cast<unsigned long long *>(p);
    void *at;
    if ((st = b->reserve(n, &at))) return st;
    a.out = at;
    unsigned epoch = next_epoch(ctx);
    bool aligned = (reinterpret_cast<uintptr_t>(a.x) & 15) == 0 &&
                   (reinterpret_cast<uintptr_t>(a.m) & 15) == 0;
    using O = typename Word<KIND == SEL_WHERE ? 8 : W>::T;
    const size_t smem = sizeof(O) * SEL_TILE;
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(select_kernel<KIND, W, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        cudaFuncSetAttribute(select_kernel<KIND, W, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        configured = true;
    }
    if (aligned)
        select_kernel<KIND, W, true><<<tiles, SEL_THREADS, smem, ctx->stream>>>(a, tiles, words, epoch, ctx->counters, ctx->status);
    else
        select_kernel<KIND, W, false><<<tiles, SEL_THREADS, smem, ctx->stream>>>(a, tiles, words, epoch, ctx->counters, ctx->status);
    if ((st = launched(ctx, "select"))) return st;
    DevStatus ds;
    if ((st = read_status(ctx, &ds))) return st;
    void *h;
    if ((st = pinned(ctx, 8, &h))) return st;
    VKC_CUDA(ctx, cudaMemcpyAsync(h, a.total, 8, cudaMemcpyDeviceToHost, ctx->stream));
    VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    unsigned long long k = *static_cast<unsigned long long *>(h);
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

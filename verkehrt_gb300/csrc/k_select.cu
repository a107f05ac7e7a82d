// Selections: filter_<cmp>_f64, compress_T and where (src/kernels/scalar/select.rs:81-104,
// src/kernels/scalar/fused.rs:225-236).
//
// One pass: each 4096-row tile computes its keep flags, the tile's survivor count goes through
// a decoupled lookback for the tile's output offset, and the survivors are compacted in shared
// memory and written out contiguously. The output is the rows in input order, so it does not
// depend on the tiling (select.rs:36-57 writes the same rows).
#include "lookback.cuh"
#include "reduce_common.h"

namespace vkc {

constexpr int SEL_THREADS = 256;
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

// Loads 16 consecutive items starting at item `row` (16-byte aligned when ALIGNED).
template <int W, bool ALIGNED>
__device__ __forceinline__ void load16(const void *p, int64_t row, int64_t n,
                                       typename Word<W>::T (&v)[SEL_ITEMS]) {
    using T = typename Word<W>::T;
    const T *src = static_cast<const T *>(p) + row;
    if (ALIGNED && row + SEL_ITEMS <= n) {
        const uint4 *q = reinterpret_cast<const uint4 *>(src);
#pragma unroll
        for (int j = 0; j < SEL_ITEMS * W / 16; ++j) {
            uint4 u = __ldcs(q + j);
            const T *e = reinterpret_cast<const T *>(&u);
#pragma unroll
            for (int k = 0; k < 16 / W; ++k) v[j * (16 / W) + k] = e[k];
        }
    } else {
#pragma unroll
        for (int j = 0; j < SEL_ITEMS; ++j) v[j] = row + j < n ? src[j] : T(0);
    }
}

template <int KIND, int W, bool ALIGNED>
__global__ void __launch_bounds__(SEL_THREADS) select_kernel(SelArgs a, int tiles,
                                                             LookbackTiles<unsigned long long> lb,
                                                             unsigned epoch, unsigned *counters,
                                                             DevStatus *status) {
    using T = typename Word<W>::T;
    using O = typename Word<KIND == SEL_WHERE ? 8 : W>::T;
    __shared__ O s_out[SEL_TILE];
    __shared__ unsigned long long s_prefix, s_count;
    const int tile = take_ticket(counters);
    const int64_t row0 = static_cast<int64_t>(tile) * SEL_TILE + threadIdx.x * SEL_ITEMS;

    T v[SEL_ITEMS];
    unsigned keep = 0;
    if (KIND != SEL_WHERE) load16<W, ALIGNED>(a.x, row0, a.n, v);
    if (KIND == SEL_FILTER) {
#pragma unroll
        for (int j = 0; j < SEL_ITEMS; ++j)
            if (row0 + j < a.n && in_range(a.r, static_cast<unsigned long long>(v[j]))) keep |= 1u << j;
    } else {
        unsigned char m[SEL_ITEMS];
        load16<1, ALIGNED>(a.m, row0, a.n, m);
#pragma unroll
        for (int j = 0; j < SEL_ITEMS; ++j)
            if (m[j]) keep |= 1u << j;
    }
    unsigned long long c = __popc(keep), tile_count;
    unsigned long long off = block_exclusive_sum<unsigned long long>(c, &tile_count);
    // Compact into shared memory in row order.
    int r = static_cast<int>(off);
#pragma unroll
    for (int j = 0; j < SEL_ITEMS; ++j)
        if (keep & (1u << j)) {
            if (KIND == SEL_WHERE) s_out[r] = static_cast<O>(a.base + row0 + j);
            else s_out[r] = static_cast<O>(v[j]);
            ++r;
        }
    if (threadIdx.x == 0) {
        auto add = [](unsigned long long p, unsigned long long q) { return p + q; };
        s_prefix = lookback_exclusive<unsigned long long>(lb, tile, tile_count, 0ull, epoch, add, status);
        s_count = tile_count;
        if (tile == tiles - 1) *a.total = s_prefix + tile_count;
    }
    __syncthreads();
    O *out = static_cast<O *>(a.out) + s_prefix;
    for (int i = threadIdx.x; i < static_cast<int>(s_count); i += SEL_THREADS) out[i] = s_out[i];
    release_ticket(counters, tiles);
}

template <int KIND, int W>
static vkc_status run_select(vkc_ctx *ctx, SelArgs a, int64_t n, Builder *b) {
    int64_t tiles64 = (n + SEL_TILE - 1) / SEL_TILE;
    int tiles = static_cast<int>(tiles64);
    void *p;
    unsigned *flags;
    vkc_status st;
    if ((st = scratch(ctx, 16 * static_cast<size_t>(tiles) + 256, &p))) return st;
    if ((st = flag_arena(ctx, static_cast<size_t>(tiles), &flags))) return st;
    auto *vals = static_cast<unsigned long long *>(p);
    LookbackTiles<unsigned long long> lb{flags, vals, vals + tiles};
    a.total = vals + 2 * static_cast<size_t>(tiles);
    void *at;
    if ((st = b->reserve(n, &at))) return st;
    a.out = at;
    unsigned epoch = next_epoch(ctx);
    bool aligned = (reinterpret_cast<uintptr_t>(a.x) & 15) == 0 &&
                   (reinterpret_cast<uintptr_t>(a.m) & 15) == 0;
    if (aligned)
        select_kernel<KIND, W, true><<<tiles, SEL_THREADS, 0, ctx->stream>>>(a, tiles, lb, epoch, ctx->counters, ctx->status);
    else
        select_kernel<KIND, W, false><<<tiles, SEL_THREADS, 0, ctx->stream>>>(a, tiles, lb, epoch, ctx->counters, ctx->status);
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

// Selections: filter_<cmp>_f64, compress_T and where (src/kernels/scalar/select.rs:81-104,
// src/kernels/scalar/fused.rs:225-236).
//
// One persistent pass (tilepass.cuh): a tile's survivor count is taken while the tile streams
// from HBM, its output offset comes from the decoupled lookback, and the survivors are written
// when the tile is read a second time, from L2. The output is the rows in input order, so it
// does not depend on the tiling (select.rs:36-57 writes the same rows).
#include "reduce_common.h"
#include "tilepass.cuh"

namespace vkc {

constexpr int SEL_THREADS = 256;
constexpr int SEL_TILE = 4096;                             // rows per tile
constexpr int SEL_SLICE = SEL_TILE / (SEL_THREADS / 32);   // rows per warp
constexpr int SEL_WINDOW = 4;                              // lookback: 32 * 4 tiles per step

enum SelKind { SEL_FILTER = 0, SEL_COMPRESS = 1, SEL_WHERE = 2 };

template <int W> struct Word;
template <> struct Word<16> { using T = uint4; };
template <> struct Word<8> { using T = unsigned long long; };
template <> struct Word<4> { using T = unsigned; };
template <> struct Word<2> { using T = unsigned short; };
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

// Nonzero bytes of a 32-bit word.
__device__ __forceinline__ unsigned nonzero_bytes(unsigned v) {
    const unsigned t = ~(((v & 0x7f7f7f7fu) + 0x7f7f7f7fu) | v | 0x7f7f7f7fu);  // 0x80 per zero byte
    return 4u - __popc(t);
}

// A selection as a tile pass. A warp's slice of a tile is SEL_SLICE consecutive rows. The
// count reads the keys (the values of a filter, the mask otherwise) with 16-byte loads; the
// write reads, per step, VV rows per lane (16 bytes of values, and the mask bytes of the same
// rows), ranks the kept rows with ballots and compacts them into the warp's slice of shared
// memory, which it then copies out with consecutive lanes on consecutive rows.
template <int KIND, int W, bool ALIGNED> struct SelectPass {
    static constexpr int THREADS = SEL_THREADS;
    using R = CountRec;
    using V = unsigned long long;
    using T = typename Word<W>::T;
    using O = typename Word<KIND == SEL_WHERE ? 8 : W>::T;
    static constexpr int VK = KIND == SEL_FILTER ? 2 : 16;  // keys per lane per count step
    static constexpr int SK = SEL_SLICE / (32 * VK);
    static constexpr int VV = KIND == SEL_WHERE ? 16 : 16 / W;  // rows per lane per write step
    static constexpr int SV = SEL_SLICE / (32 * VV);
    static_assert(SK >= 1 && SV >= 1, "a slice holds whole steps");

    SelArgs a;
    O *stage;  // SEL_SLICE outputs per warp

    __device__ __forceinline__ bool keep_filter(unsigned long long v) const { return in_range(a.r, v); }

    __device__ V count(int tile) const {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const int64_t base = static_cast<int64_t>(tile) * SEL_TILE + static_cast<int64_t>(w) * SEL_SLICE;
        unsigned c = 0;
        if (KIND == SEL_FILTER) {
            const auto *x = static_cast<const unsigned long long *>(a.x);
            ulonglong2 u[SK];
#pragma unroll
            for (int s = 0; s < SK; ++s) {
                const int64_t i0 = base + s * 64 + lane * 2;
                if (ALIGNED && i0 + 2 <= a.n) {
                    u[s] = *reinterpret_cast<const ulonglong2 *>(x + i0);
                } else {
                    u[s].x = i0 < a.n ? x[i0] : 0ull;
                    u[s].y = i0 + 1 < a.n ? x[i0 + 1] : 0ull;
                }
            }
#pragma unroll
            for (int s = 0; s < SK; ++s) {
                const int64_t i0 = base + s * 64 + lane * 2;
                c += (i0 < a.n && keep_filter(u[s].x)) + (i0 + 1 < a.n && keep_filter(u[s].y));
            }
        } else {
#pragma unroll
            for (int s = 0; s < SK; ++s) {
                const int64_t i0 = base + s * 512 + lane * 16;
                if (ALIGNED && i0 + 16 <= a.n) {
                    const uint4 u = *reinterpret_cast<const uint4 *>(a.m + i0);
                    c += nonzero_bytes(u.x) + nonzero_bytes(u.y) + nonzero_bytes(u.z) + nonzero_bytes(u.w);
                } else {
                    for (int k = 0; k < 16; ++k)
                        if (i0 + k < a.n && a.m[i0 + k]) ++c;
                }
            }
        }
        return warp_sum(c);
    }

    __device__ void write(int tile, V pre) const {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const unsigned lt = (1u << lane) - 1;
        const int64_t base = static_cast<int64_t>(tile) * SEL_TILE + static_cast<int64_t>(w) * SEL_SLICE;
        O *st = stage + w * SEL_SLICE;
        // Every step's loads are issued before any is used.
        T v[SV][KIND == SEL_WHERE ? 1 : VV];
        unsigned bits[SV];
#pragma unroll
        for (int s = 0; s < SV; ++s) {
            const int64_t i0 = base + s * (32 * VV) + lane * VV;
            bits[s] = 0;
            if (KIND != SEL_WHERE) {
                const T *x = static_cast<const T *>(a.x) + i0;
                if (ALIGNED && i0 + VV <= a.n) {
                    const uint4 u = __ldcs(reinterpret_cast<const uint4 *>(x));
                    const T *e = reinterpret_cast<const T *>(&u);
#pragma unroll
                    for (int k = 0; k < VV; ++k) v[s][k] = e[k];
                } else {
#pragma unroll
                    for (int k = 0; k < VV; ++k) v[s][k] = i0 + k < a.n ? x[k] : T(0);
                }
            }
            if (KIND != SEL_FILTER) {
                const unsigned char *m = a.m + i0;
                if (ALIGNED && i0 + VV <= a.n) {
                    if (VV == 16) {
                        const uint4 u = __ldcs(reinterpret_cast<const uint4 *>(m));
                        const unsigned wd[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                        for (int k = 0; k < 16; ++k)
                            if ((wd[k >> 2] >> (8 * (k & 3))) & 0xffu) bits[s] |= 1u << k;
                    } else {
                        const unsigned wd = VV == 4 ? __ldcs(reinterpret_cast<const unsigned *>(m))
                                                    : __ldcs(reinterpret_cast<const unsigned short *>(m));
#pragma unroll
                        for (int k = 0; k < VV; ++k)
                            if ((wd >> (8 * k)) & 0xffu) bits[s] |= 1u << k;
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < VV; ++k)
                        if (i0 + k < a.n && m[k]) bits[s] |= 1u << k;
                }
            }
        }
        unsigned total = 0;
#pragma unroll
        for (int s = 0; s < SV; ++s) {
            const int64_t i0 = base + s * (32 * VV) + lane * VV;
            unsigned b = bits[s];
            if (KIND == SEL_FILTER) {
#pragma unroll
                for (int k = 0; k < VV; ++k)
                    if (i0 + k < a.n && keep_filter(static_cast<unsigned long long>(v[s][k]))) b |= 1u << k;
            }
            // In-order ranks: the lanes before this one, element by element.
            unsigned before = 0, step_total = 0;
#pragma unroll
            for (int k = 0; k < VV; ++k) {
                const unsigned m = __ballot_sync(FULL, (b >> k) & 1u);
                before += __popc(m & lt);
                step_total += __popc(m);
            }
            unsigned p = total + before;
#pragma unroll
            for (int k = 0; k < VV; ++k)
                if ((b >> k) & 1u) {
                    if (KIND == SEL_WHERE) st[p] = static_cast<O>(a.base + i0 + k);
                    else st[p] = static_cast<O>(v[s][KIND == SEL_WHERE ? 0 : k]);
                    ++p;
                }
            total += step_total;
        }
        __syncwarp();
        O *out = static_cast<O *>(a.out) + pre;
        for (unsigned i = lane; i < total; i += 32) out[i] = st[i];
        __syncwarp();  // the slice of shared memory is free again
    }

    __device__ void last_tile(V inclusive) const { *a.total = inclusive; }
};

template <int KIND, int W, bool ALIGNED>
__global__ void __launch_bounds__(SEL_THREADS, 4) select_kernel(SelArgs a, int tiles, unsigned long long *recs,
                                                             unsigned epoch, unsigned *counters,
                                                             DevStatus *status) {
    using P = SelectPass<KIND, W, ALIGNED>;
    extern __shared__ __align__(16) unsigned char sel_smem[];
    P p{a, reinterpret_cast<typename P::O *>(sel_smem)};
    tile_pass<SEL_WINDOW>(p, recs, tiles, epoch, counters, status, 0ull);
}

template <int KIND, int W>
static vkc_status run_select(vkc_ctx *ctx, SelArgs a, int64_t n, Builder *b) {
    if (n >= (int64_t(1) << 38)) return fail(ctx, VKC_USAGE, "selection of 2^38 rows or more");
    const int64_t tiles64 = (n + SEL_TILE - 1) / SEL_TILE;
    const int tiles = static_cast<int>(tiles64);
    void *p;
    unsigned *flags;
    vkc_status st;
    if ((st = scratch(ctx, 256, &p))) return st;
    if ((st = flag_arena(ctx, 2 * static_cast<size_t>(tiles), &flags))) return st;
    auto *recs = reinterpret_cast<unsigned long long *>(flags);
    a.total = static_cast<unsigned long long *>(p);
    void *at;
    if ((st = b->reserve(n, &at))) return st;
    a.out = at;
    const unsigned epoch = next_epoch(ctx);
    const bool aligned = (reinterpret_cast<uintptr_t>(a.x) & 15) == 0 &&
                         (reinterpret_cast<uintptr_t>(a.m) & 15) == 0;
    using O = typename SelectPass<KIND, W, true>::O;
    const size_t smem = sizeof(O) * SEL_TILE;
    if (aligned) {
        const int grid = tile_pass_grid(ctx, select_kernel<KIND, W, true>, SEL_THREADS, smem, tiles);
        select_kernel<KIND, W, true><<<grid, SEL_THREADS, smem, ctx->stream>>>(a, tiles, recs, epoch, ctx->counters, ctx->status);
    } else {
        const int grid = tile_pass_grid(ctx, select_kernel<KIND, W, false>, SEL_THREADS, smem, tiles);
        select_kernel<KIND, W, false><<<grid, SEL_THREADS, smem, ctx->stream>>>(a, tiles, recs, epoch, ctx->counters, ctx->status);
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

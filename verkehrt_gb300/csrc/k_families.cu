// The kernel families on every element type: the entries of the reference's registry that the
// specialised files (f64 sums, f64/i64 extremes, i64 scans and buckets, i64 sort and group ids)
// do not hold.
//
//   reductions  reduce_add/mul/min/max_T, reduce_and/or/xor_T, argmin/argmax_T, any, all
//               (src/kernels/scalar/reduce.rs:331-726)
//   fused       dot/sumsq/count_<cmp>/filter_<cmp>/condsum_<cmp> on f32, i64, u64, i32
//               (src/kernels/scalar/fused.rs:73-379)
//   scans       scan_<fold>_T, scan_by_<fold>_T, reduce_into_<fold>_T, prev_T
//               (src/kernels/scalar/scan.rs:16-439)
//   whole       argsort_T, group_id_T, group_id2_A_B (index.rs:159-173, group.rs:259-363),
//               fill_T, same_len_T (construct.rs:49-120), slice_T (index.rs:240-258)
//
// Values travel as 64-bit words: i32 sign-extended, u8 and bool zero-extended, f32 as its 32
// bits. Every fold except the canonical float sum and product is order-free (wrapping integer
// arithmetic, the 754-2019 minimum/maximum, bit operations), so those reductions are a plain
// grid fold and the scans a reduce-then-scan over 4096-row tiles. The canonical float order
// (f32 sums, every float product) is sixteen chains of dependent IEEE operations: one block
// stages the rows in shared memory while sixteen threads run the chains (fast enough for these
// secondary entries; the f64 sums have their own exact parallel path in k_canon.cu).
#include <climits>
#include <cstring>

#include "kcommon.cuh"
#include "reduce_common.h"

namespace vkc {

vkc_status bucket_key_error(vkc_ctx *ctx, const long long *k, int64_t n, int64_t nb, bool *found);

namespace {

typedef unsigned long long u64;

enum Fold { F_ADD = 0, F_MUL = 1, F_MIN = 2, F_MAX = 3, F_AND = 4, F_OR = 5, F_XOR = 6 };
const char *FOLD_NAMES[7] = {"add", "mul", "min", "max", "and", "or", "xor"};
const char *CMP_NAME[6] = {"eq", "ne", "lt", "le", "gt", "ge"};

__host__ __device__ constexpr int width_of(vkc_type t) {
    return t == VKC_F64 || t == VKC_I64 || t == VKC_U64 ? 8 : (t == VKC_F32 || t == VKC_I32 ? 4 : 1);
}
__host__ __device__ constexpr vkc_type sum_type(vkc_type t) {
    return t == VKC_I32 ? VKC_I64 : (t == VKC_U8 ? VKC_U64 : t);
}
__host__ __device__ constexpr bool is_float(vkc_type t) { return t == VKC_F64 || t == VKC_F32; }
__host__ __device__ constexpr bool is_signed_t(vkc_type t) { return t == VKC_I64 || t == VKC_I32; }

// Element load and store as words.
template <vkc_type T> __device__ __forceinline__ u64 ld_word(const void *p, int64_t i) {
    if (width_of(T) == 8) return static_cast<const u64 *>(p)[i];
    if (T == VKC_F32) return static_cast<const unsigned *>(p)[i];
    if (T == VKC_I32) return static_cast<u64>(static_cast<long long>(static_cast<const int *>(p)[i]));
    return static_cast<const unsigned char *>(p)[i];
}
template <int W> __device__ __forceinline__ void st_word(void *p, int64_t i, u64 v) {
    if (W == 8) static_cast<u64 *>(p)[i] = v;
    else if (W == 4) static_cast<unsigned *>(p)[i] = static_cast<unsigned>(v);
    else static_cast<unsigned char *>(p)[i] = static_cast<unsigned char>(v);
}

// Num::wrapping on the element type (elementwise.rs:386-400): truncate and widen back.
template <vkc_type T> __host__ __device__ constexpr u64 wrap(u64 v) {
    return T == VKC_I32 ? static_cast<u64>(static_cast<long long>(static_cast<int>(static_cast<unsigned>(v))))
           : (T == VKC_U8 || T == VKC_BOOL) ? (v & 0xffull) : v;
}

__device__ __forceinline__ bool nan64(u64 b) { return (b & ~(1ull << 63)) > 0x7ff0000000000000ull; }
__device__ __forceinline__ bool nan32(u64 b) { return (b & 0x7fffffffull) > 0x7f800000ull; }
template <vkc_type T> __device__ __forceinline__ bool is_nan(u64 w) {
    return T == VKC_F64 ? nan64(w) : (T == VKC_F32 ? nan32(w) : false);
}

// elementwise.rs:413-440: min2/max2 (NaN propagates, -0 below +0); Ord on integers.
template <vkc_type T, bool MAX> __device__ __forceinline__ u64 ext2(u64 a, u64 b) {
    if (T == VKC_F64) {
        if (nan64(a) || nan64(b)) return 0x7ff8000000000000ull;
        const double x = __longlong_as_double(static_cast<long long>(a)), y = __longlong_as_double(static_cast<long long>(b));
        if (x == y) return ((a >> 63) != 0) == !MAX ? a : b;
        return (MAX ? x > y : x < y) ? a : b;
    }
    if (T == VKC_F32) {
        if (nan32(a) || nan32(b)) return 0x7fc00000ull;
        const float x = __uint_as_float(static_cast<unsigned>(a)), y = __uint_as_float(static_cast<unsigned>(b));
        if (x == y) return ((a >> 31) & 1u) == (MAX ? 0u : 1u) ? a : b;
        return (MAX ? x > y : x < y) ? a : b;
    }
    if (is_signed_t(T)) {
        const long long x = static_cast<long long>(a), y = static_cast<long long>(b);
        return (MAX ? x >= y : x <= y) ? a : b;
    }
    return (MAX ? a >= b : a <= b) ? a : b;
}

// One step of fold F (scan.rs:130-233 ScanOp::step, the reductions' Accum steps): the
// accumulator of add is in the sum type.
template <vkc_type T, int F> __device__ __forceinline__ u64 step(u64 acc, u64 x) {
    if (F == F_ADD) return acc + x;
    if (F == F_MUL) return wrap<T>(acc * x);
    if (F == F_MIN) return ext2<T, false>(acc, x);
    if (F == F_MAX) return ext2<T, true>(acc, x);
    if (F == F_AND) return acc & x;
    if (F == F_OR) return acc | x;
    return acc ^ x;
}

// scan.rs:99-120, :130-233 (identity): add/or/xor 0, mul 1, and all ones (bool: true), min the
// highest value (+inf), max the lowest (-inf).
template <vkc_type T, int F> __host__ __device__ constexpr u64 identity() {
    return F == F_ADD || F == F_OR || F == F_XOR ? 0ull
           : F == F_MUL ? 1ull
           : F == F_AND ? (T == VKC_BOOL ? 1ull : wrap<T>(~0ull))
           : F == F_MIN ? (T == VKC_F64 ? 0x7ff0000000000000ull
                           : T == VKC_F32 ? 0x7f800000ull
                           : T == VKC_I64 ? 0x7fffffffffffffffull
                           : T == VKC_I32 ? 0x7fffffffull
                           : T == VKC_U8 ? 0xffull : ~0ull)
                        : (T == VKC_F64 ? 0xfff0000000000000ull
                           : T == VKC_F32 ? 0xff800000ull
                           : T == VKC_I64 ? 0x8000000000000000ull
                           : T == VKC_I32 ? 0xffffffff80000000ull : 0ull);
}

// fused.rs:41-54: the comparison of the single-op kernels (IEEE for floats: NaN is unordered).
template <vkc_type T> __device__ __forceinline__ bool cmp_test(int cmp, u64 a, u64 b) {
    bool lt, eq, unord = false;
    if (T == VKC_F64) {
        const double x = __longlong_as_double(static_cast<long long>(a)), y = __longlong_as_double(static_cast<long long>(b));
        unord = x != x || y != y;
        lt = x < y;
        eq = x == y;
    } else if (T == VKC_F32) {
        const float x = __uint_as_float(static_cast<unsigned>(a)), y = __uint_as_float(static_cast<unsigned>(b));
        unord = x != x || y != y;
        lt = x < y;
        eq = x == y;
    } else if (is_signed_t(T)) {
        lt = static_cast<long long>(a) < static_cast<long long>(b);
        eq = a == b;
    } else {
        lt = a < b;
        eq = a == b;
    }
    if (unord) return cmp == 1;
    switch (cmp) {
    case 0: return eq;
    case 1: return !eq;
    case 2: return lt;
    case 3: return lt || eq;
    case 4: return !lt && !eq;
    default: return !lt;
    }
}

// Num::mul on the element type: one IEEE multiply (no contraction) or a wrapping product.
template <vkc_type T> __device__ __forceinline__ u64 mul_t(u64 a, u64 b) {
    if (T == VKC_F64)
        return static_cast<u64>(__double_as_longlong(__dmul_rn(__longlong_as_double(static_cast<long long>(a)),
                                                               __longlong_as_double(static_cast<long long>(b)))));
    if (T == VKC_F32)
        return __float_as_uint(__fmul_rn(__uint_as_float(static_cast<unsigned>(a)), __uint_as_float(static_cast<unsigned>(b))));
    return wrap<T>(a * b);
}

// Row values of the folds (fused.rs:73-212): the row itself, x*y, x*x, (x <cmp> c ? x : e),
// the predicate as 0/1, or a bool byte as 0/1.
enum Row { R_PLAIN = 0, R_DOT = 1, R_SUMSQ = 2, R_COND = 3, R_PRED = 4 };
struct RowArgs {
    const void *x;
    const void *y;
    int cmp;
    u64 c, e;
};
template <vkc_type T, int ROW> __device__ __forceinline__ u64 row_value(const RowArgs &a, int64_t i) {
    const u64 v = ld_word<T>(a.x, i);
    if (ROW == R_DOT) return mul_t<T>(v, ld_word<T>(a.y, i));
    if (ROW == R_SUMSQ) return mul_t<T>(v, v);
    if (ROW == R_COND) return cmp_test<T>(a.cmp, v, a.c) ? v : a.e;
    if (ROW == R_PRED) return cmp_test<T>(a.cmp, v, a.c) ? 1ull : 0ull;
    return v;
}

// ------------------------------------------------------------------ order-free folds

// Every block folds its rows (grid-stride, four rows in flight per thread), the warps and the
// block combine (the fold is commutative), and the last block to finish folds the block
// partials into the reducer's state word.
template <vkc_type T, int F, int ROW>
__global__ void __launch_bounds__(256) fam_fold_kernel(RowArgs a, int64_t n, u64 *partials, unsigned *done, u64 *state) {
    constexpr vkc_type AT = ROW == R_PRED ? VKC_U64 : T;  // predicate counts add as u64
    u64 acc = identity<AT, F>();
    const int64_t tid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = tid; i < n; i += 4 * stride) {
        u64 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = i + u * stride < n ? row_value<T, ROW>(a, i + u * stride) : identity<AT, F>();
#pragma unroll
        for (int u = 0; u < 4; ++u) acc = step<AT, F>(acc, v[u]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = step<AT, F>(acc, __shfl_xor_sync(FULL, acc, o));
    __shared__ u64 ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        u64 s = ws[0];
        for (int w = 1; w < 8; ++w) s = step<AT, F>(s, ws[w]);
        partials[blockIdx.x] = s;
    }
    if (last_block(done) && threadIdx.x < 32) {
        u64 s = identity<AT, F>();
        for (unsigned b = threadIdx.x; b < gridDim.x; b += 32) s = step<AT, F>(s, partials[b]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = step<AT, F>(s, __shfl_xor_sync(FULL, s, o));
        if (threadIdx.x == 0) {
            state[0] = step<AT, F>(state[0], s);
            state[1] = 1;  // rows seen
        }
    }
}

// argmin/argmax (reduce.rs:417-468): the first NaN's row, else the first row of the extreme
// (-0 below +0). Each row is the pair (h, row) with h = 0 for a NaN, else the order key (argmin)
// or its complement (argmax); the result is the least pair. Non-NaN keys of floats are never 0.
template <vkc_type T> __device__ __forceinline__ u64 order_key(u64 w) {
    if (T == VKC_F64) return (w >> 63) ? ~w : (w | (1ull << 63));
    if (T == VKC_F32) return ((w >> 31) & 1u) ? (~w & 0xffffffffull) : (w | 0x80000000ull);
    if (is_signed_t(T)) return w ^ (1ull << 63);
    return w;
}
template <vkc_type T, bool MAX> __device__ __forceinline__ u64 arg_key(u64 w) {
    if (is_nan<T>(w)) return 0;
    return MAX ? ~order_key<T>(w) : order_key<T>(w);
}
__device__ __forceinline__ void arg_better(u64 &h, u64 &r, u64 h2, u64 r2) {
    if (h2 < h || (h2 == h && r2 < r)) {
        h = h2;
        r = r2;
    }
}

template <vkc_type T, bool MAX>
__global__ void __launch_bounds__(256) fam_arg_kernel(const void *x, int64_t n, u64 base, ulonglong2 *partials,
                                                      unsigned *done, u64 *state) {
    u64 h = ~0ull, r = ~0ull;
    const int64_t tid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = tid; i < n; i += stride) arg_better(h, r, arg_key<T, MAX>(ld_word<T>(x, i)), base + static_cast<u64>(i));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) arg_better(h, r, __shfl_xor_sync(FULL, h, o), __shfl_xor_sync(FULL, r, o));
    __shared__ u64 wh[8], wr[8];
    if ((threadIdx.x & 31) == 0) {
        wh[threadIdx.x >> 5] = h;
        wr[threadIdx.x >> 5] = r;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; ++w) arg_better(h, r, wh[w], wr[w]);
        partials[blockIdx.x] = make_ulonglong2(h, r);
    }
    if (last_block(done) && threadIdx.x < 32) {
        u64 bh = ~0ull, br = ~0ull;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += 32) arg_better(bh, br, partials[b].x, partials[b].y);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) arg_better(bh, br, __shfl_xor_sync(FULL, bh, o), __shfl_xor_sync(FULL, br, o));
        if (threadIdx.x == 0) {
            u64 sh = state[0], sr = state[1];
            arg_better(sh, sr, bh, br);
            state[0] = sh;
            state[1] = sr;
            state[2] = 1;
        }
    }
}

// The result word as a scalar of type t.
vkc_scalar word_scalar(vkc_type t, u64 w) {
    vkc_scalar s;
    s.type = t;
    s.bits = width_of(t) == 8 ? w : (width_of(t) == 4 ? (w & 0xffffffffull) : (w & 0xffull));
    return s;
}

// A scalar argument of type t as a word (i32 sign-extended).
u64 scalar_word(vkc_type t, const vkc_scalar &s) {
    if (t == VKC_I32) return static_cast<u64>(static_cast<long long>(static_cast<int>(static_cast<unsigned>(s.bits))));
    if (width_of(t) == 4) return s.bits & 0xffffffffull;
    if (width_of(t) == 1) return s.bits & 0xffull;
    return s.bits;
}

// Reducers of the order-free folds. State: [0] the folded word, [1] rows seen (argmin/argmax:
// [0] key, [1] row, [2] rows seen). `base` counts the rows of earlier updates.
struct FamReducer : DevReducer {
    vkc_type in, out;
    int fold;      // F_*, or -1 argmin, -2 argmax
    int row;       // R_*
    int nargs_want;
    int cmp = 0;
    bool empty_error = false;  // min/max/argmin/argmax of no rows fail
    const char *what = "";
    u64 base = 0;
    using Launch = void (*)(vkc_ctx *, const RowArgs &, int64_t, int, void *, u64, u64 *);
    Launch launch = nullptr;

    vkc_status init(vkc_ctx *ctx, u64 id0, u64 id1) { return fill(ctx, 3, id0, id1, 0); }
    vkc_status update(vkc_ctx *ctx, const Arg *args, int nargs) override {
        vkc_status st;
        if (nargs != nargs_want) return fail(ctx, VKC_RUNTIME, arity_error(nargs_want, nargs));
        if (!rows_arg(ctx, args[0], in, &st)) return st;
        RowArgs a{args[0].a->data(), nullptr, cmp, 0, 0};
        if (row == R_DOT) {
            if (!rows_arg(ctx, args[1], in, &st)) return st;
            if (args[0].len() != args[1].len())
                return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(args[0].len()) + " vs " +
                                                  std::to_string(args[1].len()));
            a.y = args[1].a->data();
        } else if (row == R_COND || row == R_PRED) {
            for (int i = 1; i < nargs; ++i)
                if (!splat_arg(ctx, args[i], in, &st)) return st;
            a.c = scalar_word(in, args[1].s);
            if (row == R_COND) a.e = scalar_word(in, args[2].s);
        }
        const int64_t n = args[0].len();
        if (n == 0) return VKC_OK;
        const int grid = stream_grid(ctx, n, 256, tune(ctx, TK_STREAM_BLOCKS, n), 4096);
        void *part;
        if ((st = scratch(ctx, 16 * static_cast<size_t>(grid), &part))) return st;
        launch(ctx, a, n, grid, part, base, static_cast<u64 *>(state));
        base += static_cast<u64>(n);
        return launched(ctx, "family_fold");
    }
    vkc_status finish(vkc_ctx *ctx, vkc_scalar *out_s) override {
        u64 h[3];
        vkc_status st = download(ctx, h, sizeof h);
        if (st) return st;
        const bool arg = fold < 0;
        if (empty_error && !(arg ? h[2] : h[1])) return fail(ctx, VKC_RUNTIME, std::string(what) + " of an empty array");
        *out_s = arg ? scalar_i64(static_cast<int64_t>(h[1])) : word_scalar(out, h[0]);
        return VKC_OK;
    }
    vkc_status finish_into(vkc_ctx *ctx, void *dst) override {
        if (empty_error && base == 0) return fail(ctx, VKC_RUNTIME, std::string(what) + " of an empty array");
        // Words are little-endian: the result type's bytes are the word's low bytes.
        return fold < 0 ? copy_out(ctx, dst, 8, 8) : copy_out(ctx, dst, static_cast<size_t>(width_of(out)));
    }
};

template <vkc_type T, int F, int ROW>
void launch_fold(vkc_ctx *ctx, const RowArgs &a, int64_t n, int grid, void *part, u64, u64 *state) {
    fam_fold_kernel<T, F, ROW><<<grid, 256, 0, ctx->stream>>>(a, n, static_cast<u64 *>(part), ctx->counters + 1, state);
}
template <vkc_type T, bool MAX>
void launch_arg(vkc_ctx *ctx, const RowArgs &a, int64_t n, int grid, void *part, u64 base, u64 *state) {
    fam_arg_kernel<T, MAX><<<grid, 256, 0, ctx->stream>>>(a.x, n, base, static_cast<ulonglong2 *>(part),
                                                          ctx->counters + 1, state);
}

template <vkc_type T, int F, int ROW, int NARGS>
ReducerImpl *make_fold(vkc_ctx *ctx, vkc_type out, int cmp, bool empty_error, const char *what) {
    auto *r = new FamReducer;
    if (r->alloc(ctx, 24)) {
        delete r;
        return nullptr;
    }
    r->in = T;
    r->out = out;
    r->fold = F;
    r->row = ROW;
    r->nargs_want = NARGS;
    r->cmp = cmp;
    r->empty_error = empty_error;
    r->what = what;
    r->launch = launch_fold<T, F, ROW>;
    constexpr vkc_type AT = ROW == R_PRED ? VKC_U64 : T;
    if (r->init(ctx, identity<AT, F>(), 0)) {
        delete r;
        return nullptr;
    }
    return r;
}

template <vkc_type T, bool MAX> ReducerImpl *make_arg(vkc_ctx *ctx) {
    auto *r = new FamReducer;
    if (r->alloc(ctx, 24)) {
        delete r;
        return nullptr;
    }
    r->in = T;
    r->out = VKC_I64;
    r->fold = MAX ? -2 : -1;
    r->row = R_PLAIN;
    r->nargs_want = 1;
    r->empty_error = true;
    r->what = MAX ? "argmax" : "argmin";
    r->launch = launch_arg<T, MAX>;
    if (r->init(ctx, ~0ull, ~0ull)) {
        delete r;
        return nullptr;
    }
    return r;
}

// ------------------------------------------------------------------ canonical float chains
//
// reduce.rs:45-91: lane j adds (multiplies) rows 16b + j in order from the identity; then +8,
// +4, +2, +1; then the tail. One block: warps 1..7 stage chunk k + 1 (FC_ROWS rows, as row values)
// in shared memory while the first sixteen threads of warp 0 run their lane chains over chunk k.
constexpr int FC_BLOCKS = 128;               // 16-row blocks per chunk
constexpr int FC_ROWS = FC_BLOCKS * 16;      // rows per chunk

template <vkc_type T> __device__ __forceinline__ u64 fop(u64 a, u64 b, bool mul) {
    if (T == VKC_F64) {
        const double x = __longlong_as_double(static_cast<long long>(a)), y = __longlong_as_double(static_cast<long long>(b));
        return static_cast<u64>(__double_as_longlong(mul ? __dmul_rn(x, y) : __dadd_rn(x, y)));
    }
    const float x = __uint_as_float(static_cast<unsigned>(a)), y = __uint_as_float(static_cast<unsigned>(b));
    return __float_as_uint(mul ? __fmul_rn(x, y) : __fadd_rn(x, y));
}

template <vkc_type T, int ROW, bool MUL>
__global__ void __launch_bounds__(256) fam_chain_kernel(RowArgs a, int64_t nb, u64 *lanes) {
    __shared__ u64 buf[2][FC_ROWS];
    const int t = threadIdx.x;
    const int64_t chunks = (nb + FC_BLOCKS - 1) / FC_BLOCKS;
    auto stage = [&](int64_t k, int first, int step) {
        const int64_t r0 = k * FC_ROWS, rows = min(static_cast<int64_t>(FC_ROWS), nb * 16 - r0);
        for (int i = first; i < rows; i += step) buf[k & 1][i] = row_value<T, ROW>(a, r0 + i);
    };
    u64 s = t < 16 ? lanes[t] : 0ull;
    if (chunks > 0) stage(0, t, 256);
    __syncthreads();
    for (int64_t k = 0; k < chunks; ++k) {
        if (t >= 32) {
            if (k + 1 < chunks) stage(k + 1, t - 32, 224);
        } else if (t < 16) {
            const int blocks = static_cast<int>(min(static_cast<int64_t>(FC_BLOCKS), nb - k * FC_BLOCKS));
            const u64 *b = buf[k & 1];
            for (int i = 0; i < blocks; ++i) s = fop<T>(s, b[i * 16 + t], MUL);
        }
        __syncthreads();
    }
    if (t < 16) lanes[t] = s;
}

// The tail rows (fewer than 16) as row values, kept until finish.
template <vkc_type T, int ROW>
__global__ void fam_chain_tail(RowArgs a, int64_t first, int rest, u64 *tail) {
    if (static_cast<int>(threadIdx.x) < rest) tail[threadIdx.x] = row_value<T, ROW>(a, first + threadIdx.x);
}

// reduce.rs:77-91 (finish_lanes).
template <vkc_type T, bool MUL> __global__ void fam_chain_finish(u64 *st, int tail_len) {
    u64 acc[16];
    for (int j = 0; j < 16; ++j) acc[j] = st[j];
    for (int s = 8; s > 0; s >>= 1)
        for (int j = 0; j < s; ++j) acc[j] = fop<T>(acc[j], acc[j + s], MUL);
    u64 r = acc[0];
    for (int j = 0; j < tail_len; ++j) r = fop<T>(r, st[16 + j], MUL);
    st[32] = r;
}

// CanonicalAcc (reduce.rs:253-323) on the device. State: [0..15] lanes, [16..31] tail, [32] result.
struct ChainReducer : DevReducer {
    vkc_type in;
    int row, nargs_want, cmp = 0;
    int tail_len = 0;
    using Launch = void (*)(vkc_ctx *, const RowArgs &, int64_t nb, int64_t first, int rest, u64 *state);
    Launch launch = nullptr;
    using Fin = void (*)(vkc_ctx *, u64 *, int);
    Fin fin = nullptr;

    vkc_status update(vkc_ctx *ctx, const Arg *args, int nargs) override {
        vkc_status st;
        if (nargs != nargs_want) return fail(ctx, VKC_RUNTIME, arity_error(nargs_want, nargs));
        if (!rows_arg(ctx, args[0], in, &st)) return st;
        RowArgs a{args[0].a->data(), nullptr, cmp, 0, 0};
        if (row == R_DOT) {
            if (!rows_arg(ctx, args[1], in, &st)) return st;
            if (args[0].len() != args[1].len())
                return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(args[0].len()) + " vs " +
                                                  std::to_string(args[1].len()));
            a.y = args[1].a->data();
        } else if (row == R_COND) {
            if (!splat_arg(ctx, args[1], in, &st) || !splat_arg(ctx, args[2], in, &st)) return st;
            a.c = scalar_word(in, args[1].s);
            a.e = scalar_word(in, args[2].s);
        }
        const int64_t n = args[0].len();
        if (tail_len != 0) return fail(ctx, VKC_RUNTIME, "canonical update after a partial block");
        const int64_t nb = n / 16;
        const int rest = static_cast<int>(n % 16);
        launch(ctx, a, nb, nb * 16, rest, static_cast<u64 *>(state));
        tail_len = rest;
        return launched(ctx, "family_chain");
    }
    vkc_status finish(vkc_ctx *ctx, vkc_scalar *out) override {
        fin(ctx, static_cast<u64 *>(state), tail_len);
        vkc_status st = launched(ctx, "family_chain_finish");
        if (st) return st;
        u64 r = 0;
        if ((st = download(ctx, &r, 8, 32 * 8))) return st;
        *out = word_scalar(in, r);
        return VKC_OK;
    }
    vkc_status finish_into(vkc_ctx *ctx, void *dst) override {
        fin(ctx, static_cast<u64 *>(state), tail_len);
        vkc_status st = launched(ctx, "family_chain_finish");
        return st ? st : copy_out(ctx, dst, static_cast<size_t>(width_of(in)), 32 * 8);
    }
};

template <vkc_type T, int ROW, bool MUL>
void launch_chain(vkc_ctx *ctx, const RowArgs &a, int64_t nb, int64_t first, int rest, u64 *state) {
    if (nb > 0) fam_chain_kernel<T, ROW, MUL><<<1, 256, 0, ctx->stream>>>(a, nb, state);
    if (rest > 0) fam_chain_tail<T, ROW><<<1, 16, 0, ctx->stream>>>(a, first, rest, state + 16);
}
template <vkc_type T, bool MUL> void finish_chain(vkc_ctx *ctx, u64 *state, int tail_len) {
    fam_chain_finish<T, MUL><<<1, 1, 0, ctx->stream>>>(state, tail_len);
}

template <vkc_type T, int ROW, bool MUL, int NARGS> ReducerImpl *make_chain(vkc_ctx *ctx, int cmp) {
    auto *r = new ChainReducer;
    if (r->alloc(ctx, 33 * 8)) {
        delete r;
        return nullptr;
    }
    r->in = T;
    r->row = ROW;
    r->nargs_want = NARGS;
    r->cmp = cmp;
    r->launch = launch_chain<T, ROW, MUL>;
    r->fin = finish_chain<T, MUL>;
    const u64 one = T == VKC_F64 ? 0x3ff0000000000000ull : 0x3f800000ull;
    const u64 v = MUL ? one : 0ull;
    if (r->fill(ctx, 33, v, v, v, v)) {
        delete r;
        return nullptr;
    }
    return r;
}

// ------------------------------------------------------------------ scans
//
// scan.rs:248-282: row 0 and every row whose start flag is set lift their value, every other
// row steps the running value; state carries across updates. With the fold's identity as the
// state before the first row (step(identity, x) = lift(x)), out[i] is the fold of the state and
// the rows from the last start through i: an associative fold of (flag, value) pairs,
// (f1, v1) then (f2, v2) = (f1 | f2, f2 ? v2 : v1 op v2). Three kernels: tile aggregates, one
// block's exclusive scan of them from the carried state, and each tile's rows from its prefix.
constexpr int SC_T = 256, SC_I = 16, SC_ROWS = SC_T * SC_I;

struct SegVal {
    u64 v;
    unsigned f;
};

template <vkc_type T, int F> __device__ __forceinline__ SegVal seg_op(SegVal a, SegVal b) {
    return SegVal{b.f ? b.v : step<T, F>(a.v, b.v), a.f | b.f};
}

// Inclusive block scan of one pair per thread, in thread order; *total gets the block's pair.
template <vkc_type T, int F> __device__ SegVal block_scan(SegVal x, SegVal *total) {
    __shared__ u64 wv[SC_T / 32];
    __shared__ unsigned wf[SC_T / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        SegVal y{__shfl_up_sync(FULL, x.v, o), __shfl_up_sync(FULL, x.f, o)};
        if (lane >= o) x = seg_op<T, F>(y, x);
    }
    if (lane == 31) {
        wv[w] = x.v;
        wf[w] = x.f;
    }
    __syncthreads();
    SegVal before{identity<T, F>(), 0};
    for (int i = 0; i < w; ++i) before = seg_op<T, F>(before, SegVal{wv[i], wf[i]});
    SegVal t{identity<T, F>(), 0};
    for (int i = 0; i < SC_T / 32; ++i) t = seg_op<T, F>(t, SegVal{wv[i], wf[i]});
    *total = t;
    __syncthreads();
    return w ? seg_op<T, F>(before, x) : x;
}

// IT: the element type; OT: the word domain of the fold (the sum type for add).
template <vkc_type IT, vkc_type OT, int F, bool BY>
__device__ __forceinline__ SegVal thread_rows(const void *x, const unsigned char *s, int64_t r0, int64_t n, u64 *v) {
    SegVal acc{identity<OT, F>(), 0};
#pragma unroll
    for (int j = 0; j < SC_I; ++j) {
        const int64_t r = r0 + j;
        v[j] = r < n ? ld_word<IT>(x, r) : identity<OT, F>();
        const unsigned f = (BY && r < n) ? (s[r] != 0) : 0u;
        acc = f ? SegVal{v[j], 1u} : SegVal{step<OT, F>(acc.v, v[j]), acc.f};
    }
    return acc;
}

template <vkc_type IT, vkc_type OT, int F, bool BY>
__global__ void __launch_bounds__(SC_T) fam_scan_agg(const void *x, const unsigned char *s, int64_t n, u64 *aggv,
                                                     unsigned *aggf) {
    const int64_t r0 = static_cast<int64_t>(blockIdx.x) * SC_ROWS + threadIdx.x * SC_I;
    u64 v[SC_I];
    SegVal mine = thread_rows<IT, OT, F, BY>(x, s, r0, n, v);
    SegVal tot;
    block_scan<OT, F>(mine, &tot);
    if (threadIdx.x == 0) {
        aggv[blockIdx.x] = tot.v;
        aggf[blockIdx.x] = tot.f;
    }
}

// One block: the exclusive prefix of every tile from the carried state (carry[0]).
template <vkc_type OT, int F>
__global__ void __launch_bounds__(1024) fam_scan_prefix(u64 *aggv, const unsigned *aggf, int tiles, const u64 *carry) {
    __shared__ u64 tv[1024];
    __shared__ unsigned tf[1024];
    const int per = (tiles + 1023) / 1024;
    const int t0 = threadIdx.x * per, t1 = min(tiles, t0 + per);
    SegVal acc{identity<OT, F>(), 0};
    for (int t = t0; t < t1; ++t) acc = seg_op<OT, F>(acc, SegVal{aggv[t], aggf[t]});
    tv[threadIdx.x] = acc.v;
    tf[threadIdx.x] = acc.f;
    __syncthreads();
    if (threadIdx.x == 0) {
        SegVal run{carry[0], 0};
        for (int i = 0; i < 1024; ++i) {
            const SegVal mine{tv[i], tf[i]};
            tv[i] = run.v;
            run = seg_op<OT, F>(run, mine);
        }
    }
    __syncthreads();
    SegVal run{tv[threadIdx.x], 0};
    for (int t = t0; t < t1; ++t) {
        const SegVal mine{aggv[t], aggf[t]};
        aggv[t] = run.v;  // exclusive prefix of tile t
        run = seg_op<OT, F>(run, mine);
    }
}

template <vkc_type IT, vkc_type OT, int F, bool BY>
__global__ void __launch_bounds__(SC_T) fam_scan_apply(const void *x, const unsigned char *s, int64_t n,
                                                       const u64 *prefix, void *out, u64 *carry) {
    const int64_t r0 = static_cast<int64_t>(blockIdx.x) * SC_ROWS + threadIdx.x * SC_I;
    u64 v[SC_I];
    SegVal mine = thread_rows<IT, OT, F, BY>(x, s, r0, n, v);
    SegVal tot;
    const SegVal incl = block_scan<OT, F>(mine, &tot);
    // The value before this thread's rows: the tile's prefix, then the earlier threads' rows (the
    // inclusive scan of the thread before).
    SegVal before{prefix[blockIdx.x], 0};
    {
        __shared__ u64 pv[SC_T];
        __shared__ unsigned pf[SC_T];
        pv[threadIdx.x] = incl.v;
        pf[threadIdx.x] = incl.f;
        __syncthreads();
        if (threadIdx.x) before = seg_op<OT, F>(before, SegVal{pv[threadIdx.x - 1], pf[threadIdx.x - 1]});
    }
    u64 acc = before.v;
#pragma unroll
    for (int j = 0; j < SC_I; ++j) {
        const int64_t r = r0 + j;
        if (r >= n) break;
        const bool f = BY && s[r] != 0;
        acc = f ? v[j] : step<OT, F>(acc, v[j]);
        if (F != F_ADD) acc = wrap<OT>(acc);
        st_word<width_of(OT)>(out, r, acc);
        if (r == n - 1) carry[0] = acc;
    }
}

// Scanner of one fold. carry[0]: the output of the last row so far, the identity before any.
struct FamScan : ScannerImpl {
    vkc_type in, out;
    bool by;
    u64 *carry = nullptr;
    DeviceMem mem;
    using Launch = void (*)(vkc_ctx *, const void *, const unsigned char *, int64_t, void *, u64 *, u64 *, unsigned *);
    Launch launch = nullptr;
    vkc_status update(vkc_ctx *ctx, const Arg *args, int nargs, vkc_array *o) override {
        vkc_status st;
        const int want = by ? 2 : 1;
        if (nargs != want) return fail(ctx, VKC_RUNTIME, arity_error(want, nargs));
        if (!rows_arg(ctx, args[0], in, &st)) return st;
        if (by && !rows_arg(ctx, args[1], VKC_BOOL, &st)) return st;
        if (o->type != out) return fail(ctx, VKC_RUNTIME, "bad destination");
        const int64_t n = args[0].len();
        if (o->len != n || (by && args[1].len() != n))
            return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(n) + " rows for a destination of " +
                                              std::to_string(o->len) + " rows");
        if (n == 0) return VKC_OK;
        const int64_t tiles = (n + SC_ROWS - 1) / SC_ROWS;
        void *p;
        if ((st = scratch(ctx, static_cast<size_t>(tiles) * 12 + 256, &p))) return st;
        launch(ctx, args[0].a->data(), by ? static_cast<const unsigned char *>(args[1].a->data()) : nullptr, n,
               o->data(), carry, static_cast<u64 *>(p), reinterpret_cast<unsigned *>(static_cast<u64 *>(p) + tiles));
        return launched(ctx, "family_scan");
    }
};

template <vkc_type IT, vkc_type OT, int F, bool BY>
void launch_scan_fam(vkc_ctx *ctx, const void *x, const unsigned char *s, int64_t n, void *out, u64 *carry,
                     u64 *aggv, unsigned *aggf) {
    const int tiles = static_cast<int>((n + SC_ROWS - 1) / SC_ROWS);
    fam_scan_agg<IT, OT, F, BY><<<tiles, SC_T, 0, ctx->stream>>>(x, s, n, aggv, aggf);
    fam_scan_prefix<OT, F><<<1, 1024, 0, ctx->stream>>>(aggv, aggf, tiles, carry);
    fam_scan_apply<IT, OT, F, BY><<<tiles, SC_T, 0, ctx->stream>>>(x, s, n, aggv, out, carry);
}

template <vkc_type IT, int F, bool BY> ScannerImpl *make_scan_fam(vkc_ctx *ctx) {
    constexpr vkc_type OT = F == F_ADD ? sum_type(IT) : IT;
    auto *s = new FamScan;
    s->in = IT;
    s->out = OT;
    s->by = BY;
    s->launch = launch_scan_fam<IT, OT, F, BY>;
    if (cudaMallocAsync(reinterpret_cast<void **>(&s->carry), 8, ctx->stream) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return nullptr;
    }
    s->mem.ptr = s->carry;
    s->mem.box = ctx->box;
    const u64 id = identity<OT, F>();
    void *h;
    if (pinned(ctx, 8, &h) || cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return nullptr;
    }
    memcpy(h, &id, 8);
    if (cudaMemcpyAsync(s->carry, h, 8, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return nullptr;
    }
    return s;
}

// prev_T (scan.rs:16-73): out[0] is the fill on the first update, else the last row of the
// previous update; out[i] = x[i - 1]. carry: [0] last row, [1] seen.
template <int W>
__global__ void fam_prev_kernel(const void *x, void *out, int64_t n, u64 fill, const u64 *carry) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        u64 v;
        if (i == 0) v = carry[1] ? carry[0] : fill;
        else if (W == 8) v = static_cast<const u64 *>(x)[i - 1];
        else if (W == 4) v = static_cast<const unsigned *>(x)[i - 1];
        else v = static_cast<const unsigned char *>(x)[i - 1];
        st_word<W>(out, i, v);
    }
}
template <int W> __global__ void fam_prev_carry(const void *x, int64_t n, u64 *carry) {
    carry[0] = W == 8 ? static_cast<const u64 *>(x)[n - 1]
                      : (W == 4 ? static_cast<const unsigned *>(x)[n - 1] : static_cast<const unsigned char *>(x)[n - 1]);
    carry[1] = 1;
}

struct FamPrev : ScannerImpl {
    vkc_type t;
    u64 *carry = nullptr;
    DeviceMem mem;
    vkc_status update(vkc_ctx *ctx, const Arg *args, int nargs, vkc_array *o) override {
        vkc_status st;
        if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
        if (!rows_arg(ctx, args[0], t, &st) || !splat_arg(ctx, args[1], t, &st)) return st;
        const int64_t n = args[0].len();
        if (o->len != n)
            return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(n) + " rows for a destination of " +
                                              std::to_string(o->len) + " rows");
        if (n == 0) return VKC_OK;
        const int grid = stream_grid(ctx, n, 256, 8, 2048);
        const void *x = args[0].a->data();
        const u64 fill = args[1].s.bits;
        switch (width_of(t)) {
        case 8:
            fam_prev_kernel<8><<<grid, 256, 0, ctx->stream>>>(x, o->data(), n, fill, carry);
            fam_prev_carry<8><<<1, 1, 0, ctx->stream>>>(x, n, carry);
            break;
        case 4:
            fam_prev_kernel<4><<<grid, 256, 0, ctx->stream>>>(x, o->data(), n, fill, carry);
            fam_prev_carry<4><<<1, 1, 0, ctx->stream>>>(x, n, carry);
            break;
        default:
            fam_prev_kernel<1><<<grid, 256, 0, ctx->stream>>>(x, o->data(), n, fill, carry);
            fam_prev_carry<1><<<1, 1, 0, ctx->stream>>>(x, n, carry);
            break;
        }
        return launched(ctx, "family_prev");
    }
};

template <vkc_type T> ScannerImpl *make_prev_fam(vkc_ctx *ctx) {
    auto *s = new FamPrev;
    s->t = T;
    if (cudaMallocAsync(reinterpret_cast<void **>(&s->carry), 16, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(s->carry, 0, 16, ctx->stream) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return nullptr;
    }
    s->mem.ptr = s->carry;
    s->mem.box = ctx->box;
    return s;
}

// ------------------------------------------------------------------ reduce_into

// Each bucket word starts at the fold's identity; rows step their bucket with an atomic of the
// fold (a compare-and-swap loop for products and float extremes), then the words narrow to
// the output type. The fold is order-free, so the result is the reference's sequential one.
template <vkc_type IT, vkc_type OT, int F>
__device__ __forceinline__ void bucket_step(u64 *p, u64 v) {
    if (F == F_ADD) atomicAdd(p, v);
    else if (F == F_AND) atomicAnd(p, v);
    else if (F == F_OR) atomicOr(p, v);
    else if (F == F_XOR) atomicXor(p, v);
    else if ((F == F_MIN || F == F_MAX) && is_signed_t(IT)) {
        if (F == F_MIN) atomicMin(reinterpret_cast<long long *>(p), static_cast<long long>(v));
        else atomicMax(reinterpret_cast<long long *>(p), static_cast<long long>(v));
    } else if ((F == F_MIN || F == F_MAX) && !is_float(IT)) {
        if (F == F_MIN) atomicMin(p, v);
        else atomicMax(p, v);
    } else {
        u64 old = *reinterpret_cast<volatile u64 *>(p);
        for (;;) {
            const u64 want = F == F_MUL ? wrap<IT>(old * v) : step<IT, F>(old, v);
            if (want == old) break;
            const u64 seen = atomicCAS(p, old, want);
            if (seen == old) break;
            old = seen;
        }
    }
}

template <vkc_type OT, int F> __global__ void fam_bucket_init(u64 *w, int64_t nb) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < nb; i += stride)
        w[i] = identity<OT, F>();
}

template <vkc_type IT, vkc_type OT, int F>
__global__ void __launch_bounds__(256) fam_bucket_kernel(const long long *keys, const void *vals, int64_t n, u64 *w) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        bucket_step<IT, OT, F>(w + keys[i], ld_word<IT>(vals, i));
}

template <int W> __global__ void fam_narrow(const u64 *w, void *out, int64_t nb) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < nb; i += stride)
        st_word<W>(out, i, w[i]);
}

// index.rs:194-222 (ReduceInto): the values' kind, then checked_keys (:116-130: the keys' kind,
// the count, a negative count, the first key out of range), then the lengths, then the result.
template <vkc_type IT, int F>
vkc_status reduce_into_fam(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    constexpr vkc_type OT = F == F_ADD ? sum_type(IT) : IT;
    vkc_status st;
    if (nargs != 3) return fail(ctx, VKC_RUNTIME, arity_error(3, nargs));
    if (!array_arg(ctx, args[1], IT, &st)) return st;
    int64_t nb;
    if (!array_arg(ctx, args[0], VKC_I64, &st) || !i64_arg(ctx, args[2], &nb, &st)) return st;
    if (nb < 0) return fail(ctx, VKC_RUNTIME, "negative bucket count " + std::to_string(nb));
    const vkc_array *keys = args[0].array, *vals = args[1].array;
    const int64_t n = keys->len;
    const auto *k = static_cast<const long long *>(keys->data());
    bool found;
    if ((st = bucket_key_error(ctx, k, n, nb, &found)) || found) return st;
    if (vals->len != n)
        return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(n) + " keys for " + std::to_string(vals->len) +
                                          " values");
    vkc_array *o;
    if ((st = new_array(ctx, OT, nb, false, &o))) return st;
    if (nb > 0) {
        u64 *w = static_cast<u64 *>(o->data());
        vkc_array *tmp = nullptr;
        if (width_of(OT) != 8) {
            if ((st = new_array(ctx, VKC_U64, nb, false, &tmp))) {
                vkc_array_release(o);
                return st;
            }
            w = static_cast<u64 *>(tmp->data());
        }
        const int g0 = stream_grid(ctx, nb, 256, 8, 2048);
        fam_bucket_init<OT, F><<<g0, 256, 0, ctx->stream>>>(w, nb);
        if (n > 0) {
            const int g = stream_grid(ctx, n, 256, 8, 2048);
            fam_bucket_kernel<IT, OT, F><<<g, 256, 0, ctx->stream>>>(k, vals->data(), n, w);
        }
        if (tmp) {
            if (width_of(OT) == 4) fam_narrow<4><<<g0, 256, 0, ctx->stream>>>(w, o->data(), nb);
            else fam_narrow<1><<<g0, 256, 0, ctx->stream>>>(w, o->data(), nb);
            vkc_array_release(tmp);
        }
        if ((st = launched(ctx, "family_reduce_into"))) {
            vkc_array_release(o);
            return st;
        }
    }
    out->kind = VKC_VALUE_ARRAY;
    out->array = o;
    return VKC_OK;
}

// ------------------------------------------------------------------ filter on other types

// filter_<cmp>_T (fused.rs:214-236): the rows with x <cmp> c, in order, through compress_T with
// the comparison's mask.
template <vkc_type T>
__global__ void fam_mask_kernel(const void *x, int64_t n, int cmp, u64 c, unsigned char *m) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        m[i] = cmp_test<T>(cmp, ld_word<T>(x, i), c) ? 1 : 0;
}

template <vkc_type T, int C>
vkc_status filter_fam(vkc_ctx *ctx, const Arg *args, int nargs, int64_t base, Builder *out) {
    vkc_status st;
    if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
    if (!rows_arg(ctx, args[0], T, &st) || !splat_arg(ctx, args[1], T, &st)) return st;
    const int64_t n = args[0].len();
    if (n == 0) return VKC_OK;
    vkc_array *m;
    if ((st = new_array(ctx, VKC_BOOL, n, false, &m))) return st;
    const int g = stream_grid(ctx, n, 256, 8, 2048);
    fam_mask_kernel<T><<<g, 256, 0, ctx->stream>>>(args[0].a->data(), n, C, scalar_word(T, args[1].s),
                                                   static_cast<unsigned char *>(m->data()));
    if ((st = launched(ctx, "family_mask"))) {
        vkc_array_release(m);
        return st;
    }
    static const KernelDef *comp = nullptr;
    if (!comp) comp = kernel_def((std::string("compress_") + type_name(T)).c_str());
    Arg ca[2] = {args[0], Arg{true, m, vkc_scalar{}}};
    st = comp->sel(ctx, ca, 2, base, out);
    vkc_array_release(m);
    return st;
}

// ------------------------------------------------------------------ whole kernels

// Widens keys to i64 for the i64 entries: for argsort an image whose i64 order is the key
// order (u64: flip the top bit; i32 and u8: the value), for group ids any one-to-one image.
template <vkc_type T, bool ORDER>
__global__ void fam_widen_kernel(const void *x, int64_t n, long long *o) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        u64 w = ld_word<T>(x, i);
        if (ORDER && T == VKC_U64) w ^= 1ull << 63;
        o[i] = static_cast<long long>(w);
    }
}

template <vkc_type T, bool ORDER> vkc_status widen(vkc_ctx *ctx, const vkc_array *a, vkc_array **out) {
    vkc_status st;
    if ((st = new_array(ctx, VKC_I64, a->len, false, out))) return st;
    if (a->len > 0) {
        const int g = stream_grid(ctx, a->len, 256, 8, 2048);
        fam_widen_kernel<T, ORDER><<<g, 256, 0, ctx->stream>>>(a->data(), a->len, static_cast<long long *>((*out)->data()));
        if ((st = launched(ctx, "family_widen"))) {
            vkc_array_release(*out);
            return st;
        }
    }
    return VKC_OK;
}

// argsort_T (index.rs:159-173): the stable ascending positions, those of the widened keys.
template <vkc_type T> vkc_status argsort_fam(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 1) return fail(ctx, VKC_RUNTIME, arity_error(1, nargs));
    if (!array_arg(ctx, args[0], T, &st)) return st;
    vkc_array *w;
    if ((st = widen<T, true>(ctx, args[0].array, &w))) return st;
    static const KernelDef *d = kernel_def("argsort_i64");
    vkc_value a{};
    a.kind = VKC_VALUE_ARRAY;
    a.array = w;
    st = d->whole(ctx, &a, 1, out);
    vkc_array_release(w);
    return st;
}

// group_id_T (group.rs:259-274): ids by first occurrence depend only on which rows are equal.
template <vkc_type T> vkc_status group_id_fam(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 1) return fail(ctx, VKC_RUNTIME, arity_error(1, nargs));
    if (!array_arg(ctx, args[0], T, &st)) return st;
    vkc_array *w;
    if ((st = widen<T, false>(ctx, args[0].array, &w))) return st;
    static const KernelDef *d = kernel_def("group_id_i64");
    vkc_value a{};
    a.kind = VKC_VALUE_ARRAY;
    a.array = w;
    st = d->whole(ctx, &a, 1, out);
    vkc_array_release(w);
    return st;
}

// group_id2_A_B (group.rs:276-299): both columns' kinds, then the lengths, as the reference.
template <vkc_type A, vkc_type B> vkc_status group_id2_fam(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
    if (!array_arg(ctx, args[0], A, &st) || !array_arg(ctx, args[1], B, &st)) return st;
    if (args[0].array->len != args[1].array->len)
        return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(args[0].array->len) + " vs " +
                                          std::to_string(args[1].array->len));
    vkc_array *wa, *wb;
    if ((st = widen<A, false>(ctx, args[0].array, &wa))) return st;
    if ((st = widen<B, false>(ctx, args[1].array, &wb))) {
        vkc_array_release(wa);
        return st;
    }
    static const KernelDef *d = kernel_def("group_id2_i64_i64");
    vkc_value a[2]{};
    a[0].kind = a[1].kind = VKC_VALUE_ARRAY;
    a[0].array = wa;
    a[1].array = wb;
    st = d->whole(ctx, a, 2, out);
    vkc_array_release(wa);
    vkc_array_release(wb);
    return st;
}

// fill_T (construct.rs:49-61): n copies of v; "negative length" for n < 0, the value's type,
// then the size.
template <int W> __global__ void fam_fill_kernel(void *o, int64_t n, u64 v) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) st_word<W>(o, i, v);
}

template <vkc_type T> vkc_status fill_fam(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
    int64_t n;
    if (!i64_arg(ctx, args[0], &n, &st)) return st;
    if (n < 0) return fail(ctx, VKC_RUNTIME, "negative length " + std::to_string(n));
    if (args[1].kind != VKC_VALUE_SCALAR || args[1].scalar.type != T)
        return fail(ctx, VKC_RUNTIME, std::string("expected ") + type_name(T) + ", got " + value_type_name(args[1]));
    vkc_array *o;
    if ((st = new_array(ctx, T, n, false, &o))) return st;
    if (n > 0) {
        const int g = stream_grid(ctx, n, 256, 8, 4096);
        const u64 v = args[1].scalar.bits;
        switch (width_of(T)) {
        case 8: fam_fill_kernel<8><<<g, 256, 0, ctx->stream>>>(o->data(), n, v); break;
        case 4: fam_fill_kernel<4><<<g, 256, 0, ctx->stream>>>(o->data(), n, v); break;
        default: fam_fill_kernel<1><<<g, 256, 0, ctx->stream>>>(o->data(), n, v); break;
        }
        if ((st = launched(ctx, "family_fill"))) {
            vkc_array_release(o);
            return st;
        }
    }
    out->kind = VKC_VALUE_ARRAY;
    out->array = o;
    return VKC_OK;
}

// slice_T (index.rs:240-258): a view of rows start..end, or "slice s..e out of range for length n".
template <vkc_type T> vkc_status slice_fam(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 3) return fail(ctx, VKC_RUNTIME, arity_error(3, nargs));
    if (!array_arg(ctx, args[0], T, &st)) return st;
    int64_t s, e;
    if (!i64_arg(ctx, args[1], &s, &st) || !i64_arg(ctx, args[2], &e, &st)) return st;
    const int64_t len = args[0].array->len;
    if (s < 0 || e < 0 || s > e || e > len)
        return fail(ctx, VKC_RUNTIME, "slice " + std::to_string(s) + ".." + std::to_string(e) +
                                          " out of range for length " + std::to_string(len));
    vkc_array *v;
    if ((st = vkc_array_slice(ctx, args[0].array, s, e - s, &v))) return st;
    out->kind = VKC_VALUE_ARRAY;
    out->array = v;
    return VKC_OK;
}

// same_len_T (construct.rs:108-120): the array itself when its length is n.
template <vkc_type T> vkc_status same_len_fam(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
    if (!array_arg(ctx, args[0], T, &st)) return st;
    int64_t n;
    if (!i64_arg(ctx, args[1], &n, &st)) return st;
    const int64_t len = args[0].array->len;
    if (len != n) return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(len) + " vs " + std::to_string(n));
    vkc_array_retain(args[0].array);
    out->kind = VKC_VALUE_ARRAY;
    out->array = args[0].array;
    return VKC_OK;
}

// ------------------------------------------------------------------ registration helpers

InSpec arr(vkc_type t) { return InSpec{IN_ARRAY, t}; }
InSpec sca(vkc_type t) { return InSpec{IN_SCALAR, t}; }

void add_red(std::vector<KernelDef> &t, const std::string &name, std::vector<InSpec> in, vkc_type out, uint64_t cost,
             ReducerMake make) {
    KernelDef d{name, VKC_REDUCTION, std::move(in), false, out, cost};
    d.red = make;
    t.push_back(d);
}
void add_whole(std::vector<KernelDef> &t, const std::string &name, std::vector<InSpec> in, vkc_type out, uint64_t cost,
               WholeFn f, bool out_array = true) {
    KernelDef d{name, VKC_WHOLE, std::move(in), out_array, out, cost};
    d.whole = f;
    t.push_back(d);
}
void add_scan(std::vector<KernelDef> &t, const std::string &name, std::vector<InSpec> in, vkc_type out, uint64_t cost,
              ScanMake make) {
    KernelDef d{name, VKC_SCAN, std::move(in), true, out, cost};
    d.scan = make;
    t.push_back(d);
}

bool has(const std::vector<KernelDef> &t, const std::string &name) {
    for (const KernelDef &d : t)
        if (d.name == name) return true;
    return false;
}

// Reductions of one numeric type (reduce.rs:664-686): add (sum type), mul, min, max, argmin,
// argmax, each with cost = the input width.
template <vkc_type T> void reg_numeric(std::vector<KernelDef> &t) {
    const std::string n = type_name(T);
    const uint64_t w = width_of(T);
    if (is_float(T)) {
        add_red(t, "reduce_add_" + n, {arr(T)}, T, w, [](vkc_ctx *c) { return make_chain<T, R_PLAIN, false, 1>(c, 0); });
        add_red(t, "reduce_mul_" + n, {arr(T)}, T, w, [](vkc_ctx *c) { return make_chain<T, R_PLAIN, true, 1>(c, 0); });
    } else {
        add_red(t, "reduce_add_" + n, {arr(T)}, sum_type(T), w,
                [](vkc_ctx *c) { return make_fold<T, F_ADD, R_PLAIN, 1>(c, sum_type(T), 0, false, ""); });
        add_red(t, "reduce_mul_" + n, {arr(T)}, T, w,
                [](vkc_ctx *c) { return make_fold<T, F_MUL, R_PLAIN, 1>(c, T, 0, false, ""); });
    }
    add_red(t, "reduce_min_" + n, {arr(T)}, T, w,
            [](vkc_ctx *c) { return make_fold<T, F_MIN, R_PLAIN, 1>(c, T, 0, true, "reduce_min"); });
    add_red(t, "reduce_max_" + n, {arr(T)}, T, w,
            [](vkc_ctx *c) { return make_fold<T, F_MAX, R_PLAIN, 1>(c, T, 0, true, "reduce_max"); });
    add_red(t, "argmin_" + n, {arr(T)}, VKC_I64, w, make_arg<T, false>);
    add_red(t, "argmax_" + n, {arr(T)}, VKC_I64, w, make_arg<T, true>);
}

// Bit folds (reduce.rs:688-702, :704-712 for bool).
template <vkc_type T> void reg_bits(std::vector<KernelDef> &t) {
    const std::string n = type_name(T);
    const uint64_t w = width_of(T);
    add_red(t, "reduce_and_" + n, {arr(T)}, T, w, [](vkc_ctx *c) { return make_fold<T, F_AND, R_PLAIN, 1>(c, T, 0, false, ""); });
    add_red(t, "reduce_or_" + n, {arr(T)}, T, w, [](vkc_ctx *c) { return make_fold<T, F_OR, R_PLAIN, 1>(c, T, 0, false, ""); });
    add_red(t, "reduce_xor_" + n, {arr(T)}, T, w, [](vkc_ctx *c) { return make_fold<T, F_XOR, R_PLAIN, 1>(c, T, 0, false, ""); });
}

// Fused kernels of one type (fused.rs:290-371): dot (2 widths), sumsq (1), count_<cmp> (1),
// filter_<cmp> (2), condsum_<cmp> (1); sums in the sum type.
template <vkc_type T, int C> void reg_cmp(std::vector<KernelDef> &t) {
    const std::string n = type_name(T), c = CMP_NAME[C];
    const uint64_t w = width_of(T);
    add_red(t, "count_" + c + "_" + n, {arr(T), sca(T)}, VKC_I64, w,
            [](vkc_ctx *x) { return make_fold<T, F_ADD, R_PRED, 2>(x, VKC_I64, C, false, ""); });
    KernelDef f{"filter_" + c + "_" + n, VKC_SELECTION, {arr(T), sca(T)}, true, T, 2 * w};
    f.sel = filter_fam<T, C>;
    t.push_back(f);
    if (is_float(T))
        add_red(t, "condsum_" + c + "_" + n, {arr(T), sca(T), sca(T)}, T, w,
                [](vkc_ctx *x) { return make_chain<T, R_COND, false, 3>(x, C); });
    else
        add_red(t, "condsum_" + c + "_" + n, {arr(T), sca(T), sca(T)}, sum_type(T), w,
                [](vkc_ctx *x) { return make_fold<T, F_ADD, R_COND, 3>(x, sum_type(T), C, false, ""); });
}

template <vkc_type T> void reg_fused(std::vector<KernelDef> &t) {
    const std::string n = type_name(T);
    const uint64_t w = width_of(T);
    if (is_float(T)) {
        add_red(t, "dot_" + n, {arr(T), arr(T)}, T, 2 * w, [](vkc_ctx *c) { return make_chain<T, R_DOT, false, 2>(c, 0); });
        add_red(t, "sumsq_" + n, {arr(T)}, T, w, [](vkc_ctx *c) { return make_chain<T, R_SUMSQ, false, 1>(c, 0); });
    } else {
        add_red(t, "dot_" + n, {arr(T), arr(T)}, sum_type(T), 2 * w,
                [](vkc_ctx *c) { return make_fold<T, F_ADD, R_DOT, 2>(c, sum_type(T), 0, false, ""); });
        add_red(t, "sumsq_" + n, {arr(T)}, sum_type(T), w,
                [](vkc_ctx *c) { return make_fold<T, F_ADD, R_SUMSQ, 1>(c, sum_type(T), 0, false, ""); });
    }
    reg_cmp<T, 0>(t);
    reg_cmp<T, 1>(t);
    reg_cmp<T, 2>(t);
    reg_cmp<T, 3>(t);
    reg_cmp<T, 4>(t);
    reg_cmp<T, 5>(t);
}

// scan_<f>_T, scan_by_<f>_T, reduce_into_<f>_T (scan.rs:330-385): costs in+out widths, +1 for
// scan_by, 8 + in + 2 out for reduce_into.
template <vkc_type T, int F> void reg_fold(std::vector<KernelDef> &t) {
    constexpr vkc_type OT = F == F_ADD ? sum_type(T) : T;
    const std::string n = std::string(FOLD_NAMES[F]) + "_" + type_name(T);
    const uint64_t cost = width_of(T) + width_of(OT);
    if (!has(t, "scan_" + n)) add_scan(t, "scan_" + n, {arr(T)}, OT, cost, make_scan_fam<T, F, false>);
    if (!has(t, "scan_by_" + n)) add_scan(t, "scan_by_" + n, {arr(T), arr(VKC_BOOL)}, OT, cost + 1, make_scan_fam<T, F, true>);
    if (!has(t, "reduce_into_" + n))
        add_whole(t, "reduce_into_" + n, {arr(VKC_I64), arr(T), sca(VKC_I64)}, OT, 8 + width_of(T) + 2 * width_of(OT),
                  reduce_into_fam<T, F>);
}

template <vkc_type T> void reg_int_folds(std::vector<KernelDef> &t) {
    reg_fold<T, F_ADD>(t);
    reg_fold<T, F_MUL>(t);
    reg_fold<T, F_MIN>(t);
    reg_fold<T, F_MAX>(t);
    reg_fold<T, F_AND>(t);
    reg_fold<T, F_OR>(t);
    reg_fold<T, F_XOR>(t);
}

template <vkc_type T> void reg_prev(std::vector<KernelDef> &t) {
    const std::string n = std::string("prev_") + type_name(T);
    if (!has(t, n)) add_scan(t, n, {arr(T), sca(T)}, T, 2 * width_of(T), make_prev_fam<T>);
}

template <vkc_type T> void reg_whole_of(std::vector<KernelDef> &t) {
    const std::string n = type_name(T);
    const uint64_t w = width_of(T);
    add_whole(t, "fill_" + n, {sca(VKC_I64), sca(T)}, T, w, fill_fam<T>);
    add_whole(t, "slice_" + n, {arr(T), sca(VKC_I64), sca(VKC_I64)}, T, 0, slice_fam<T>);
    add_whole(t, "same_len_" + n, {arr(T), sca(VKC_I64)}, T, 0, same_len_fam<T>);
}

template <vkc_type A> void reg_group2(std::vector<KernelDef> &t) {
    const vkc_type bs[4] = {VKC_I64, VKC_U64, VKC_I32, VKC_U8};
    const WholeFn fs[4] = {group_id2_fam<A, VKC_I64>, group_id2_fam<A, VKC_U64>, group_id2_fam<A, VKC_I32>,
                           group_id2_fam<A, VKC_U8>};
    for (int i = 0; i < 4; ++i) {
        const std::string n = std::string("group_id2_") + type_name(A) + "_" + type_name(bs[i]);
        if (!has(t, n)) add_whole(t, n, {arr(A), arr(bs[i])}, VKC_I64, width_of(A) + width_of(bs[i]) + 8, fs[i]);
    }
}

}  // namespace

void register_families(std::vector<KernelDef> &t) {
    // reduce.rs:714-726
    reg_numeric<VKC_F32>(t);
    reg_numeric<VKC_I32>(t);
    reg_numeric<VKC_U8>(t);
    reg_numeric<VKC_U64>(t);
    add_red(t, "reduce_mul_f64", {arr(VKC_F64)}, VKC_F64, 8,
            [](vkc_ctx *c) { return make_chain<VKC_F64, R_PLAIN, true, 1>(c, 0); });
    add_red(t, "reduce_mul_i64", {arr(VKC_I64)}, VKC_I64, 8,
            [](vkc_ctx *c) { return make_fold<VKC_I64, F_MUL, R_PLAIN, 1>(c, VKC_I64, 0, false, ""); });
    reg_bits<VKC_I64>(t);
    reg_bits<VKC_I32>(t);
    reg_bits<VKC_U8>(t);
    reg_bits<VKC_U64>(t);
    add_red(t, "reduce_and_bool", {arr(VKC_BOOL)}, VKC_BOOL, 1,
            [](vkc_ctx *c) { return make_fold<VKC_BOOL, F_AND, R_PLAIN, 1>(c, VKC_BOOL, 0, false, ""); });
    add_red(t, "reduce_or_bool", {arr(VKC_BOOL)}, VKC_BOOL, 1,
            [](vkc_ctx *c) { return make_fold<VKC_BOOL, F_OR, R_PLAIN, 1>(c, VKC_BOOL, 0, false, ""); });
    add_red(t, "reduce_xor_bool", {arr(VKC_BOOL)}, VKC_BOOL, 1,
            [](vkc_ctx *c) { return make_fold<VKC_BOOL, F_XOR, R_PLAIN, 1>(c, VKC_BOOL, 0, false, ""); });
    add_red(t, "any", {arr(VKC_BOOL)}, VKC_BOOL, 1,
            [](vkc_ctx *c) { return make_fold<VKC_BOOL, F_OR, R_PLAIN, 1>(c, VKC_BOOL, 0, false, ""); });
    add_red(t, "all", {arr(VKC_BOOL)}, VKC_BOOL, 1,
            [](vkc_ctx *c) { return make_fold<VKC_BOOL, F_AND, R_PLAIN, 1>(c, VKC_BOOL, 0, false, ""); });
    // fused.rs:373-379
    reg_fused<VKC_F32>(t);
    reg_fused<VKC_I64>(t);
    reg_fused<VKC_U64>(t);
    reg_fused<VKC_I32>(t);
    // scan.rs:424-439
    reg_int_folds<VKC_I64>(t);
    reg_int_folds<VKC_U64>(t);
    reg_int_folds<VKC_I32>(t);
    reg_int_folds<VKC_U8>(t);
    reg_fold<VKC_F64, F_MIN>(t);
    reg_fold<VKC_F64, F_MAX>(t);
    reg_fold<VKC_F32, F_MIN>(t);
    reg_fold<VKC_F32, F_MAX>(t);
    reg_fold<VKC_BOOL, F_AND>(t);
    reg_fold<VKC_BOOL, F_OR>(t);
    reg_fold<VKC_BOOL, F_XOR>(t);
    reg_prev<VKC_F64>(t);
    reg_prev<VKC_F32>(t);
    reg_prev<VKC_U64>(t);
    reg_prev<VKC_I32>(t);
    reg_prev<VKC_U8>(t);
    reg_prev<VKC_BOOL>(t);
    // index.rs:290-325, group.rs:352-363, construct.rs:214-270
    add_whole(t, "argsort_u64", {arr(VKC_U64)}, VKC_I64, 16, argsort_fam<VKC_U64>);
    add_whole(t, "argsort_i32", {arr(VKC_I32)}, VKC_I64, 12, argsort_fam<VKC_I32>);
    add_whole(t, "argsort_u8", {arr(VKC_U8)}, VKC_I64, 9, argsort_fam<VKC_U8>);
    add_whole(t, "group_id_u64", {arr(VKC_U64)}, VKC_I64, 16, group_id_fam<VKC_U64>);
    add_whole(t, "group_id_i32", {arr(VKC_I32)}, VKC_I64, 12, group_id_fam<VKC_I32>);
    add_whole(t, "group_id_u8", {arr(VKC_U8)}, VKC_I64, 9, group_id_fam<VKC_U8>);
    reg_group2<VKC_I64>(t);
    reg_group2<VKC_U64>(t);
    reg_group2<VKC_I32>(t);
    reg_group2<VKC_U8>(t);
    reg_whole_of<VKC_F64>(t);
    reg_whole_of<VKC_F32>(t);
    reg_whole_of<VKC_I64>(t);
    reg_whole_of<VKC_U64>(t);
    reg_whole_of<VKC_I32>(t);
    reg_whole_of<VKC_U8>(t);
    reg_whole_of<VKC_BOOL>(t);
}

}  // namespace vkc

// Reductions: count_<cmp>_f64, count, reduce_min/max and argmin/argmax on f64 and i64, and
// reduce_add_i64 (src/kernels/scalar/reduce.rs:331-468, src/kernels/scalar/fused.rs:145-179).
// The canonical float sums live in k_canon.cu.
//
// Each reducer keeps its running state in a small device buffer. An update is one kernel: every
// block folds its rows, and the last block to finish (last-block-done) folds the block
// partials into the state, so the only host sync is the download at finish.
#include <cmath>
#include <cstring>

#include "kcommon.cuh"
#include "reduce_common.h"

namespace vkc {

// ------------------------------------------------------------------ comparison ranges

CmpRange cmp_range(int cmp, double c) {
    CmpRange r{1, 0, 0};  // empty
    if (std::isnan(c)) {
        r.negate = cmp == 1;  // ne is true on everything, the others on nothing
        return r;
    }
    unsigned long long pz = 0, nz = 0x8000000000000000ull, cb;
    memcpy(&cb, &c, 8);
    const bool zero = c == 0.0;
    auto key = [](unsigned long long b) { return key_of_bits(b); };
    switch (cmp) {
    case 0:  // eq
    case 1:  // ne
        r.lo = zero ? key(nz) : key(cb);
        r.hi = zero ? key(pz) : key(cb);
        r.negate = cmp == 1;
        break;
    case 2:  // lt: keys below c, with -0 standing for both zeros
        r.lo = KEY_NEG_INF;
        r.hi = (zero ? key(nz) : key(cb)) - 1;
        break;
    case 3:  // le
        r.lo = KEY_NEG_INF;
        r.hi = zero ? key(pz) : key(cb);
        break;
    case 4:  // gt: keys above c, with +0 standing for both zeros
        r.lo = (zero ? key(pz) : key(cb)) + 1;
        r.hi = KEY_POS_INF;
        break;
    default:  // ge
        r.lo = zero ? key(nz) : key(cb);
        r.hi = KEY_POS_INF;
        break;
    }
    return r;
}

// ------------------------------------------------------------------ count

// Counts rows with x <cmp> c (as a key range) or, for `count` over bool, nonzero bytes.
template <bool BOOL, bool POS>
__global__ void __launch_bounds__(256) count_kernel(const void *__restrict__ xv, int64_t n,
                                                    CmpRange r, unsigned long long *partials,
                                                    unsigned *done, unsigned long long *state) {
    unsigned long long c = 0;
    int64_t tid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    if (BOOL) {
        const uint8_t *x = static_cast<const uint8_t *>(xv);
        int64_t head = (16 - (reinterpret_cast<uintptr_t>(x) & 15)) & 15;
        if (head > n) head = n;
        for (int64_t i = tid; i < head; i += stride) c += x[i] != 0;
        const uint4 *x16 = reinterpret_cast<const uint4 *>(x + head);
        int64_t n16 = (n - head) >> 4;
        for (int64_t i = tid; i < n16; i += stride) {
            uint4 v = __ldcs(&x16[i]);
            unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                // A byte is nonzero when any of its bits is set.
                unsigned t = w[j] | (w[j] >> 4);
                t |= t >> 2;
                t |= t >> 1;
                c += __popc(t & 0x01010101u);
            }
        }
        for (int64_t i = head + (n16 << 4) + tid; i < n; i += stride) c += x[i] != 0;
    } else {
        const unsigned long long *x = static_cast<const unsigned long long *>(xv);
        int64_t head = (reinterpret_cast<uintptr_t>(x) & 15) ? 1 : 0;
        if (head > n) head = n;
        if (head && tid == 0) c += in_range_t<POS>(r, x[0]);
        const ulonglong2 *x2 = reinterpret_cast<const ulonglong2 *>(x + head);
        int64_t n2 = (n - head) >> 1;
        // Four independent 16-byte loads per thread in flight.
        for (int64_t i = tid; i < n2; i += 4 * stride) {
            ulonglong2 v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                v[u] = i + u * stride < n2 ? __ldcs(&x2[i + u * stride]) : make_ulonglong2(~0ull, ~0ull);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (i + u * stride < n2) c += in_range_t<POS>(r, v[u].x) + in_range_t<POS>(r, v[u].y);
        }
        if (((n - head) & 1) && tid == 0) c += in_range_t<POS>(r, x[n - 1]);
    }
    c = warp_sum(c);
    __shared__ unsigned long long ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        for (int w = 0; w < 8; ++w) s += ws[w];
        partials[blockIdx.x] = s;
    }
    if (last_block(done) && threadIdx.x < 32) {
        unsigned long long s = 0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += 32) s += partials[b];
        s = warp_sum(s);
        if (threadIdx.x == 0) *state += s;
    }
}

struct CountReducer : DevReducer {
    int cmp;  // -1 for `count` over bool
    vkc_status update(vkc_ctx *ctx, const Arg *args, int nargs) override {
        vkc_status st;
        if (cmp < 0) {
            if (nargs != 1) return fail(ctx, VKC_RUNTIME, arity_error(1, nargs));
            if (!rows_arg(ctx, args[0], VKC_BOOL, &st)) return st;
        } else {
            if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
            if (!rows_arg(ctx, args[0], VKC_F64, &st) || !splat_arg(ctx, args[1], VKC_F64, &st))
                return st;
        }
        int64_t n = args[0].len();
        if (n == 0) return VKC_OK;
        int grid = stream_grid(ctx, n, 256, tune(ctx, TK_STREAM_BLOCKS, n), cmp < 0 ? 16384 : 4096);
        void *part;
        if ((st = scratch(ctx, sizeof(unsigned long long) * grid, &part))) return st;
        auto *s = static_cast<unsigned long long *>(state);
        auto *pp = static_cast<unsigned long long *>(part);
        if (cmp < 0) {
            count_kernel<true, false><<<grid, 256, 0, ctx->stream>>>(args[0].a->data(), n, CmpRange{}, pp, ctx->counters + 1, s);
        } else {
            const CmpRange r = cmp_range(cmp, args[1].f64());
            if (pos_range(r)) count_kernel<false, true><<<grid, 256, 0, ctx->stream>>>(args[0].a->data(), n, r, pp, ctx->counters + 1, s);
            else count_kernel<false, false><<<grid, 256, 0, ctx->stream>>>(args[0].a->data(), n, r, pp, ctx->counters + 1, s);
        }
        return launched(ctx, "count");
    }
    vkc_status finish(vkc_ctx *ctx, vkc_scalar *out) override {
        unsigned long long v = 0;
        vkc_status st = download(ctx, &v, sizeof v);
        if (st) return st;
        *out = scalar_i64(static_cast<int64_t>(v));
        return VKC_OK;
    }
    vkc_status finish_into(vkc_ctx *ctx, void *dst) override { return copy_out(ctx, dst, 8); }
};

// ------------------------------------------------------------------ extremes

// State of reduce_min / reduce_max / argmin / argmax: the best key and its row, the first NaN
// row, and whether any row was seen.
struct ExtState {
    long long key;
    unsigned long long idx;
    unsigned long long nan_idx;  // ~0 when no NaN
    unsigned long long seen;
};

// Combines two candidates: for MAX the larger key, else the smaller, ties to the earlier row.
template <bool MAX>
__device__ __forceinline__ void better(long long &k, unsigned long long &i, long long k2,
                                       unsigned long long i2) {
    bool b = MAX ? (k2 > k || (k2 == k && i2 < i)) : (k2 < k || (k2 == k && i2 < i));
    if (b) {
        k = k2;
        i = i2;
    }
}

// One pass over x[0, n) at global row offset `base`. F64 rows are compared as order keys;
// NaN rows only record their first position, which decides argmin/argmax and makes min/max
// NaN. A thread visits its rows in increasing order, four 16-byte loads per step, so within a
// thread a strict comparison keeps the first index of the extreme, and a thread's position is
// kept as (step * 8 + slot) until the end.
template <bool MAX, bool F64, bool ARG>
__global__ void __launch_bounds__(256) extreme_kernel(const long long *__restrict__ x, int64_t n,
                                                      unsigned long long base, ExtState *partials,
                                                      unsigned *done, ExtState *state) {
    long long bk = MAX ? LLONG_MIN : LLONG_MAX;
    unsigned bpos = ~0u, npos = ~0u;  // best and first-NaN positions (step * 8 + slot)
    unsigned long long maxabs = 0;     // min/max only: NaN when above +inf's bits
    const int64_t tid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const int64_t head = ((reinterpret_cast<uintptr_t>(x) & 15) && n > 0) ? 1 : 0;
    const longlong2 *x2 = reinterpret_cast<const longlong2 *>(x + head);
    const int64_t n2 = (n - head) >> 1;
    unsigned step = 0;
    bool any = false;
    for (int64_t i = tid; i < n2; i += 4 * stride, ++step) {
        any = true;
        longlong2 v[4];
        bool ok[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            ok[u] = i + u * stride < n2;
            v[u] = ok[u] ? __ldcs(&x2[i + u * stride]) : make_longlong2(0, 0);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (!ok[u]) continue;
            long long e[2] = {v[u].x, v[u].y};
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                long long k = e[j];
                if (F64) {
                    const unsigned long long b = static_cast<unsigned long long>(k);
                    if (!ARG) {
                        maxabs = max(maxabs, b & 0x7fffffffffffffffull);
                        k = f64_key(b);
                    } else {
                        if ((b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) {
                            npos = min(npos, step * 8 + u * 2 + j);
                            continue;
                        }
                        k = f64_key(b);
                    }
                }
                if (ARG) {
                    if (MAX ? k > bk : k < bk) {
                        bk = k;
                        bpos = step * 8 + u * 2 + j;
                    }
                } else {
                    bk = MAX ? max(bk, k) : min(bk, k);
                }
            }
        }
    }
    // Rows: position (step, slot) of this thread is row head + 2 * (tid + (step*4 + slot/2) * stride) + slot%2.
    auto row_of = [&](unsigned p) -> unsigned long long {
        const int64_t q = tid + (static_cast<int64_t>(p >> 3) * 4 + ((p >> 1) & 3)) * stride;
        return static_cast<unsigned long long>(head + 2 * q + (p & 1));
    };
    unsigned long long bi = ~0ull, nan = ~0ull;
    if (ARG) {
        if (bpos != ~0u) bi = row_of(bpos);
        if (npos != ~0u) nan = row_of(npos);
    } else {
        if (any) bi = 0;  // a row was seen
        if (maxabs > 0x7ff0000000000000ull) nan = 0;
    }
    // The head and tail rows (views that start or end off the 16-byte grid).
    auto visit = [&](int64_t r) {
        const unsigned long long b = static_cast<unsigned long long>(x[r]);
        long long k = static_cast<long long>(b);
        if (F64) {
            if ((b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) {
                nan = ARG ? min(nan, static_cast<unsigned long long>(r)) : 0;
                return;
            }
            k = f64_key(b);
        }
        if (ARG) better<MAX>(bk, bi, k, static_cast<unsigned long long>(r));
        else {
            bk = MAX ? max(bk, k) : min(bk, k);
            bi = 0;
        }
    };
    if (tid == 0 && head) visit(0);
    if (tid == 0 && ((n - head) & 1)) visit(n - 1);
    // Warp, then block.
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        long long k2 = __shfl_xor_sync(FULL, bk, o);
        unsigned long long i2 = __shfl_xor_sync(FULL, bi, o);
        unsigned long long n2v = __shfl_xor_sync(FULL, nan, o);
        if (ARG) better<MAX>(bk, bi, k2, i2);
        else if (i2 != ~0ull) {
            bk = MAX ? max(bk, k2) : min(bk, k2);
            bi = 0;
        }
        nan = n2v < nan ? n2v : nan;
    }
    __shared__ ExtState ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = ExtState{bk, bi, nan, 0};
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; ++w) {
            if (ARG) better<MAX>(bk, bi, ws[w].key, ws[w].idx);
            else if (ws[w].idx != ~0ull) {
                bk = MAX ? max(bk, ws[w].key) : min(bk, ws[w].key);
                bi = 0;
            }
            if (ws[w].nan_idx < nan) nan = ws[w].nan_idx;
        }
        partials[blockIdx.x] = ExtState{bk, bi, nan, 0};
    }
    if (last_block(done)) {
        // The block's threads combine the partials (strided), then the warps, then warp 0 with
        // the carried state. (key, row) is a total order, so the grouping does not matter.
        long long k = MAX ? LLONG_MIN : LLONG_MAX;
        unsigned long long i = ~0ull, nn = ~0ull;
        auto take = [&](long long k2, unsigned long long i2, unsigned long long n2) {
            if (i2 != ~0ull) {
                if (ARG) better<MAX>(k, i, k2, i2);
                else {
                    k = (i == ~0ull) ? k2 : (MAX ? max(k, k2) : min(k, k2));
                    i = 0;
                }
            }
            if (n2 < nn) nn = n2;
        };
        for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
            const ExtState q = partials[b];
            take(q.key, q.idx == ~0ull ? ~0ull : q.idx + base, q.nan_idx == ~0ull ? ~0ull : q.nan_idx + base);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const long long k2 = __shfl_xor_sync(FULL, k, o);
            const unsigned long long i2 = __shfl_xor_sync(FULL, i, o), n2 = __shfl_xor_sync(FULL, nn, o);
            take(k2, i2, n2);
        }
        __syncthreads();
        if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = ExtState{k, i, nn, 0};
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < 8; ++w) take(ws[w].key, ws[w].idx, ws[w].nan_idx);
            const ExtState s = *state;
            if (s.seen) take(s.key, s.idx, s.nan_idx);
            *state = ExtState{k, i, nn, 1};
        }
    }
}

// finish on the device: the result's bits as ExtremeReducer::finish makes them (rows seen).
static __global__ void ext_result_kernel(const ExtState *s, bool arg, bool f64, unsigned long long *dst) {
    if (arg) *dst = s->nan_idx != ~0ull ? s->nan_idx : s->idx;
    else if (f64) *dst = s->nan_idx != ~0ull ? 0x7ff8000000000000ull : bits_of_key(s->key);
    else *dst = static_cast<unsigned long long>(s->key);
}

struct ExtremeReducer : DevReducer {
    bool max, arg;
    vkc_type type;
    unsigned long long consumed = 0;
    vkc_status init(vkc_ctx *ctx) { return fill(ctx, 4, 0, ~0ull, ~0ull, 0); }  // ExtState{0, ~0, ~0, 0}
    vkc_status update(vkc_ctx *ctx, const Arg *args, int nargs) override {
        vkc_status st;
        if (nargs != 1) return fail(ctx, VKC_RUNTIME, arity_error(1, nargs));
        if (!rows_arg(ctx, args[0], type, &st)) return st;
        int64_t n = args[0].len();
        if (n == 0) return VKC_OK;
        int grid = stream_grid(ctx, n, 256, tune(ctx, TK_STREAM_BLOCKS, n), 4096);
        void *part;
        if ((st = scratch(ctx, sizeof(ExtState) * grid, &part))) return st;
        auto *p = static_cast<ExtState *>(part);
        auto *s = static_cast<ExtState *>(state);
        const long long *x = static_cast<const long long *>(args[0].a->data());
        bool f = type == VKC_F64;
#define EXT_LAUNCH(MX, F, A) extreme_kernel<MX, F, A><<<grid, 256, 0, ctx->stream>>>(x, n, consumed, p, ctx->counters + 1, s)
        if (arg) {
            if (max && f) EXT_LAUNCH(true, true, true);
            else if (max) EXT_LAUNCH(true, false, true);
            else if (f) EXT_LAUNCH(false, true, true);
            else EXT_LAUNCH(false, false, true);
        } else {
            if (max && f) EXT_LAUNCH(true, true, false);
            else if (max) EXT_LAUNCH(true, false, false);
            else if (f) EXT_LAUNCH(false, true, false);
            else EXT_LAUNCH(false, false, false);
        }
#undef EXT_LAUNCH
        consumed += static_cast<unsigned long long>(n);
        return launched(ctx, "extreme");
    }
    // reduce.rs:401-411 and :454-467: empty input is an error; a NaN decides the result.
    vkc_status finish(vkc_ctx *ctx, vkc_scalar *out) override {
        ExtState s;
        vkc_status st = download(ctx, &s, sizeof s);
        if (st) return st;
        if (!s.seen) {
            std::string what = arg ? (max ? "argmax" : "argmin") : (max ? "reduce_max" : "reduce_min");
            return fail(ctx, VKC_RUNTIME, what + " of an empty array");
        }
        if (arg) {
            unsigned long long i = s.nan_idx != ~0ull ? s.nan_idx : s.idx;
            *out = scalar_i64(static_cast<int64_t>(i));
        } else if (type == VKC_F64) {
            if (s.nan_idx != ~0ull) *out = scalar_f64(NAN);
            else {
                out->type = VKC_F64;
                out->bits = bits_of_key(s.key);
            }
        } else {
            *out = scalar_i64(s.key);
        }
        return VKC_OK;
    }
    vkc_status finish_into(vkc_ctx *ctx, void *dst) override {
        if (consumed == 0) {
            std::string what = arg ? (max ? "argmax" : "argmin") : (max ? "reduce_max" : "reduce_min");
            return fail(ctx, VKC_RUNTIME, what + " of an empty array");
        }
        ext_result_kernel<<<1, 1, 0, ctx->stream>>>(static_cast<const ExtState *>(state), arg, type == VKC_F64,
                                                     static_cast<unsigned long long *>(dst));
        return launched(ctx, "extreme_result");
    }
};

// ------------------------------------------------------------------ integer sum

__global__ void __launch_bounds__(256) isum_kernel(const unsigned long long *__restrict__ x, int64_t n,
                                                   unsigned long long *partials, unsigned *done,
                                                   unsigned long long *state) {
    unsigned long long c = 0;
    int64_t tid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    int64_t head = (reinterpret_cast<uintptr_t>(x) & 15) ? 1 : 0;
    if (head > n) head = n;
    if (head && tid == 0) c += x[0];
    const ulonglong2 *x2 = reinterpret_cast<const ulonglong2 *>(x + head);
    int64_t n2 = (n - head) >> 1;
    for (int64_t i = tid; i < n2; i += 4 * stride) {
        ulonglong2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = i + u * stride < n2 ? __ldcs(&x2[i + u * stride]) : make_ulonglong2(0, 0);
#pragma unroll
        for (int u = 0; u < 4; ++u) c += v[u].x + v[u].y;
    }
    if (((n - head) & 1) && tid == 0) c += x[n - 1];
    c = warp_sum(c);
    __shared__ unsigned long long ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        for (int w = 0; w < 8; ++w) s += ws[w];
        partials[blockIdx.x] = s;
    }
    if (last_block(done) && threadIdx.x < 32) {
        unsigned long long s = 0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += 32) s += partials[b];
        s = warp_sum(s);
        if (threadIdx.x == 0) *state += s;
    }
}

// reduce.rs:331-377 (IntSum<i64>): wrapping, so any grouping gives the same bits.
struct IntSumReducer : DevReducer {
    vkc_status update(vkc_ctx *ctx, const Arg *args, int nargs) override {
        vkc_status st;
        if (nargs != 1) return fail(ctx, VKC_RUNTIME, arity_error(1, nargs));
        if (!rows_arg(ctx, args[0], VKC_I64, &st)) return st;
        int64_t n = args[0].len();
        if (n == 0) return VKC_OK;
        int grid = stream_grid(ctx, n, 256, tune(ctx, TK_STREAM_BLOCKS, n), 4096);
        void *part;
        if ((st = scratch(ctx, sizeof(unsigned long long) * grid, &part))) return st;
        isum_kernel<<<grid, 256, 0, ctx->stream>>>(
            static_cast<const unsigned long long *>(args[0].a->data()), n,
            static_cast<unsigned long long *>(part), ctx->counters + 1,
            static_cast<unsigned long long *>(state));
        return launched(ctx, "isum");
    }
    vkc_status finish(vkc_ctx *ctx, vkc_scalar *out) override {
        unsigned long long v = 0;
        vkc_status st = download(ctx, &v, sizeof v);
        if (st) return st;
        *out = scalar_i64(static_cast<int64_t>(v));
        return VKC_OK;
    }
    vkc_status finish_into(vkc_ctx *ctx, void *dst) override { return copy_out(ctx, dst, 8); }
};

// ------------------------------------------------------------------ registration

template <class R> static R *alloc_reducer(vkc_ctx *ctx, size_t bytes) {
    R *r = new R;
    if (r->alloc(ctx, bytes)) {
        delete r;
        return nullptr;
    }
    return r;
}

static const char *CMP_NAMES[6] = {"eq", "ne", "lt", "le", "gt", "ge"};

template <int C> static ReducerImpl *make_count(vkc_ctx *ctx) {
    auto *r = alloc_reducer<CountReducer>(ctx, 8);
    if (r) r->cmp = C;
    return r;
}

template <bool MAX, bool ARG, vkc_type T> static ReducerImpl *make_ext(vkc_ctx *ctx) {
    auto *r = alloc_reducer<ExtremeReducer>(ctx, sizeof(ExtState));
    if (!r) return nullptr;
    r->max = MAX;
    r->arg = ARG;
    r->type = T;
    if (r->init(ctx)) {
        delete r;
        return nullptr;
    }
    return r;
}

static ReducerImpl *make_isum(vkc_ctx *ctx) { return alloc_reducer<IntSumReducer>(ctx, 8); }

void register_reduce(std::vector<KernelDef> &t) {
    InSpec xa{IN_ARRAY, VKC_F64}, xs{IN_SCALAR, VKC_F64};
    ReducerMake counts[6] = {make_count<0>, make_count<1>, make_count<2>,
                             make_count<3>, make_count<4>, make_count<5>};
    for (int c = 0; c < 6; ++c) {
        // fused.rs:293-306: count_<cmp>_f64, cost 1 width.
        KernelDef d{std::string("count_") + CMP_NAMES[c] + "_f64", VKC_REDUCTION, {xa, xs}, false, VKC_I64, 8};
        d.red = counts[c];
        t.push_back(d);
    }
    KernelDef d{"count", VKC_REDUCTION, {InSpec{IN_ARRAY, VKC_BOOL}}, false, VKC_I64, 1};
    d.red = make_count<-1>;
    t.push_back(d);
    struct E { const char *name; ReducerMake make; vkc_type in, out; };
    const E ext[] = {
        {"reduce_min_f64", make_ext<false, false, VKC_F64>, VKC_F64, VKC_F64},
        {"reduce_max_f64", make_ext<true, false, VKC_F64>, VKC_F64, VKC_F64},
        {"argmin_f64", make_ext<false, true, VKC_F64>, VKC_F64, VKC_I64},
        {"argmax_f64", make_ext<true, true, VKC_F64>, VKC_F64, VKC_I64},
        {"reduce_min_i64", make_ext<false, false, VKC_I64>, VKC_I64, VKC_I64},
        {"reduce_max_i64", make_ext<true, false, VKC_I64>, VKC_I64, VKC_I64},
        {"argmin_i64", make_ext<false, true, VKC_I64>, VKC_I64, VKC_I64},
        {"argmax_i64", make_ext<true, true, VKC_I64>, VKC_I64, VKC_I64},
        {"reduce_add_i64", make_isum, VKC_I64, VKC_I64},
    };
    for (const E &e : ext) {
        KernelDef k{e.name, VKC_REDUCTION, {InSpec{IN_ARRAY, e.in}}, false, e.out, 8};
        k.red = e.make;
        t.push_back(k);
    }
    register_canon(t);
}

}  // namespace vkc

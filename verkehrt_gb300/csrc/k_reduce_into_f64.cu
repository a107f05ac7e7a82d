// reduce_into_add_f64: per-bucket float sums. The reference has no float reduce_into (the gap
// is listed at src/kernels/scalar/scan.rs:408-415); its tier-2 design notes
// (docs/superpowers/specs/2026-10-31-verkehrt-tier2-design.md:171-172) give the candidate order
// this entry computes: rows below b = n - n % 16 go to stripe i mod 16 of their bucket, each
// stripe adds its rows in index order from +0.0, and the 16 stripes combine pairwise (+8, +4,
// +2, +1). The bucket's rows from b on then fold into the result in index order, the canonical
// sum's tail rule (reduce.rs:77-91, finish_lanes): under that reading the notes' property holds,
// with every key equal the bucket's sum has the bits of reduce_add_f64.
//
// Equivalently, out[k] is the canonical sum of the rows with every row of another bucket read as
// +0.0: a stripe starts at +0.0 and never holds -0.0 (a sum is -0.0 only when both terms are), so
// adding +0.0 leaves it unchanged. Two paths:
//  * few buckets (at most 16): that identity, per bucket: the masked rows, then reduce_add_f64
//    (one canonical pass each, about 1 ms per bucket at 2^27 rows);
//  * otherwise: a stable argsort of the rows below b by (key, stripe), after which each stripe of
//    each bucket is a contiguous chain that one warp adds in index order (32 rows per load, the
//    adds in order through shuffles); the chains of a bucket combine pairwise, and one thread
//    folds the tail rows in order.
// Arguments and errors follow reduce_into_add_i64 (index.rs:194-222): the values' kind first,
// then the keys (checked_keys, index.rs:116-130), a length mismatch, the result's allocation.
#include "reduce_common.h"

namespace vkc {

int64_t scan_counts_sum_words(int64_t m);
void scan_counts(vkc_ctx *ctx, const unsigned *c, int64_t m, unsigned *sums, unsigned *out);
vkc_status bucket_key_error(vkc_ctx *ctx, const long long *k, int64_t n, int64_t nb, bool *found);

constexpr int64_t RIF_MASKED_BUCKETS = 16;

__device__ __forceinline__ double rif_f64(unsigned long long b) { return __longlong_as_double(static_cast<long long>(b)); }

// v[i] = x[i] for rows of bucket k, else +0.0.
__global__ void rif_mask_kernel(const long long *__restrict__ keys, const unsigned long long *__restrict__ x,
                                int64_t n, long long k, unsigned long long *__restrict__ v) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        v[i] = keys[i] == k ? x[i] : 0ull;
}

__global__ void rif_store_kernel(unsigned long long *out, int64_t k, unsigned long long bits) { out[k] = bits; }

// c[i] = key * 16 + stripe for the rows below b (keys are in range, below 2^59).
__global__ void rif_composite_kernel(const long long *__restrict__ keys, int64_t b, long long *__restrict__ c) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < b; i += stride)
        c[i] = keys[i] * 16 + (i & 15);
}

// heads[p] = 1 where a chain (one stripe of one bucket, in sorted order) starts.
__global__ void rif_heads_kernel(const long long *__restrict__ cs, int64_t b, unsigned *__restrict__ heads) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < b; p += stride)
        heads[p] = p == 0 || cs[p] != cs[p - 1];
}

// A warp per 32-row window of sorted positions: for each chain that starts in the window, in
// order, the warp reads the chain RIF_U x 32 rows at a time (all the loads in flight together;
// the rows of a chain are contiguous, so the lanes still in it are a prefix of each 32) and adds
// them in order from +0.0, every lane holding the same running sum; chain o (its ordinal among
// the heads) gets its composite key and sum. The window of the last row writes the number of
// chains.
constexpr int RIF_U = 8;
__global__ void __launch_bounds__(256) rif_chain_kernel(const long long *__restrict__ cs,
                                                        const unsigned long long *__restrict__ v, int64_t b,
                                                        const unsigned *__restrict__ heads,
                                                        const unsigned *__restrict__ ord,
                                                        long long *__restrict__ chain_key,
                                                        unsigned long long *__restrict__ chain_sum,
                                                        unsigned *__restrict__ nchains) {
    const int lane = threadIdx.x & 31;
    const int64_t p0 = (static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32;
    if (p0 >= b) return;
    const int64_t pl = p0 + lane;
    if (pl == b - 1) *nchains = ord[pl] + heads[pl];
    unsigned hm = __ballot_sync(FULL, pl < b && heads[pl] != 0);
    while (hm) {
        const int i = __ffs(hm) - 1;
        hm &= hm - 1;
        const int64_t p = p0 + i;
        const long long key = cs[p];
        double s = 0.0;
        for (int64_t q0 = p;; q0 += 32 * RIF_U) {
            bool in[RIF_U];
            double x[RIF_U];
#pragma unroll
            for (int u = 0; u < RIF_U; ++u) {
                const int64_t q = q0 + u * 32 + lane;
                in[u] = q < b && cs[q] == key;
                x[u] = q < b ? rif_f64(v[q]) : 0.0;
            }
            bool more = true;
#pragma unroll
            for (int u = 0; u < RIF_U; ++u) {
                const unsigned m = __ballot_sync(FULL, in[u]);
                if (more) {
                    const int len = m == FULL ? 32 : __ffs(~m) - 1;
#pragma unroll 8
                    for (int j = 0; j < len; ++j) s = __dadd_rn(s, __shfl_sync(FULL, x[u], j));
                    more = len == 32;
                }
            }
            if (!more) break;
        }
        if (lane == 0) {
            chain_key[ord[p]] = key;
            chain_sum[ord[p]] = static_cast<unsigned long long>(__double_as_longlong(s));
        }
    }
}

// One thread per bucket that has chains: its stripes (+0.0 where a stripe has no rows) combine
// pairwise, +8, +4, +2, +1, into out[bucket].
__global__ void rif_combine_kernel(const long long *__restrict__ chain_key,
                                   const unsigned long long *__restrict__ chain_sum,
                                   const unsigned *__restrict__ nchains, unsigned long long *__restrict__ out) {
    const int64_t m = *nchains;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t o = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; o < m; o += stride) {
        const long long k = chain_key[o] >> 4;
        if (o > 0 && (chain_key[o - 1] >> 4) == k) continue;
        double s[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) s[j] = 0.0;
        for (int64_t o2 = o; o2 < m && (chain_key[o2] >> 4) == k; ++o2) s[chain_key[o2] & 15] = rif_f64(chain_sum[o2]);
#pragma unroll
        for (int step = 8; step > 0; step >>= 1)
#pragma unroll
            for (int j = 0; j < step; ++j) s[j] = __dadd_rn(s[j], s[j + step]);
        out[k] = static_cast<unsigned long long>(__double_as_longlong(s[0]));
    }
}

// The rows from b on, fewer than 16, fold into their buckets in index order.
__global__ void rif_tail_kernel(const long long *__restrict__ keys, const unsigned long long *__restrict__ x,
                                int64_t b, int64_t n, unsigned long long *__restrict__ out) {
    for (int64_t i = b; i < n; ++i)
        out[keys[i]] = static_cast<unsigned long long>(__double_as_longlong(__dadd_rn(rif_f64(out[keys[i]]), rif_f64(x[i]))));
}

// A whole entry of the table by name, on array arguments; the result array in *res.
static vkc_status call_whole(vkc_ctx *ctx, const char *name, std::initializer_list<const vkc_array *> arrays,
                             vkc_array **res) {
    const KernelDef *d = kernel_def(name);
    if (!d || !d->whole) return fail(ctx, VKC_USAGE, std::string("no entry ") + name);
    vkc_value in[4] = {};
    int k = 0;
    for (const vkc_array *a : arrays) {
        in[k].kind = VKC_VALUE_ARRAY;
        in[k].array = const_cast<vkc_array *>(a);
        ++k;
    }
    vkc_value out{};
    vkc_status st = d->whole(ctx, in, k, &out);
    *res = st ? nullptr : out.array;
    return st;
}

// The masked path: for each bucket, reduce_add_f64 of the rows with the others read as +0.0.
static vkc_status rif_masked(vkc_ctx *ctx, const long long *keys, const unsigned long long *x, int64_t n,
                             int64_t nb, unsigned long long *out) {
    vkc_array *v;
    vkc_status st = new_array(ctx, VKC_F64, n, false, &v);
    if (st) return st;
    const KernelDef *sum = kernel_def("reduce_add_f64");
    for (int64_t k = 0; k < nb && !st; ++k) {
        rif_mask_kernel<<<stream_grid(ctx, n, 256, 8, 4096), 256, 0, ctx->stream>>>(
            keys, x, n, k, static_cast<unsigned long long *>(v->data()));
        if ((st = launched(ctx, "rif_mask"))) break;
        ReducerImpl *r = sum->red(ctx);
        if (!r) {
            st = VKC_ALLOC;
            break;
        }
        Arg a{true, v, {}};
        vkc_scalar s{};
        st = r->update(ctx, &a, 1);
        if (!st) st = r->finish(ctx, &s);
        delete r;
        if (st) break;
        rif_store_kernel<<<1, 1, 0, ctx->stream>>>(out, k, s.bits);
        st = launched(ctx, "rif_store");
    }
    vkc_array_release(v);
    return st;
}

// The sorted path over the rows below b (b > 0).
static vkc_status rif_sorted(vkc_ctx *ctx, const vkc_array *keys, const vkc_array *vals, int64_t b,
                             unsigned long long *out) {
    vkc_array *c = nullptr, *perm = nullptr, *cs = nullptr, *v = nullptr, *heads = nullptr, *ord = nullptr,
              *sums = nullptr, *ckey = nullptr, *csum = nullptr;
    auto done = [&](vkc_status st) {
        for (vkc_array *a : {c, perm, cs, v, heads, ord, sums, ckey, csum})
            if (a) vkc_array_release(a);
        return st;
    };
    vkc_status st;
    if ((st = new_array(ctx, VKC_I64, b, false, &c))) return done(st);
    const int grid = stream_grid(ctx, b, 256, 8, 4096);
    rif_composite_kernel<<<grid, 256, 0, ctx->stream>>>(static_cast<const long long *>(keys->data()), b,
                                                        static_cast<long long *>(c->data()));
    if ((st = launched(ctx, "rif_composite"))) return done(st);
    if ((st = call_whole(ctx, "argsort_i64", {c}, &perm))) return done(st);
    if ((st = call_whole(ctx, "gather_i64", {c, perm}, &cs))) return done(st);
    if ((st = call_whole(ctx, "gather_f64", {vals, perm}, &v))) return done(st);
    const int64_t sw = scan_counts_sum_words(b);
    if ((st = new_array(ctx, VKC_I32, b, false, &heads)) || (st = new_array(ctx, VKC_I32, b, false, &ord)) ||
        (st = new_array(ctx, VKC_I32, sw + 1, false, &sums)) || (st = new_array(ctx, VKC_I64, b, false, &ckey)) ||
        (st = new_array(ctx, VKC_F64, b, false, &csum)))
        return done(st);
    auto *h = static_cast<unsigned *>(heads->data());
    auto *od = static_cast<unsigned *>(ord->data());
    auto *nchains = static_cast<unsigned *>(sums->data()) + sw;
    const auto *csp = static_cast<const long long *>(cs->data());
    rif_heads_kernel<<<grid, 256, 0, ctx->stream>>>(csp, b, h);
    scan_counts(ctx, h, b, static_cast<unsigned *>(sums->data()), od);
    rif_chain_kernel<<<static_cast<int>((b + 255) / 256), 256, 0, ctx->stream>>>(csp, static_cast<const unsigned long long *>(v->data()), b, h, od,
                                                    static_cast<long long *>(ckey->data()),
                                                    static_cast<unsigned long long *>(csum->data()), nchains);
    rif_combine_kernel<<<grid, 256, 0, ctx->stream>>>(static_cast<const long long *>(ckey->data()),
                                                      static_cast<const unsigned long long *>(csum->data()), nchains,
                                                      out);
    return done(launched(ctx, "rif_chains"));
}

static vkc_status reduce_into_add_f64(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 3) return fail(ctx, VKC_RUNTIME, arity_error(3, nargs));
    if (!array_arg(ctx, args[1], VKC_F64, &st)) return st;
    int64_t nb;
    if (!array_arg(ctx, args[0], VKC_I64, &st) || !i64_arg(ctx, args[2], &nb, &st)) return st;
    if (nb < 0) return fail(ctx, VKC_RUNTIME, "negative bucket count " + std::to_string(nb));
    const vkc_array *keys = args[0].array, *vals = args[1].array;
    const int64_t n = keys->len;
    const auto *k = static_cast<const long long *>(keys->data());
    bool found;
    if (vals->len != n) {
        if ((st = bucket_key_error(ctx, k, n, nb, &found))) return st;
        return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(n) + " keys for " +
                                          std::to_string(vals->len) + " values");
    }
    vkc_array *o;
    st = new_array(ctx, VKC_F64, nb, true, &o);  // +0.0 in every bucket
    if (st) {
        std::string msg = ctx->err;
        vkc_status kst = bucket_key_error(ctx, k, n, nb, &found);
        if (kst) return kst;
        return fail(ctx, st, msg);
    }
    if ((st = bucket_key_error(ctx, k, n, nb, &found))) {
        vkc_array_release(o);
        return st;
    }
    auto *ov = static_cast<unsigned long long *>(o->data());
    const auto *x = static_cast<const unsigned long long *>(vals->data());
    const int64_t b = n - n % 16;
    if (n > 0 && nb <= RIF_MASKED_BUCKETS) {
        st = rif_masked(ctx, k, x, n, nb, ov);
    } else if (n > 0) {
        if (b > 0) st = rif_sorted(ctx, keys, vals, b, ov);
        if (!st && b < n) {
            rif_tail_kernel<<<1, 1, 0, ctx->stream>>>(k, x, b, n, ov);
            st = launched(ctx, "rif_tail");
        }
    }
    if (st) {
        vkc_array_release(o);
        return st;
    }
    out->kind = VKC_VALUE_ARRAY;
    out->array = o;
    return VKC_OK;
}

void register_reduce_into_f64(std::vector<KernelDef> &t) {
    // The i64 entry's inputs (keys, values, bucket count) and cost (index.rs:241-255).
    KernelDef d{"reduce_into_add_f64", VKC_WHOLE,
                {InSpec{IN_ARRAY, VKC_I64}, InSpec{IN_ARRAY, VKC_F64}, InSpec{IN_SCALAR, VKC_I64}}, true, VKC_F64, 32};
    d.whole = reduce_into_add_f64;
    t.push_back(d);
}

}  // namespace vkc

// Construction kernels: rand_f64, rand_i64 and length_T
// (src/kernels/scalar/construct.rs:12-17, :64-76, :99-106, :233-251).
#include <algorithm>

#include "kcommon.cuh"
#include "registry.h"

namespace vkc {

// construct.rs:12-17 (splitmix64).
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
    unsigned long long z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// (bits >> 11) * 2^-53 as IEEE bits, built with integer ops: m < 2^53 is exact in f64, so its
// value is 2^e * (1 + mantissa) with e the position of its top bit.
__device__ __forceinline__ unsigned long long unit53_bits(unsigned long long bits) {
    unsigned long long m = bits >> 11;
    if (m == 0) return 0;
    int e = 63 - __clzll(static_cast<long long>(m));
    unsigned long long mant = (m << (52 - e)) & 0xfffffffffffffull;
    return (static_cast<unsigned long long>(970 + e) << 52) | mant;
}

template <bool F64>
__global__ void __launch_bounds__(256) rand_kernel(unsigned long long *__restrict__ out, int64_t n,
                                                   unsigned long long seed) {
    int64_t pairs = n >> 1;
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    ulonglong2 *o2 = reinterpret_cast<ulonglong2 *>(out);
    for (int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < pairs; p += stride) {
        unsigned long long i = static_cast<unsigned long long>(p) * 2;
        unsigned long long a = splitmix64(seed + i), b = splitmix64(seed + i + 1);
        if (F64) {
            a = unit53_bits(a);
            b = unit53_bits(b);
        }
        __stcs(&o2[p], make_ulonglong2(a, b));
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        unsigned long long a = splitmix64(seed + static_cast<unsigned long long>(n - 1));
        out[n - 1] = F64 ? unit53_bits(a) : a;
    }
}

// construct.rs:21-34 (count_arg): negative lengths are errors.
static vkc_status run_rand(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out,
                           bool f64) {
    if (nargs != 2) return fail(ctx, VKC_USAGE, arity_error(2, nargs));
    int64_t n, seed;
    vkc_status st;
    if (!i64_arg(ctx, args[0], &n, &st) || !i64_arg(ctx, args[1], &seed, &st)) return st;
    if (n < 0) return fail(ctx, VKC_RUNTIME, "negative length " + std::to_string(n));
    vkc_array *a;
    st = new_array(ctx, f64 ? VKC_F64 : VKC_I64, n, false, &a);
    if (st) return st;
    if (n > 0) {
        int grid = stream_grid(ctx, (n + 1) / 2, 256, 8, 1024);
        if (f64)
            rand_kernel<true><<<grid, 256, 0, ctx->stream>>>(
                static_cast<unsigned long long *>(a->data()), n, static_cast<unsigned long long>(seed));
        else
            rand_kernel<false><<<grid, 256, 0, ctx->stream>>>(
                static_cast<unsigned long long *>(a->data()), n, static_cast<unsigned long long>(seed));
        st = launched(ctx, "rand");
        if (st) {
            vkc_array_release(a);
            return st;
        }
    }
    out->kind = VKC_VALUE_ARRAY;
    out->array = a;
    return VKC_OK;
}

static vkc_status rand_f64(vkc_ctx *c, const vkc_value *a, int n, vkc_value *o) {
    return run_rand(c, a, n, o, true);
}
static vkc_status rand_i64(vkc_ctx *c, const vkc_value *a, int n, vkc_value *o) {
    return run_rand(c, a, n, o, false);
}

// ------------------------------------------------------------------ batched generators
//
// Many rand_f64/rand_i64 statements (one per request of a batch) in one launch: block row y
// fills statement y's array, each value the generator's value at its own (seed, row), so every
// array equals its own rand call. The arrays are views of one allocation, each starting on a
// 256-byte boundary.
constexpr int RB_MAX = 512;  // statements per launch
struct RandBatch {
    int count;
    long long start[RB_MAX], len[RB_MAX];
    unsigned long long seed[RB_MAX];
};

template <bool F64>
__global__ void __launch_bounds__(256) batch_rand_kernel(const RandBatch B, unsigned long long *__restrict__ base) {
    const int sg = blockIdx.y;
    const int64_t n = B.len[sg];
    const unsigned long long seed = B.seed[sg];
    unsigned long long *out = base + B.start[sg];
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned long long a = splitmix64(seed + static_cast<unsigned long long>(i));
        __stcs(out + i, F64 ? unit53_bits(a) : a);
    }
}

// construct.rs:99-106 (run_length): the handle knows its length, no kernel runs.
static vkc_status length(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    if (nargs != 1) return fail(ctx, VKC_USAGE, arity_error(1, nargs));
    out->kind = VKC_VALUE_SCALAR;
    out->scalar = scalar_i64(args[0].array->len);
    return VKC_OK;
}

void register_construct(std::vector<KernelDef> &t) {
    auto i64s = InSpec{IN_SCALAR, VKC_I64};
    KernelDef d;
    d = KernelDef{"rand_f64", VKC_WHOLE, {i64s, i64s}, true, VKC_F64, 8};
    d.whole = rand_f64;
    t.push_back(d);
    d = KernelDef{"rand_i64", VKC_WHOLE, {i64s, i64s}, true, VKC_I64, 8};
    d.whole = rand_i64;
    t.push_back(d);
    const vkc_type types[] = {VKC_F64, VKC_F32, VKC_I64, VKC_U64, VKC_I32, VKC_U8, VKC_BOOL};
    for (vkc_type ty : types) {
        d = KernelDef{std::string("length_") + type_name(ty), VKC_WHOLE, {InSpec{IN_ARRAY, ty}},
                      false, VKC_I64, 0};
        d.whole = length;
        t.push_back(d);
    }
}

}  // namespace vkc

using namespace vkc;

extern "C" VKC_API vkc_status vkc_batch_rand(vkc_ctx *ctx, vkc_type type, int count, const int64_t *lens,
                                            const int64_t *seeds, vkc_array **outs) {
    if (!ctx || count < 0 || (count > 0 && (!lens || !seeds || !outs))) return VKC_USAGE;
    if (type != VKC_F64 && type != VKC_I64) return fail(ctx, VKC_USAGE, "batch rand: f64 or i64 arrays");
    for (int i = 0; i < count; ++i) {
        outs[i] = nullptr;
        if (lens[i] < 0) return fail(ctx, VKC_RUNTIME, "negative length " + std::to_string(lens[i]));
    }
    vkc_status st = VKC_OK;
    for (int c0 = 0; c0 < count && !st; c0 += RB_MAX) {
        const int m = std::min(count - c0, RB_MAX);
        RandBatch B;
        B.count = m;
        int64_t total = 0, longest = 0;
        for (int i = 0; i < m; ++i) {
            B.start[i] = total;
            B.len[i] = lens[c0 + i];
            B.seed[i] = static_cast<unsigned long long>(seeds[c0 + i]);
            total += (lens[c0 + i] + 31) / 32 * 32;  // 256-byte starts
            longest = std::max<int64_t>(longest, lens[c0 + i]);
        }
        vkc_array *all;
        if ((st = new_array(ctx, type, total, false, &all))) break;
        if (longest > 0) {
            const dim3 grid(static_cast<unsigned>(std::min<int64_t>((longest + 1023) / 1024, 64)), static_cast<unsigned>(m));
            auto *base = static_cast<unsigned long long *>(all->data());
            if (type == VKC_F64) batch_rand_kernel<true><<<grid, 256, 0, ctx->stream>>>(B, base);
            else batch_rand_kernel<false><<<grid, 256, 0, ctx->stream>>>(B, base);
            st = launched(ctx, "batch_rand");
        }
        for (int i = 0; i < m && !st; ++i) st = vkc_array_slice(ctx, all, B.start[i], B.len[i], &outs[c0 + i]);
        vkc_array_release(all);  // the views hold the allocation
    }
    if (st)
        for (int i = 0; i < count; ++i) {
            vkc_array_release(outs[i]);
            outs[i] = nullptr;
        }
    return st;
}

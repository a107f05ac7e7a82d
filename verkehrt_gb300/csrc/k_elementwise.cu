// Elementwise kernels for unfused plans and the group-by idioms: mul/add/sub/min/max on f64
// and i64, the six comparisons on f64 and i64, select_f64/select_i64, and/or/not on bool, and
// iota (src/kernels/scalar/elementwise.rs:378-445, :757-804; construct.rs:36-45).
//
// Every operand is an array or a scalar splat (InputSpec::Either). f64 arithmetic is one IEEE
// operation per row (built with -fmad=false), so `mul_f64` then `reduce_add_f64` gives the bits
// of `dot_f64`.
#include "reduce_common.h"

namespace vkc {

struct Opnd {
    const void *p;
    unsigned long long s;
    int arr;
};

template <class T> __device__ __forceinline__ T get(const Opnd &o, int64_t i) {
    if (o.arr) return __ldcs(static_cast<const T *>(o.p) + i);
    T v;
    memcpy(&v, &o.s, sizeof(T));
    return v;
}

// Comparisons come last: an op at or after EW_EQ produces bool.
enum EwOp {
    EW_ADD, EW_SUB, EW_MUL, EW_MIN, EW_MAX, EW_AND, EW_OR, EW_XOR, EW_NOT,
    EW_EQ, EW_NE, EW_LT, EW_LE, EW_GT, EW_GE
};

// IEEE 754-2019 minimum/maximum, elementwise.rs:412-440.
__device__ __forceinline__ double fmin2(double a, double b) {
    if (isnan(a) || isnan(b)) return __longlong_as_double(0x7ff8000000000000ll);
    if (a == b) return signbit(a) ? a : b;
    return a < b ? a : b;
}
__device__ __forceinline__ double fmax2(double a, double b) {
    if (isnan(a) || isnan(b)) return __longlong_as_double(0x7ff8000000000000ll);
    if (a == b) return !signbit(a) ? a : b;
    return a > b ? a : b;
}

template <class T, int OP> struct Bin;
template <int OP> struct Bin<double, OP> {
    using Out = typename std::conditional<(OP >= EW_EQ), unsigned char, double>::type;
    __device__ static Out f(double a, double b) {
        switch (OP) {
        case EW_ADD: return __dadd_rn(a, b);
        case EW_SUB: return __dsub_rn(a, b);
        case EW_MUL: return __dmul_rn(a, b);
        case EW_MIN: return fmin2(a, b);
        case EW_MAX: return fmax2(a, b);
        case EW_EQ: return a == b;
        case EW_NE: return a != b;
        case EW_LT: return a < b;
        case EW_LE: return a <= b;
        case EW_GT: return a > b;
        default: return a >= b;
        }
    }
};
template <int OP> struct Bin<long long, OP> {
    using Out = typename std::conditional<(OP >= EW_EQ), unsigned char, long long>::type;
    __device__ static Out f(long long a, long long b) {
        // Integer arithmetic wraps (elementwise.rs:391-400).
        unsigned long long ua = static_cast<unsigned long long>(a), ub = static_cast<unsigned long long>(b);
        switch (OP) {
        case EW_ADD: return static_cast<long long>(ua + ub);
        case EW_SUB: return static_cast<long long>(ua - ub);
        case EW_MUL: return static_cast<long long>(ua * ub);
        case EW_MIN: return a < b ? a : b;
        case EW_MAX: return a > b ? a : b;
        case EW_AND: return a & b;
        case EW_OR: return a | b;
        case EW_XOR: return a ^ b;
        case EW_EQ: return a == b;
        case EW_NE: return a != b;
        case EW_LT: return a < b;
        case EW_LE: return a <= b;
        case EW_GT: return a > b;
        default: return a >= b;
        }
    }
};
template <int OP> struct Bin<unsigned char, OP> {
    using Out = unsigned char;
    __device__ static Out f(unsigned char a, unsigned char b) {
        switch (OP) {
        case EW_AND: return a & b;
        case EW_OR: return a | b;
        case EW_EQ: return a == b;
        case EW_NE: return a != b;
        default: return static_cast<unsigned char>(a ^ 1u);  // not
        }
    }
};

template <class T, int OP>
__global__ void __launch_bounds__(256) binary_kernel(Opnd a, Opnd b, typename Bin<T, OP>::Out *__restrict__ out,
                                                     int64_t n) {
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = Bin<T, OP>::f(get<T>(a, i), get<T>(b, i));
}

template <class T>
__global__ void __launch_bounds__(256) select_kernel(Opnd m, Opnd a, Opnd b, T *__restrict__ out, int64_t n) {
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = get<unsigned char>(m, i) ? get<T>(a, i) : get<T>(b, i);
}

static Opnd opnd(const Arg &a) {
    Opnd o;
    o.arr = a.rows;
    o.p = a.rows ? a.a->data() : nullptr;
    o.s = a.rows ? 0 : a.s.bits;
    return o;
}

template <class T, int OP>
static vkc_status run_binary(vkc_ctx *ctx, const Arg *args, int nargs, int64_t n, vkc_array *out) {
    if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
    int grid = stream_grid(ctx, n, 256, 8, 2048);
    binary_kernel<T, OP><<<grid, 256, 0, ctx->stream>>>(opnd(args[0]), opnd(args[1]),
        static_cast<typename Bin<T, OP>::Out *>(out->data()), n);
    return launched(ctx, "binary");
}

template <class T>
static vkc_status run_select(vkc_ctx *ctx, const Arg *args, int nargs, int64_t n, vkc_array *out) {
    if (nargs != 3) return fail(ctx, VKC_RUNTIME, arity_error(3, nargs));
    int grid = stream_grid(ctx, n, 256, 8, 2048);
    select_kernel<T><<<grid, 256, 0, ctx->stream>>>(opnd(args[0]), opnd(args[1]), opnd(args[2]),
                                                    static_cast<T *>(out->data()), n);
    return launched(ctx, "select");
}

static vkc_status run_not(vkc_ctx *ctx, const Arg *args, int nargs, int64_t n, vkc_array *out) {
    if (nargs != 1) return fail(ctx, VKC_RUNTIME, arity_error(1, nargs));
    int grid = stream_grid(ctx, n, 256, 8, 2048);
    Opnd z{nullptr, 0, 0};
    binary_kernel<unsigned char, EW_NOT><<<grid, 256, 0, ctx->stream>>>(opnd(args[0]), z,
        static_cast<unsigned char *>(out->data()), n);
    return launched(ctx, "not");
}

__global__ void iota_kernel(long long *out, int64_t n) {
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) out[i] = i;
}

// construct.rs:36-45 (run_iota).
static vkc_status iota(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 1) return fail(ctx, VKC_USAGE, arity_error(1, nargs));
    int64_t n;
    if (!i64_arg(ctx, args[0], &n, &st)) return st;
    if (n < 0) return fail(ctx, VKC_RUNTIME, "negative length " + std::to_string(n));
    vkc_array *a;
    if ((st = new_array(ctx, VKC_I64, n, false, &a))) return st;
    if (n > 0) {
        iota_kernel<<<stream_grid(ctx, n, 256, 8, 2048), 256, 0, ctx->stream>>>(static_cast<long long *>(a->data()), n);
        if ((st = launched(ctx, "iota"))) {
            vkc_array_release(a);
            return st;
        }
    }
    out->kind = VKC_VALUE_ARRAY;
    out->array = a;
    return VKC_OK;
}

void register_elementwise(std::vector<KernelDef> &t) {
    InSpec fe{IN_EITHER, VKC_F64}, ie{IN_EITHER, VKC_I64}, be{IN_EITHER, VKC_BOOL};
    struct E { const char *name; std::vector<InSpec> in; vkc_type out; uint64_t cost; ElemFn f; };
    const E es[] = {
        {"add_f64", {fe, fe}, VKC_F64, 24, run_binary<double, EW_ADD>},
        {"sub_f64", {fe, fe}, VKC_F64, 24, run_binary<double, EW_SUB>},
        {"mul_f64", {fe, fe}, VKC_F64, 24, run_binary<double, EW_MUL>},
        {"min_f64", {fe, fe}, VKC_F64, 24, run_binary<double, EW_MIN>},
        {"max_f64", {fe, fe}, VKC_F64, 24, run_binary<double, EW_MAX>},
        {"eq_f64", {fe, fe}, VKC_BOOL, 17, run_binary<double, EW_EQ>},
        {"ne_f64", {fe, fe}, VKC_BOOL, 17, run_binary<double, EW_NE>},
        {"lt_f64", {fe, fe}, VKC_BOOL, 17, run_binary<double, EW_LT>},
        {"le_f64", {fe, fe}, VKC_BOOL, 17, run_binary<double, EW_LE>},
        {"gt_f64", {fe, fe}, VKC_BOOL, 17, run_binary<double, EW_GT>},
        {"ge_f64", {fe, fe}, VKC_BOOL, 17, run_binary<double, EW_GE>},
        {"add_i64", {ie, ie}, VKC_I64, 24, run_binary<long long, EW_ADD>},
        {"sub_i64", {ie, ie}, VKC_I64, 24, run_binary<long long, EW_SUB>},
        {"mul_i64", {ie, ie}, VKC_I64, 24, run_binary<long long, EW_MUL>},
        {"min_i64", {ie, ie}, VKC_I64, 24, run_binary<long long, EW_MIN>},
        {"max_i64", {ie, ie}, VKC_I64, 24, run_binary<long long, EW_MAX>},
        {"and_i64", {ie, ie}, VKC_I64, 24, run_binary<long long, EW_AND>},
        {"or_i64", {ie, ie}, VKC_I64, 24, run_binary<long long, EW_OR>},
        {"xor_i64", {ie, ie}, VKC_I64, 24, run_binary<long long, EW_XOR>},
        {"eq_i64", {ie, ie}, VKC_BOOL, 17, run_binary<long long, EW_EQ>},
        {"ne_i64", {ie, ie}, VKC_BOOL, 17, run_binary<long long, EW_NE>},
        {"lt_i64", {ie, ie}, VKC_BOOL, 17, run_binary<long long, EW_LT>},
        {"le_i64", {ie, ie}, VKC_BOOL, 17, run_binary<long long, EW_LE>},
        {"gt_i64", {ie, ie}, VKC_BOOL, 17, run_binary<long long, EW_GT>},
        {"ge_i64", {ie, ie}, VKC_BOOL, 17, run_binary<long long, EW_GE>},
        {"and_bool", {be, be}, VKC_BOOL, 3, run_binary<unsigned char, EW_AND>},
        {"or_bool", {be, be}, VKC_BOOL, 3, run_binary<unsigned char, EW_OR>},
        {"eq_bool", {be, be}, VKC_BOOL, 3, run_binary<unsigned char, EW_EQ>},
        {"ne_bool", {be, be}, VKC_BOOL, 3, run_binary<unsigned char, EW_NE>},
        {"not_bool", {be}, VKC_BOOL, 2, run_not},
        {"select_f64", {be, fe, fe}, VKC_F64, 25, run_select<double>},
        {"select_i64", {be, ie, ie}, VKC_I64, 25, run_select<long long>},
        {"select_bool", {be, be, be}, VKC_BOOL, 4, run_select<unsigned char>},
    };
    for (const E &e : es) {
        KernelDef d{e.name, VKC_ELEMENTWISE, e.in, true, e.out, e.cost};
        d.elem = e.f;
        t.push_back(d);
    }
    KernelDef d{"iota", VKC_WHOLE, {InSpec{IN_SCALAR, VKC_I64}}, true, VKC_I64, 8};
    d.whole = iota;
    t.push_back(d);
}

}  // namespace vkc

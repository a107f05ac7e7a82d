// Elementwise kernels of every array type (src/kernels/scalar/elementwise.rs:757-873 register
// them; the array kernels exist for the v1 array types f64, f32, i64, i32, u8, u64 and bool,
// value.rs:23-31), and iota (construct.rs:36-45):
//  * Num on every numeric type: add, sub, mul, min, max and the four orderings (:757-769);
//    integers wrap, floats are one IEEE operation (built with -fmad=false), min/max are the
//    754-2019 minimum/maximum (:403-445);
//  * Signed (i32, i64, f32, f64): neg and abs, wrapping on integers, the sign bit on floats
//    (:447-476); Float: div and sqrt, correctly rounded (:478-495, :777-781);
//  * eq, ne and select on every type (:789-804); and, or, xor, not on i32, i64, u8, u64 (bits)
//    and on bool (0/1 storage) (:806-823);
//  * casts between every array type and every numeric array type by Rust `as` (:572-613,
//    :858-871): float to integer truncates toward zero, saturates and maps NaN to 0;
//  * div_const on i64, u64, i32, u8 (:615-755): truncating division by a scalar with the
//    round-up multiply-high method of Granlund and Montgomery ("Division by invariant integers
//    using multiplication", 1994), the divisor's constants derived once on the host; signed
//    types divide magnitudes and fix the sign, so MIN / -1 = MIN as wrapping_div gives.
// Every operand is an array or a scalar splat (InputSpec::Either; the divisor is a scalar).
// One row per thread per grid-stride step; the cost of an entry is its row bytes.
#include <type_traits>

#include "reduce_common.h"
#include "region.h"

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

// ------------------------------------------------------------------ row operations

template <class T> using Wide = typename std::make_unsigned<T>::type;

// Arithmetic: wrapping integers (elementwise.rs:386-401), IEEE floats.
template <class T> __device__ __forceinline__ T ew_add(T a, T b) { return static_cast<T>(static_cast<Wide<T>>(a) + static_cast<Wide<T>>(b)); }
template <class T> __device__ __forceinline__ T ew_sub(T a, T b) { return static_cast<T>(static_cast<Wide<T>>(a) - static_cast<Wide<T>>(b)); }
template <class T> __device__ __forceinline__ T ew_mul(T a, T b) { return static_cast<T>(static_cast<Wide<T>>(a) * static_cast<Wide<T>>(b)); }
template <> __device__ __forceinline__ double ew_add(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ double ew_sub(double a, double b) { return __dsub_rn(a, b); }
template <> __device__ __forceinline__ double ew_mul(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ float ew_add(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ float ew_sub(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ float ew_mul(float a, float b) { return __fmul_rn(a, b); }

// min/max: Ord on integers; IEEE 754-2019 minimum/maximum on floats (elementwise.rs:413-440).
template <class T> __device__ __forceinline__ T ew_min(T a, T b) {
    if constexpr (std::is_floating_point<T>::value) {
        if (a != a || b != b) return a != a ? a + b : b + a;  // a NaN operand: a NaN result
        if (a == b) return (std::is_same<T, double>::value ? __double_as_longlong(a) < 0 : __float_as_int(a) < 0) ? a : b;
    }
    return a < b ? a : b;
}
template <class T> __device__ __forceinline__ T ew_max(T a, T b) {
    if constexpr (std::is_floating_point<T>::value) {
        if (a != a || b != b) return a != a ? a + b : b + a;
        if (a == b) return (std::is_same<T, double>::value ? __double_as_longlong(a) < 0 : __float_as_int(a) < 0) ? b : a;
    }
    return a > b ? a : b;
}

// neg/abs: wrapping on integers (:452-462), the sign bit on floats (:464-474).
template <class T> __device__ __forceinline__ T ew_neg(T a) { return static_cast<T>(Wide<T>(0) - static_cast<Wide<T>>(a)); }
template <> __device__ __forceinline__ double ew_neg(double a) { return __longlong_as_double(__double_as_longlong(a) ^ (1ll << 63)); }
template <> __device__ __forceinline__ float ew_neg(float a) { return __int_as_float(__float_as_int(a) ^ static_cast<int>(0x80000000u)); }
template <class T> __device__ __forceinline__ T ew_abs(T a) { return a < 0 ? ew_neg(a) : a; }
template <> __device__ __forceinline__ double ew_abs(double a) { return __longlong_as_double(__double_as_longlong(a) & 0x7fffffffffffffffll); }
template <> __device__ __forceinline__ float ew_abs(float a) { return __int_as_float(__float_as_int(a) & 0x7fffffff); }

__device__ __forceinline__ double ew_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float ew_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double ew_sqrt(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ float ew_sqrt(float a) { return __fsqrt_rn(a); }

// Operation tags: f(a, b) or f(a) on storage type T, giving U.
#define EW_BIN(NAME, EXPR, CODE)                                                               \
    struct NAME {                                                                              \
        static constexpr int code = CODE;                                                      \
        template <class T, class U> __device__ static U f(T a, T b) { return static_cast<U>(EXPR); } \
    };
EW_BIN(OpAdd, ew_add(a, b), EF_ADD)
EW_BIN(OpSub, ew_sub(a, b), EF_SUB)
EW_BIN(OpMul, ew_mul(a, b), EF_MUL)
EW_BIN(OpMin, ew_min(a, b), EF_MIN)
EW_BIN(OpMax, ew_max(a, b), EF_MAX)
EW_BIN(OpLt, a < b, EF_LT)
EW_BIN(OpLe, a <= b, EF_LE)
EW_BIN(OpGt, a > b, EF_GT)
EW_BIN(OpGe, a >= b, EF_GE)
EW_BIN(OpEq, a == b, EF_EQ)
EW_BIN(OpNe, a != b, EF_NE)
EW_BIN(OpAnd, a & b, EF_AND)
EW_BIN(OpOr, a | b, EF_OR)
EW_BIN(OpXor, a ^ b, EF_XOR)
EW_BIN(OpDiv, ew_div(a, b), EF_DIV)
#undef EW_BIN

#define EW_UN(NAME, EXPR, CODE)                                                                \
    struct NAME {                                                                              \
        static constexpr int code = CODE;                                                      \
        template <class T, class U> __device__ static U f(T a) { return static_cast<U>(EXPR); } \
    };
EW_UN(OpNeg, ew_neg(a), EF_NEG)
EW_UN(OpAbs, ew_abs(a), EF_ABS)
EW_UN(OpSqrt, ew_sqrt(a), EF_SQRT)
EW_UN(OpBitNot, ~a, EF_NOT)
EW_UN(OpBoolNot, a ^ 1u, EF_BNOT)
#undef EW_UN

// Rust `as` (elementwise.rs:572-613).
template <class S, class D> struct CastAs {
    __device__ static D f(S x) {
        if constexpr (std::is_floating_point<S>::value && std::is_integral<D>::value) {
            // Truncation toward zero, saturated at D's bounds; NaN maps to 0.
            const double v = static_cast<double>(x);
            if (v != v) return D(0);
            const double hi = std::is_same<D, unsigned char>::value ? 256.0
                              : std::is_same<D, int>::value         ? 2147483648.0
                              : std::is_same<D, long long>::value   ? 9223372036854775808.0
                                                                    : 18446744073709551616.0;
            const double lo = std::is_signed<D>::value ? -hi : 0.0;
            if (v >= hi) return static_cast<D>(std::is_signed<D>::value ? (hi == 2147483648.0 ? 2147483647ll : 9223372036854775807ll)
                                                                        : (hi == 256.0 ? 255ull : 18446744073709551615ull));
            if (v <= lo) return std::is_signed<D>::value ? static_cast<D>(hi == 2147483648.0 ? -2147483648ll : (-9223372036854775807ll - 1)) : D(0);
            return static_cast<D>(v);
        } else {
            return static_cast<D>(x);  // integer truncation or extension; to float: round to nearest even
        }
    }
};
template <class S, class D> struct OpCast {
    static constexpr int code = EF_CAST;
    template <class T, class U> __device__ static U f(T a) { return CastAs<S, D>::f(a); }
};

// ------------------------------------------------------------------ kernels

template <class T, class U, class F>
__global__ void __launch_bounds__(256) ew_binary_kernel(Opnd a, Opnd b, U *__restrict__ out, int64_t n) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = F::template f<T, U>(get<T>(a, i), get<T>(b, i));
}

template <class T, class U, class F>
__global__ void __launch_bounds__(256) ew_unary_kernel(Opnd a, U *__restrict__ out, int64_t n) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = F::template f<T, U>(get<T>(a, i));
}

template <class T>
__global__ void __launch_bounds__(256) select_kernel(Opnd m, Opnd a, Opnd b, T *__restrict__ out, int64_t n) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = get<unsigned char>(m, i) ? get<T>(a, i) : get<T>(b, i);
}

// The divider of an unsigned divisor d of B bits (elementwise.rs:627-666): with l = ceil(log2 d),
// m = floor(2^B (2^l - d) / d) + 1, t = mulhi(m, n), q = (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0).
__device__ __forceinline__ unsigned long long div_u(unsigned long long x, const Divider &v, int bits) {
    unsigned long long t;
    if (bits == 64) t = __umul64hi(v.m, x);
    else t = (v.m * x) >> bits;  // m and x below 2^bits <= 2^32: the product fits
    return (t + ((x - t) >> v.sh1)) >> v.sh2;
}

template <class T> __device__ __forceinline__ T ew_div_const(T x, const Divider &v) {
    using UT = Wide<T>;
    constexpr int B = 8 * sizeof(T);
    if constexpr (std::is_signed<T>::value) {
        // Magnitudes, then the sign: MIN's magnitude 2^(B-1) divided by 1 reads back as MIN.
        const UT xneg = static_cast<UT>(x < 0 ? ~UT(0) : UT(0));
        const UT mag = x < 0 ? static_cast<UT>(UT(0) - static_cast<UT>(x)) : static_cast<UT>(x);
        const UT q = static_cast<UT>(div_u(mag, v, B));
        const UT mask = static_cast<UT>(xneg ^ static_cast<UT>(v.dneg));
        return static_cast<T>(static_cast<UT>((q ^ mask) - mask));
    } else {
        return static_cast<T>(div_u(static_cast<unsigned long long>(x), v, B));
    }
}

template <class T>
__global__ void __launch_bounds__(256) div_const_kernel(Opnd a, Divider v, T *__restrict__ out, int64_t n) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = ew_div_const<T>(get<T>(a, i), v);
}

// ------------------------------------------------------------------ entries

static Opnd opnd(const Arg &a) {
    Opnd o;
    o.arr = a.rows;
    o.p = a.rows ? a.a->data() : nullptr;
    o.s = a.rows ? 0 : a.s.bits;
    return o;
}

static int ew_grid(vkc_ctx *ctx, int64_t n) { return stream_grid(ctx, n, 256, 8, 2048); }

template <class T, class U, class F>
static vkc_status run_bin(vkc_ctx *ctx, const Arg *args, int nargs, int64_t n, vkc_array *out) {
    if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
    ew_binary_kernel<T, U, F><<<ew_grid(ctx, n), 256, 0, ctx->stream>>>(opnd(args[0]), opnd(args[1]),
                                                                         static_cast<U *>(out->data()), n);
    return launched(ctx, "elementwise");
}

template <class T, class U, class F>
static vkc_status run_un(vkc_ctx *ctx, const Arg *args, int nargs, int64_t n, vkc_array *out) {
    if (nargs != 1) return fail(ctx, VKC_RUNTIME, arity_error(1, nargs));
    ew_unary_kernel<T, U, F><<<ew_grid(ctx, n), 256, 0, ctx->stream>>>(opnd(args[0]), static_cast<U *>(out->data()), n);
    return launched(ctx, "elementwise");
}

template <class T>
static vkc_status run_select(vkc_ctx *ctx, const Arg *args, int nargs, int64_t n, vkc_array *out) {
    if (nargs != 3) return fail(ctx, VKC_RUNTIME, arity_error(3, nargs));
    select_kernel<T><<<ew_grid(ctx, n), 256, 0, ctx->stream>>>(opnd(args[0]), opnd(args[1]), opnd(args[2]),
                                                               static_cast<T *>(out->data()), n);
    return launched(ctx, "select");
}

// The divider of |d| (B bits), elementwise.rs:640-656.
static Divider make_divider(unsigned long long d, int bits) {
    int l = 0;
    while (l < bits && (1ull << l) < d) ++l;  // ceil(log2 d); 0 for d = 1
    unsigned __int128 num = (static_cast<unsigned __int128>(1) << bits) *
                            ((static_cast<unsigned __int128>(1) << l) - d);
    const unsigned __int128 m = num / d + 1;
    Divider v;
    v.m = static_cast<unsigned long long>(m);
    v.sh1 = l < 1 ? l : 1;
    v.sh2 = l > 0 ? l - 1 : 0;
    v.dneg = 0;
    return v;
}

// The divider of the divisor d of type T (a signed divisor by its magnitude and sign).
template <class T> static Divider typed_divider(T d) {
    using UT = Wide<T>;
    const bool neg = std::is_signed<T>::value && d < 0;
    const UT mag = neg ? static_cast<UT>(UT(0) - static_cast<UT>(d)) : static_cast<UT>(d);
    Divider v = make_divider(static_cast<unsigned long long>(mag), 8 * sizeof(T));
    v.dneg = neg ? ~0ull : 0ull;
    return v;
}

bool make_ew_divider(int ty, unsigned long long bits, Divider *out) {
    switch (ty) {
    case ET_I64: if (static_cast<long long>(bits) == 0) return false; *out = typed_divider<long long>(static_cast<long long>(bits)); return true;
    case ET_U64: if (bits == 0) return false; *out = typed_divider<unsigned long long>(bits); return true;
    case ET_I32: if (static_cast<int>(static_cast<unsigned>(bits)) == 0) return false; *out = typed_divider<int>(static_cast<int>(static_cast<unsigned>(bits))); return true;
    case ET_U8: if ((bits & 0xff) == 0) return false; *out = typed_divider<unsigned char>(static_cast<unsigned char>(bits)); return true;
    default: return false;
    }
}

template <class T>
static vkc_status run_div_const(vkc_ctx *ctx, const Arg *args, int nargs, int64_t n, vkc_array *out) {
    if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
    T d;
    memcpy(&d, &args[1].s.bits, sizeof(T));
    if (d == 0) return fail(ctx, VKC_RUNTIME, "div_const: division by zero");  // elementwise.rs:725-727
    div_const_kernel<T><<<ew_grid(ctx, n), 256, 0, ctx->stream>>>(opnd(args[0]), typed_divider<T>(d),
                                                                   static_cast<T *>(out->data()), n);
    return launched(ctx, "div_const");
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

// ------------------------------------------------------------------ regions
//
// A region's rows pass through its kernels in post-order on chip. Values are 64-bit words
// holding a type's bytes in their low bytes (bool as u8 0/1); every kernel applies the same row
// operation as its own entry above, so a region gives the bits of its kernels run one by one.

template <class T> __device__ __forceinline__ T from_word(unsigned long long w) {
    T v;
    memcpy(&v, &w, sizeof(T));
    return v;
}
template <class T> __device__ __forceinline__ unsigned long long to_word(T v) {
    unsigned long long w = 0;
    memcpy(&w, &v, sizeof(T));
    return w;
}

constexpr int RG_THREADS = 128, RG_ROWS = 4, RG_BLOCK_ROWS = RG_THREADS * RG_ROWS;

// NaN test on the bits (the region folds' NaN rule).
__device__ __forceinline__ bool f64_nan(unsigned long long b) { return (b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull; }

// One kernel of a region over a thread's RG_ROWS rows: the operation is chosen once (uniform
// branches), then the rows run through it.
#define RG_EACH(EXPR)                                      \
    {                                                      \
        _Pragma("unroll") for (int r = 0; r < RG_ROWS; ++r) { \
            const T x = from_word<T>(a[0][r]);             \
            const T y = from_word<T>(a[1][r]);             \
            (void)x;                                       \
            (void)y;                                       \
            out[r] = (EXPR);                               \
        }                                                  \
        return;                                            \
    }

template <class T>
__device__ __forceinline__ void rg_typed(const RgOp &o, const unsigned long long (&a)[3][RG_ROWS],
                                         unsigned long long (&out)[RG_ROWS]) {
    constexpr bool FL = std::is_floating_point<T>::value;
    constexpr bool SG = FL || std::is_signed<T>::value;
    switch (o.fn) {
    case EF_ADD: RG_EACH(to_word(ew_add(x, y)))
    case EF_SUB: RG_EACH(to_word(ew_sub(x, y)))
    case EF_MUL: RG_EACH(to_word(ew_mul(x, y)))
    case EF_MIN: RG_EACH(to_word(ew_min(x, y)))
    case EF_MAX: RG_EACH(to_word(ew_max(x, y)))
    case EF_LT: RG_EACH(static_cast<unsigned long long>(x < y))
    case EF_LE: RG_EACH(static_cast<unsigned long long>(x <= y))
    case EF_GT: RG_EACH(static_cast<unsigned long long>(x > y))
    case EF_GE: RG_EACH(static_cast<unsigned long long>(x >= y))
    case EF_EQ: RG_EACH(static_cast<unsigned long long>(x == y))
    case EF_NE: RG_EACH(static_cast<unsigned long long>(x != y))
    // select(mask, a, b): the mask is the first operand.
    case EF_SELECT: RG_EACH((a[0][r] & 0xffu) ? a[1][r] : a[2][r])
    case EF_BNOT: RG_EACH(a[0][r] ^ 1u)
    case EF_CAST:
        switch (o.dst) {
        case ET_F64: RG_EACH(to_word(CastAs<T, double>::f(x)))
        case ET_F32: RG_EACH(to_word(CastAs<T, float>::f(x)))
        case ET_I64: RG_EACH(to_word(CastAs<T, long long>::f(x)))
        case ET_U64: RG_EACH(to_word(CastAs<T, unsigned long long>::f(x)))
        case ET_I32: RG_EACH(to_word(CastAs<T, int>::f(x)))
        default: RG_EACH(to_word(CastAs<T, unsigned char>::f(x)))
        }
    default: break;
    }
    if constexpr (SG) {
        if (o.fn == EF_NEG) RG_EACH(to_word(ew_neg(x)))
        if (o.fn == EF_ABS) RG_EACH(to_word(ew_abs(x)))
    }
    if constexpr (FL) {
        if (o.fn == EF_DIV) RG_EACH(to_word(ew_div(x, y)))
        if (o.fn == EF_SQRT) RG_EACH(to_word(ew_sqrt(x)))
    }
    if constexpr (!FL) {
        if (o.fn == EF_AND) RG_EACH(to_word(static_cast<T>(x & y)))
        if (o.fn == EF_OR) RG_EACH(to_word(static_cast<T>(x | y)))
        if (o.fn == EF_XOR) RG_EACH(to_word(static_cast<T>(x ^ y)))
        if (o.fn == EF_NOT) RG_EACH(to_word(static_cast<T>(~x)))
        if (o.fn == EF_DIVC) RG_EACH(to_word(ew_div_const<T>(x, o.dv)))
    }
#pragma unroll
    for (int r = 0; r < RG_ROWS; ++r) out[r] = 0;
}
#undef RG_EACH

__device__ __forceinline__ void rg_eval(const RgOp &o, const unsigned long long (&a)[3][RG_ROWS],
                                        unsigned long long (&out)[RG_ROWS]) {
    switch (o.ty) {
    case ET_F64: rg_typed<double>(o, a, out); return;
    case ET_F32: rg_typed<float>(o, a, out); return;
    case ET_I64: rg_typed<long long>(o, a, out); return;
    case ET_U64: rg_typed<unsigned long long>(o, a, out); return;
    case ET_I32: rg_typed<int>(o, a, out); return;
    default: rg_typed<unsigned char>(o, a, out); return;
    }
}

__device__ __forceinline__ unsigned long long rg_load(const RgIn in, int64_t i) {
    switch (in.width) {
    case 8: return __ldcs(static_cast<const unsigned long long *>(in.p) + i);
    case 4: return __ldcs(static_cast<const unsigned *>(in.p) + i);
    default: return __ldcs(static_cast<const unsigned char *>(in.p) + i);
    }
}

// Each block takes RG_BLOCK_ROWS rows per step, four per thread (t, t + 128, ...), and loads
// every array input's rows of the step first. A kernel's operands come from those inputs,
// constants, the previous kernel's value in registers, or
// a shared-memory slot (a value that a kernel after the next one reads; a thread touches only
// its own rows, so no barrier is needed). COUNT: instead of storing the result rows, count the
// nonzero ones (a region under `count`) into *out (an unsigned 64-bit counter).
// The values of the region's last kernel for the thread's rows of the step from row b0.
__device__ __forceinline__ void rg_values(const RegionProg &P, int64_t b0, int64_t n, unsigned long long *s_w,
                                          unsigned long long (&prev)[RG_ROWS]) {
    const int t = threadIdx.x;
    // Every array input's rows of the step, all loads in flight together.
    unsigned long long inv[RG_MAX_ARR][RG_ROWS];
    const int64_t base = b0 + t;
#pragma unroll
    for (int j = 0; j < RG_MAX_ARR; ++j) {
        if (j >= P.narr) continue;
        const RgIn in = P.in[j];
        if (in.width == 8) {
            const unsigned long long *q = static_cast<const unsigned long long *>(in.p) + base;
#pragma unroll
            for (int r = 0; r < RG_ROWS; ++r) inv[j][r] = base + r * RG_THREADS < n ? __ldcs(q + r * RG_THREADS) : 0ull;
        } else {
#pragma unroll
            for (int r = 0; r < RG_ROWS; ++r) {
                const int64_t i = base + r * RG_THREADS;
                inv[j][r] = i < n ? rg_load(in, i) : 0ull;
            }
        }
    }
    for (int k = 0; k < P.nk; ++k) {
        const RgOp &o = P.op[k];
        unsigned long long a[3][RG_ROWS];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int kind = o.kind[j], idx = o.idx[j];
            if (kind == RK_IN) {
                // A uniform branch per input keeps the register array statically indexed.
                switch (idx) {
#define RG_IN_CASE(q)                                                \
    case q:                                                          \
        for (int r = 0; r < RG_ROWS; ++r) a[j][r] = inv[q][r];       \
        break;
                    RG_IN_CASE(0) RG_IN_CASE(1) RG_IN_CASE(2) default: RG_IN_CASE(3)
#undef RG_IN_CASE
                }
            } else if (kind == RK_CONST) {
#pragma unroll
                for (int r = 0; r < RG_ROWS; ++r) a[j][r] = o.c[j];
            } else if (kind == RK_PREV) {
#pragma unroll
                for (int r = 0; r < RG_ROWS; ++r) a[j][r] = prev[r];
            } else {
#pragma unroll
                for (int r = 0; r < RG_ROWS; ++r) a[j][r] = s_w[idx * RG_BLOCK_ROWS + t + r * RG_THREADS];
            }
        }
        rg_eval(o, a, prev);
        if (o.keep) {
#pragma unroll
            for (int r = 0; r < RG_ROWS; ++r) s_w[o.slot * RG_BLOCK_ROWS + t + r * RG_THREADS] = prev[r];
        }
    }
}

template <bool COUNT>
__global__ void __launch_bounds__(RG_THREADS) region_kernel(const RegionProg P, int64_t n, void *__restrict__ out) {
    extern __shared__ unsigned long long s_w[];
    const int t = threadIdx.x;
    unsigned long long nonzero = 0;
    for (int64_t b0 = static_cast<int64_t>(blockIdx.x) * RG_BLOCK_ROWS; b0 < n;
         b0 += static_cast<int64_t>(gridDim.x) * RG_BLOCK_ROWS) {
        unsigned long long prev[RG_ROWS];
        rg_values(P, b0, n, s_w, prev);
#pragma unroll
        for (int r = 0; r < RG_ROWS; ++r) {
            const int64_t i = b0 + t + r * RG_THREADS;
            if (i >= n) break;
            const unsigned long long w = prev[r];
            if (COUNT) {
                nonzero += w != 0;
                continue;
            }
            switch (P.out_width) {
            case 8: static_cast<unsigned long long *>(out)[i] = w; break;
            case 4: static_cast<unsigned *>(out)[i] = static_cast<unsigned>(w); break;
            default: static_cast<unsigned char *>(out)[i] = static_cast<unsigned char>(w); break;
            }
        }
    }
    if (COUNT) {
        nonzero = warp_sum(nonzero);
        if ((t & 31) == 0 && nonzero) atomicAdd(static_cast<unsigned long long *>(out), nonzero);
    }
}

// ------------------------------------------------------------------ region folds
//
// A reduction over a region's value in the same pass: reduce_min/max and argmin/argmax on f64
// and i64 (f64 rows by their order keys, the first NaN row deciding, as the extreme reducers of
// k_reduce.cu do: src/kernels/scalar/reduce.rs:380-468) and the wrapping i64 sum
// (reduce.rs:331-377).

__device__ __forceinline__ void rg_fold_take(int kind, RgFold &a, const RgFold &b) {
    a.nan_idx = min(a.nan_idx, b.nan_idx);
    a.sum += b.sum;
    if (b.idx == ~0ull) return;
    const bool mx = kind == RF_MAX || kind == RF_ARGMAX;
    const bool better = a.idx == ~0ull || (mx ? b.key > a.key : b.key < a.key) || (b.key == a.key && b.idx < a.idx);
    if (better) {
        a.key = b.key;
        a.idx = b.idx;
    }
}

__device__ __forceinline__ RgFold rg_fold_shfl(const RgFold &v, int o) {
    return RgFold{static_cast<long long>(__shfl_xor_sync(FULL, static_cast<unsigned long long>(v.key), o)),
                  __shfl_xor_sync(FULL, v.idx, o), __shfl_xor_sync(FULL, v.nan_idx, o), __shfl_xor_sync(FULL, v.sum, o)};
}

// The block's fold of `v` into thread 0's return value (every thread calls it).
__device__ __forceinline__ RgFold rg_fold_block(int kind, RgFold v) {
    __shared__ RgFold s_f[RG_THREADS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rg_fold_take(kind, v, rg_fold_shfl(v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) s_f[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 1; w < RG_THREADS / 32; ++w) rg_fold_take(kind, v, s_f[w]);
    return v;
}

__global__ void __launch_bounds__(RG_THREADS) region_fold_kernel(const RegionProg P, int64_t n, int kind, bool f64,
                                                                 RgFold *partials, unsigned *done, RgFold *result) {
    extern __shared__ unsigned long long s_w[];
    const int t = threadIdx.x;
    RgFold me{0, ~0ull, ~0ull, 0};
    for (int64_t b0 = static_cast<int64_t>(blockIdx.x) * RG_BLOCK_ROWS; b0 < n;
         b0 += static_cast<int64_t>(gridDim.x) * RG_BLOCK_ROWS) {
        unsigned long long prev[RG_ROWS];
        rg_values(P, b0, n, s_w, prev);
#pragma unroll
        for (int r = 0; r < RG_ROWS; ++r) {
            const int64_t i = b0 + t + r * RG_THREADS;
            if (i >= n) break;
            const unsigned long long w = prev[r];
            if (kind == RF_SUM) {
                me.sum += w;
                continue;
            }
            if (f64 && f64_nan(w)) {
                me.nan_idx = min(me.nan_idx, static_cast<unsigned long long>(i));
                continue;
            }
            rg_fold_take(kind, me, RgFold{f64 ? f64_key(w) : static_cast<long long>(w), static_cast<unsigned long long>(i), ~0ull, 0});
        }
    }
    const RgFold b = rg_fold_block(kind, me);
    if (t == 0) partials[blockIdx.x] = b;
    if (last_block(done)) {
        RgFold v{0, ~0ull, ~0ull, 0};
        for (unsigned q = t; q < gridDim.x; q += RG_THREADS) rg_fold_take(kind, v, partials[q]);
        v = rg_fold_block(kind, v);
        if (t == 0) *result = v;
    }
}

vkc_status launch_region_fold(vkc_ctx *ctx, const RegionProg &p, int64_t n, int kind, bool f64, RgFold *work,
                              unsigned *done) {
    if (n <= 0) return VKC_OK;
    const size_t smem = static_cast<size_t>(p.nslots) * RG_BLOCK_ROWS * sizeof(unsigned long long);
    static std::atomic<unsigned long long> configured{0};
    once_per_device(configured, ctx->device, [] {
        cudaFuncSetAttribute(region_fold_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(RG_MAX_K * RG_BLOCK_ROWS * sizeof(unsigned long long)));
    });
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, region_fold_kernel, RG_THREADS, smem);
    const int64_t blocks = (n + RG_BLOCK_ROWS - 1) / RG_BLOCK_ROWS;
    int64_t g = std::min<int64_t>(blocks, static_cast<int64_t>(ctx->sms) * std::max(1, per_sm));
    const int grid = static_cast<int>(std::min<int64_t>(g, RG_FOLD_MAX_GRID));
    region_fold_kernel<<<grid, RG_THREADS, smem, ctx->stream>>>(p, n, kind, f64, work + 1, done, work);
    return launched(ctx, "region_fold");
}

// The IEEE orderings of doubles on their bits (kcommon.cuh's order keys rank -0 just below +0;
// a NaN is unordered and unequal), so that comparisons leave the FP64 unit to the arithmetic,
// and a comparison's result as 1.0 or +0.0, tested on its bits.
__device__ __forceinline__ bool f64_nan_v(double v) {
    return (static_cast<unsigned long long>(__double_as_longlong(v)) & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}
__device__ __forceinline__ bool f64_zeros_v(double x, double y) {
    return ((static_cast<unsigned long long>(__double_as_longlong(x)) | static_cast<unsigned long long>(__double_as_longlong(y))) &
            0x7fffffffffffffffull) == 0;
}
__device__ __forceinline__ bool f64_less(double x, double y) {
    const unsigned long long a = __double_as_longlong(x), b = __double_as_longlong(y);
    return !f64_nan_v(x) && !f64_nan_v(y) && f64_key(a) < f64_key(b) && !f64_zeros_v(x, y);
}
__device__ __forceinline__ bool f64_less_eq(double x, double y) {
    const unsigned long long a = __double_as_longlong(x), b = __double_as_longlong(y);
    return !f64_nan_v(x) && !f64_nan_v(y) && (f64_key(a) <= f64_key(b) || f64_zeros_v(x, y));
}
__device__ __forceinline__ bool f64_equal(double x, double y) {
    return !f64_nan_v(x) && (__double_as_longlong(x) == __double_as_longlong(y) || f64_zeros_v(x, y));
}
// ew_min / ew_max with the order keys where no row is a NaN (the key order ranks -0 below +0, as
// the 754-2019 minimum and maximum do); a NaN row takes ew_min / ew_max itself.
__device__ __forceinline__ double rg_min(double x, double y) {
    if (f64_nan_v(x) || f64_nan_v(y)) return ew_min(x, y);
    return f64_key(__double_as_longlong(x)) <= f64_key(__double_as_longlong(y)) ? x : y;
}
__device__ __forceinline__ double rg_max(double x, double y) {
    if (f64_nan_v(x) || f64_nan_v(y)) return ew_max(x, y);
    return f64_key(__double_as_longlong(x)) >= f64_key(__double_as_longlong(y)) ? x : y;
}
__device__ __forceinline__ double rg_one(bool c) { return __longlong_as_double(c ? 0x3ff0000000000000ll : 0ll); }
__device__ __forceinline__ bool rg_true(double v) { return __double_as_longlong(v) != 0; }

// Regions of f64 arithmetic and comparisons over f64 inputs: values held as doubles (a
// comparison's result as 1.0 or 0.0, read back by select_f64 and by the output as a bool), the
// same row operations as the kernels' own entries, no type dispatch and no word conversions.
__global__ void __launch_bounds__(RG_THREADS) region_f64_kernel(const RegionProg P, int64_t n, void *__restrict__ out) {
    extern __shared__ double s_d[];
    const int t = threadIdx.x;
    for (int64_t b0 = static_cast<int64_t>(blockIdx.x) * RG_BLOCK_ROWS; b0 < n;
         b0 += static_cast<int64_t>(gridDim.x) * RG_BLOCK_ROWS) {
        const int64_t base = b0 + t;
        double inv[RG_MAX_ARR][RG_ROWS];
#pragma unroll
        for (int j = 0; j < RG_MAX_ARR; ++j) {
            const double *q = static_cast<const double *>(P.in[j].p);
#pragma unroll
            for (int r = 0; r < RG_ROWS; ++r) inv[j][r] = (q && base + r * RG_THREADS < n) ? __ldcs(q + base + r * RG_THREADS) : 0.0;
        }
        double prev[RG_ROWS];
        for (int k = 0; k < P.nk; ++k) {
            const RgOp &o = P.op[k];
            double a[3][RG_ROWS];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int kind = o.kind[j], idx = o.idx[j];
                if (kind == RK_IN) {
                    switch (idx) {
#define RG_IN_CASE(q)                                                          \
    case q:                                                                    \
        _Pragma("unroll") for (int r = 0; r < RG_ROWS; ++r) a[j][r] = inv[q][r]; \
        break;
                        RG_IN_CASE(0) RG_IN_CASE(1) RG_IN_CASE(2) default: RG_IN_CASE(3)
#undef RG_IN_CASE
                    }
                } else if (kind == RK_CONST) {
#pragma unroll
                    for (int r = 0; r < RG_ROWS; ++r) a[j][r] = __longlong_as_double(static_cast<long long>(o.c[j]));
                } else if (kind == RK_PREV) {
#pragma unroll
                    for (int r = 0; r < RG_ROWS; ++r) a[j][r] = prev[r];
                } else {
#pragma unroll
                    for (int r = 0; r < RG_ROWS; ++r) a[j][r] = s_d[idx * RG_BLOCK_ROWS + t + r * RG_THREADS];
                }
            }
#define RG_F(EXPR)                                                                     \
    {                                                                                  \
        _Pragma("unroll") for (int r = 0; r < RG_ROWS; ++r) {                          \
            const double x = a[0][r], y = a[1][r];                                     \
            (void)y;                                                                   \
            prev[r] = (EXPR);                                                          \
        }                                                                              \
        break;                                                                         \
    }
            switch (o.fn) {
            case EF_ADD: RG_F(ew_add(x, y))
            case EF_SUB: RG_F(ew_sub(x, y))
            case EF_MUL: RG_F(ew_mul(x, y))
            case EF_DIV: RG_F(ew_div(x, y))
            case EF_MIN: RG_F(rg_min(x, y))
            case EF_MAX: RG_F(rg_max(x, y))
            case EF_NEG: RG_F(ew_neg(x))
            case EF_ABS: RG_F(ew_abs(x))
            case EF_SQRT: RG_F(ew_sqrt(x))
            case EF_LT: RG_F(rg_one(f64_less(x, y)))
            case EF_LE: RG_F(rg_one(f64_less_eq(x, y)))
            case EF_GT: RG_F(rg_one(f64_less(y, x)))
            case EF_GE: RG_F(rg_one(f64_less_eq(y, x)))
            case EF_EQ: RG_F(rg_one(f64_equal(x, y)))
            case EF_NE: RG_F(rg_one(!f64_equal(x, y)))
            default: RG_F(rg_true(x) ? y : a[2][r])  // EF_SELECT: the mask is 1.0 or +0.0
            }
#undef RG_F
            if (o.keep) {
#pragma unroll
                for (int r = 0; r < RG_ROWS; ++r) s_d[o.slot * RG_BLOCK_ROWS + t + r * RG_THREADS] = prev[r];
            }
        }
#pragma unroll
        for (int r = 0; r < RG_ROWS; ++r) {
            const int64_t i = base + r * RG_THREADS;
            if (i >= n) break;
            if (P.out_width == 8) static_cast<double *>(out)[i] = prev[r];
            else static_cast<unsigned char *>(out)[i] = rg_true(prev[r]);
        }
    }
}

vkc_status launch_region(vkc_ctx *ctx, const RegionProg &p, int64_t n, void *out, bool count) {
    if (n <= 0) return VKC_OK;
    const size_t smem = static_cast<size_t>(p.nslots) * RG_BLOCK_ROWS * sizeof(unsigned long long);
    static std::atomic<unsigned long long> configured{0};
    once_per_device(configured, ctx->device, [] {
        const int most = static_cast<int>(RG_MAX_K * RG_BLOCK_ROWS * sizeof(unsigned long long));
        cudaFuncSetAttribute(region_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
        cudaFuncSetAttribute(region_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
    });
    static std::atomic<unsigned long long> configured_f64{0};
    once_per_device(configured_f64, ctx->device, [] {
        const int most = static_cast<int>(RG_MAX_K * RG_BLOCK_ROWS * sizeof(double));
        cudaFuncSetAttribute(region_f64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
    });
    // Counted regions take the word evaluator: measured at 2^28, count(x*y > 0.25) ran in 1.29 ms
    // there and in 1.65-1.71 ms in the f64 one (with FP64 or with integer comparisons alike).
    const bool f64 = p.f64only && !count;
    int per_sm = 0;
    const void *kern = f64 ? reinterpret_cast<const void *>(region_f64_kernel)
                           : (count ? reinterpret_cast<const void *>(region_kernel<true>)
                                    : reinterpret_cast<const void *>(region_kernel<false>));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, RG_THREADS, smem);
    const int64_t blocks = (n + RG_BLOCK_ROWS - 1) / RG_BLOCK_ROWS;
    const int grid = static_cast<int>(std::min<int64_t>(blocks, static_cast<int64_t>(ctx->sms) * std::max(1, per_sm)));
    if (f64) {
        region_f64_kernel<<<grid, RG_THREADS, smem, ctx->stream>>>(p, n, out);
    } else {
        if (count) region_kernel<true><<<grid, RG_THREADS, smem, ctx->stream>>>(p, n, out);
        else region_kernel<false><<<grid, RG_THREADS, smem, ctx->stream>>>(p, n, out);
    }
    return launched(ctx, "region");
}

// ------------------------------------------------------------------ registration

template <class T> struct TypeOf;
template <> struct TypeOf<double> { static constexpr vkc_type v = VKC_F64; };
template <> struct TypeOf<float> { static constexpr vkc_type v = VKC_F32; };
template <> struct TypeOf<long long> { static constexpr vkc_type v = VKC_I64; };
template <> struct TypeOf<unsigned long long> { static constexpr vkc_type v = VKC_U64; };
template <> struct TypeOf<int> { static constexpr vkc_type v = VKC_I32; };
template <> struct TypeOf<unsigned char> { static constexpr vkc_type v = VKC_U8; };

static std::string tname(vkc_type t) { return type_name(t); }

template <class T> constexpr int tcode() {
    return std::is_same<T, double>::value               ? ET_F64
           : std::is_same<T, float>::value              ? ET_F32
           : std::is_same<T, long long>::value          ? ET_I64
           : std::is_same<T, unsigned long long>::value ? ET_U64
           : std::is_same<T, int>::value                ? ET_I32
                                                        : ET_U8;
}

// An elementwise entry with its row operation for the region evaluator.
struct EwEntry {
    ElemFn f;
    int fn, ty, dst;
};
template <class T, class U, class F> static EwEntry bin() { return {run_bin<T, U, F>, F::code, tcode<T>(), tcode<U>()}; }
template <class T, class U, class F> static EwEntry un() { return {run_un<T, U, F>, F::code, tcode<T>(), tcode<U>()}; }
template <class T> static EwEntry sel() { return {run_select<T>, EF_SELECT, tcode<T>(), tcode<T>()}; }
template <class T> static EwEntry divc() { return {run_div_const<T>, EF_DIVC, tcode<T>(), tcode<T>()}; }

// KernelDef of an elementwise entry; cost = the row bytes (elementwise.rs:272).
static void add(std::vector<KernelDef> &t, const std::string &name, std::vector<InSpec> in, vkc_type out, EwEntry e) {
    uint64_t cost = static_cast<uint64_t>(type_width(out));
    for (const InSpec &s : in) cost += static_cast<uint64_t>(type_width(s.type));
    KernelDef d{name, VKC_ELEMENTWISE, std::move(in), true, out, cost};
    d.elem = e.f;
    d.ew_fn = e.fn;
    d.ew_ty = e.ty;
    d.ew_dst = e.dst;
    t.push_back(d);
}

// register_num (:757-769).
template <class T> static void reg_num(std::vector<KernelDef> &t) {
    const vkc_type ty = TypeOf<T>::v;
    const std::string n = tname(ty);
    const InSpec e{IN_EITHER, ty};
    add(t, "add_" + n, {e, e}, ty, bin<T, T, OpAdd>());
    add(t, "sub_" + n, {e, e}, ty, bin<T, T, OpSub>());
    add(t, "mul_" + n, {e, e}, ty, bin<T, T, OpMul>());
    add(t, "min_" + n, {e, e}, ty, bin<T, T, OpMin>());
    add(t, "max_" + n, {e, e}, ty, bin<T, T, OpMax>());
    add(t, "lt_" + n, {e, e}, VKC_BOOL, bin<T, unsigned char, OpLt>());
    add(t, "le_" + n, {e, e}, VKC_BOOL, bin<T, unsigned char, OpLe>());
    add(t, "gt_" + n, {e, e}, VKC_BOOL, bin<T, unsigned char, OpGt>());
    add(t, "ge_" + n, {e, e}, VKC_BOOL, bin<T, unsigned char, OpGe>());
}

// register_signed (:771-775) and register_float (:777-781).
template <class T> static void reg_signed(std::vector<KernelDef> &t) {
    const vkc_type ty = TypeOf<T>::v;
    const InSpec e{IN_EITHER, ty};
    add(t, "neg_" + tname(ty), {e}, ty, un<T, T, OpNeg>());
    add(t, "abs_" + tname(ty), {e}, ty, un<T, T, OpAbs>());
}
template <class T> static void reg_float(std::vector<KernelDef> &t) {
    const vkc_type ty = TypeOf<T>::v;
    const InSpec e{IN_EITHER, ty};
    add(t, "div_" + tname(ty), {e, e}, ty, bin<T, T, OpDiv>());
    add(t, "sqrt_" + tname(ty), {e}, ty, un<T, T, OpSqrt>());
}

// register_any (:789-804): eq, ne, select; `ty` is bool for the bool instantiation on u8.
template <class T> static void reg_any(std::vector<KernelDef> &t, vkc_type ty) {
    const std::string n = tname(ty);
    const InSpec e{IN_EITHER, ty}, b{IN_EITHER, VKC_BOOL};
    add(t, "eq_" + n, {e, e}, VKC_BOOL, bin<T, unsigned char, OpEq>());
    add(t, "ne_" + n, {e, e}, VKC_BOOL, bin<T, unsigned char, OpNe>());
    add(t, "select_" + n, {b, e, e}, ty, sel<T>());
}

// register_bits (:806-813).
template <class T> static void reg_bits(std::vector<KernelDef> &t) {
    const vkc_type ty = TypeOf<T>::v;
    const std::string n = tname(ty);
    const InSpec e{IN_EITHER, ty};
    add(t, "and_" + n, {e, e}, ty, bin<T, T, OpAnd>());
    add(t, "or_" + n, {e, e}, ty, bin<T, T, OpOr>());
    add(t, "xor_" + n, {e, e}, ty, bin<T, T, OpXor>());
    add(t, "not_" + n, {e}, ty, un<T, T, OpBitNot>());
}

// register_div_const (:739-755): the divisor is a scalar.
template <class T> static void reg_div_const(std::vector<KernelDef> &t) {
    const vkc_type ty = TypeOf<T>::v;
    add(t, "div_const_" + tname(ty), {InSpec{IN_EITHER, ty}, InSpec{IN_SCALAR, ty}}, ty, divc<T>());
}

// register_casts (:858-871): one source type to every numeric array type.
template <class S> static void reg_casts_from(std::vector<KernelDef> &t, vkc_type src) {
    const std::string s = "cast_" + tname(src) + "_";
    const InSpec e{IN_EITHER, src};
    add(t, s + "f64", {e}, VKC_F64, un<S, double, OpCast<S, double>>());
    add(t, s + "f32", {e}, VKC_F32, un<S, float, OpCast<S, float>>());
    add(t, s + "i64", {e}, VKC_I64, un<S, long long, OpCast<S, long long>>());
    add(t, s + "u64", {e}, VKC_U64, un<S, unsigned long long, OpCast<S, unsigned long long>>());
    add(t, s + "i32", {e}, VKC_I32, un<S, int, OpCast<S, int>>());
    add(t, s + "u8", {e}, VKC_U8, un<S, unsigned char, OpCast<S, unsigned char>>());
}

void register_elementwise(std::vector<KernelDef> &t) {
    reg_num<double>(t);
    reg_num<float>(t);
    reg_num<long long>(t);
    reg_num<unsigned long long>(t);
    reg_num<int>(t);
    reg_num<unsigned char>(t);
    reg_signed<double>(t);
    reg_signed<float>(t);
    reg_signed<long long>(t);
    reg_signed<int>(t);
    reg_float<double>(t);
    reg_float<float>(t);
    reg_div_const<long long>(t);
    reg_div_const<unsigned long long>(t);
    reg_div_const<int>(t);
    reg_div_const<unsigned char>(t);
    reg_any<double>(t, VKC_F64);
    reg_any<float>(t, VKC_F32);
    reg_any<long long>(t, VKC_I64);
    reg_any<unsigned long long>(t, VKC_U64);
    reg_any<int>(t, VKC_I32);
    reg_any<unsigned char>(t, VKC_U8);
    reg_any<unsigned char>(t, VKC_BOOL);
    reg_bits<long long>(t);
    reg_bits<unsigned long long>(t);
    reg_bits<int>(t);
    reg_bits<unsigned char>(t);
    // register_bool (:815-823): on the 0/1 storage.
    const InSpec be{IN_EITHER, VKC_BOOL};
    add(t, "and_bool", {be, be}, VKC_BOOL, bin<unsigned char, unsigned char, OpAnd>());
    add(t, "or_bool", {be, be}, VKC_BOOL, bin<unsigned char, unsigned char, OpOr>());
    add(t, "xor_bool", {be, be}, VKC_BOOL, bin<unsigned char, unsigned char, OpXor>());
    add(t, "not_bool", {be}, VKC_BOOL, un<unsigned char, unsigned char, OpBoolNot>());
    reg_casts_from<double>(t, VKC_F64);
    reg_casts_from<float>(t, VKC_F32);
    reg_casts_from<long long>(t, VKC_I64);
    reg_casts_from<unsigned long long>(t, VKC_U64);
    reg_casts_from<int>(t, VKC_I32);
    reg_casts_from<unsigned char>(t, VKC_U8);
    reg_casts_from<unsigned char>(t, VKC_BOOL);
    KernelDef d{"iota", VKC_WHOLE, {InSpec{IN_SCALAR, VKC_I64}}, true, VKC_I64, 8};
    d.whole = iota;
    t.push_back(d);
}

}  // namespace vkc

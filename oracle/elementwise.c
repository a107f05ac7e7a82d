/*
 * CPU oracle, elementwise kernels of every array type: TEST INFRASTRUCTURE ONLY.
 *
 * Restates src/kernels/scalar/elementwise.rs (antiguru/verkehrt): the Num ops (:378-445,
 * integers wrap, floats IEEE with the 754-2019 minimum/maximum), Signed (:447-476, integer
 * neg/abs wrap), Float div/sqrt (:478-495), bits and bool ops (:524-570), Rust `as` casts
 * (:572-613: float to int truncates toward zero, saturates and maps NaN to 0; int to int
 * truncates or extends; to float rounds to nearest even) and div_const (:615-737, truncating
 * division that wraps like wrapping_div; a zero divisor is an error). Type codes are those of
 * vkc_type. Built with the rest of the oracle (-O3 -ffp-contract=off).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "oracle.h"

enum { T_F64 = 0, T_F32 = 1, T_I64 = 2, T_U64 = 3, T_I32 = 4, T_U8 = 5, T_BOOL = 6 };

enum {
    OP_ADD, OP_SUB, OP_MUL, OP_MIN, OP_MAX, OP_LT, OP_LE, OP_GT, OP_GE, OP_EQ, OP_NE,
    OP_AND, OP_OR, OP_XOR, OP_NOT, OP_NEG, OP_ABS, OP_DIV, OP_SQRT, OP_BAD
};

static int op_code(const char *op) {
    static const char *names[] = {"add", "sub", "mul", "min", "max", "lt", "le", "gt", "ge", "eq", "ne",
                                  "and", "or", "xor", "not", "neg", "abs", "div", "sqrt"};
    for (int i = 0; i < OP_BAD; ++i)
        if (strcmp(op, names[i]) == 0) return i;
    return OP_BAD;
}

/* elementwise.rs:413-440: NaN propagates, -0 < +0. */
static double min2_d(double a, double b) {
    if (isnan(a) || isnan(b)) return NAN;
    if (a == b) return signbit(a) ? a : b;
    return a < b ? a : b;
}
static double max2_d(double a, double b) {
    if (isnan(a) || isnan(b)) return NAN;
    if (a == b) return signbit(a) ? b : a;
    return a > b ? a : b;
}
static float min2_f(float a, float b) {
    if (isnan(a) || isnan(b)) return NAN;
    if (a == b) return signbit(a) ? a : b;
    return a < b ? a : b;
}
static float max2_f(float a, float b) {
    if (isnan(a) || isnan(b)) return NAN;
    if (a == b) return signbit(a) ? b : a;
    return a > b ? a : b;
}

/* Float negation and abs act on the sign bit (Rust -x and abs). */
static double neg_d(double a) { uint64_t u; memcpy(&u, &a, 8); u ^= 1ull << 63; memcpy(&a, &u, 8); return a; }
static double abs_d(double a) { uint64_t u; memcpy(&u, &a, 8); u &= ~(1ull << 63); memcpy(&a, &u, 8); return a; }
static float neg_f(float a) { uint32_t u; memcpy(&u, &a, 4); u ^= 1u << 31; memcpy(&a, &u, 4); return a; }
static float abs_f(float a) { uint32_t u; memcpy(&u, &a, 4); u &= ~(1u << 31); memcpy(&a, &u, 4); return a; }

#define AT(T, p, splat, i) (((const T *)(p))[(splat) ? 0 : (i)])

/* Integers: arithmetic in the unsigned twin, so it wraps. */
#define INT_BINARY(T, U)                                                                       \
    for (int64_t i = 0; i < n; ++i) {                                                          \
        T x = AT(T, a, as, i), y = AT(T, b, bs, i);                                            \
        switch (op) {                                                                          \
        case OP_ADD: ((T *)out)[i] = (T)((U)x + (U)y); break;                                  \
        case OP_SUB: ((T *)out)[i] = (T)((U)x - (U)y); break;                                  \
        case OP_MUL: ((T *)out)[i] = (T)((U)x * (U)y); break;                                  \
        case OP_MIN: ((T *)out)[i] = x < y ? x : y; break;                                     \
        case OP_MAX: ((T *)out)[i] = x > y ? x : y; break;                                     \
        case OP_AND: ((T *)out)[i] = (T)(x & y); break;                                        \
        case OP_OR: ((T *)out)[i] = (T)(x | y); break;                                         \
        case OP_XOR: ((T *)out)[i] = (T)(x ^ y); break;                                        \
        case OP_LT: ((uint8_t *)out)[i] = x < y; break;                                        \
        case OP_LE: ((uint8_t *)out)[i] = x <= y; break;                                       \
        case OP_GT: ((uint8_t *)out)[i] = x > y; break;                                        \
        case OP_GE: ((uint8_t *)out)[i] = x >= y; break;                                       \
        case OP_EQ: ((uint8_t *)out)[i] = x == y; break;                                       \
        case OP_NE: ((uint8_t *)out)[i] = x != y; break;                                       \
        default: return -1;                                                                    \
        }                                                                                      \
    }

#define FLOAT_BINARY(T, MIN2, MAX2)                                                            \
    for (int64_t i = 0; i < n; ++i) {                                                          \
        T x = AT(T, a, as, i), y = AT(T, b, bs, i);                                            \
        switch (op) {                                                                          \
        case OP_ADD: ((T *)out)[i] = x + y; break;                                             \
        case OP_SUB: ((T *)out)[i] = x - y; break;                                             \
        case OP_MUL: ((T *)out)[i] = x * y; break;                                             \
        case OP_DIV: ((T *)out)[i] = x / y; break;                                             \
        case OP_MIN: ((T *)out)[i] = MIN2(x, y); break;                                        \
        case OP_MAX: ((T *)out)[i] = MAX2(x, y); break;                                        \
        case OP_LT: ((uint8_t *)out)[i] = x < y; break;                                        \
        case OP_LE: ((uint8_t *)out)[i] = x <= y; break;                                       \
        case OP_GT: ((uint8_t *)out)[i] = x > y; break;                                        \
        case OP_GE: ((uint8_t *)out)[i] = x >= y; break;                                       \
        case OP_EQ: ((uint8_t *)out)[i] = x == y; break;                                       \
        case OP_NE: ((uint8_t *)out)[i] = x != y; break;                                       \
        default: return -1;                                                                    \
        }                                                                                      \
    }

/* out = op(a, b); a or b may be one splat row. Returns -1 for an op the type lacks. */
int orc_ew_binary(const char *opname, int type, const void *a, int as, const void *b, int bs, int64_t n,
                  void *out) {
    const int op = op_code(opname);
    switch (type) {
    case T_F64: FLOAT_BINARY(double, min2_d, max2_d) return 0;
    case T_F32: FLOAT_BINARY(float, min2_f, max2_f) return 0;
    case T_I64: INT_BINARY(int64_t, uint64_t) return 0;
    case T_U64: INT_BINARY(uint64_t, uint64_t) return 0;
    case T_I32: INT_BINARY(int32_t, uint32_t) return 0;
    case T_U8: INT_BINARY(uint8_t, uint8_t) return 0;
    case T_BOOL:
        /* elementwise.rs:534-539, :815-823: bool ops on the 0/1 storage. */
        for (int64_t i = 0; i < n; ++i) {
            uint8_t x = AT(uint8_t, a, as, i), y = AT(uint8_t, b, bs, i);
            switch (op) {
            case OP_AND: ((uint8_t *)out)[i] = x & y; break;
            case OP_OR: ((uint8_t *)out)[i] = x | y; break;
            case OP_XOR: ((uint8_t *)out)[i] = x ^ y; break;
            case OP_EQ: ((uint8_t *)out)[i] = x == y; break;
            case OP_NE: ((uint8_t *)out)[i] = x != y; break;
            default: return -1;
            }
        }
        return 0;
    }
    return -1;
}

int orc_ew_unary(const char *opname, int type, const void *a, int64_t n, void *out) {
    const int op = op_code(opname);
    for (int64_t i = 0; i < n; ++i) {
        switch (type) {
        case T_F64: {
            double x = ((const double *)a)[i];
            if (op == OP_NEG) ((double *)out)[i] = neg_d(x);
            else if (op == OP_ABS) ((double *)out)[i] = abs_d(x);
            else if (op == OP_SQRT) ((double *)out)[i] = sqrt(x);
            else return -1;
            break;
        }
        case T_F32: {
            float x = ((const float *)a)[i];
            if (op == OP_NEG) ((float *)out)[i] = neg_f(x);
            else if (op == OP_ABS) ((float *)out)[i] = abs_f(x);
            else if (op == OP_SQRT) ((float *)out)[i] = sqrtf(x);
            else return -1;
            break;
        }
        case T_I64: {
            int64_t x = ((const int64_t *)a)[i];
            int64_t ng = (int64_t)(0ull - (uint64_t)x);
            if (op == OP_NEG) ((int64_t *)out)[i] = ng;
            else if (op == OP_ABS) ((int64_t *)out)[i] = x < 0 ? ng : x;
            else if (op == OP_NOT) ((int64_t *)out)[i] = ~x;
            else return -1;
            break;
        }
        case T_I32: {
            int32_t x = ((const int32_t *)a)[i];
            int32_t ng = (int32_t)(0u - (uint32_t)x);
            if (op == OP_NEG) ((int32_t *)out)[i] = ng;
            else if (op == OP_ABS) ((int32_t *)out)[i] = x < 0 ? ng : x;
            else if (op == OP_NOT) ((int32_t *)out)[i] = ~x;
            else return -1;
            break;
        }
        case T_U64:
            if (op != OP_NOT) return -1;
            ((uint64_t *)out)[i] = ~((const uint64_t *)a)[i];
            break;
        case T_U8:
            if (op != OP_NOT) return -1;
            ((uint8_t *)out)[i] = (uint8_t)~((const uint8_t *)a)[i];
            break;
        case T_BOOL:
            if (op != OP_NOT) return -1;
            ((uint8_t *)out)[i] = ((const uint8_t *)a)[i] ^ 1;
            break;
        default: return -1;
        }
    }
    return 0;
}

/* select_T, elementwise.rs:789-804: m[i] ? a[i] : b[i], every operand may be a splat. */
void orc_ew_select(int width, const uint8_t *m, int ms, const void *a, int as, const void *b, int bs, int64_t n,
                   void *out) {
    for (int64_t i = 0; i < n; ++i) {
        const uint8_t c = m[ms ? 0 : i];
        const char *src = c ? (const char *)a + (as ? 0 : i * width) : (const char *)b + (bs ? 0 : i * width);
        memcpy((char *)out + i * width, src, (size_t)width);
    }
}

/* ---------------------------------------------------------------- casts (Rust `as`) */

static double load_num(int t, const void *p, int64_t i, int64_t *iv, uint64_t *uv, int *kind) {
    /* kind 0: signed integer in *iv, 1: unsigned in *uv, 2: float (returned) */
    switch (t) {
    case T_F64: *kind = 2; return ((const double *)p)[i];
    case T_F32: *kind = 2; return (double)((const float *)p)[i];
    case T_I64: *kind = 0; *iv = ((const int64_t *)p)[i]; return 0;
    case T_I32: *kind = 0; *iv = ((const int32_t *)p)[i]; return 0;
    case T_U64: *kind = 1; *uv = ((const uint64_t *)p)[i]; return 0;
    default: *kind = 1; *uv = ((const uint8_t *)p)[i]; return 0; /* u8 and bool storage */
    }
}

/* Float to integer: truncate toward zero, saturate at the type's bounds, NaN to 0. */
static int64_t f2i(double x, double lo, double hi_excl, int64_t lo_v, int64_t hi_v) {
    if (isnan(x)) return 0;
    if (x >= hi_excl) return hi_v;
    if (x <= lo) return lo_v;
    return (int64_t)x;
}
static uint64_t f2u(double x, double hi_excl, uint64_t hi_v) {
    if (!(x > 0)) return 0;
    if (x >= hi_excl) return hi_v;
    return (uint64_t)x;
}

int orc_ew_cast(int src, int dst, const void *a, int64_t n, void *out) {
    for (int64_t i = 0; i < n; ++i) {
        int64_t iv = 0;
        uint64_t uv = 0;
        int kind;
        const double fv = load_num(src, a, i, &iv, &uv, &kind);
        /* f32 sources convert to f32 targets and to integers from their own value. */
        const float f32v = src == T_F32 ? ((const float *)a)[i] : 0.0f;
        switch (dst) {
        case T_F64:
            ((double *)out)[i] = kind == 2 ? fv : (kind == 0 ? (double)iv : (double)uv);
            break;
        case T_F32:
            ((float *)out)[i] = src == T_F32 ? f32v : (kind == 2 ? (float)fv : (kind == 0 ? (float)iv : (float)uv));
            break;
        case T_I64:
            ((int64_t *)out)[i] = kind == 2 ? f2i(fv, -9223372036854775808.0, 9223372036854775808.0, INT64_MIN, INT64_MAX)
                                            : (kind == 0 ? iv : (int64_t)uv);
            break;
        case T_I32:
            ((int32_t *)out)[i] = kind == 2 ? (int32_t)f2i(fv, -2147483648.0, 2147483648.0, INT32_MIN, INT32_MAX)
                                            : (kind == 0 ? (int32_t)(uint32_t)(uint64_t)iv : (int32_t)(uint32_t)uv);
            break;
        case T_U64:
            ((uint64_t *)out)[i] = kind == 2 ? f2u(fv, 18446744073709551616.0, UINT64_MAX)
                                             : (kind == 0 ? (uint64_t)iv : uv);
            break;
        case T_U8:
            ((uint8_t *)out)[i] = kind == 2 ? (uint8_t)f2u(fv, 256.0, 255) : (kind == 0 ? (uint8_t)(uint64_t)iv : (uint8_t)uv);
            break;
        default: return -1;
        }
    }
    return 0;
}

/* ---------------------------------------------------------------- div_const */

/* Truncating division by the scalar *d, wrapping like wrapping_div (MIN / -1 = MIN). */
int orc_ew_div_const(int type, const void *a, const void *d, int64_t n, void *out, char *err) {
    switch (type) {
    case T_I64: {
        const int64_t q = *(const int64_t *)d;
        if (q == 0) break;
        for (int64_t i = 0; i < n; ++i) {
            const int64_t x = ((const int64_t *)a)[i];
            ((int64_t *)out)[i] = (q == -1) ? (int64_t)(0ull - (uint64_t)x) : x / q;
        }
        return 0;
    }
    case T_I32: {
        const int32_t q = *(const int32_t *)d;
        if (q == 0) break;
        for (int64_t i = 0; i < n; ++i) {
            const int32_t x = ((const int32_t *)a)[i];
            ((int32_t *)out)[i] = (q == -1) ? (int32_t)(0u - (uint32_t)x) : x / q;
        }
        return 0;
    }
    case T_U64: {
        const uint64_t q = *(const uint64_t *)d;
        if (q == 0) break;
        for (int64_t i = 0; i < n; ++i) ((uint64_t *)out)[i] = ((const uint64_t *)a)[i] / q;
        return 0;
    }
    case T_U8: {
        const uint8_t q = *(const uint8_t *)d;
        if (q == 0) break;
        for (int64_t i = 0; i < n; ++i) ((uint8_t *)out)[i] = (uint8_t)(((const uint8_t *)a)[i] / q);
        return 0;
    }
    default:
        strcpy(err, "div_const: unsupported type");
        return 1;
    }
    /* elementwise.rs:725-727 */
    strcpy(err, "div_const: division by zero");
    return 1;
}

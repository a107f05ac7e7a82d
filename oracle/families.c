/*
 * CPU oracle, part 3: the kernel families on every element type (TEST INFRASTRUCTURE ONLY).
 *
 * Plain-C restatements of the reference's generic folds, for the element types the other files
 * do not cover: the reductions of src/kernels/scalar/reduce.rs (integer sums that widen,
 * wrapping products, extremes, bit folds, bool folds, the canonical float order for f32 and
 * for products), the fused reductions of src/kernels/scalar/fused.rs on f32/i64/u64/i32, and
 * the scans, segmented scans and bucket folds of src/kernels/scalar/scan.rs for every fold.
 *
 * Values travel as 64-bit words: an element of type t is read with ld() below (i32 sign-
 * extended, u8 and bool zero-extended, f32 as its 32 bits) and results are written back in the
 * output type's width. Type numbers are vkc_type's (0 f64, 1 f32, 2 i64, 3 u64, 4 i32, 5 u8,
 * 6 bool); fold numbers are FOLD_* below, the order of ReduceOp in src/ops.rs.
 */
#include "oracle.h"

#include <math.h>
#include <stdio.h>
#include <string.h>

enum { T_F64 = 0, T_F32 = 1, T_I64 = 2, T_U64 = 3, T_I32 = 4, T_U8 = 5, T_BOOL = 6 };
enum { FOLD_ADD = 0, FOLD_MUL = 1, FOLD_MIN = 2, FOLD_MAX = 3, FOLD_AND = 4, FOLD_OR = 5, FOLD_XOR = 6 };

static int width(int t) { return t == T_F64 || t == T_I64 || t == T_U64 ? 8 : (t == T_F32 || t == T_I32 ? 4 : 1); }

static uint64_t ld(int t, const void *p, int64_t i) {
    switch (t) {
    case T_F64: case T_I64: case T_U64: return ((const uint64_t *)p)[i];
    case T_F32: return ((const uint32_t *)p)[i];
    case T_I32: return (uint64_t)(int64_t)((const int32_t *)p)[i];
    default: return ((const uint8_t *)p)[i];
    }
}

static void st(int t, void *p, int64_t i, uint64_t v) {
    switch (width(t)) {
    case 8: ((uint64_t *)p)[i] = v; break;
    case 4: ((uint32_t *)p)[i] = (uint32_t)v; break;
    default: ((uint8_t *)p)[i] = (uint8_t)v; break;
    }
}

static double as_d(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }
static uint64_t d_bits(double d) { uint64_t b; memcpy(&b, &d, 8); return b; }
static float as_f(uint64_t b) { uint32_t u = (uint32_t)b; float f; memcpy(&f, &u, 4); return f; }
static uint64_t f_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

/* elementwise.rs:413-440 (min2/max2 on floats: NaN propagates, -0 < +0; Ord on integers). */
static int is_float(int t) { return t == T_F64 || t == T_F32; }
static int is_signed(int t) { return t == T_I64 || t == T_I32; }

static uint64_t min2(int t, uint64_t a, uint64_t b, int is_max) {
    if (t == T_F64) {
        double x = as_d(a), y = as_d(b);
        if (isnan(x) || isnan(y)) return d_bits(NAN);
        if (x == y) return (signbit(x) != 0) == !is_max ? a : b;
        return (is_max ? x > y : x < y) ? a : b;
    }
    if (t == T_F32) {
        float x = as_f(a), y = as_f(b);
        if (isnan(x) || isnan(y)) return f_bits(NAN);
        if (x == y) return (signbit(x) != 0) == !is_max ? a : b;
        return (is_max ? x > y : x < y) ? a : b;
    }
    if (is_signed(t)) {
        int64_t x = (int64_t)a, y = (int64_t)b;
        return (is_max ? x >= y : x <= y) ? a : b;
    }
    return (is_max ? a >= b : a <= b) ? a : b;
}

/* Truncates a 64-bit word to the type's storage and widens it back (the wrapping of Num). */
static uint64_t wrap(int t, uint64_t v) {
    switch (t) {
    case T_I32: return (uint64_t)(int64_t)(int32_t)(uint32_t)v;
    case T_U8: case T_BOOL: return v & 0xff;
    default: return v;
    }
}

/* The sum type of reduce_add and scan add (reduce.rs:559-586 Reducible::Sum, scan.rs ScanSum):
 * i32 widens to i64, u8 to u64. */
static int sum_type(int t) { return t == T_I32 ? T_I64 : (t == T_U8 ? T_U64 : t); }

/* One step of fold f on rows of type t (scan.rs:130-233 ScanOp::step; the reductions' Accum
 * steps are the same operations, reduce.rs:331-377, :380-412, :470-545). For add the
 * accumulator is in the sum type. */
static uint64_t step(int t, int f, uint64_t acc, uint64_t x) {
    switch (f) {
    case FOLD_ADD: return acc + x; /* wrapping, in the widened type */
    case FOLD_MUL: return wrap(t, acc * x);
    case FOLD_MIN: return min2(t, acc, x, 0);
    case FOLD_MAX: return min2(t, acc, x, 1);
    case FOLD_AND: return acc & x;
    case FOLD_OR: return acc | x;
    default: return acc ^ x;
    }
}

/* scan.rs:99-120 (Extremes) and :130-233 (ScanOp::identity). */
static uint64_t identity(int t, int f) {
    switch (f) {
    case FOLD_ADD: case FOLD_OR: case FOLD_XOR: return 0;
    case FOLD_MUL: return 1;
    case FOLD_AND: return t == T_BOOL ? 1 : wrap(t, ~0ull);
    case FOLD_MIN:
        switch (t) {
        case T_F64: return d_bits(INFINITY);
        case T_F32: return f_bits(INFINITY);
        case T_I64: return (uint64_t)INT64_MAX;
        case T_I32: return (uint64_t)(int64_t)INT32_MAX;
        case T_U8: return 0xff;
        default: return ~0ull;
        }
    default:
        switch (t) {
        case T_F64: return d_bits(-INFINITY);
        case T_F32: return f_bits(-INFINITY);
        case T_I64: return (uint64_t)INT64_MIN;
        case T_I32: return (uint64_t)(int64_t)INT32_MIN;
        default: return 0;
        }
    }
}

/* ---------------------------------------------------------------- reductions */

/* reduce.rs:45-91 (the canonical order) for f32 or f64, add or mul, over row values v(i). */
typedef uint64_t (*row_fn)(const void *x, const void *y, int64_t i, int t, int cmp, uint64_t c, uint64_t e);

static uint64_t canon(int t, int mul, row_fn rv, const void *x, const void *y, int64_t n, int cmp, uint64_t c,
                      uint64_t e) {
    int64_t blocks = n / 16;
    if (t == T_F64) {
        double acc[16];
        for (int j = 0; j < 16; ++j) acc[j] = mul ? 1.0 : 0.0;
        for (int64_t b = 0; b < blocks; ++b)
            for (int j = 0; j < 16; ++j) {
                double v = as_d(rv(x, y, b * 16 + j, t, cmp, c, e));
                acc[j] = mul ? acc[j] * v : acc[j] + v;
            }
        for (int s = 8; s > 0; s /= 2)
            for (int j = 0; j < s; ++j) acc[j] = mul ? acc[j] * acc[j + s] : acc[j] + acc[j + s];
        double r = acc[0];
        for (int64_t i = blocks * 16; i < n; ++i) {
            double v = as_d(rv(x, y, i, t, cmp, c, e));
            r = mul ? r * v : r + v;
        }
        return d_bits(r);
    }
    float acc[16];
    for (int j = 0; j < 16; ++j) acc[j] = mul ? 1.0f : 0.0f;
    for (int64_t b = 0; b < blocks; ++b)
        for (int j = 0; j < 16; ++j) {
            float v = as_f(rv(x, y, b * 16 + j, t, cmp, c, e));
            acc[j] = mul ? acc[j] * v : acc[j] + v;
        }
    for (int s = 8; s > 0; s /= 2)
        for (int j = 0; j < s; ++j) acc[j] = mul ? acc[j] * acc[j + s] : acc[j] + acc[j + s];
    float r = acc[0];
    for (int64_t i = blocks * 16; i < n; ++i) {
        float v = as_f(rv(x, y, i, t, cmp, c, e));
        r = mul ? r * v : r + v;
    }
    return f_bits(r);
}

static uint64_t row_plain(const void *x, const void *y, int64_t i, int t, int cmp, uint64_t c, uint64_t e) {
    (void)y; (void)cmp; (void)c; (void)e;
    return ld(t, x, i);
}

/* reduce.rs:664-726: reduce_<fold>_t. Empty min/max fail ("reduce_min of an empty array",
 * reduce.rs:403-410); the others give the identity. Floats add and multiply in the canonical
 * order; every other fold is order-free. The result is in the sum type for add. */
int orc_fold(int t, int f, const void *x, int64_t n, uint64_t *out, char *err) {
    if ((f == FOLD_MIN || f == FOLD_MAX) && n == 0) {
        snprintf(err, ORC_ERR_LEN, "reduce_%s of an empty array", f == FOLD_MAX ? "max" : "min");
        return 1;
    }
    if (is_float(t) && (f == FOLD_ADD || f == FOLD_MUL)) {
        *out = canon(t, f == FOLD_MUL, row_plain, x, NULL, n, 0, 0, 0);
        return 0;
    }
    uint64_t acc = f == FOLD_MIN || f == FOLD_MAX ? ld(t, x, 0) : identity(f == FOLD_ADD ? sum_type(t) : t, f);
    for (int64_t i = (f == FOLD_MIN || f == FOLD_MAX) ? 1 : 0; i < n; ++i) acc = step(t, f, acc, ld(t, x, i));
    *out = f == FOLD_ADD ? acc : wrap(t, acc);
    return 0;
}

/* reduce.rs:417-468 (ArgExtreme): the first NaN's row, else the first row of the extreme, with
 * -0 below +0 (Ordered::less/greater, :171-199). */
static int less(int t, uint64_t a, uint64_t b) {
    if (t == T_F64) { double x = as_d(a), y = as_d(b); return x < y || (x == y && signbit(x) && !signbit(y)); }
    if (t == T_F32) { float x = as_f(a), y = as_f(b); return x < y || (x == y && signbit(x) && !signbit(y)); }
    if (is_signed(t)) return (int64_t)a < (int64_t)b;
    return a < b;
}

int orc_argext(int t, int is_max, const void *x, int64_t n, int64_t *out, char *err) {
    if (n == 0) {
        snprintf(err, ORC_ERR_LEN, "%s of an empty array", is_max ? "argmax" : "argmin");
        return 1;
    }
    int64_t best = -1;
    for (int64_t i = 0; i < n; ++i) {
        uint64_t v = ld(t, x, i);
        if ((t == T_F64 && isnan(as_d(v))) || (t == T_F32 && isnan(as_f(v)))) {
            *out = i;
            return 0;
        }
        if (best < 0 || (is_max ? less(t, ld(t, x, best), v) : less(t, v, ld(t, x, best)))) best = i;
    }
    *out = best;
    return 0;
}

/* ---------------------------------------------------------------- fused reductions (fused.rs) */

/* fused.rs:41-54: the comparison of the single-op kernels (IEEE: NaN compares false but ne). */
static int cmp_test(int t, int cmp, uint64_t a, uint64_t b) {
    int lt, eq, unord = 0;
    if (t == T_F64) { double x = as_d(a), y = as_d(b); unord = isnan(x) || isnan(y); lt = x < y; eq = x == y; }
    else if (t == T_F32) { float x = as_f(a), y = as_f(b); unord = isnan(x) || isnan(y); lt = x < y; eq = x == y; }
    else if (is_signed(t)) { lt = (int64_t)a < (int64_t)b; eq = a == b; }
    else { lt = a < b; eq = a == b; }
    if (unord) return cmp == ORC_NE;
    switch (cmp) {
    case ORC_EQ: return eq;
    case ORC_NE: return !eq;
    case ORC_LT: return lt;
    case ORC_LE: return lt || eq;
    case ORC_GT: return !lt && !eq;
    default: return !lt;
    }
}

/* Num::mul on the element type (wrapping for integers, one IEEE multiply for floats). */
static uint64_t mul_t(int t, uint64_t a, uint64_t b) {
    if (t == T_F64) return d_bits(as_d(a) * as_d(b));
    if (t == T_F32) return f_bits(as_f(a) * as_f(b));
    return wrap(t, a * b);
}

static uint64_t row_dot(const void *x, const void *y, int64_t i, int t, int cmp, uint64_t c, uint64_t e) {
    (void)cmp; (void)c; (void)e;
    return mul_t(t, ld(t, x, i), ld(t, y, i));
}
static uint64_t row_sumsq(const void *x, const void *y, int64_t i, int t, int cmp, uint64_t c, uint64_t e) {
    (void)y; (void)cmp; (void)c; (void)e;
    uint64_t v = ld(t, x, i);
    return mul_t(t, v, v);
}
static uint64_t row_cond(const void *x, const void *y, int64_t i, int t, int cmp, uint64_t c, uint64_t e) {
    (void)y;
    uint64_t v = ld(t, x, i);
    return cmp_test(t, cmp, v, c) ? v : e;
}

/* fused.rs:73-212: dot (what 0), sumsq (1), condsum_<cmp> (2): the row values summed as
 * reduce_add sums them (the canonical order for floats, the widening wrapping sum otherwise).
 * Scalars c and e are given in the element type's 64-bit form (ld's). */
uint64_t orc_fused_sum(int t, int what, int cmp, const void *x, const void *y, int64_t n, uint64_t c, uint64_t e) {
    row_fn rv = what == 0 ? row_dot : (what == 1 ? row_sumsq : row_cond);
    if (is_float(t)) return canon(t, 0, rv, x, y, n, cmp, c, e);
    uint64_t acc = 0;
    for (int64_t i = 0; i < n; ++i) acc += rv(x, y, i, t, cmp, c, e);
    return acc;
}

/* fused.rs:145-179 (count_<cmp>) and :214-236 (filter_<cmp>, the survivors in order). */
int64_t orc_count_cmp(int t, int cmp, const void *x, int64_t n, uint64_t c) {
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i) k += cmp_test(t, cmp, ld(t, x, i), c);
    return k;
}

int64_t orc_filter_cmp(int t, int cmp, const void *x, int64_t n, uint64_t c, void *out) {
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i) {
        uint64_t v = ld(t, x, i);
        if (cmp_test(t, cmp, v, c)) st(t, out, k++, v);
    }
    return k;
}

/* ---------------------------------------------------------------- scans (scan.rs) */

/* scan.rs:248-282 (Scan::update, one update over all rows): row 0 and (scan_by) every row whose
 * start flag is set lift their value; every other row steps the running value. The output type
 * is the sum type for add, else the element type. */
void orc_scan(int t, int f, int by, const void *x, const uint8_t *starts, int64_t n, void *out) {
    int ot = f == FOLD_ADD ? sum_type(t) : t;
    uint64_t acc = 0;
    for (int64_t i = 0; i < n; ++i) {
        uint64_t v = ld(t, x, i);
        if (i == 0 || (by && starts[i])) acc = v;
        else acc = step(t, f, acc, v);
        if (f != FOLD_ADD) acc = wrap(t, acc);
        st(ot, out, i, acc);
    }
}

/* index.rs:194-222 (ReduceInto) with the bucket checks of :116-130 (checked_keys): the value
 * kind, then keys outside [0, nb) (the first in order) or a negative nb, then the lengths;
 * each bucket starts at the fold's identity and steps its rows in order. */
int orc_reduce_into(int t, int f, const int64_t *keys, int64_t nk, const void *vals, int64_t nv, int64_t nb,
                    void *out, char *err) {
    if (nb < 0) {
        snprintf(err, ORC_ERR_LEN, "negative bucket count %lld", (long long)nb);
        return 1;
    }
    for (int64_t i = 0; i < nk; ++i)
        if ((uint64_t)keys[i] >= (uint64_t)nb) {
            snprintf(err, ORC_ERR_LEN, "bucket key %lld out of range for %lld buckets", (long long)keys[i],
                     (long long)nb);
            return 1;
        }
    if (nk != nv) {
        snprintf(err, ORC_ERR_LEN, "length mismatch: %lld keys for %lld values", (long long)nk, (long long)nv);
        return 1;
    }
    int ot = f == FOLD_ADD ? sum_type(t) : t;
    uint64_t id = identity(ot, f);
    for (int64_t b = 0; b < nb; ++b) st(ot, out, b, id);
    for (int64_t i = 0; i < nk; ++i) {
        uint64_t acc = ld(ot, out, keys[i]);
        acc = step(t, f, acc, ld(t, vals, i));
        if (f != FOLD_ADD) acc = wrap(t, acc);
        st(ot, out, keys[i], acc);
    }
    return 0;
}

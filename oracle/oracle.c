/*
 * CPU oracle for the verkehrt kernel-table primitives: TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's scalar entries (antiguru/verkehrt,
 * src/kernels/scalar/*), each function citing the file:line it follows. It is the checker
 * of the parity tests and the "port" CPU baseline of bench.py. The CUDA library never
 * links, loads or calls it. Built with -O3 -ffp-contract=off so that no multiply-add is
 * contracted (the reference uses no FMA, docs/superpowers/specs/2026-10-30-verkehrt-design.md:162).
 *
 * Parity unpinned for the float extensions orc_reduce_into_add_f64, orc_scan_add_f64 and
 * orc_scan_by_add_f64: the reference has no such kernels and no golden vectors for them; they
 * restate the candidate orders of its tier-2 design notes and are checked against the
 * properties those notes state.
 */
#include "oracle.h"

#include <inttypes.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define LANES 16

/* ---------------------------------------------------------------- construction */

/* src/kernels/scalar/construct.rs:12-17 */
uint64_t orc_splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* construct.rs:64-76 with the f64 map of :243-250: element i = (splitmix64(seed+i)>>11) * 2^-53 */
void orc_rand_f64(int64_t n, int64_t seed, double *out) {
    uint64_t s = (uint64_t)seed;
    for (int64_t i = 0; i < n; ++i)
        out[i] = (double)(orc_splitmix64(s + (uint64_t)i) >> 11) * 0x1p-53;
}

/* construct.rs:233-240: element i = splitmix64(seed+i) as i64 */
void orc_rand_i64(int64_t n, int64_t seed, int64_t *out) {
    uint64_t s = (uint64_t)seed;
    for (int64_t i = 0; i < n; ++i) out[i] = (int64_t)orc_splitmix64(s + (uint64_t)i);
}

/* ---------------------------------------------------------------- canonical float order */

static inline double canon_op(int mul, double a, double b) { return mul ? a * b : a + b; }

/* reduce.rs:253-272: accumulators and tail start at the identity */
void orc_canon_init(orc_canon *s, int mul) {
    for (int j = 0; j < LANES; ++j) s->acc[j] = s->tail[j] = mul ? 1.0 : 0.0;
    s->tail_len = 0;
    s->mul = mul;
}

/* reduce.rs:274-308 (CanonicalAcc::feed / feed_blocks) with the lane loop of :45-62 */
int orc_canon_feed(orc_canon *s, const double *xs, int64_t n, char *err) {
    if (s->tail_len != 0) {
        snprintf(err, ORC_ERR_LEN, "canonical update after a partial block");
        return 1;
    }
    int64_t blocks = n / LANES;
    for (int64_t b = 0; b < blocks; ++b)
        for (int j = 0; j < LANES; ++j) s->acc[j] = canon_op(s->mul, s->acc[j], xs[b * LANES + j]);
    int rest = (int)(n - blocks * LANES);
    for (int j = 0; j < rest; ++j) s->tail[j] = xs[blocks * LANES + j];
    s->tail_len = rest;
    return 0;
}

/* reduce.rs:77-91 (finish_lanes): +8, +4, +2, +1, then the tail into lane 0 in order */
double orc_canon_finish(const orc_canon *s) {
    double acc[LANES];
    memcpy(acc, s->acc, sizeof acc);
    for (int step = LANES / 2; step > 0; step /= 2)
        for (int j = 0; j < step; ++j) acc[j] = canon_op(s->mul, acc[j], acc[j + step]);
    double r = acc[0];
    for (int j = 0; j < s->tail_len; ++j) r = canon_op(s->mul, r, s->tail[j]);
    return r;
}

static double canon_of(const double *x, int64_t n, int mul) {
    orc_canon s;
    char err[ORC_ERR_LEN];
    orc_canon_init(&s, mul);
    orc_canon_feed(&s, x, n, err);
    return orc_canon_finish(&s);
}

/* reduce.rs:253-323, registered as reduce_add_f64 / reduce_mul_f64 at :692-695 */
double orc_reduce_add_f64(const double *x, int64_t n) { return canon_of(x, n, 0); }
double orc_reduce_mul_f64(const double *x, int64_t n) { return canon_of(x, n, 1); }

/* fused.rs:73-106: the canonical sum of fl(x*y), the product rounded on its own (no FMA) */
double orc_dot_f64(const double *x, const double *y, int64_t n) {
    double acc[LANES] = {0};
    int64_t blocks = n / LANES;
    for (int64_t b = 0; b < blocks; ++b)
        for (int j = 0; j < LANES; ++j) {
            double p = x[b * LANES + j] * y[b * LANES + j];
            acc[j] = acc[j] + p;
        }
    for (int step = LANES / 2; step > 0; step /= 2)
        for (int j = 0; j < step; ++j) acc[j] = acc[j] + acc[j + step];
    double r = acc[0];
    for (int64_t i = blocks * LANES; i < n; ++i) {
        double p = x[i] * y[i];
        r = r + p;
    }
    return r;
}

/* fused.rs:108-141 */
double orc_sumsq_f64(const double *x, int64_t n) { return orc_dot_f64(x, x, n); }

/* fused.rs:45-54 (Cmp::test): IEEE comparisons, NaN compares false except for ne */
static inline int cmp_test(int cmp, double a, double b) {
    switch (cmp) {
    case ORC_EQ: return a == b;
    case ORC_NE: return a != b;
    case ORC_LT: return a < b;
    case ORC_LE: return a <= b;
    case ORC_GT: return a > b;
    default: return a >= b;
    }
}

/* fused.rs:145-147 (count_cmp), :150-179 (CountCmp) */
int64_t orc_count_cmp_f64(const double *x, int64_t n, int cmp, double c) {
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i) k += cmp_test(cmp, x[i], c);
    return k;
}

/* fused.rs:181-212 (CondSum): the canonical sum of the picked values */
double orc_condsum_cmp_f64(const double *x, int64_t n, int cmp, double c, double e) {
    double acc[LANES] = {0};
    int64_t blocks = n / LANES;
    for (int64_t b = 0; b < blocks; ++b)
        for (int j = 0; j < LANES; ++j) {
            double v = x[b * LANES + j];
            acc[j] = acc[j] + (cmp_test(cmp, v, c) ? v : e);
        }
    for (int step = LANES / 2; step > 0; step /= 2)
        for (int j = 0; j < step; ++j) acc[j] = acc[j] + acc[j + step];
    double r = acc[0];
    for (int64_t i = blocks * LANES; i < n; ++i) r = r + (cmp_test(cmp, x[i], c) ? x[i] : e);
    return r;
}

/* fused.rs:225-236 (filter_tile): count pass, then the predicated append of select.rs:70-77 */
int64_t orc_filter_cmp_f64(const double *x, int64_t n, int cmp, double c, double *out) {
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i)
        if (cmp_test(cmp, x[i], c)) out[k++] = x[i];
    return k;
}

/* ---------------------------------------------------------------- extremes */

/* elementwise.rs:412-424 (min2) and :426-440 (max2): IEEE 754-2019 minimum / maximum */
static inline double min2(double a, double b) {
    if (isnan(a) || isnan(b)) return NAN;
    if (a == b) return signbit(a) ? a : b;
    return a < b ? a : b;
}
static inline double max2(double a, double b) {
    if (isnan(a) || isnan(b)) return NAN;
    if (a == b) return !signbit(a) ? a : b;
    return a > b ? a : b;
}

/* reduce.rs:380-412 (Extreme) */
int orc_reduce_minmax_f64(const double *x, int64_t n, int is_max, double *out, char *err) {
    if (n == 0) {
        snprintf(err, ORC_ERR_LEN, "reduce_%s of an empty array", is_max ? "max" : "min");
        return 1;
    }
    double cur = x[0];
    for (int64_t i = 1; i < n; ++i) cur = is_max ? max2(cur, x[i]) : min2(cur, x[i]);
    *out = cur;
    return 0;
}

/* reduce.rs:186-197 (Ordered::less / greater for floats): -0.0 ranks below +0.0 */
static inline int f_less(double a, double b) {
    return a < b || (a == b && signbit(a) && !signbit(b));
}
static inline int f_greater(double a, double b) {
    return a > b || (a == b && !signbit(a) && signbit(b));
}

/* reduce.rs:417-468 (ArgExtreme): the first NaN, else the first index of the extreme */
int orc_argext_f64(const double *x, int64_t n, int is_max, int64_t *out, char *err) {
    if (n == 0) {
        snprintf(err, ORC_ERR_LEN, "%s of an empty array", is_max ? "argmax" : "argmin");
        return 1;
    }
    int64_t best = -1;
    double bv = 0;
    for (int64_t i = 0; i < n; ++i) {
        double v = x[i];
        if (isnan(v)) {
            *out = i;
            return 0;
        }
        int better = best < 0 || (is_max ? f_greater(v, bv) : f_less(v, bv));
        if (better) {
            best = i;
            bv = v;
        }
    }
    *out = best;
    return 0;
}

int orc_reduce_minmax_i64(const int64_t *x, int64_t n, int is_max, int64_t *out, char *err) {
    if (n == 0) {
        snprintf(err, ORC_ERR_LEN, "reduce_%s of an empty array", is_max ? "max" : "min");
        return 1;
    }
    int64_t cur = x[0];
    for (int64_t i = 1; i < n; ++i)
        cur = is_max ? (x[i] > cur ? x[i] : cur) : (x[i] < cur ? x[i] : cur);
    *out = cur;
    return 0;
}

int orc_argext_i64(const int64_t *x, int64_t n, int is_max, int64_t *out, char *err) {
    if (n == 0) {
        snprintf(err, ORC_ERR_LEN, "%s of an empty array", is_max ? "argmax" : "argmin");
        return 1;
    }
    int64_t best = 0;
    for (int64_t i = 1; i < n; ++i)
        if (is_max ? x[i] > x[best] : x[i] < x[best]) best = i;
    *out = best;
    return 0;
}

/* reduce.rs:331-377 (IntSum<i64>): wrapping */
int64_t orc_reduce_add_i64(const int64_t *x, int64_t n) {
    uint64_t s = 0;
    for (int64_t i = 0; i < n; ++i) s += (uint64_t)x[i];
    return (int64_t)s;
}

/* ---------------------------------------------------------------- selections */

/* select.rs:81-92 (compress_append) */
int64_t orc_compress(const void *x, int width, const uint8_t *mask, int64_t n, void *out) {
    const uint8_t *src = (const uint8_t *)x;
    uint8_t *dst = (uint8_t *)out;
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i)
        if (mask[i] != 0) memcpy(dst + (size_t)(k++) * width, src + (size_t)i * width, width);
    return k;
}

/* select.rs:98-104 (where_append): global row indices base + i */
int64_t orc_where(const uint8_t *mask, int64_t n, int64_t base, int64_t *out) {
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i)
        if (mask[i] != 0) out[k++] = base + i;
    return k;
}

/* ---------------------------------------------------------------- scans */

/* scan.rs:284-326 (Scan<i64, ScanSum<i64>, false>) */
void orc_scan_add_i64(const int64_t *x, int64_t n, int64_t *out) {
    uint64_t acc = 0;
    for (int64_t i = 0; i < n; ++i) {
        acc = i == 0 ? (uint64_t)x[0] : acc + (uint64_t)x[i];
        out[i] = (int64_t)acc;
    }
}

/* scan.rs:294-316 (BY = true): row 0 always starts; a nonzero start byte restarts */
void orc_scan_by_add_i64(const int64_t *x, const uint8_t *starts, int64_t n, int64_t *out) {
    uint64_t acc = 0;
    for (int64_t i = 0; i < n; ++i) {
        acc = (i == 0 || starts[i] != 0) ? (uint64_t)x[i] : acc + (uint64_t)x[i];
        out[i] = (int64_t)acc;
    }
}

/* Float scans: the reference has none (scan.rs:408-415 lists the gap). Its tier-2 design notes
 * (docs/superpowers/specs/2026-10-31-verkehrt-tier2-design.md:172) give the candidate order
 * restated here: out[i] is the canonical sum (reduce.rs:45-91) of the prefix x[0..=i], so
 * out[n - 1] is reduce_add_f64 of the whole array. One pass keeps the 16 lane accumulators:
 * before each 16-row block the lanes combine (+8, +4, +2, +1) into the prefix's base, the
 * block's first 15 rows fold into it in order (the canonical tail), and the 16th row's prefix
 * is the combine of the lanes after the block. scan_by restarts at every row whose start flag
 * is set (row 0 always starts), with the lanes numbered from the segment's first row. */
static void scan_f64_segment(const double *x, int64_t n, double *out) {
    double lanes[LANES];
    for (int j = 0; j < LANES; ++j) lanes[j] = 0.0;
    double base = 0.0; /* the combine of lanes that all hold +0.0 */
    for (int64_t b0 = 0; b0 < n; b0 += LANES) {
        int64_t cnt = n - b0 < LANES ? n - b0 : LANES;
        double t = base;
        for (int64_t r = 0; r < cnt && r < LANES - 1; ++r) {
            t = t + x[b0 + r];
            out[b0 + r] = t;
        }
        if (cnt == LANES) {
            double acc[LANES];
            for (int j = 0; j < LANES; ++j) acc[j] = lanes[j] = lanes[j] + x[b0 + j];
            for (int step = LANES / 2; step > 0; step /= 2)
                for (int j = 0; j < step; ++j) acc[j] = acc[j] + acc[j + step];
            base = acc[0];
            out[b0 + LANES - 1] = base;
        }
    }
}

void orc_scan_add_f64(const double *x, int64_t n, double *out) { scan_f64_segment(x, n, out); }

void orc_scan_by_add_f64(const double *x, const uint8_t *starts, int64_t n, double *out) {
    int64_t s = 0;
    for (int64_t i = 1; i <= n; ++i)
        if (i == n || starts[i] != 0) {
            scan_f64_segment(x + s, i - s, out + s);
            s = i;
        }
}

/* scan.rs:16-48 (Prev) */
void orc_prev_i64(const int64_t *x, int64_t n, int64_t fill, int64_t *out) {
    for (int64_t i = 0; i < n; ++i) out[i] = i == 0 ? fill : x[i - 1];
}

/* ---------------------------------------------------------------- index kernels */

/* index.rs:102-111 (first_out_of_range): values compare as unsigned, so negatives are out */
static int64_t first_out_of_range(const int64_t *v, int64_t n, uint64_t bound, int *found) {
    for (int64_t i = 0; i < n; ++i)
        if ((uint64_t)v[i] >= bound) {
            *found = 1;
            return v[i];
        }
    *found = 0;
    return 0;
}

/* index.rs:42-73 (Gather::checked / run) */
int orc_gather(const void *src, int width, int64_t nsrc, const int64_t *idx, int64_t nidx,
               void *out, char *err) {
    int found;
    int64_t bad = first_out_of_range(idx, nidx, (uint64_t)nsrc, &found);
    if (found) {
        snprintf(err, ORC_ERR_LEN, "gather index %" PRId64 " out of range for length %" PRIu64,
                 bad, (uint64_t)nsrc);
        return 1;
    }
    const uint8_t *s = (const uint8_t *)src;
    uint8_t *d = (uint8_t *)out;
    for (int64_t i = 0; i < nidx; ++i)
        memcpy(d + (size_t)i * width, s + (size_t)idx[i] * width, width);
    return 0;
}

/* value.rs:285-289 (byte_size) for an i64 result array */
static int check_i64_array_size(int64_t len, char *err) {
    if ((uint64_t)len > (uint64_t)INT64_MAX / 8) {
        snprintf(err, ORC_ERR_LEN, "array of %" PRIu64 " elements is too large", (uint64_t)len);
        return 1;
    }
    return 0;
}

/* index.rs:116-130 (checked_keys) */
static int checked_keys(const int64_t *keys, int64_t n, int64_t buckets, char *err) {
    if (buckets < 0) {
        snprintf(err, ORC_ERR_LEN, "negative bucket count %" PRId64, buckets);
        return 1;
    }
    int found;
    int64_t k = first_out_of_range(keys, n, (uint64_t)buckets, &found);
    if (found) {
        snprintf(err, ORC_ERR_LEN, "bucket key %" PRId64 " out of range for %" PRId64 " buckets",
                 k, buckets);
        return 1;
    }
    return 0;
}

/* index.rs:138-155 (Histogram): wrapping per-bucket counts */
int orc_histogram(const int64_t *keys, int64_t n, int64_t buckets, int64_t *out, char *err) {
    if (checked_keys(keys, n, buckets, err)) return 1;
    if (check_i64_array_size(buckets, err)) return 1;
    memset(out, 0, (size_t)buckets * 8);
    for (int64_t i = 0; i < n; ++i) out[keys[i]] += 1;
    return 0;
}

/* index.rs:194-222 (ReduceInto with ScanSum<i64>): empty buckets hold 0 */
int orc_reduce_into_add_i64(const int64_t *keys, const int64_t *vals, int64_t n,
                            int64_t buckets, int64_t *out, char *err) {
    if (checked_keys(keys, n, buckets, err)) return 1;
    if (check_i64_array_size(buckets, err)) return 1;
    memset(out, 0, (size_t)buckets * 8);
    for (int64_t i = 0; i < n; ++i) out[keys[i]] = (int64_t)((uint64_t)out[keys[i]] + (uint64_t)vals[i]);
    return 0;
}

/* reduce_into with f64 add: the reference has no such kernel (scan.rs:408-415). Its tier-2
 * design notes (docs/superpowers/specs/2026-10-31-verkehrt-tier2-design.md:171-172) give the
 * candidate order restated here: rows below b = n - n % 16 go to lane i % 16 of their bucket,
 * each lane adds its rows in index order from +0.0, the lanes combine pairwise (+8, +4, +2, +1),
 * and the bucket's rows from b on fold into the result in index order, the canonical sum's tail
 * rule (reduce.rs:77-91, finish_lanes). With every key equal this is reduce_add_f64, bit for
 * bit, the property the notes give. Empty buckets hold +0.0. */
int orc_reduce_into_add_f64(const int64_t *keys, const double *vals, int64_t n, int64_t buckets,
                            double *out, char *err) {
    if (checked_keys(keys, n, buckets, err)) return 1;
    if (check_i64_array_size(buckets, err)) return 1;
    double *lanes = (double *)calloc((size_t)buckets * 16 + 1, sizeof(double));
    if (!lanes) {
        snprintf(err, ORC_ERR_LEN, "cannot allocate an array of %" PRId64 " elements", buckets * 16);
        return 1;
    }
    const int64_t b = n - n % 16;
    for (int64_t i = 0; i < b; ++i) {
        double *l = lanes + keys[i] * 16 + (i & 15);
        *l = *l + vals[i];
    }
    for (int64_t k = 0; k < buckets; ++k) {
        double *l = lanes + k * 16;
        for (int step = 8; step > 0; step /= 2)
            for (int j = 0; j < step; ++j) l[j] = l[j] + l[j + step];
        out[k] = l[0];
    }
    for (int64_t i = b; i < n; ++i) out[keys[i]] = out[keys[i]] + vals[i];
    free(lanes);
    return 0;
}

/* ---------------------------------------------------------------- argsort */

typedef struct {
    uint64_t key;
    int64_t pos;
} kp;

static int kp_cmp(const void *a, const void *b) {
    const kp *x = (const kp *)a, *y = (const kp *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->pos < y->pos ? -1 : (x->pos > y->pos);
}

/* radix.rs:58-61: the sign-flip image maps signed order onto unsigned order */
static inline uint64_t image_i64(int64_t v) { return (uint64_t)v ^ (1ull << 63); }

/* index.rs:178-188 (argsort_reference): sort (key, position), which is stable */
void orc_argsort_reference_i64(const int64_t *x, int64_t n, int64_t *out) {
    kp *t = (kp *)malloc(sizeof(kp) * (size_t)(n ? n : 1));
    for (int64_t i = 0; i < n; ++i) {
        t[i].key = image_i64(x[i]);
        t[i].pos = i;
    }
    qsort(t, (size_t)n, sizeof(kp), kp_cmp);
    for (int64_t i = 0; i < n; ++i) out[i] = t[i].pos;
    free(t);
}

/* radix.rs:126-137 (argsort_into) and :190-259 (radix_into): one counting pass for all byte
 * digits, constant digits skipped, LSD scatter passes over (image, position) pairs. */
int orc_argsort_i64(const int64_t *x, int64_t n, int64_t *out, char *err) {
    if (n <= 1024) {
        orc_argsort_reference_i64(x, n, out);
        return 0;
    }
    static const int PASSES = 8;
    size_t (*counts)[256] = (size_t(*)[256])calloc(PASSES, sizeof(size_t[256]));
    for (int64_t i = 0; i < n; ++i) {
        uint64_t k = image_i64(x[i]);
        for (int p = 0; p < PASSES; ++p) counts[p][(k >> (8 * p)) & 255]++;
    }
    int active[8], passes = 0;
    uint64_t first = image_i64(x[0]);
    for (int p = 0; p < PASSES; ++p)
        if (counts[p][(first >> (8 * p)) & 255] != (size_t)n) active[passes++] = p;
    if (passes == 0) {
        for (int64_t i = 0; i < n; ++i) out[i] = i;
        free(counts);
        return 0;
    }
    kp *a = (kp *)malloc(sizeof(kp) * (size_t)n);
    kp *b = (kp *)malloc(sizeof(kp) * (size_t)n);
    if (!a || !b) {
        snprintf(err, ORC_ERR_LEN, "cannot allocate argsort scratch for %" PRId64 " rows", n);
        free(a);
        free(b);
        free(counts);
        return 1;
    }
    for (int64_t i = 0; i < n; ++i) {
        a[i].key = image_i64(x[i]);
        a[i].pos = i;
    }
    for (int ap = 0; ap < passes; ++ap) {
        int p = active[ap];
        size_t off[256], sum = 0;
        for (int d = 0; d < 256; ++d) {
            off[d] = sum;
            sum += counts[p][d];
        }
        for (int64_t i = 0; i < n; ++i) b[off[(a[i].key >> (8 * p)) & 255]++] = a[i];
        kp *t = a;
        a = b;
        b = t;
    }
    for (int64_t i = 0; i < n; ++i) out[i] = a[i].pos;
    free(a);
    free(b);
    free(counts);
    return 0;
}

/* ---------------------------------------------------------------- group_id */

/* group.rs:40-47 (mix), with a fixed odd multiplier: the ids do not depend on it */
static const uint64_t GROUP_MUL = 0x9E3779B97F4A7C15ull;
static inline uint64_t mix(uint64_t x, uint64_t mul) { return (x ^ (x >> 32)) * mul; }

static uint64_t next_pow2(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

typedef struct {
    uint64_t a, b;
    int64_t tag;
} gslot;

/* group.rs:207-257 (probe_into) with growth of :170-197: tags are id + 1, 0 is empty,
 * linear probing, growth right after an insert leaves the table more than half full. */
static int group_ids(const uint64_t *ka, const uint64_t *kb, int64_t n, int64_t *out,
                     char *err) {
    uint64_t max_slots = next_pow2((uint64_t)n * 2);
    uint64_t slots = max_slots < 2 ? 2 : (max_slots > 256 ? 256 : max_slots);
    if (max_slots < slots) max_slots = slots;
    int shift = 64 - __builtin_ctzll(slots);
    gslot *tab = (gslot *)calloc(slots, sizeof(gslot));
    if (!tab) {
        snprintf(err, ORC_ERR_LEN, "cannot allocate a group_id table of %" PRIu64 " slots", slots);
        return 1;
    }
    int64_t groups = 0;
    for (int64_t row = 0; row < n; ++row) {
        uint64_t a = ka[row], b = kb ? kb[row] : 0;
        uint64_t h = kb ? mix(mix(a, GROUP_MUL) ^ b, GROUP_MUL) : mix(a, GROUP_MUL);
        uint64_t i = h >> shift;
        for (;;) {
            if (tab[i].tag == 0) {
                tab[i].a = a;
                tab[i].b = b;
                tab[i].tag = ++groups;
                out[row] = groups - 1;
                break;
            }
            if (tab[i].a == a && tab[i].b == b) {
                out[row] = tab[i].tag - 1;
                break;
            }
            i = (i + 1) & (slots - 1);
        }
        if ((uint64_t)(2 * groups) > slots) {
            int distinct = 8 * groups >= 7 * (row + 1);
            uint64_t grown = slots << (distinct ? 3 : 1);
            if (grown > max_slots) grown = max_slots;
            int new_shift = shift - __builtin_ctzll(grown / slots);
            gslot *nt = (gslot *)calloc(grown, sizeof(gslot));
            if (!nt) {
                snprintf(err, ORC_ERR_LEN, "cannot allocate a group_id table of %" PRIu64
                         " slots for %" PRId64 " rows", grown, n);
                free(tab);
                return 1;
            }
            for (uint64_t s = 0; s < slots; ++s) {
                if (tab[s].tag == 0) continue;
                uint64_t hh = kb ? mix(mix(tab[s].a, GROUP_MUL) ^ tab[s].b, GROUP_MUL)
                                 : mix(tab[s].a, GROUP_MUL);
                uint64_t j = hh >> new_shift;
                while (nt[j].tag != 0) j = (j + 1) & (grown - 1);
                nt[j] = tab[s];
            }
            free(tab);
            tab = nt;
            slots = grown;
            shift = new_shift;
        }
    }
    free(tab);
    return 0;
}

/* group.rs:260-277 (GroupId<i64>) */
int orc_group_id_i64(const int64_t *x, int64_t n, int64_t *out, char *err) {
    return group_ids((const uint64_t *)x, NULL, n, out, err);
}

/* group.rs:280-301 (GroupId2<i64, i64>) */
int orc_group_id2_i64_i64(const int64_t *x, const int64_t *y, int64_t n, int64_t *out,
                          char *err) {
    return group_ids((const uint64_t *)x, (const uint64_t *)y, n, out, err);
}

/* ---------------------------------------------------------------- elementwise */

/* elementwise.rs:757-769 (mul_f64) */
void orc_mul_f64(const double *x, const double *y, int64_t n, double *out) {
    for (int64_t i = 0; i < n; ++i) out[i] = x[i] * y[i];
}

/* elementwise.rs:764-768 (lt/le/gt/ge) and the eq/ne of register_any */
void orc_cmp_f64(const double *x, const double *y, int64_t n, int cmp, uint8_t *out) {
    for (int64_t i = 0; i < n; ++i) out[i] = (uint8_t)cmp_test(cmp, x[i], y[i]);
}

/* elementwise.rs:231-239 (run_select): the first operand where the mask byte is nonzero */
void orc_select_f64(const uint8_t *m, const double *a, const double *b, int64_t n, double *out) {
    for (int64_t i = 0; i < n; ++i) out[i] = m[i] ? a[i] : b[i];
}

/* ---------------------------------------------------------------- accuracy helpers */

/* Neumaier, "Rundungsfehleranalyse einiger Verfahren zur Summation endlicher Summen" (1974) */
double orc_neumaier_sum(const double *x, int64_t n) {
    double s = 0, c = 0;
    for (int64_t i = 0; i < n; ++i) {
        double t = s + x[i];
        if (fabs(s) >= fabs(x[i])) c += (s - t) + x[i];
        else c += (x[i] - t) + s;
        s = t;
    }
    return s + c;
}

/* Ogita, Rump, Oishi, "Accurate Sum and Dot Product" (2005), Algorithm 4.4 (Sum2) with
 * Knuth's TwoSum, returned unnormalised as hi + lo. */
void orc_dd_sum(const double *x, int64_t n, double *hi, double *lo) {
    double s = 0, e = 0;
    for (int64_t i = 0; i < n; ++i) {
        double t = s + x[i];
        double z = t - s;
        double err = (s - (t - z)) + (x[i] - z);
        s = t;
        e += err;
    }
    *hi = s;
    *lo = e;
}

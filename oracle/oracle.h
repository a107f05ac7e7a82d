/*
 * CPU oracle for the verkehrt kernel-table primitives.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference's scalar
 * kernel entries (antiguru/verkehrt, src/kernels/scalar/*). It is the checker the
 * parity tests compare the CUDA library against, and the "port" CPU baseline that
 * bench.py times. The product library (libvkcuda.so) never links or calls it.
 *
 * Parity pin: the restatement is checked against the reference's own golden vectors
 * (src/kernels/tests.rs, src/kernels/scalar/index/tests.rs, tests/programs/*.dd and the
 * README example outputs), see tests/test_oracle_golden.py.
 *
 * Error strings are byte-identical to the reference's messages. Functions that can fail
 * return 0 on success and 1 on a kernel error, with the message in `err` (ORC_ERR_LEN).
 */
#ifndef VERKEHRT_ORACLE_H
#define VERKEHRT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_ERR_LEN 256

/* Comparison numbers, the order of CMPS in src/kernels/scalar/fused.rs:31-38. */
enum { ORC_EQ = 0, ORC_NE = 1, ORC_LT = 2, ORC_LE = 3, ORC_GT = 4, ORC_GE = 5 };

/* construct.rs:12-17, :64-76, :233-251 */
uint64_t orc_splitmix64(uint64_t x);
void orc_rand_f64(int64_t n, int64_t seed, double *out);
void orc_rand_i64(int64_t n, int64_t seed, int64_t *out);

/* Canonical 16-lane float state, reduce.rs:253-323. `mul` selects the product. */
typedef struct {
    double acc[16];
    double tail[16];
    int tail_len;
    int mul;
} orc_canon;
void orc_canon_init(orc_canon *s, int mul);
/* Feeds n rows. Fails like CanonicalAcc::feed_blocks (a partial block pending). */
int orc_canon_feed(orc_canon *s, const double *xs, int64_t n, char *err);
double orc_canon_finish(const orc_canon *s);

double orc_reduce_add_f64(const double *x, int64_t n);
double orc_reduce_mul_f64(const double *x, int64_t n);
/* fused.rs:73-106 (dot), :108-141 (sumsq) */
double orc_dot_f64(const double *x, const double *y, int64_t n);
double orc_sumsq_f64(const double *x, int64_t n);
/* fused.rs:145-179 */
int64_t orc_count_cmp_f64(const double *x, int64_t n, int cmp, double c);
/* fused.rs:181-212, the sum of x where x <cmp> c, and e elsewhere */
double orc_condsum_cmp_f64(const double *x, int64_t n, int cmp, double c, double e);
/* fused.rs:225-236 + select.rs:36-77: returns the survivor count, writes them to out */
int64_t orc_filter_cmp_f64(const double *x, int64_t n, int cmp, double c, double *out);

/* reduce.rs:380-412 with min2/max2 of elementwise.rs:414-440 */
int orc_reduce_minmax_f64(const double *x, int64_t n, int is_max, double *out, char *err);
/* reduce.rs:417-468 */
int orc_argext_f64(const double *x, int64_t n, int is_max, int64_t *out, char *err);
int orc_reduce_minmax_i64(const int64_t *x, int64_t n, int is_max, int64_t *out, char *err);
int orc_argext_i64(const int64_t *x, int64_t n, int is_max, int64_t *out, char *err);
/* reduce.rs:331-377, wrapping i64 sum */
int64_t orc_reduce_add_i64(const int64_t *x, int64_t n);

/* select.rs:81-104: width is the element size in bytes */
int64_t orc_compress(const void *x, int width, const uint8_t *mask, int64_t n, void *out);
int64_t orc_where(const uint8_t *mask, int64_t n, int64_t base, int64_t *out);

/* scan.rs:284-326: inclusive wrapping prefix sum, and the segmented one */
void orc_scan_add_i64(const int64_t *x, int64_t n, int64_t *out);
void orc_scan_by_add_i64(const int64_t *x, const uint8_t *starts, int64_t n, int64_t *out);
/* the tier-2 notes' candidate float scan order (no reference kernel): prefix canonical sums */
void orc_scan_add_f64(const double *x, int64_t n, double *out);
void orc_scan_by_add_f64(const double *x, const uint8_t *starts, int64_t n, double *out);
/* scan.rs:16-48 */
void orc_prev_i64(const int64_t *x, int64_t n, int64_t fill, int64_t *out);

/* index.rs:42-73, :102-111 */
int orc_gather(const void *src, int width, int64_t nsrc, const int64_t *idx, int64_t nidx,
               void *out, char *err);
/* index.rs:116-155 and :194-222 */
int orc_histogram(const int64_t *keys, int64_t n, int64_t buckets, int64_t *out, char *err);
int orc_reduce_into_add_f64(const int64_t *keys, const double *vals, int64_t n, int64_t buckets,
                            double *out, char *err);
int orc_reduce_into_add_i64(const int64_t *keys, const int64_t *vals, int64_t n,
                            int64_t buckets, int64_t *out, char *err);

/* radix.rs:126-259 (LSD radix with constant-digit skip; comparison sort at <= 1024 rows) */
int orc_argsort_i64(const int64_t *x, int64_t n, int64_t *out, char *err);
/* index.rs:178-188, the comparison-sort restatement that pins the radix sort */
void orc_argsort_reference_i64(const int64_t *x, int64_t n, int64_t *out);

/* group.rs:207-301: first-occurrence ids, open addressing with linear probing */
int orc_group_id_i64(const int64_t *x, int64_t n, int64_t *out, char *err);
int orc_group_id2_i64_i64(const int64_t *x, const int64_t *y, int64_t n, int64_t *out,
                          char *err);

/* elementwise.rs: mul_f64, the comparisons, select_f64 */
void orc_mul_f64(const double *x, const double *y, int64_t n, double *out);
void orc_cmp_f64(const double *x, const double *y, int64_t n, int cmp, uint8_t *out);
void orc_select_f64(const uint8_t *m, const double *a, const double *b, int64_t n, double *out);

/* elementwise.c: every array type (type codes of vkc_type). */
int orc_ew_binary(const char *op, int type, const void *a, int as, const void *b, int bs, int64_t n, void *out);
int orc_ew_unary(const char *op, int type, const void *a, int64_t n, void *out);
void orc_ew_select(int width, const uint8_t *m, int ms, const void *a, int as, const void *b, int bs, int64_t n,
                   void *out);
int orc_ew_cast(int src, int dst, const void *a, int64_t n, void *out);
int orc_ew_div_const(int type, const void *a, const void *d, int64_t n, void *out, char *err);

/* Accuracy helpers (not reference semantics): Neumaier's compensated sum and an exact
 * double-double accumulation, used to state error bounds. */
double orc_neumaier_sum(const double *x, int64_t n);
void orc_dd_sum(const double *x, int64_t n, double *hi, double *lo);

/* families.c: the kernel families on every element type. Types are vkc_type numbers (0 f64,
 * 1 f32, 2 i64, 3 u64, 4 i32, 5 u8, 6 bool); folds 0 add, 1 mul, 2 min, 3 max, 4 and, 5 or, 6 xor.
 * Values are 64-bit words (i32 sign-extended, u8/bool zero-extended, f32 as its 32 bits). */
int orc_fold(int t, int f, const void *x, int64_t n, uint64_t *out, char *err);
int orc_argext(int t, int is_max, const void *x, int64_t n, int64_t *out, char *err);
uint64_t orc_fused_sum(int t, int what, int cmp, const void *x, const void *y, int64_t n, uint64_t c, uint64_t e);
int64_t orc_count_cmp(int t, int cmp, const void *x, int64_t n, uint64_t c);
int64_t orc_filter_cmp(int t, int cmp, const void *x, int64_t n, uint64_t c, void *out);
void orc_scan(int t, int f, int by, const void *x, const uint8_t *starts, int64_t n, void *out);
int orc_reduce_into(int t, int f, const int64_t *keys, int64_t nk, const void *vals, int64_t nv, int64_t nb,
                    void *out, char *err);

#ifdef __cplusplus
}
#endif
#endif

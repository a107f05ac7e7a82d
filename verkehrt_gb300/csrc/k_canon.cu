// The canonical f64 sums: reduce_add_f64, dot_f64, sumsq_f64 and condsum_<cmp>_f64, bit-exact
// to the reference's canonical order at every length; and, built on the same pass, the float
// scans scan_add_f64 and scan_by_add_f64 (prefix canonical sums, at the end of the file).
//
// Reference order (src/kernels/scalar/reduce.rs:45-91, :253-323; the spec in
// docs/superpowers/specs/2026-10-30-verkehrt-design.md:155-160): lane j (0..15) starts at +0.0
// and adds rows j, j+16, j+32, ... below b = n - n%16 one after another; then lanes combine
// +8, +4, +2, +1; then the tail rows are added to lane 0 in order. dot/sumsq/condsum feed
// the row values fl(x*y), fl(x*x), (x <cmp> c ? x : e) to the same order
// (src/kernels/scalar/fused.rs:73-212).
//
// A lane is a chain of n/16 dependent roundings, which a plain GPU tree cannot reproduce. This
// kernel reproduces it exactly and in parallel:
//
//  * While a lane's running sum s stays in one binade [2^E, 2^(E+1)), with u = 2^(E-52),
//    s = S*u for an integer S in [2^52, 2^53), and for x >= 0 the rounded step is
//    fl(s + x) = (S + RNE(x/u)) * u, exactly, as long as the result stays below 2^53 * u.
//    RNE(x/u) depends on S only through its parity when x/u is exactly halfway. So the effect
//    of a run of rows on S is a pair of integer increments (d0, d1) for even and odd S: a
//    "transfer function". Transfer functions compose associatively.
//  * The rows are cut into 4096-row tiles (256 blocks of 16 rows, 256 rows per lane, in 32
//    segments of 8 blocks), and these kernels, none of which waits on another block, find the
//    exact lane states:
//      K1  the approximate (float) lane sums of every tile, estimated from one 16-row block
//          per segment (an eighth of the rows);
//      K2  per lane, their exclusive prefix over the tiles from the lane's exact state (group
//          sums, then a scan inside each group), and each tile's candidate binades (the
//          approximate range widened by 2^-12 must lie in one binade or two adjacent ones);
//      K3  each tile's transfer function per lane and candidate binade, in one read of the
//          rows; then the check: K2 again on K3's own sums, and K3 again on the few tiles whose
//          binades the sampled candidates missed or that hold negative rows;
//      K4a per lane and 32-tile chunk, the composed transfer function when the chunk's tiles
//          share one;
//      K4b per lane, a walk from the exact state: whole chunks while their transfer function
//          holds, single tiles in mixed chunks, and the tiles none carries (binade crossings,
//          negative, infinite or NaN rows, the first rows of a lane) resolved from the rows by
//          a warp that recomputes their segments' transfer functions and adds the rows of any
//          segment without one one by one with IEEE f64 adds (the reference's own operation).
//    So the result is the reference's in every case.
//
// All of the per-row work is integer arithmetic: GB300 executes FP64 adds at about 1/66 of
// its integer op rate, so an FP64 tree would be compute-bound well below the HBM roofline.
#include <algorithm>
#include <climits>
#include <cmath>

#include "lookback.cuh"
#include "reduce_common.h"

namespace vkc {

int64_t scan_counts_sum_words(int64_t m);
void scan_counts(vkc_ctx *ctx, const unsigned *c, int64_t m, unsigned *sums, unsigned *out);

constexpr int CT_THREADS = 256;
constexpr int CT_SEGS = 32;       // segments per tile
constexpr int CT_SEG_BLOCKS = 8;  // 16-row blocks per segment
constexpr int CT_BLOCKS = CT_SEGS * CT_SEG_BLOCKS;  // 256 blocks = 4096 rows per tile
constexpr unsigned long long MANT = 0xfffffffffffffull;
constexpr unsigned long long ONE52 = 1ull << 52;
constexpr unsigned long long SAT = 1ull << 60;
constexpr int NO_E = INT_MIN;

enum RowOp { ROW_SUM = 0, ROW_DOT = 1, ROW_SUMSQ = 2, ROW_CONDSUM = 3 };

struct RowArgs {
    const unsigned long long *x;
    const unsigned long long *y;
    CmpRange r;
    unsigned long long e;
};

__device__ __forceinline__ double as_f64(unsigned long long b) { return __longlong_as_double(static_cast<long long>(b)); }
__device__ __forceinline__ unsigned long long as_bits(double d) { return static_cast<unsigned long long>(__double_as_longlong(d)); }

// The row value fed to the lane (fused.rs:77-98, :112-127, :190-203). Products are single
// IEEE multiplies (no FMA contraction: the file is built with -fmad=false).
template <int OP>
__device__ __forceinline__ unsigned long long row_value(const RowArgs &a, unsigned long long xv,
                                                        unsigned long long yv) {
    if (OP == ROW_DOT) return as_bits(__dmul_rn(as_f64(xv), as_f64(yv)));
    if (OP == ROW_SUMSQ) return as_bits(__dmul_rn(as_f64(xv), as_f64(xv)));
    if (OP == ROW_CONDSUM) return in_range(a.r, xv) ? xv : a.e;
    return xv;
}

// A transfer function: the increment of S for an even (d0) and odd (d1) start, saturated.
struct TF {
    unsigned long long d0, d1;
};

__device__ __forceinline__ unsigned long long sat_add(unsigned long long a, unsigned long long b) {
    unsigned long long s = a + b;
    return s > SAT ? SAT : s;
}

// Rows of both signs: a signed transfer function {up, dn | SIGNED_TF}, for rows with no tie
// (no parity dependence): up and dn are the sums of the increments of the positive and the
// negative rows, so the net increment is up - dn and every state between stays within
// [S - dn, S + up]. An unsigned one without a parity dependence (d0 == d1) has the signed
// form {d0, 0}. Saturated parts (at SAT) never apply. (Exact running bounds, the prefix's
// maximum and minimum stored as rounded-up floats, were slower: a sum that wanders around
// zero crosses binades whatever the bounds, and the encoding lengthened the walk.)
constexpr unsigned long long SIGNED_TF = 1ull << 63;

__device__ __forceinline__ bool as_signed(TF f, unsigned long long *up, unsigned long long *dn) {
    if (f.d1 & SIGNED_TF) {
        *up = f.d0;
        *dn = f.d1 & ~SIGNED_TF;
        return true;
    }
    if (f.d0 != f.d1) return false;
    *up = f.d0;
    *dn = 0;
    return true;
}

// a, then b. SIGNED = false: both are known to be unsigned (the code without the signed case).
template <bool SIGNED = true>
__device__ __forceinline__ TF compose(TF a, TF b) {
    if (!SIGNED || !((a.d1 | b.d1) & SIGNED_TF)) {
        TF r;
        r.d0 = sat_add(a.d0, (a.d0 & 1) ? b.d1 : b.d0);
        r.d1 = sat_add(a.d1, (a.d1 & 1) ? b.d0 : b.d1);
        return r;
    }
    unsigned long long au, ad, bu, bd;
    if (!as_signed(a, &au, &ad) || !as_signed(b, &bu, &bd)) return TF{SAT, SAT | SIGNED_TF};  // never applies
    return TF{sat_add(au, bu), sat_add(ad, bd) | SIGNED_TF};
}

// Applies f (valid in binade E) to the lane state with bits s. Fails when |s| is not a normal
// in binade E or when a state on the way could leave the binade. A negative state is the
// mirror image: round-to-nearest-even is symmetric, so its magnitude moves by the negated
// increments (only for functions without a parity dependence). A signed function keeps every
// state on the way at least one ulp above 2^E, so each exact sum lies in the binade.
// SIGNED = false: positive states and unsigned functions only (fails otherwise).
template <bool SIGNED = true>
__device__ __forceinline__ bool apply(unsigned long long s, int E, TF f, unsigned long long *out) {
    const unsigned long long ef = static_cast<unsigned long long>(E + 1023);
    const unsigned long long neg = SIGNED ? s >> 63 : 0;
    if (!SIGNED && (s >> 63)) return false;
    if (((s >> 52) & 0x7ff) != ef) return false;
    const unsigned long long S = (s & MANT) | ONE52;
    unsigned long long S2;
    if (!SIGNED || (!neg && !(f.d1 & SIGNED_TF))) {
        S2 = S + ((S & 1) ? f.d1 : f.d0);
        if (S2 >= (ONE52 << 1)) return false;
    } else {
        unsigned long long up, dn;
        if (!as_signed(f, &up, &dn)) return false;
        if (neg) {
            const unsigned long long x = up;
            up = dn;
            dn = x;
        }
        if (up >= ONE52 || dn >= ONE52 || S + up >= (ONE52 << 1) || (dn && S - dn <= ONE52)) return false;
        S2 = S + up - dn;
    }
    *out = (neg << 63) | (ef << 52) | (S2 & MANT);
    return true;
}

// The transfer function of 16 row values in binade E (KE = 1023 + E >= 64). Returns false
// when a row is negative, infinite, NaN or not below 2^E (k < 1), where the integer step does
// not hold. For x = M * 2^(ex-1075), x/u = M / 2^k with k = KE - ex, and
// RNE(x/u) = (M + 2^(k-1)) >> k unless M mod 2^k is exactly 2^(k-1) (a tie).
// seg_tf of a segment with negative rows (exmax: the largest exponent field, below KE): the
// increments of the magnitudes, positive and negative rows apart, as a signed function; a
// segment with a halfway row has none (the walk adds it from the rows).
__device__ __forceinline__ bool seg_tf_signed(const unsigned long long (&v)[CT_SEG_BLOCKS][2], int h, int KE,
                                              unsigned exmax, TF *out) {
    const unsigned kmin = static_cast<unsigned>(KE) - exmax;
    const unsigned low = kmin > 32 ? 0xffffffffu : (1u << (kmin - 1)) - 1u;
    unsigned long long tp = 0, tn = 0;
    unsigned op = 0, on = 0;
    bool maybe_tie = false;
#pragma unroll
    for (int i = 0; i < CT_SEG_BLOCKS; ++i) {
        const unsigned long long b = v[i][h];
        const unsigned k = min(static_cast<unsigned>(KE) - (static_cast<unsigned>(b >> 52) & 0x7ffu), 63u);
        const unsigned long long t = ((b & MANT) | ONE52) >> (k - 1);
        if (b >> 63) {
            tn += t;
            on += static_cast<unsigned>(t) & 1u;
        } else {
            tp += t;
            op += static_cast<unsigned>(t) & 1u;
        }
        maybe_tie |= (k <= 53u) & ((static_cast<unsigned>(b) & low) == 0u);
    }
    if (!maybe_tie) {
        *out = TF{(tp + op) >> 1, ((tn + on) >> 1) | SIGNED_TF};
        return true;
    }
    unsigned long long up = 0, dn = 0;
#pragma unroll
    for (int i = 0; i < CT_SEG_BLOCKS; ++i) {
        const unsigned long long b = v[i][h];
        const unsigned k = min(static_cast<unsigned>(KE) - (static_cast<unsigned>(b >> 52) & 0x7ffu), 63u);
        const unsigned long long w = ((b & MANT) | ONE52) + (1ull << (k - 1));
        if ((w << (64 - k)) == 0) return false;  // a halfway row
        if (b >> 63) dn += w >> k;
        else up += w >> k;
    }
    *out = TF{up, dn | SIGNED_TF};
    return true;
}

// SIGNED: rows of either sign (seg_tf_signed for a segment with a negative row); otherwise a
// negative row's exponent field with its sign bit is at least 2048, above any KE, and the
// segment has no function.
template <bool SIGNED>
__device__ __forceinline__ bool seg_tf(const unsigned long long (&v)[CT_SEG_BLOCKS][2], int h,
                                       int KE, TF *out) {
    unsigned exmax = 0, sgn = 0;
#pragma unroll
    for (int i = 0; i < CT_SEG_BLOCKS; ++i) {
        exmax = max(exmax, static_cast<unsigned>(v[i][h] >> 52) & (SIGNED ? 0x7ffu : 0xfffu));
        if (SIGNED) sgn |= static_cast<unsigned>(v[i][h] >> 63);
    }
    if (exmax >= static_cast<unsigned>(KE)) return false;
    if (SIGNED && sgn) return seg_tf_signed(v, h, KE, exmax, out);
    // (A 32-bit form of this loop for segments with kmin >= 26, every t below 2^28, needs more
    // registers: at 3 blocks per SM instead of 4 it made K3 slower, 0.75 against 0.72 ms.)
    // Every row has k = KE - ex >= kmin >= 1. With t = floor(M / 2^(k-1)) (the quotient with
    // one more bit), round-half-up gives (t + 1) >> 1, so the sum of the increments is
    // (sum of t + number of odd t) / 2. That is RNE unless a row is exactly halfway: k <= 53 and
    // no bit of M below the half bit (k - 1); bits 0 .. kmin - 2 are among those bits, so a
    // row with one of them set is no tie. Zero and subnormal rows have k = 63: t = 0, no tie.
    const unsigned kmin = static_cast<unsigned>(KE) - exmax;
    const unsigned low = kmin > 32 ? 0xffffffffu : (1u << (kmin - 1)) - 1u;
    unsigned long long tsum = 0;
    unsigned odd = 0;
    bool maybe_tie = false;
#pragma unroll
    for (int i = 0; i < CT_SEG_BLOCKS; ++i) {
        const unsigned long long b = v[i][h];
        const unsigned k = min(static_cast<unsigned>(KE) - static_cast<unsigned>(b >> 52), 63u);
        const unsigned long long t = ((b & MANT) | ONE52) >> (k - 1);
        tsum += t;
        odd += static_cast<unsigned>(t) & 1u;
        maybe_tie |= (k <= 53u) & ((static_cast<unsigned>(b) & low) == 0u);
    }
    if (!maybe_tie) {
        const unsigned long long D = (tsum + odd) >> 1;
        *out = TF{D, D};
        return true;
    }
    unsigned long long D = 0;
    bool tie = false;
#pragma unroll
    for (int i = 0; i < CT_SEG_BLOCKS; ++i) {
        unsigned long long b = v[i][h];
        unsigned k = min(static_cast<unsigned>(KE - static_cast<int>(b >> 52)), 63u);
        unsigned long long M = (b & MANT) | ONE52;
        unsigned long long w = M + (1ull << (k - 1));
        D += w >> k;
        tie |= (w << (64 - k)) == 0;
    }
    if (!tie) {
        *out = TF{D, D};
        return true;
    }
    // Ties: both parities, in row order. A tie rounds S + floor(x/u) + 1/2 to the even
    // neighbour, so the increment is floor(x/u) plus the parity of S + floor(x/u).
    unsigned long long d0 = 0, d1 = 0;
    for (int i = 0; i < CT_SEG_BLOCKS; ++i) {
        unsigned long long b = v[i][h];
        unsigned k = min(static_cast<unsigned>(KE - static_cast<int>(b >> 52)), 63u);
        unsigned long long M = (b & MANT) | ONE52;
        unsigned long long w = M + (1ull << (k - 1));
        unsigned long long inc = w >> k;
        if ((w << (64 - k)) == 0) {
            unsigned long long q = inc - 1;
            d0 += q + ((d0 + q) & 1);
            d1 += q + ((1 + d1 + q) & 1);
        } else {
            d0 += inc;
            d1 += inc;
        }
    }
    *out = TF{d0, d1};
    return true;
}

// A float approximation of a double from its high word: exponent rebias and mantissa
// truncation, values below 2^-126 flushed to 0 and above 2^127 clamped. Only used to find the
// binade of the running sum, with a margin far above its error.
__device__ __forceinline__ float approx_f32(unsigned long long b) {
    unsigned hi = static_cast<unsigned>(b >> 32);
    unsigned mag = hi & 0x7fffffffu;
    unsigned r = mag < (897u << 20) ? 0u : (mag >= (1151u << 20) ? 0x7f7fffffu : (mag - (896u << 20)) << 3);
    return __uint_as_float(r | (hi & 0x80000000u));
}

// Binade of a positive normal double, NO_E otherwise.
__device__ __forceinline__ int binade(double v) {
    if (!(v >= 0x1p-900) || !(v < 0x1p1000)) return NO_E;
    return static_cast<int>(as_bits(v) >> 52) - 1023;
}

// Reducer state on the device.
struct CanonState {
    unsigned long long lanes[16];
    unsigned long long tail[16];
    unsigned long long result;
};

// Per-launch work arrays, in the context scratch arena. T = number of 4096-row tiles.
struct CanonWork {
    float *apx;                // [16][T] approximate lane sums of each tile
    int *cand;                 // [T][16][2] candidate binades (NO_E when absent)
    int *recE;                 // [16][T][2] binade of each tile transfer function (NO_E: none)
    TF *recD;                  // [16][T][2]
    int *chunkE;               // [16][C] binade of each 32-tile chunk's transfer function
    TF *chunkD;                // [16][C]
    double *gsum;              // [16][G] approximate sum of each group of CAND_GROUP tiles
    int *flags;                // [T] tiles whose transfer functions are recomputed (K3 again);
                               // [T]: some tile has a negative row; [T + 1]: the number of
                               // flagged tiles, listed from [T + 2]
    unsigned long long *tstate = nullptr;  // scans: [16][T + 1] exact lane state before each tile
    int *whole = nullptr;                  // scans: [16][C] chunks the walk took whole
    int *resume = nullptr;                 // reductions: [16] tile where the lane chain takes over
                                           // from the walk (T: the walk finished the lane)
};

constexpr int CAND_GROUP = 1024;  // tiles per K2 block

__device__ __forceinline__ TF shfl_tf(TF v, int src) {
    return TF{__shfl_sync(FULL, v.d0, src), __shfl_sync(FULL, v.d1, src)};
}
__device__ __forceinline__ TF shfl_up_tf(TF v, int o) {
    return TF{__shfl_up_sync(FULL, v.d0, o), __shfl_up_sync(FULL, v.d1, o)};
}

// Loads the thread's 8 blocks x 2 lanes of tile `tile` and computes the row values. Rows past
// the last block read as +0.0, which leaves every lane state unchanged (a lane is never -0).
template <int OP, bool ALIGNED>
__device__ __forceinline__ void load_tile(const RowArgs &args, int64_t nb, int tile, int lp, int seg,
                                          unsigned long long (&v)[CT_SEG_BLOCKS][2]) {
    const int64_t blk0 = static_cast<int64_t>(tile) * CT_BLOCKS;
#pragma unroll
    for (int i = 0; i < CT_SEG_BLOCKS; ++i) {
        int64_t b = blk0 + seg * CT_SEG_BLOCKS + i;
        unsigned long long x0 = 0, x1 = 0, y0 = 0, y1 = 0;
        if (b < nb) {
            int64_t r = b * 16 + 2 * lp;
            if (ALIGNED) {
                ulonglong2 xv = __ldcs(reinterpret_cast<const ulonglong2 *>(args.x + r));
                x0 = xv.x;
                x1 = xv.y;
                if (OP == ROW_DOT) {
                    ulonglong2 yv = __ldcs(reinterpret_cast<const ulonglong2 *>(args.y + r));
                    y0 = yv.x;
                    y1 = yv.y;
                }
            } else {
                x0 = __ldcs(args.x + r);
                x1 = __ldcs(args.x + r + 1);
                if (OP == ROW_DOT) {
                    y0 = __ldcs(args.y + r);
                    y1 = __ldcs(args.y + r + 1);
                }
            }
            v[i][0] = row_value<OP>(args, x0, y0);
            v[i][1] = row_value<OP>(args, x1, y1);
        } else {
            v[i][0] = 0;
            v[i][1] = 0;
        }
    }
}

// The float image of a row value: products are taken of the float images (the sums only
// choose the candidate binades, so their error costs time, never exactness).
template <int OP>
__device__ __forceinline__ float approx_row(const RowArgs &a, unsigned long long xv, unsigned long long yv) {
    if (OP == ROW_DOT) return approx_f32(xv) * approx_f32(yv);
    if (OP == ROW_SUMSQ) {
        const float f = approx_f32(xv);
        return f * f;
    }
    if (OP == ROW_CONDSUM) return approx_f32(in_range(a.r, xv) ? xv : a.e);
    return approx_f32(xv);
}

// K1: the approximate lane sums of every tile (float sums of float images), from the first
// 16-row block of each segment only (one 128-byte line in CT_SEG_BLOCKS, scaled up): the sums
// choose K3's candidate binades, and K3's own sums check them afterwards (K2c), so an estimate
// that sampling got wrong costs a second transfer function for that tile, never exactness.
constexpr int CT_SAMPLE = CT_SEG_BLOCKS;
constexpr int APX_TILES = 8;
template <int OP, bool ALIGNED>
__global__ void __launch_bounds__(CT_THREADS) canon_apx_kernel(RowArgs args, int64_t nb, int T, CanonWork wk) {
    // APX_TILES tiles per block: each thread has one sampled load per tile in flight at once.
    __shared__ float s_apx[APX_TILES][CT_SEGS][16];
    const int t = threadIdx.x, lp = t & 7, seg = t >> 3;
    const int tile0 = blockIdx.x * APX_TILES;
    unsigned long long x[APX_TILES][2], y[APX_TILES][2];
    unsigned in = 0;  // bit q: the sampled block of tile q exists
#pragma unroll
    for (int q = 0; q < APX_TILES; ++q) {
        const int64_t b = static_cast<int64_t>(tile0 + q) * CT_BLOCKS + seg * CT_SEG_BLOCKS;
        x[q][0] = x[q][1] = y[q][0] = y[q][1] = 0;
        if (tile0 + q < T && b < nb) {
            in |= 1u << q;
            const int64_t r = b * 16 + 2 * lp;
            if (ALIGNED) {
                const ulonglong2 xv = __ldcs(reinterpret_cast<const ulonglong2 *>(args.x + r));
                x[q][0] = xv.x;
                x[q][1] = xv.y;
                if (OP == ROW_DOT) {
                    const ulonglong2 yv = __ldcs(reinterpret_cast<const ulonglong2 *>(args.y + r));
                    y[q][0] = yv.x;
                    y[q][1] = yv.y;
                }
            } else {
                x[q][0] = __ldcs(args.x + r);
                x[q][1] = __ldcs(args.x + r + 1);
                if (OP == ROW_DOT) {
                    y[q][0] = __ldcs(args.y + r);
                    y[q][1] = __ldcs(args.y + r + 1);
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < APX_TILES; ++q) {
        const bool ok = (in >> q) & 1u;
        s_apx[q][seg][2 * lp] = ok ? approx_row<OP>(args, x[q][0], y[q][0]) * static_cast<float>(CT_SAMPLE) : 0.f;
        s_apx[q][seg][2 * lp + 1] = ok ? approx_row<OP>(args, x[q][1], y[q][1]) * static_cast<float>(CT_SAMPLE) : 0.f;
    }
    __syncthreads();
    if (t < 16 * APX_TILES) {
        const int q = t >> 4, L = t & 15;
        float A = 0.f;
        for (int sg = 0; sg < CT_SEGS; ++sg) A += s_apx[q][sg][L];
        if (tile0 + q < T) wk.apx[static_cast<int64_t>(L) * T + tile0 + q] = A;
    }
}

// K2a: per lane and group of CAND_GROUP tiles (one block each), the approximate sum of the
// group's tiles.
__global__ void __launch_bounds__(256) canon_gsum_kernel(int T, int G, CanonWork wk) {
    const int L = blockIdx.x / G, g = blockIdx.x % G;
    const float *a = wk.apx + static_cast<int64_t>(L) * T;
    double s = 0;
    for (int k = g * CAND_GROUP + threadIdx.x; k < min(T, (g + 1) * CAND_GROUP); k += 256) s += static_cast<double>(a[k]);
    s = warp_sum(s);
    __shared__ double s_w[8];
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < 8; ++w) t += s_w[w];
        wk.gsum[L * G + g] = t;
    }
}

// K2b: per lane and group (one block each, CAND_PER tiles per thread), the exclusive prefix
// of the approximate sums over the lane's tiles from its exact state, and each tile's
// candidate binades: the range [start, end] widened by 2^-12 on each side must lie in one
// binade or two adjacent ones. The prefix inside the group is a float scan (its error, a few
// float roundings, is far inside the margin); the groups before it and the state are added in
// double.
constexpr int CAND_THREADS = 256;
constexpr int CAND_PER = CAND_GROUP / CAND_THREADS;

// CHECK (K2c, after K3 and the refined sums of canon_refine_kernel): a tile whose new
// candidates include a binade that its K3 candidates did not gets the new ones and a flag.
template <bool CHECK>
__global__ void __launch_bounds__(CAND_THREADS) canon_cand_kernel(int T, int G, CanonWork wk, const CanonState *state) {
    __shared__ double s_base;
    const int L = blockIdx.x / G, g = blockIdx.x % G, t = threadIdx.x;
    const int k0 = g * CAND_GROUP + t * CAND_PER;
    const float *apx = wk.apx + static_cast<int64_t>(L) * T;
    float a[CAND_PER], tot = 0.f;
#pragma unroll
    for (int j = 0; j < CAND_PER; ++j) {
        a[j] = k0 + j < T ? apx[k0 + j] : 0.f;
        tot += a[j];
    }
    if (t < 32) {
        double b = 0.0;
        for (int i = t; i < g; i += 32) b += wk.gsum[L * G + i];
        b = warp_sum(b);
        if (t == 0) s_base = as_f64(state->lanes[L]) + b;
    }
    float total;
    float run = block_exclusive_sum<float>(tot, &total);  // synchronises the block
    const double start = s_base;
    // With the lane's base in a comfortable float range the prefixes are float sums (their
    // error, a few float roundings of 2^-24, is far inside the 2^-12 margin) and the margins
    // are tests of the exponent and mantissa bits: no FP64 arithmetic per tile, the scarce unit
    // on this part. Otherwise double arithmetic.
    const double as = fabs(start);
    const bool in_float = as == 0.0 || (as > 0x1p-100 && as < 0x1p100);
    const float sf = in_float ? __double2float_rn(start) : 0.f;
#pragma unroll
    for (int j = 0; j < CAND_PER; ++j) {
        const int k = k0 + j;
        if (k >= T) break;
        int elo, ehi;
        if (in_float) {
            const float A = a[j], pre = sf + run;
            run += A;
            float lo = A < 0 ? pre + A : pre, hi = A < 0 ? pre : pre + A;
            if (hi < 0) {
                const float m = -hi;
                hi = -lo;
                lo = m;
            }
            // binade(lo (1 - 2^-12)) and binade(hi (1 + 2^-12)) of positive normal floats.
            const unsigned bl = __float_as_uint(lo), bh = __float_as_uint(hi);
            const unsigned xl = bl >> 23, xh = bh >> 23;  // a sign bit makes these >= 256
            elo = (lo > 0.f && xl >= 1u && xl <= 254u) ? static_cast<int>(xl) - 127 - ((bl & 0x7fffffu) <= (1u << 11) ? 1 : 0)
                                                        : NO_E;
            ehi = (hi > 0.f && xh >= 1u && xh <= 254u)
                      ? static_cast<int>(xh) - 127 + ((bh & 0x7fffffu) >= (1u << 23) - (1u << 12) ? 1 : 0)
                      : NO_E;
        } else {
            const double A = static_cast<double>(a[j]);
            const double pre = start + static_cast<double>(run);
            run += a[j];
            double lo = A < 0 ? pre + A : pre, hi = A < 0 ? pre : pre + A;
            if (hi < 0) {  // a negative sum: the binades of its magnitude
                const double m = -hi;
                hi = -lo;
                lo = m;
            }
            elo = binade(lo * (1.0 - 0x1p-12));
            ehi = binade(hi * (1.0 + 0x1p-12));
        }
        int c0 = NO_E, c1 = NO_E;
        if (elo != NO_E && ehi != NO_E && elo >= -959) {
            if (ehi == elo) c0 = elo;
            else if (ehi == elo + 1) {
                c0 = elo;
                c1 = ehi;
            }
        }
        int2 *at = reinterpret_cast<int2 *>(&wk.cand[(static_cast<int64_t>(k) * 16 + L) * 2]);
        if (CHECK) {
            const int2 old = *at;
            const bool covered = (c0 == NO_E || c0 == old.x || c0 == old.y) && (c1 == NO_E || c1 == old.x || c1 == old.y);
            if (covered) continue;
            wk.flags[k] = 1;
        }
        *at = make_int2(c0, c1);
    }
}

// K2c input: each tile's lane sum from its transfer function where K3 made one (the increment
// in ulps of that binade is the sum to within half an ulp a row), else the sampled sum.
__global__ void __launch_bounds__(256) canon_refine_kernel(int T, CanonWork wk) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<int64_t>(16) * T) return;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        const int E = wk.recE[i * 2 + c];
        if (E == NO_E) continue;
        const TF f = wk.recD[i * 2 + c];
        const long long d = (f.d1 & SIGNED_TF) ? static_cast<long long>(f.d0) - static_cast<long long>(f.d1 & ~SIGNED_TF)
                                               : static_cast<long long>(f.d0);
        if (E - 52 >= -126 && E - 52 <= 40) {
            // The sum in float: the increment below 2^62 times the ulp 2^(E-52), no FP64 unit.
            wk.apx[i] = __ll2float_rn(d) * __uint_as_float(static_cast<unsigned>(E - 52 + 127) << 23);
        } else {
            const double v = __dmul_rn(__ll2double_rn(d), __longlong_as_double(static_cast<long long>(E - 52 + 1023) << 52));
            wk.apx[i] = v < 3.0e38 ? (v > -3.0e38 ? __double2float_rn(v) : -3.0e38f) : 3.0e38f;
        }
        return;
    }
}

// K3: each tile's transfer function per lane and candidate binade (NO_E when a segment does
// not take the integer step in that binade).
// The thread's segment functions for its two lanes and both candidates.
template <bool SIGNED>
__device__ __forceinline__ void seg_tfs(const unsigned long long (&v)[CT_SEG_BLOCKS][2], const int (*s_E)[2], int lp,
                                        TF (&fv)[2][2], int &okv, bool &plain) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int L = 2 * lp + h;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const int E = s_E[L][c];
            TF f{0, 0};
            const bool ok = E != NO_E && seg_tf<SIGNED>(v, h, 1023 + E, &f);
            plain = plain && f.d0 == f.d1;
            fv[h][c] = f;
            okv |= static_cast<int>(ok) << (2 * h + c);
        }
    }
}

// FLAGGED (K3c): only the tiles flagged by K3 (a negative row) or K2c (new candidates), with
// the signed functions where a tile has a negative row. Otherwise (K3) a tile with a negative
// row is only flagged, so that this kernel holds no signed code.
template <int OP, bool ALIGNED, bool FLAGGED>
__device__ __forceinline__ void tf_tile(const RowArgs &args, int64_t nb, int T, const CanonWork &wk, int tile) {
    __shared__ TF s_tf[2][CT_SEGS][16];
    __shared__ unsigned char s_ok[2][CT_SEGS][16];
    __shared__ int s_E[16][2];
    const int t = threadIdx.x, lp = t & 7, seg = t >> 3;
    if (t < 32) (&s_E[0][0])[t] = wk.cand[tile * 32 + t];
    unsigned long long v[CT_SEG_BLOCKS][2];
    load_tile<OP, ALIGNED>(args, nb, tile, lp, seg, v);
    TF fv[2][2];
    int okv = 0;  // bit 2h + c: the segment takes the integer step for lane 2lp+h, candidate c
    bool plain = true;
    // Tiles with a negative row take the signed functions (a separate path, so that tiles
    // without one keep the shorter code).
    unsigned sgn = 0;
#pragma unroll
    for (int i = 0; i < CT_SEG_BLOCKS; ++i) sgn |= static_cast<unsigned>((v[i][0] | v[i][1]) >> 63);
    if (__syncthreads_or(sgn)) {  // also the barrier after s_E
        if (!FLAGGED) {
            if (t == 0) {
                wk.flags[tile] = 2;
                wk.flags[T] = 1;  // some tile has a negative row
            }
            if (t < 32) wk.recE[(static_cast<int64_t>(t & 15) * T + tile) * 2 + (t >> 4)] = NO_E;
            return;
        }
        seg_tfs<true>(v, s_E, lp, fv, okv, plain);
    } else {
        seg_tfs<false>(v, s_E, lp, fv, okv, plain);
    }
    static_assert(CT_SEGS == 32 && CT_THREADS == 256, "four segments per warp, eight warps");
    const int sl = t & 31, wp = t >> 5;
    if (__syncthreads_and(plain)) {
        // No segment has a halfway row: every transfer function adds one increment whatever
        // the parity, so composing them is a saturated sum (the terms are below 2^57, their
        // sum below 2^62). The warp's four segments combine by shuffles (lanes 8 and 16 apart
        // hold the same lanes), the eight warps' partials through shared memory.
        unsigned long long d[2][2];
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                d[h][c] = fv[h][c].d0;
                d[h][c] += __shfl_xor_sync(FULL, d[h][c], 8);
                d[h][c] += __shfl_xor_sync(FULL, d[h][c], 16);
            }
        okv &= __shfl_xor_sync(FULL, okv, 8);
        okv &= __shfl_xor_sync(FULL, okv, 16);
        unsigned long long(*s_part)[32] = reinterpret_cast<unsigned long long(*)[32]>(&s_tf[0][0][0]);  // [warp][c*16 + L]
        unsigned char(*s_pok)[32] = reinterpret_cast<unsigned char(*)[32]>(&s_ok[0][0][0]);
        if (sl < 8) {
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    s_part[wp][c * 16 + 2 * lp + h] = d[h][c];
                    s_pok[wp][c * 16 + 2 * lp + h] = static_cast<unsigned char>((okv >> (2 * h + c)) & 1);
                }
        }
        __syncthreads();
        if (t < 32) {
            const int c = t >> 4, L = t & 15;
            unsigned long long sum = 0;
            int ok = 1;
#pragma unroll
            for (int w = 0; w < CT_THREADS / 32; ++w) {
                sum += s_part[w][t];
                ok &= s_pok[w][t];
            }
            const int E = s_E[L][c];
            const int64_t at = (static_cast<int64_t>(L) * T + tile) * 2 + c;
            wk.recE[at] = (E != NO_E && ok) ? E : NO_E;
            sum = sum > SAT ? SAT : sum;
            wk.recD[at] = TF{sum, sum};
        }
        return;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            s_tf[c][seg][2 * lp + h] = fv[h][c];
            s_ok[c][seg][2 * lp + h] = static_cast<unsigned char>((okv >> (2 * h + c)) & 1);
        }
    __syncthreads();
    // The 32 (lane, candidate) pairs, four per warp: lane s of the warp holds segment s, and an
    // ordered scan (earlier segments on the left) composes them.
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int pair = wp * 4 + q, L = pair >> 1, c = pair & 1;
        const int E = s_E[L][c];
        if (E == NO_E) {
            if (sl == 0) wk.recE[(static_cast<int64_t>(L) * T + tile) * 2 + c] = NO_E;
            continue;
        }
        TF f = s_tf[c][sl][L];
        const bool ok = __all_sync(FULL, s_ok[c][sl][L] != 0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const TF y = shfl_up_tf(f, o);
            if (sl >= o) f = compose<FLAGGED>(y, f);
        }
        if (sl == 31) {
            const int64_t at = (static_cast<int64_t>(L) * T + tile) * 2 + c;
            wk.recE[at] = ok ? E : NO_E;
            wk.recD[at] = f;
        }
    }
}

template <int OP, bool ALIGNED>
__global__ void __launch_bounds__(CT_THREADS, 4) canon_tf_kernel(RowArgs args, int64_t nb, int T, CanonWork wk) {
    tf_tile<OP, ALIGNED, false>(args, nb, T, wk, blockIdx.x);
}

// The flagged tiles in a list (any order): wk.flags[T + 1] counts them, wk.flags[T + 2 ..]
// holds them.
__global__ void __launch_bounds__(256) canon_flag_list_kernel(int T, CanonWork wk) {
    const int stride = gridDim.x * blockDim.x;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += stride)
        if (wk.flags[t]) wk.flags[T + 2 + atomicAdd(&wk.flags[T + 1], 1)] = t;
}

// K3c: persistent blocks over the list of flagged tiles.
template <int OP, bool ALIGNED>
__global__ void __launch_bounds__(CT_THREADS, 4) canon_tf_flagged_kernel(RowArgs args, int64_t nb, int T, CanonWork wk) {
    const int count = wk.flags[T + 1];
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        __syncthreads();  // the previous tile's shared arrays are free
        tf_tile<OP, ALIGNED, true>(args, nb, T, wk, wk.flags[T + 2 + i]);
    }
}


// The transfer function of tile `tp` for lane L in binade E, if it has one.
__device__ __forceinline__ bool tile_tf(const CanonWork &wk, int T, int L, int tp, int E, TF *f) {
    const int64_t at = (static_cast<int64_t>(L) * T + tp) * 2;
    if (E == NO_E) return false;
    if (wk.recE[at] == E) {
        *f = wk.recD[at];
        return true;
    }
    if (wk.recE[at + 1] == E) {
        *f = wk.recD[at + 1];
        return true;
    }
    return false;
}

// K4a: per lane and 32-tile chunk (one warp each), the composed transfer function when every
// tile of the chunk has one in the same binade (the binade of candidate 0 of the chunk's
// first tile).
__global__ void __launch_bounds__(256) canon_chunk_kernel(int T, int C, CanonWork wk) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (gw >= static_cast<int64_t>(16) * C) return;
    const int L = static_cast<int>(gw / C), k = static_cast<int>(gw % C);
    const int tp = k * 32 + lane;
    const int E = __shfl_sync(FULL, tp < T ? wk.recE[(static_cast<int64_t>(L) * T + tp) * 2] : NO_E, 0);
    TF f{0, 0};
    bool ok = tp >= T || tile_tf(wk, T, L, tp, E, &f);
    if (!__all_sync(FULL, ok) || E == NO_E) {
        if (lane == 0) wk.chunkE[static_cast<int64_t>(L) * C + k] = NO_E;
        return;
    }
    // Ordered composition: lane i holds tile 32k + i, the lower lane is the earlier tile.
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        TF other = TF{__shfl_down_sync(FULL, f.d0, o), __shfl_down_sync(FULL, f.d1, o)};
        if (lane + o < 32) f = compose(f, other);
    }
    if (lane == 0) {
        wk.chunkE[static_cast<int64_t>(L) * C + k] = E;
        wk.chunkD[static_cast<int64_t>(L) * C + k] = f;
    }
}

// The binade of |s| (s normal and finite), NO_E otherwise.
__device__ __forceinline__ int state_binade(unsigned long long s) {
    const unsigned long long e = (s >> 52) & 0x7ff;
    return (e >= 1 && e <= 2046) ? static_cast<int>(e) - 1023 : NO_E;
}

// Inclusive ordered prefix composition over the warp (lane 0 first), then the number of
// leading lanes whose prefix applies to state s (usable and inside the binade). Returns that
// count and, in *out, the state after them.
template <bool SIGNED = true>
__device__ __forceinline__ int apply_prefix(TF f, bool usable, unsigned long long s, int E,
                                            unsigned long long *out, unsigned long long *mine = nullptr) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        TF y = shfl_up_tf(f, o);
        if (lane >= o) f = compose<SIGNED>(y, f);
    }
    unsigned long long r = 0;
    const bool ok = usable && apply<SIGNED>(s, E, f, &r);
    if (mine) *mine = r;  // this lane's state (valid below the returned count)
    const unsigned bad = __ballot_sync(FULL, !ok);
    const int m = bad ? __ffs(bad) - 1 : 32;
    if (m > 0) *out = __shfl_sync(FULL, r, m - 1);
    return m;
}

// Resolves tile `tp` for lane L from the state s: the warp recomputes the tile's 32 segment
// transfer functions from the rows (lane j = segment j) for the state's binade and the next,
// applies them in order, and adds the rows of any segment they do not carry one by one.
template <int OP, bool SIGNED>
__device__ unsigned long long resolve_tile(const RowArgs &args, int64_t nb, int tp, int L, unsigned long long s) {
    const int lane = threadIdx.x & 31;
    unsigned long long v[CT_SEG_BLOCKS][2];
    const int64_t blk0 = static_cast<int64_t>(tp) * CT_BLOCKS + lane * CT_SEG_BLOCKS;
#pragma unroll
    for (int i = 0; i < CT_SEG_BLOCKS; ++i) {
        int64_t b = blk0 + i;
        unsigned long long xv = 0, yv = 0;
        if (b < nb) {
            xv = args.x[b * 16 + L];
            if (OP == ROW_DOT) yv = args.y[b * 16 + L];
            v[i][0] = row_value<OP>(args, xv, yv);
        } else {
            v[i][0] = 0;
        }
        v[i][1] = 0;
    }
    int seg = 0;
    while (seg < CT_SEGS) {
        const int E = state_binade(s);
        if (E != NO_E && E >= -959) {
            TF f{0, 0};
            bool ok = lane >= seg && seg_tf<SIGNED>(v, 0, 1023 + E, &f);
            if (lane < seg) {
                f = TF{0, 0};
                ok = true;  // already consumed: identity
            }
            unsigned long long r = s;
            int m = apply_prefix<SIGNED>(f, ok, s, E, &r);
            if (m > seg) {
                s = r;
                seg = m;
                continue;
            }
        }
        // Segment `seg` is not carried: its owner adds its rows one by one.
        unsigned long long r = 0;
        if (lane == seg) {
            double d = as_f64(s);
#pragma unroll
            for (int i = 0; i < CT_SEG_BLOCKS; ++i) d = __dadd_rn(d, as_f64(v[i][0]));
            r = as_bits(d);
        }
        s = __shfl_sync(FULL, r, seg);
        ++seg;
    }
    return s;
}

// K4b: one block per lane. The block first copies the lane's chunk records, and the tile
// records of the chunks without one ("mixed"), into shared memory; then warp 0 walks the tiles
// from the lane's exact state: whole 32-tile chunks while their transfer function holds, single
// tiles inside mixed chunks, and resolves from the rows the tiles that none carries (binade
// crossings, negative or special rows, the first rows of the lane).
constexpr int WK_THREADS = 256;
constexpr int WK_MAX_CHUNKS = 4096;  // chunk records held in shared memory
constexpr int WK_MAX_MIXED = 48;     // mixed chunks whose tile records are held there

// The walk's progress over windows of the SM clock: a window in which it advanced fewer tiles
// than the lane chain would (WALK_MIN_TILES in WALK_WINDOW cycles, about 2 tiles a microsecond)
// hands the lane to the chain. A growing sum advances hundreds of tiles a microsecond between
// its few binade crossings; a wandering one resolves tile after tile from the rows.
constexpr long long WALK_WINDOW = 1ll << 18;
constexpr int WALK_MIN_TILES = 256;
struct WalkClock {
    long long start;
    int tile;  // the first tile of the window
    __device__ __forceinline__ bool slower(int tp) {
        const long long now = clock64();
        // The first window is four times as long: the lane's first tiles cross many binades.
        if (now - start < (tile == 0 ? 4 * WALK_WINDOW : WALK_WINDOW)) return false;
        if (tp - tile < WALK_MIN_TILES) return true;
        start = now;
        tile = tp;
        return false;
    }
};

struct WalkSmem {
    int chunkE[WK_MAX_CHUNKS];
    TF chunkD[WK_MAX_CHUNKS];
    short mixed_of[WK_MAX_CHUNKS];
    int chunk_of[WK_MAX_MIXED];
    int mE[WK_MAX_MIXED][32][2];
    TF mD[WK_MAX_MIXED][32][2];
    int nmixed;
};

// Chunk k of lane L tile by tile from state s (one warp): runs of tiles whose transfer
// functions hold, and the tiles none carries resolved from the rows. RECORD (scans) stores the
// exact state before each tile. sm and slot give the chunk's tile records when the walk holds
// them in shared memory (slot >= 0).
// Without RECORD, the walk stops at the first round of the tile loop (a run of tiles whose
// functions apply, or one tile resolved from the rows) at which `clk` finds it slower than the
// lane chain: *stop gets that tile and the state before it is returned (the chain goes on from
// there).
template <int OP, bool SIGNED, bool RECORD>
__device__ __forceinline__ unsigned long long walk_chunk_tiles(const RowArgs &args, int64_t nb, int T, const CanonWork &wk,
                                                               const WalkSmem *sm, int slot, int L, int k,
                                                               unsigned long long s, WalkClock *clk = nullptr,
                                                               int *stop = nullptr) {
    const int lane = threadIdx.x & 31;
    unsigned long long *rec = RECORD ? wk.tstate + static_cast<int64_t>(L) * (T + 1) : nullptr;
    int tp = k * 32;
    const int end = min(T, tp + 32);
    while (tp < end) {
        if (!RECORD && stop && clk->slower(tp)) {
            *stop = tp;
            return s;
        }
        if (RECORD && lane == 0) rec[tp] = s;
        const int Et = state_binade(s);
        const int tl = tp + lane;
        TF g{0, 0};
        bool usable = false;
        if (tl < end && Et != NO_E) {
            if (slot >= 0) {
                const int j = tl - k * 32;
                if (sm->mE[slot][j][0] == Et) {
                    g = sm->mD[slot][j][0];
                    usable = true;
                } else if (sm->mE[slot][j][1] == Et) {
                    g = sm->mD[slot][j][1];
                    usable = true;
                }
            } else {
                usable = tile_tf(wk, T, L, tl, Et, &g);
            }
        }
        unsigned long long r = s, mine = 0;
        const int mt = Et == NO_E ? 0 : apply_prefix<SIGNED>(g, usable, s, Et, &r, RECORD ? &mine : nullptr);
        if (mt > 0) {
            if (RECORD && lane + 1 < mt) rec[tp + lane + 1] = mine;
            s = r;
            tp += mt;
        } else {
            s = resolve_tile<OP, SIGNED>(args, nb, tp, L, s);
            ++tp;
        }
    }
    return s;
}

// The walk of lane L from state s (warp 0 of the lane's block), with the signed functions
// when some tile has a negative row or the state is negative (SIGNED), else the shorter code.
// RECORD (scans) stores the state before each chunk it takes whole, marks it in wk.whole, and
// the state before each tile of the others.
template <int OP, bool SIGNED, bool RECORD>
__device__ __forceinline__ unsigned long long walk_lane(const RowArgs &args, int64_t nb, int T, int C, const CanonWork &wk,
                                                        const WalkSmem &sm, bool held, const int *gE, const TF *gD,
                                                        int L, unsigned long long s, int *stop) {
    const int lane = threadIdx.x;
    // Reductions only: the walk goes on while it is faster than the lane chain (WalkClock).
    WalkClock clk{clock64(), 0};
    int k = 0;  // next chunk
    while (k < C) {
        if (!RECORD && clk.slower(k * 32)) {
            *stop = k * 32;
            return s;
        }
        // Whole chunks k .. k+31.
        const int E = state_binade(s);
        const int kc = k + lane;
        int ce = NO_E;
        TF f{0, 0};
        if (kc < C) {
            ce = held ? sm.chunkE[kc] : gE[kc];
            if (ce != NO_E && ce == E) f = held ? sm.chunkD[kc] : gD[kc];
        }
        unsigned long long r = s, mine = 0;
        int m = E == NO_E ? 0
                          : apply_prefix<SIGNED>(f, kc < C && ce != NO_E && ce == E, s, E, &r,
                                                 RECORD ? &mine : nullptr);
        if (m > 0) {
            if (RECORD) {
                unsigned long long *rec = wk.tstate + static_cast<int64_t>(L) * (T + 1);
                if (lane == 0) rec[k * 32] = s;
                if (lane + 1 < m) rec[(k + lane + 1) * 32] = mine;
                if (lane < m) wk.whole[static_cast<int64_t>(L) * C + kc] = 1;
            }
            s = r;
            k += m;
            continue;
        }
        // Chunk k, tile by tile.
        s = walk_chunk_tiles<OP, SIGNED, RECORD>(args, nb, T, wk, &sm, held ? sm.mixed_of[k] : -1, L, k, s,
                                                 &clk, RECORD ? nullptr : stop);
        if (*stop >= 0) return s;
        ++k;
    }
    return s;
}

template <int OP, bool RECORD>
__global__ void __launch_bounds__(WK_THREADS) canon_walk_kernel(RowArgs args, int64_t nb, int T, int C, CanonWork wk,
                                                                CanonState *state) {
    extern __shared__ __align__(16) unsigned char walk_smem[];
    WalkSmem &sm = *reinterpret_cast<WalkSmem *>(walk_smem);
    const int L = blockIdx.x, t = threadIdx.x;
    const bool held = C <= WK_MAX_CHUNKS;
    const int *gE = wk.chunkE + static_cast<int64_t>(L) * C;
    const TF *gD = wk.chunkD + static_cast<int64_t>(L) * C;
    if (t == 0) sm.nmixed = 0;
    __syncthreads();
    if (held) {
        for (int c = t; c < C; c += WK_THREADS) {
            int e = gE[c];
            sm.chunkE[c] = e;
            sm.chunkD[c] = gD[c];
            short slot = -1;
            if (e == NO_E) {
                int k = atomicAdd(&sm.nmixed, 1);
                if (k < WK_MAX_MIXED) {
                    slot = static_cast<short>(k);
                    sm.chunk_of[k] = c;
                }
            }
            sm.mixed_of[c] = slot;
        }
    }
    __syncthreads();
    if (held) {
        // Tile records of the mixed chunks with a slot: 32 tiles x 2 candidates each.
        const int nm = min(sm.nmixed, WK_MAX_MIXED);
        for (int idx = t; idx < nm * 64; idx += WK_THREADS) {
            const int slot = idx >> 6, j = (idx >> 1) & 31, cand = idx & 1;
            const int tp = sm.chunk_of[slot] * 32 + j;
            int e = NO_E;
            TF d{0, 0};
            if (tp < T) {
                const int64_t at = (static_cast<int64_t>(L) * T + tp) * 2 + cand;
                e = wk.recE[at];
                d = wk.recD[at];
            }
            sm.mE[slot][j][cand] = e;
            sm.mD[slot][j][cand] = d;
        }
    }
    __syncthreads();
    if (t >= 32) return;
    const int lane = t;
    unsigned long long s = state->lanes[L];
    int stop = -1;
    s = (wk.flags[T] != 0 || (s >> 63)) ? walk_lane<OP, true, RECORD>(args, nb, T, C, wk, sm, held, gE, gD, L, s, &stop)
                                        : walk_lane<OP, false, RECORD>(args, nb, T, C, wk, sm, held, gE, gD, L, s, &stop);
    if (lane == 0) {
        state->lanes[L] = s;
        if (RECORD) wk.tstate[static_cast<int64_t>(L) * (T + 1) + T] = s;
        else wk.resume[L] = stop >= 0 ? stop : T;
    }
}

// Scans, after the walk: the state before every tile of the chunks it took whole, one warp per
// lane and chunk, by the walk's own tile steps from the chunk's recorded state (any prefix of a
// chunk whose composed function applied applies as well: increments only add up, and a signed
// function's bounds cover its prefixes').
template <int OP>
__global__ void __launch_bounds__(256) canon_fill_kernel(RowArgs args, int64_t nb, int T, int C, CanonWork wk) {
    const int64_t gw = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (gw >= static_cast<int64_t>(16) * C) return;
    const int L = static_cast<int>(gw / C), k = static_cast<int>(gw % C);
    if (!wk.whole[static_cast<int64_t>(L) * C + k]) return;
    const unsigned long long s = wk.tstate[static_cast<int64_t>(L) * (T + 1) + k * 32];
    if (wk.flags[T] != 0 || (s >> 63))
        walk_chunk_tiles<OP, true, true>(args, nb, T, wk, nullptr, -1, L, k, s);
    else
        walk_chunk_tiles<OP, false, true>(args, nb, T, wk, nullptr, -1, L, k, s);
}

// Short inputs: the reference's own order, each lane a chain of IEEE adds over its rows
// (reduce.rs:45-62), from the lane states. The block first stages every row value in shared
// memory (coalesced, all loads in flight at once); then 16 threads run the lane chains.
constexpr int64_t CANON_SEQ_BLOCKS = 256;  // 16-row blocks (4096 rows) up to which this path runs

template <int OP>
__global__ void __launch_bounds__(256) canon_seq_kernel(RowArgs args, int nb, CanonState *state) {
    __shared__ unsigned long long s_v[CANON_SEQ_BLOCKS * 16];
    const int rows = nb * 16;
    for (int i = threadIdx.x; i < rows; i += blockDim.x)
        s_v[i] = row_value<OP>(args, args.x[i], OP == ROW_DOT ? args.y[i] : 0ull);
    __syncthreads();
    const int j = threadIdx.x;
    if (j >= 16) return;
    double s = as_f64(state->lanes[j]);
    for (int b = 0; b < nb; ++b) s = __dadd_rn(s, as_f64(s_v[b * 16 + j]));
    state->lanes[j] = as_bits(s);
}

// Stores the row values of the rest rows (fewer than 16) as the pending tail.
template <int OP>
__global__ void canon_tail(RowArgs args, int64_t first, int rest, CanonState *state) {
    int j = threadIdx.x;
    if (j < rest) {
        unsigned long long y = OP == ROW_DOT ? args.y[first + j] : 0ull;
        state->tail[j] = row_value<OP>(args, args.x[first + j], y);
    }
}

// reduce.rs:77-91 (finish_lanes): +8, +4, +2, +1, then the tail into lane 0 in order.
__global__ void canon_finish(CanonState *state, int tail_len) {
    double acc[16];
    for (int j = 0; j < 16; ++j) acc[j] = as_f64(state->lanes[j]);
    for (int step = 8; step > 0; step >>= 1)
        for (int j = 0; j < step; ++j) acc[j] = __dadd_rn(acc[j], acc[j + step]);
    double r = acc[0];
    for (int j = 0; j < tail_len; ++j) r = __dadd_rn(r, as_f64(state->tail[j]));
    state->result = as_bits(r);
}

// ---------------------------------------------------------------------------- the lane chain
// Reductions whose lane sums keep leaving their binade (rows of both signs whose sum wanders
// around zero, magnitudes as large as the sum) make the walk resolve most tiles from the rows,
// one at a time. When the walk falls behind this kernel's pace (WalkClock) it stops, and this
// kernel runs each stopped lane to the end from its exact state. One warp per lane; each step
// takes 32 * ROWS of the lane's rows, ROWS consecutive ones per thread (the autotuner's
// canon_chain_rows), prefetched CH_SLOTS - 1 steps ahead with cp.async into the thread's own row
// of a shared ring (each thread reads only what it copied). The cost is one warp round per
// binade crossing, each with ROWS
// dependent IEEE adds (63 cycles each on GB300), so the rows per thread are few (measured at
// 2^26 mean-centred rows: 8 rows 43 ms, 32 rows 92 ms; eight warps a lane, or 32 rows in four
// 8-row fallback units, were slower again: every crossing costs a whole round).
//
// A thread's ROWS rows act on the state's magnitude S (in ulps u = 2^(E-52) of its binade E) as
// integer increments, the integer step of seg_tf: +-RNE(|x|/u) by the row's sign relative to
// the state's, and for a row exactly halfway the even neighbour, which depends on the parity of
// S at that row; so each thread keeps its increments for both parities of S before its rows,
// with the lowest (mn) and highest (mx) partial sum, and a warp scan composes the parity pairs
// in order. This is exact while every state on the way stays inside the binade: the state
// passes every thread whose states all stay in [2^52 + 1, 2^53 - 1] ulps (the margin keeps the
// exact sum of a downward step above 2^E); the first thread whose rows fail (a crossing, a row
// not below 2^E or not finite) adds its rows with IEEE adds, the reference's own operation, and
// the rest are computed again for the new state. So the result is the chain's, bit for bit.
constexpr int CH_SLOTS = 8;  // steps in the shared ring

__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Doubles per thread row of the ring: ROWS + 1 (odd: spreads the banks).
template <int OP, int ROWS> constexpr size_t chain_smem() {
    return static_cast<size_t>(CH_SLOTS) * (OP == ROW_DOT ? 2 : 1) * 32 * (ROWS + 1) * sizeof(unsigned long long);
}

template <int OP, int ROWS>
__global__ void __launch_bounds__(32) canon_chain_kernel(RowArgs args, int64_t nb, int T, CanonWork wk,
                                                         CanonState *state) {
    extern __shared__ __align__(16) unsigned long long chain_smem_buf[];
    constexpr int NA = OP == ROW_DOT ? 2 : 1;
    constexpr int STEP = 32 * ROWS, PITCH = ROWS + 1;
    const int L = blockIdx.x, j = threadIdx.x;
    const int t0 = wk.resume[L];
    if (t0 >= T) return;
    const int64_t b0 = static_cast<int64_t>(t0) * CT_BLOCKS;
    const int64_t steps = (nb - b0 + STEP - 1) / STEP;
    auto row_at = [&](int64_t k, int a) {
        return chain_smem_buf + ((k % CH_SLOTS) * NA + a) * (32 * PITCH) + j * PITCH;
    };
    // Copies of step k (an empty group past the end keeps the group count uniform).
    auto issue = [&](int64_t k) {
        if (k < steps) {
            const int64_t bb = b0 + k * STEP + static_cast<int64_t>(j) * ROWS;
            unsigned long long *dx = row_at(k, 0);
            unsigned long long *dy = row_at(k, NA - 1);
#pragma unroll 8
            for (int i = 0; i < ROWS; ++i) {
                if (bb + i < nb) {
                    cp_async8(dx + i, args.x + (bb + i) * 16 + L);
                    if (OP == ROW_DOT) cp_async8(dy + i, args.y + (bb + i) * 16 + L);
                }
            }
        }
        cp_async_commit();
    };
    for (int k = 0; k < CH_SLOTS - 1; ++k) issue(k);
    unsigned long long s = state->lanes[L];
    for (int64_t k = 0; k < steps; ++k) {
        cp_async_wait<CH_SLOTS - 2>();  // this thread's copies of step k have landed
        unsigned long long v[ROWS];
        {
            const int64_t bb = b0 + k * STEP + static_cast<int64_t>(j) * ROWS;
            const unsigned long long *rx = row_at(k, 0);
            const unsigned long long *ry = row_at(k, NA - 1);
#pragma unroll
            for (int i = 0; i < ROWS; ++i)
                v[i] = bb + i < nb ? row_value<OP>(args, rx[i], OP == ROW_DOT ? ry[i] : 0ull) : 0ull;
        }
        issue(k + CH_SLOTS - 1);  // into the slot of step k - 1, read by the previous step
        if ((s & ~(1ull << 63)) > 0x7ff0000000000000ull) continue;  // NaN stays NaN
        int cur = 0;  // threads already applied
        // The thread's function depends on the binade and the state's sign only (in magnitude
        // space a negative state adds the negated rows), so it is computed again only when a
        // fallback changes either. A halfway row rounds to the even neighbour, so the function
        // is kept for both parities of the state before the thread's rows: (P0, mn0, mx0) for an
        // even start, (P1, mn1, mx1) for an odd one.
        unsigned fkey = ~0u;
        long long fP0 = 0, fP1 = 0, fmn0 = 0, fmx0 = 0, fmn1 = 0, fmx1 = 0;
        bool fok = false, ftie = false;
        while (cur < 32) {
            const unsigned es = static_cast<unsigned>(s >> 52) & 0x7ffu;
            const unsigned long long neg = s >> 63;
            const bool usable = es >= 64u && es <= 2046u;
            const unsigned key = es | static_cast<unsigned>(neg << 11);
            if (usable && j >= cur && key != fkey) {
                fkey = key;
                fP0 = fP1 = 0;
                fmn0 = fmn1 = LLONG_MAX;
                fmx0 = fmx1 = LLONG_MIN;
                fok = true;
                ftie = false;
#pragma unroll
                for (int i = 0; i < ROWS; ++i) {
                    const unsigned long long b = v[i];
                    const unsigned ex = static_cast<unsigned>(b >> 52) & 0x7ffu;
                    fok &= ex < es;  // below 2^E and finite
                    const unsigned k2 = min(es - ex, 63u);
                    const unsigned long long w = ((b & MANT) | ONE52) + (1ull << ((k2 - 1) & 63));
                    const long long q = static_cast<long long>(w >> k2);
                    long long i0 = q, i1 = q;
                    if ((w << ((64 - k2) & 63)) == 0) {  // halfway: to the even magnitude
                        const long long qf = q - 1;
                        i0 = qf + ((fP0 + qf) & 1);
                        i1 = qf + ((1 + fP1 + qf) & 1);
                        ftie = true;
                    }
                    const bool down = ((b >> 63) ^ neg) != 0;  // the row moves the magnitude down
                    fP0 += down ? -i0 : i0;
                    fP1 += down ? -i1 : i1;
                    fmn0 = min(fmn0, fP0);
                    fmx0 = max(fmx0, fP0);
                    fmn1 = min(fmn1, fP1);
                    fmx1 = max(fmx1, fP1);
                }
            }
            const bool live = j >= cur;
            const bool ok = !live || (usable && fok);
            const long long M = static_cast<long long>((s & MANT) | ONE52);
            const long long p0 = M & 1;
            long long c0 = live ? fP0 : 0, c1 = live ? fP1 : 0, pre;
            if (!__any_sync(FULL, live && ftie)) {
                // No halfway row: every function is one increment whatever the parity, and the
                // composition is a plain sum.
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const long long a0 = __shfl_up_sync(FULL, c0, o);
                    if (j >= o) c0 += a0;
                }
                c1 = c0;
                const long long e0 = __shfl_up_sync(FULL, c0, 1);
                pre = j == 0 ? 0 : e0;
            } else {
                // Ordered composition of the parity pairs (the state's parity after a function).
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const long long a0 = __shfl_up_sync(FULL, c0, o), a1 = __shfl_up_sync(FULL, c1, o);
                    if (j >= o) {
                        const long long n0 = a0 + ((a0 & 1) ? c1 : c0);
                        const long long n1 = a1 + (((1 + a1) & 1) ? c1 : c0);
                        c0 = n0;
                        c1 = n1;
                    }
                }
                const long long e0 = __shfl_up_sync(FULL, c0, 1), e1 = __shfl_up_sync(FULL, c1, 1);
                pre = j == 0 ? 0 : (p0 ? e1 : e0);  // increments before this thread
            }
            const bool odd = ((p0 + pre) & 1) != 0;
            const long long mn = odd ? fmn1 : fmn0, mx = odd ? fmx1 : fmx0;
            const long long lo = static_cast<long long>(ONE52) + 1, hi = static_cast<long long>(2 * ONE52) - 1;
            bool valid = !live;
            if (!valid && ok) valid = M + pre + mn >= lo && M + pre + mx <= hi;
            const unsigned bad = __ballot_sync(FULL, !valid);
            const int js = bad ? __ffs(bad) - 1 : 32;
            if (js > cur) {
                const long long tot = p0 ? __shfl_sync(FULL, c1, 31) : __shfl_sync(FULL, c0, 31);
                const long long adv = js < 32 ? __shfl_sync(FULL, pre, js) : tot;
                const unsigned long long Mn = static_cast<unsigned long long>(M + adv);
                s = (neg << 63) | (static_cast<unsigned long long>(es) << 52) | (Mn & MANT);
            }
            if (js == 32) break;
            unsigned long long r = 0;
            if (j == js) {
                double d = as_f64(s);
#pragma unroll
                for (int i = 0; i < ROWS; ++i) d = __dadd_rn(d, as_f64(v[i]));
                r = as_bits(d);
            }
            s = __shfl_sync(FULL, r, js);
            cur = js + 1;
        }
    }
    cp_async_wait<0>();
    if (j == 0) state->lanes[L] = s;
}

// RECORD (scans): the walk also stores the exact lane state before every tile in wk.tstate.
template <int OP, bool ALIGNED, bool RECORD = false>
static vkc_status launch_canon(vkc_ctx *ctx, const RowArgs &a, int64_t nb, int T, int C, const CanonWork &wk,
                               CanonState *state) {
    vkc_status st;
    canon_apx_kernel<OP, ALIGNED><<<(T + APX_TILES - 1) / APX_TILES, CT_THREADS, 0, ctx->stream>>>(a, nb, T, wk);
    if ((st = launched(ctx, "canon_apx"))) return st;
    const int G = (T + CAND_GROUP - 1) / CAND_GROUP;
    canon_gsum_kernel<<<16 * G, 256, 0, ctx->stream>>>(T, G, wk);
    if ((st = launched(ctx, "canon_gsum"))) return st;
    canon_cand_kernel<false><<<16 * G, CAND_THREADS, 0, ctx->stream>>>(T, G, wk, state);
    if ((st = launched(ctx, "canon_cand"))) return st;
    VKC_CUDA(ctx, cudaMemsetAsync(wk.flags, 0, static_cast<size_t>(T + 2) * sizeof(int), ctx->stream));
    canon_tf_kernel<OP, ALIGNED><<<T, CT_THREADS, 0, ctx->stream>>>(a, nb, T, wk);
    if ((st = launched(ctx, "canon_tf"))) return st;
    // The check of the sampled candidates: K3's sums, the prefixes again, K3 again on the tiles
    // whose binades the first candidates missed and on the tiles with negative rows.
    canon_refine_kernel<<<static_cast<int>((16 * static_cast<int64_t>(T) + 255) / 256), 256, 0, ctx->stream>>>(T, wk);
    canon_gsum_kernel<<<16 * G, 256, 0, ctx->stream>>>(T, G, wk);
    canon_cand_kernel<true><<<16 * G, CAND_THREADS, 0, ctx->stream>>>(T, G, wk, state);
    canon_flag_list_kernel<<<std::min(T / 256 + 1, 1024), 256, 0, ctx->stream>>>(T, wk);
    canon_tf_flagged_kernel<OP, ALIGNED><<<std::min(T, 4 * ctx->sms), CT_THREADS, 0, ctx->stream>>>(a, nb, T, wk);
    if ((st = launched(ctx, "canon_check"))) return st;
    int warps = 16 * C;
    canon_chunk_kernel<<<(warps + 7) / 8, 256, 0, ctx->stream>>>(T, C, wk);
    if ((st = launched(ctx, "canon_chunk"))) return st;
    static std::atomic<unsigned long long> configured{0};
    once_per_device(configured, ctx->device, [] {
        cudaFuncSetAttribute(canon_walk_kernel<OP, RECORD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(sizeof(WalkSmem)));
    });
    if constexpr (RECORD) VKC_CUDA(ctx, cudaMemsetAsync(wk.whole, 0, static_cast<size_t>(C) * 16 * sizeof(int), ctx->stream));
    canon_walk_kernel<OP, RECORD><<<16, WK_THREADS, sizeof(WalkSmem), ctx->stream>>>(a, nb, T, C, wk, state);
    if ((st = launched(ctx, "canon_walk"))) return st;
    if constexpr (!RECORD) {
        static std::atomic<unsigned long long> chain_configured{0};
        once_per_device(chain_configured, ctx->device, [] {
            cudaFuncSetAttribute(canon_chain_kernel<OP, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(chain_smem<OP, 4>()));
            cudaFuncSetAttribute(canon_chain_kernel<OP, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(chain_smem<OP, 8>()));
            cudaFuncSetAttribute(canon_chain_kernel<OP, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(chain_smem<OP, 16>()));
        });
        switch (tune(ctx, TK_CHAIN_ROWS, nb * 16)) {
        case 4: canon_chain_kernel<OP, 4><<<16, 32, chain_smem<OP, 4>(), ctx->stream>>>(a, nb, T, wk, state); break;
        case 16: canon_chain_kernel<OP, 16><<<16, 32, chain_smem<OP, 16>(), ctx->stream>>>(a, nb, T, wk, state); break;
        default: canon_chain_kernel<OP, 8><<<16, 32, chain_smem<OP, 8>(), ctx->stream>>>(a, nb, T, wk, state); break;
        }
        if ((st = launched(ctx, "canon_chain"))) return st;
    }
    if constexpr (RECORD) {
        canon_fill_kernel<OP><<<(warps + 7) / 8, 256, 0, ctx->stream>>>(a, nb, T, C, wk);
        if ((st = launched(ctx, "canon_fill"))) return st;
    }
    return VKC_OK;
}

// The work arrays of one canonical pass over T tiles (C chunks) in one scratch block starting
// at b; SCAN adds the tile states, the whole-chunk marks and the pass's own lane state. Returns
// the block's size (b == nullptr: only the size).
static size_t canon_layout(int T, int C, bool scan, char *b, CanonWork *wk, CanonState **cs) {
    auto up = [](size_t v) { return (v + 255) & ~size_t(255); };
    const size_t t16 = static_cast<size_t>(T) * 16, c16 = static_cast<size_t>(C) * 16;
    const size_t o_cand = up(t16 * sizeof(float));
    const size_t o_recE = o_cand + up(t16 * 2 * sizeof(int));
    const size_t o_recD = o_recE + up(t16 * 2 * sizeof(int));
    const size_t o_chE = o_recD + up(t16 * 2 * sizeof(TF));
    const size_t o_chD = o_chE + up(c16 * sizeof(int));
    const size_t g16 = static_cast<size_t>((T + CAND_GROUP - 1) / CAND_GROUP) * 16;
    const size_t o_gs = o_chD + up(c16 * sizeof(TF));
    const size_t o_fl = o_gs + up(g16 * sizeof(double));
    const size_t o_ts = o_fl + up(static_cast<size_t>(2 * T + 2) * sizeof(int));
    const size_t o_wh = o_ts + up(static_cast<size_t>(T + 1) * 16 * sizeof(unsigned long long));
    const size_t o_cs = o_wh + up(c16 * sizeof(int));
    const size_t o_rs = up(o_fl + static_cast<size_t>(2 * T + 2) * sizeof(int));
    const size_t total = scan ? o_cs + sizeof(CanonState) : o_rs + 16 * sizeof(int);
    if (b) {
        *wk = CanonWork{reinterpret_cast<float *>(b), reinterpret_cast<int *>(b + o_cand),
                        reinterpret_cast<int *>(b + o_recE), reinterpret_cast<TF *>(b + o_recD),
                        reinterpret_cast<int *>(b + o_chE), reinterpret_cast<TF *>(b + o_chD),
                        reinterpret_cast<double *>(b + o_gs), reinterpret_cast<int *>(b + o_fl)};
        if (!scan) wk->resume = reinterpret_cast<int *>(b + o_rs);
        if (scan) {
            wk->tstate = reinterpret_cast<unsigned long long *>(b + o_ts);
            wk->whole = reinterpret_cast<int *>(b + o_wh);
            *cs = reinterpret_cast<CanonState *>(b + o_cs);
        }
    }
    return total;
}

// The canonical reducer of one row operation.
struct CanonReducer : DevReducer {
    int op;
    int cmp = -1;
    int tail_len = 0;

    vkc_status update(vkc_ctx *ctx, const Arg *args, int nargs) override {
        vkc_status st;
        RowArgs a{};
        // Argument checks in the order of each reducer's update (fused.rs:77-203, reduce.rs:612-617).
        switch (op) {
        case ROW_SUM:
        case ROW_SUMSQ:
            if (nargs != 1) return fail(ctx, VKC_RUNTIME, arity_error(1, nargs));
            if (!rows_arg(ctx, args[0], VKC_F64, &st)) return st;
            break;
        case ROW_DOT:
            if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
            if (!rows_arg(ctx, args[0], VKC_F64, &st) || !rows_arg(ctx, args[1], VKC_F64, &st)) return st;
            if (args[0].len() != args[1].len())
                return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(args[0].len()) +
                                                  " vs " + std::to_string(args[1].len()));
            a.y = args[1].ptr<unsigned long long>();
            break;
        default:
            if (nargs != 3) return fail(ctx, VKC_RUNTIME, arity_error(3, nargs));
            if (!rows_arg(ctx, args[0], VKC_F64, &st) || !splat_arg(ctx, args[1], VKC_F64, &st) ||
                !splat_arg(ctx, args[2], VKC_F64, &st))
                return st;
            a.r = cmp_range(cmp, args[1].f64());
            a.e = args[2].s.bits;
            break;
        }
        a.x = args[0].ptr<unsigned long long>();
        const int64_t n = args[0].len();
        // reduce.rs:297-303: rows may only follow whole blocks.
        if (tail_len != 0) return fail(ctx, VKC_RUNTIME, "canonical update after a partial block");
        const int64_t nb = n / 16;
        const int rest = static_cast<int>(n % 16);
        auto *cs = static_cast<CanonState *>(state);
        if (nb > 0 && nb <= CANON_SEQ_BLOCKS) {
            const int nbi = static_cast<int>(nb);
            switch (op) {
            case ROW_SUM: canon_seq_kernel<ROW_SUM><<<1, 256, 0, ctx->stream>>>(a, nbi, cs); break;
            case ROW_DOT: canon_seq_kernel<ROW_DOT><<<1, 256, 0, ctx->stream>>>(a, nbi, cs); break;
            case ROW_SUMSQ: canon_seq_kernel<ROW_SUMSQ><<<1, 256, 0, ctx->stream>>>(a, nbi, cs); break;
            default: canon_seq_kernel<ROW_CONDSUM><<<1, 256, 0, ctx->stream>>>(a, nbi, cs); break;
            }
            if ((st = launched(ctx, "canon_seq"))) return st;
        } else if (nb > 0) {
            const int64_t T64 = (nb + CT_BLOCKS - 1) / CT_BLOCKS;
            if (T64 > (int64_t(1) << 26)) return fail(ctx, VKC_USAGE, "array too long for one update");
            const int T = static_cast<int>(T64), C = (T + 31) / 32;
            void *p;
            if ((st = scratch(ctx, canon_layout(T, C, false, nullptr, nullptr, nullptr), &p))) return st;
            CanonWork wk;
            canon_layout(T, C, false, static_cast<char *>(p), &wk, nullptr);
            const bool aligned = (reinterpret_cast<uintptr_t>(a.x) & 15) == 0 &&
                                 (op != ROW_DOT || (reinterpret_cast<uintptr_t>(a.y) & 15) == 0);
            switch (op) {
            case ROW_SUM: st = aligned ? launch_canon<ROW_SUM, true>(ctx, a, nb, T, C, wk, cs) : launch_canon<ROW_SUM, false>(ctx, a, nb, T, C, wk, cs); break;
            case ROW_DOT: st = aligned ? launch_canon<ROW_DOT, true>(ctx, a, nb, T, C, wk, cs) : launch_canon<ROW_DOT, false>(ctx, a, nb, T, C, wk, cs); break;
            case ROW_SUMSQ: st = aligned ? launch_canon<ROW_SUMSQ, true>(ctx, a, nb, T, C, wk, cs) : launch_canon<ROW_SUMSQ, false>(ctx, a, nb, T, C, wk, cs); break;
            default: st = aligned ? launch_canon<ROW_CONDSUM, true>(ctx, a, nb, T, C, wk, cs) : launch_canon<ROW_CONDSUM, false>(ctx, a, nb, T, C, wk, cs); break;
            }
            if (st) return st;
        }
        if (rest > 0) {
            const int64_t first = nb * 16;
            switch (op) {
            case ROW_SUM: canon_tail<ROW_SUM><<<1, 16, 0, ctx->stream>>>(a, first, rest, cs); break;
            case ROW_DOT: canon_tail<ROW_DOT><<<1, 16, 0, ctx->stream>>>(a, first, rest, cs); break;
            case ROW_SUMSQ: canon_tail<ROW_SUMSQ><<<1, 16, 0, ctx->stream>>>(a, first, rest, cs); break;
            default: canon_tail<ROW_CONDSUM><<<1, 16, 0, ctx->stream>>>(a, first, rest, cs); break;
            }
            if ((st = launched(ctx, "canon_tail"))) return st;
            tail_len = rest;
        }
        return VKC_OK;
    }

    vkc_status finish(vkc_ctx *ctx, vkc_scalar *out) override {
        auto *cs = static_cast<CanonState *>(state);
        canon_finish<<<1, 1, 0, ctx->stream>>>(cs, tail_len);
        vkc_status st = launched(ctx, "canon_finish");
        if (st) return st;
        out->type = VKC_F64;
        return download(ctx, &out->bits, 8, offsetof(CanonState, result));
    }
    vkc_status finish_into(vkc_ctx *ctx, void *dst) override {
        canon_finish<<<1, 1, 0, ctx->stream>>>(static_cast<CanonState *>(state), tail_len);
        vkc_status st = launched(ctx, "canon_finish");
        return st ? st : copy_out(ctx, dst, 8, offsetof(CanonState, result));
    }
};

// ---------------------------------------------------------------------------- float scans
// scan_add_f64 and scan_by_add_f64: the reference has no float scans (scan.rs:408-415 lists the
// gap); its tier-2 design notes (docs/superpowers/specs/2026-10-31-verkehrt-tier2-design.md:172)
// give the candidate order built here: out[i] is the canonical sum of the prefix x[0..=i], so
// out[n - 1] is reduce_add_f64 of the array. With the exact lane states before each 16-row
// block, the prefix ending at row 16k + r (r < 15) is the combine (+8, +4, +2, +1) of the lane
// states before block k followed by rows 16k .. 16k + r in order (the canonical tail), and the
// prefix ending at row 16k + 15 is the combine of the lane states after block k.
//
// The lane states before each 4096-row tile come from the canonical pass in record mode (the
// walk, then canon_fill_kernel); one block per tile then runs the 16 lane chains over the
// tile's blocks with IEEE adds, each block's combine and each block's tail chain. Shared rows
// are padded to 17 doubles per 16 so that the threads of a warp, one per block, read different
// banks.
constexpr int SCAN_PAD = 17;
struct ScanSmem {
    unsigned long long v[CT_BLOCKS * SCAN_PAD];  // the tile's rows (bits), then its outputs
    union {
        unsigned long long st[(CT_BLOCKS + 1) * SCAN_PAD];  // lane states before block j, j = 0 .. 256
        struct {
            TF tf[16][CT_SEGS];  // each lane's segment transfer functions
            int ok[16][CT_SEGS];
        } seg;
    };
    double c[CT_BLOCKS + 1];  // the combines of st[j]
    int serial[16];           // lanes whose segments do not all carry a transfer function
};

// fl(s + x) on bits. When s is a positive normal in binade E >= -959, x is non-negative and below
// that binade and the sum stays in it, s = S u with u = 2^(E-52) and fl(s + x) = (S + RNE(x/u)) u
// with ties to the even S (the integer steps of seg_tf for one row); otherwise the FP64 add.
__device__ __forceinline__ unsigned long long add_bits(unsigned long long s, unsigned long long x) {
    const unsigned KE = static_cast<unsigned>(s >> 52);  // with the sign bit: a negative s is above 2047
    const unsigned ex = static_cast<unsigned>(x >> 52);  // likewise a negative x
    if (KE >= 64u && KE <= 2046u && ex < KE) {
        const unsigned k = min(KE - ex, 63u);  // zero and subnormal rows: k = 63, no increment
        const unsigned long long w = ((x & MANT) | ONE52) + (1ull << (k - 1));
        unsigned long long inc = w >> k;
        const unsigned long long S = (s & MANT) | ONE52;
        if ((w << (64 - k)) == 0) {  // exactly halfway: to the even neighbour
            inc -= 1;
            inc += (S + inc) & 1;
        }
        const unsigned long long S2 = S + inc;
        if (S2 < (ONE52 << 1)) return (static_cast<unsigned long long>(KE) << 52) | (S2 & MANT);
    }
    return as_bits(__dadd_rn(as_f64(s), as_f64(x)));
}

// One block per tile. (1) Each (segment, lane pair) thread computes its segments' transfer
// functions at the binade of the lane's state before the tile (K3's layout: 8 lane pairs x 32
// segments of 8 blocks). (2) Per lane, a warp composes them in segment order from that state;
// where all 32 apply, the states before each segment follow. (3) Each thread then adds its
// segments' rows one at a time (add_bits) for the state after every block; a lane whose segments
// do not all apply (a binade crossing, a negative row or state, the first tile) runs its whole
// chain in one thread instead. (4) The combines of the states, (5) the tails, in add_bits.
__global__ void __launch_bounds__(256, 3) canon_scan_kernel(const unsigned long long *__restrict__ x, int64_t n, int64_t nb,
                                                         int T, const unsigned long long *__restrict__ tstate,
                                                         unsigned long long *__restrict__ out) {
    extern __shared__ __align__(16) unsigned char scan_smem[];
    ScanSmem &sm = *reinterpret_cast<ScanSmem *>(scan_smem);
    const int t = blockIdx.x, tid = threadIdx.x;
    const int64_t row0 = static_cast<int64_t>(t) * (CT_BLOCKS * 16);
    const int64_t left = n - row0;
    const int rows = left < CT_BLOCKS * 16 ? static_cast<int>(left) : CT_BLOCKS * 16;
    {  // all 16 loads of a thread in flight before the first store
        unsigned long long pre[CT_BLOCKS * 16 / 256];
#pragma unroll
        for (int q = 0; q < CT_BLOCKS * 16 / 256; ++q) {
            const int i = tid + q * 256;
            pre[q] = i < rows ? x[row0 + i] : 0ull;
        }
#pragma unroll
        for (int q = 0; q < CT_BLOCKS * 16 / 256; ++q) {
            const int i = tid + q * 256;
            if (i < rows) sm.v[(i >> 4) * SCAN_PAD + (i & 15)] = pre[q];
        }
    }
    // The tile's whole blocks (all but a partial last one) feed the lanes.
    const int64_t whole = nb - static_cast<int64_t>(t) * CT_BLOCKS;
    const int fb = whole <= 0 ? 0 : (whole < CT_BLOCKS ? static_cast<int>(whole) : CT_BLOCKS);
    __syncthreads();
    // (1)
    const int lp = tid & 7, seg = tid >> 3;
    unsigned long long r[CT_SEG_BLOCKS][2];
#pragma unroll
    for (int i = 0; i < CT_SEG_BLOCKS; ++i) {
        const int blk = seg * CT_SEG_BLOCKS + i;
        r[i][0] = blk < fb ? sm.v[blk * SCAN_PAD + 2 * lp] : 0ull;
        r[i][1] = blk < fb ? sm.v[blk * SCAN_PAD + 2 * lp + 1] : 0ull;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int L = 2 * lp + h;
        const int E = tstate ? state_binade(tstate[static_cast<int64_t>(L) * (T + 1) + t]) : NO_E;
        TF f{0, 0};
        const bool ok = E != NO_E && E >= -959 && seg_tf<false>(r, h, 1023 + E, &f);
        sm.seg.tf[L][seg] = f;
        sm.seg.ok[L][seg] = ok;
    }
    __syncthreads();
    // (2) warp w: lanes 2w and 2w + 1, thread `sl` of the warp = segment sl.
    const int w = tid >> 5, sl = tid & 31;
    unsigned long long before[2];
    bool carried[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int L = 2 * w + h;
        const unsigned long long s0 = tstate ? tstate[static_cast<int64_t>(L) * (T + 1) + t] : 0ull;
        const int E = state_binade(s0);
        unsigned long long after = s0, mine = 0;
        const int m = E == NO_E ? 0 : apply_prefix<false>(sm.seg.tf[L][sl], sm.seg.ok[L][sl] != 0, s0, E, &after, &mine);
        carried[h] = m == CT_SEGS;
        const unsigned long long prev = __shfl_up_sync(FULL, mine, 1);
        before[h] = sl == 0 ? s0 : prev;
    }
    __syncthreads();  // the segment functions are read; their space holds the states from here
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int L = 2 * w + h;
        if (carried[h]) sm.st[(sl * CT_SEG_BLOCKS) * SCAN_PAD + L] = before[h];
        if (sl == 0) sm.serial[L] = !carried[h];
    }
    __syncthreads();
    // (3)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int L = 2 * lp + h;
        if (sm.serial[L]) continue;
        unsigned long long st = sm.st[(seg * CT_SEG_BLOCKS) * SCAN_PAD + L];
#pragma unroll
        for (int i = 0; i < CT_SEG_BLOCKS; ++i) {
            st = add_bits(st, r[i][h]);
            // the state after the segment's last block is the next segment's, stored in (2)
            if (i < CT_SEG_BLOCKS - 1 || seg == CT_SEGS - 1) sm.st[(seg * CT_SEG_BLOCKS + i + 1) * SCAN_PAD + L] = st;
        }
    }
    if (tid < 16 && sm.serial[tid]) {
        unsigned long long st = tstate ? tstate[static_cast<int64_t>(tid) * (T + 1) + t] : 0ull;
        sm.st[tid] = st;
        if (st >> 63) {  // a negative state: the integer steps do not apply
            for (int j = 0; j < fb; ++j) {
                st = as_bits(__dadd_rn(as_f64(st), as_f64(sm.v[j * SCAN_PAD + tid])));
                sm.st[(j + 1) * SCAN_PAD + tid] = st;
            }
        } else {
            for (int j = 0; j < fb; ++j) {
                st = add_bits(st, sm.v[j * SCAN_PAD + tid]);
                sm.st[(j + 1) * SCAN_PAD + tid] = st;
            }
        }
    }
    __syncthreads();
    // (4)
    for (int j = tid; j <= fb; j += 256) {
        double a[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) a[q] = as_f64(sm.st[j * SCAN_PAD + q]);
#pragma unroll
        for (int step = 8; step > 0; step >>= 1)
#pragma unroll
            for (int q = 0; q < step; ++q) a[q] = __dadd_rn(a[q], a[q + step]);
        sm.c[j] = a[0];
    }
    __syncthreads();
    // (5)
    const int nbt = (rows + 15) >> 4;  // blocks in the tile, a partial last one included
    for (int j = tid; j < nbt; j += 256) {
        unsigned long long c = as_bits(sm.c[j]);
        const int cnt = min(16, rows - 16 * j);
        unsigned long long *v = sm.v + j * SCAN_PAD;
#pragma unroll
        for (int q = 0; q < 15; ++q) {
            if (q < cnt) {
                c = add_bits(c, v[q]);
                v[q] = c;
            }
        }
        if (cnt == 16) v[15] = as_bits(sm.c[j + 1]);  // a whole block: j < fb
    }
    __syncthreads();
    for (int i = tid; i < rows; i += 256) out[row0 + i] = sm.v[(i >> 4) * SCAN_PAD + (i & 15)];
}

// The prefix canonical sums of rows x[0 .. n) into out[0 .. n).
static vkc_status canon_scan_rows(vkc_ctx *ctx, const unsigned long long *x, int64_t n, unsigned long long *out) {
    if (n == 0) return VKC_OK;
    vkc_status st;
    const int64_t nb = n / 16;
    const int64_t tiles = ((n + 15) / 16 + CT_BLOCKS - 1) / CT_BLOCKS;
    if (tiles > (int64_t(1) << 26)) return fail(ctx, VKC_USAGE, "array too long for one scan");
    const unsigned long long *tstate = nullptr;
    int T = 0;
    if (tiles > 1) {  // then nb >= CT_BLOCKS
        T = static_cast<int>((nb + CT_BLOCKS - 1) / CT_BLOCKS);
        const int C = (T + 31) / 32;
        void *p;
        if ((st = scratch(ctx, canon_layout(T, C, true, nullptr, nullptr, nullptr), &p))) return st;
        CanonWork wk;
        CanonState *cs = nullptr;
        canon_layout(T, C, true, static_cast<char *>(p), &wk, &cs);
        VKC_CUDA(ctx, cudaMemsetAsync(cs, 0, sizeof(CanonState), ctx->stream));
        RowArgs a{};
        a.x = x;
        st = (reinterpret_cast<uintptr_t>(x) & 15) == 0 ? launch_canon<ROW_SUM, true, true>(ctx, a, nb, T, C, wk, cs)
                                                        : launch_canon<ROW_SUM, false, true>(ctx, a, nb, T, C, wk, cs);
        if (st) return st;
        tstate = wk.tstate;
    }
    static std::atomic<unsigned long long> configured{0};
    once_per_device(configured, ctx->device, [] {
        cudaFuncSetAttribute(canon_scan_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(sizeof(ScanSmem)));
    });
    canon_scan_kernel<<<static_cast<unsigned>(tiles), 256, sizeof(ScanSmem), ctx->stream>>>(x, n, nb, T, tstate, out);
    return launched(ctx, "canon_scan");
}

static vkc_status scan_add_f64(vkc_ctx *ctx, const vkc_value *args, int, vkc_value *out) {
    vkc_status st;
    if (!array_arg(ctx, args[0], VKC_F64, &st)) return st;
    const vkc_array *xa = args[0].array;
    vkc_array *o;
    if ((st = new_array(ctx, VKC_F64, xa->len, false, &o))) return st;
    st = canon_scan_rows(ctx, static_cast<const unsigned long long *>(xa->data()), xa->len,
                         static_cast<unsigned long long *>(o->data()));
    if (st) {
        vkc_array_release(o);
        return st;
    }
    out->kind = VKC_VALUE_ARRAY;
    out->array = o;
    return VKC_OK;
}

// scan_by_add_f64: each segment (from a row whose start flag is set, row 0 always, to the next)
// is scanned with its lanes numbered from its first row. Segment heads are listed in order (a
// count per 1024-row tile, a scan, an ordered write). One block per tile then takes the segments
// whose heads lie in the tile: consecutive segments packed into runs of at most SBP_CAP rows,
// staged in shared memory; a segment longer than that in windows of SBP_CAP rows that carry its
// lane states; segments longer than SB_SHORT are listed for the host and take the tiled scan.
constexpr int SB_TILE = 1024;
constexpr int64_t SB_SHORT = int64_t(1) << 16;
constexpr int SBP_CAP = 1536, SBP_THREADS = 128, SBP_RPT = SBP_CAP / SBP_THREADS;  // 12 rows a thread

// The head bits of rows r0 .. r0 + 15: one 16-byte load where the flags allow it.
__device__ __forceinline__ unsigned sb_heads(const unsigned char *__restrict__ starts, int64_t n, int64_t r0, unsigned *mask) {
    unsigned m = 0;
    if (r0 + 16 <= n && (reinterpret_cast<uintptr_t>(starts + r0) & 15) == 0) {
        const uint4 q = *reinterpret_cast<const uint4 *>(starts + r0);
        const unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int b = 0; b < 4; ++b)
                if ((w[k] >> (8 * b)) & 0xffu) m |= 1u << (4 * k + b);
        if (r0 == 0) m |= 1u;
    } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int64_t i = r0 + j;
            if (i < n && (i == 0 || starts[i] != 0)) m |= 1u << j;
        }
    }
    *mask = m;
    return __popc(m);
}

__global__ void __launch_bounds__(SB_TILE / 16) sb_count_kernel(const unsigned char *__restrict__ starts, int64_t n,
                                                                unsigned *__restrict__ counts) {
    unsigned m, total;
    const unsigned c = sb_heads(starts, n, static_cast<int64_t>(blockIdx.x) * SB_TILE + threadIdx.x * 16, &m);
    block_exclusive_sum<unsigned>(c, &total);
    if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SB_TILE / 16) sb_list_kernel(const unsigned char *__restrict__ starts, int64_t n,
                                                               const unsigned *__restrict__ offs, long long *__restrict__ heads) {
    unsigned m, total;
    const int64_t r0 = static_cast<int64_t>(blockIdx.x) * SB_TILE + threadIdx.x * 16;
    const unsigned c = sb_heads(starts, n, r0, &m);
    unsigned at = offs[blockIdx.x] + block_exclusive_sum<unsigned>(c, &total);
    while (m) {
        const int j = __ffs(m) - 1;
        m &= m - 1;
        heads[at++] = r0 + j;
    }
}

// Rows of a pack in shared memory: row i at i ^ ((i >> 4) & 15), so that the threads of a
// half-warp reading the same position of 16 consecutive 16-row blocks hit different banks.
__device__ __forceinline__ int sbp(int i) { return i ^ ((i >> 4) & 15); }

struct SbSmem {
    unsigned long long x[SBP_CAP];    // the pack's rows (bits)
    unsigned long long out[SBP_CAP];  // the lane states after each whole block at their rows, then the outputs
    unsigned long long carried[16];   // a long segment: its lane states at the window's first row
    unsigned long long carried_c;     // and their combine
    long long tile_end;               // the row after the tile's last segment
    unsigned bm[SBP_CAP / 32 + 2];    // the pack's segment heads (two words past the end stay 0)
    unsigned items[SBP_CAP / 16];     // segments with a whole block: first row | blocks << 16
    int n_items;
    int warp_max[32];
    unsigned short hs[SB_TILE];  // the tile's heads, from the tile's first row
};

// Block-wide exclusive maximum (-1 before the first thread); blockDim.x a multiple of 32.
__device__ __forceinline__ int sb_exclusive_max(int v, int *warp_max) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x = max(x, y);
    }
    int before = __shfl_up_sync(FULL, x, 1);
    if (lane == 0) before = -1;
    if (lane == 31) warp_max[w] = x;
    __syncthreads();
    int carry = -1;
    for (int j = 0; j < w && j < nw; ++j) carry = max(carry, warp_max[j]);
    __syncthreads();
    return max(carry, before);
}

// One pack: rows [p0, p0 + rows) of x. `window`: a window of one long segment, whose lanes start
// from `carried` (+0.0 in its first window) and whose first block's tail from `carried_c`;
// otherwise the consecutive segments m .. m2 - 1 of the tile, each of at most SBP_CAP rows,
// their lanes and first tails from +0.0. In the order of the oracle's restatement: lane l of a
// segment adds its rows l, l + 16, ... of the whole blocks (add_bits, which equals the IEEE add
// and takes the FP64 add itself from +0.0); the row closing a whole block gets the pairwise
// combine (+8, +4, +2, +1) of the lane states after it; the other rows of a block are the chain
// from the combine before the block (+0.0 for the segment's first block).
__device__ __forceinline__ void sb_pack(SbSmem &sm, const unsigned long long *__restrict__ x,
                                        unsigned long long *__restrict__ out, int64_t p0, int rows, bool window,
                                        bool first, int m, int m2, int64_t trow, int cnt) {
    const int tid = threadIdx.x;
    unsigned long long v[SBP_RPT];
#pragma unroll
    for (int q = 0; q < SBP_RPT; ++q) {
        const int i = tid + q * SBP_THREADS;
        v[q] = i < rows ? x[p0 + i] : 0ull;
    }
#pragma unroll
    for (int q = 0; q < SBP_RPT; ++q) {
        const int i = tid + q * SBP_THREADS;
        if (i < rows) sm.x[sbp(i)] = v[q];
    }
    if (window) {
        if (first && tid < 16) sm.carried[tid] = 0ull;
        if (first && tid == 0) sm.carried_c = 0ull;
        if (tid == 0) {
            sm.items[0] = static_cast<unsigned>(rows >> 4) << 16;
            sm.n_items = rows >= 16 ? 1 : 0;
        }
    } else {
        for (int j = m + tid; j < m2; j += SBP_THREADS) {
            const int64_t sj = trow + sm.hs[j];
            const int64_t ej = j + 1 < cnt ? trow + sm.hs[j + 1] : sm.tile_end;
            const int off = static_cast<int>(sj - p0);
            atomicOr(&sm.bm[off >> 5], 1u << (off & 31));
            const unsigned nb = static_cast<unsigned>((ej - sj) >> 4);
            if (nb > 0) sm.items[atomicAdd(&sm.n_items, 1)] = static_cast<unsigned>(off) | (nb << 16);
        }
    }
    __syncthreads();
    // The lane chains: 16 consecutive threads take the 16 lanes of one segment.
    const int total = 16 * sm.n_items;
    for (int i = tid; i < total; i += SBP_THREADS) {
        const unsigned it = sm.items[i >> 4];
        const int l = i & 15, off = static_cast<int>(it & 0xffffu), nb = static_cast<int>(it >> 16);
        unsigned long long st = window ? sm.carried[l] : 0ull;
        for (int b = 0; b < nb; ++b) {
            const int r = off + l + 16 * b;
            st = add_bits(st, sm.x[sbp(r)]);
            sm.out[sbp(r)] = st;
        }
        if (window) sm.carried[l] = st;  // read by this thread only, in the next window
    }
    // Each thread's rows r0 .. r0 + SBP_RPT - 1 and the segment start before them.
    const int r0 = tid * SBP_RPT;
    unsigned mine = 0;
    int sr0 = 0;
    if (!window) {
        const unsigned long long w2 = sm.bm[r0 >> 5] | (static_cast<unsigned long long>(sm.bm[(r0 >> 5) + 1]) << 32);
        mine = static_cast<unsigned>(w2 >> (r0 & 31)) & ((1u << SBP_RPT) - 1);
        sr0 = sb_exclusive_max(mine ? r0 + 31 - __clz(mine) : -1, sm.warp_max);  // synchronises the block
    } else {
        __syncthreads();
    }
    // Each thread's block starts and the one block end (at most one block closes in 16 or fewer
    // consecutive rows), found first so that a warp runs one combine and the tails side by side.
    int sr = sr0, rend = -1;
    unsigned smask = 0;
#pragma unroll
    for (int q = 0; q < SBP_RPT; ++q) {
        const int r = r0 + q;
        if ((mine >> q) & 1u) sr = r;
        if (r < rows) {
            if (((r - sr) & 15) == 0) smask |= 1u << q;
            if (((r - sr) & 15) == 15) rend = r;
        }
    }
    if (rend >= 0) {
        double a[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) a[k] = as_f64(sm.out[sbp(rend - 15 + k)]);
#pragma unroll
        for (int step = 8; step > 0; step >>= 1)
#pragma unroll
            for (int k = 0; k < step; ++k) a[k] = __dadd_rn(a[k], a[k + step]);
        sm.out[sbp(rend)] = as_bits(a[0]);
    }
    __syncthreads();
    // The tails, from each block's first row: the combine before it, +0.0 at a segment's head.
    while (smask) {
        const int q = __ffs(smask) - 1;
        smask &= smask - 1;
        const int r = r0 + q;
        const bool head = window ? r == 0 : ((mine >> q) & 1u) != 0;
        unsigned long long c = head ? (window ? sm.carried_c : 0ull) : sm.out[sbp(r - 1)];
        // rows r .. r + 14 up to the next head or the pack's end
        const int b1 = r + 1, sh = b1 & 31;
        const unsigned next = (sm.bm[b1 >> 5] >> sh) | (sh ? sm.bm[(b1 >> 5) + 1] << (32 - sh) : 0u);
        const int len = min((next & 0x3fffu) ? __ffs(next & 0x3fffu) : 15, rows - r);
        for (int k = 0; k < len; ++k) {
            c = add_bits(c, sm.x[sbp(r + k)]);
            sm.out[sbp(r + k)] = c;
        }
    }
    __syncthreads();
    if (window && tid == 0) sm.carried_c = sm.out[sbp(rows - 1)];  // the next window's, when this one is whole
#pragma unroll
    for (int q = 0; q < SBP_RPT; ++q) {
        const int i = tid + q * SBP_THREADS;
        if (i < rows) out[p0 + i] = sm.out[sbp(i)];
    }
    if (!window)
        for (int i = tid; i < SBP_CAP / 32 + 2; i += SBP_THREADS) sm.bm[i] = 0;
    if (tid == 0) sm.n_items = 0;
    __syncthreads();
}

// One block per tile of SB_TILE rows: the segments whose heads lie in it, the long ones (more
// than SB_SHORT rows) listed as (first row, rows) pairs after a count in longs[0].
__global__ void __launch_bounds__(SBP_THREADS, 8) sb_pack_kernel(const unsigned long long *__restrict__ x, int64_t n,
                                                                 const long long *__restrict__ heads,
                                                                 const unsigned *__restrict__ offs,
                                                                 const unsigned *__restrict__ counts, int tiles,
                                                                 unsigned long long *__restrict__ out,
                                                                 unsigned long long *__restrict__ longs) {
    extern __shared__ __align__(16) unsigned char sb_smem[];
    SbSmem &sm = *reinterpret_cast<SbSmem *>(sb_smem);
    const int c = blockIdx.x, tid = threadIdx.x;
    const int cnt = static_cast<int>(counts[c]);
    if (cnt == 0) return;
    const int64_t k0 = offs[c];
    const int64_t G = static_cast<int64_t>(offs[tiles - 1]) + counts[tiles - 1];
    const int64_t trow = static_cast<int64_t>(c) * SB_TILE;
    for (int i = tid; i < cnt; i += SBP_THREADS) sm.hs[i] = static_cast<unsigned short>(heads[k0 + i] - trow);
    for (int i = tid; i < SBP_CAP / 32 + 2; i += SBP_THREADS) sm.bm[i] = 0;
    if (tid == 0) {
        sm.tile_end = k0 + cnt < G ? heads[k0 + cnt] : n;
        sm.n_items = 0;
    }
    __syncthreads();
    const int64_t tile_end = sm.tile_end;
    auto end_of = [&](int j) { return j + 1 < cnt ? trow + sm.hs[j + 1] : tile_end; };
    int m = 0;
    while (m < cnt) {
        const int64_t s = trow + sm.hs[m], e = end_of(m);
        if (e - s > SB_SHORT) {
            if (tid == 0) {
                const unsigned long long k = atomicAdd(longs, 1ull);
                longs[1 + 2 * k] = static_cast<unsigned long long>(s);
                longs[2 + 2 * k] = static_cast<unsigned long long>(e - s);
            }
            ++m;
            continue;
        }
        if (e - s > SBP_CAP) {
            for (int64_t w0 = s; w0 < e; w0 += SBP_CAP)
                sb_pack(sm, x, out, w0, static_cast<int>(e - w0 < SBP_CAP ? e - w0 : SBP_CAP), true, w0 == s, 0, 0, trow, cnt);
            ++m;
            continue;
        }
        // The longest run of segments from m within SBP_CAP rows.
        int lo = m + 1, hi = cnt;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (end_of(mid - 1) - s <= SBP_CAP) lo = mid;
            else hi = mid - 1;
        }
        sb_pack(sm, x, out, s, static_cast<int>(end_of(lo - 1) - s), false, false, m, lo, trow, cnt);
        m = lo;
    }
}

// One block per listed long segment (first row, rows): the windows of sb_pack in order.
__global__ void __launch_bounds__(SBP_THREADS, 8) sb_long_kernel(const unsigned long long *__restrict__ x,
                                                                 const unsigned long long *__restrict__ list,
                                                                 unsigned long long *__restrict__ out) {
    extern __shared__ __align__(16) unsigned char sb_smem[];
    SbSmem &sm = *reinterpret_cast<SbSmem *>(sb_smem);
    const int64_t s = static_cast<int64_t>(list[2 * blockIdx.x]), e = s + static_cast<int64_t>(list[2 * blockIdx.x + 1]);
    for (int i = threadIdx.x; i < SBP_CAP / 32 + 2; i += SBP_THREADS) sm.bm[i] = 0;
    if (threadIdx.x == 0) sm.n_items = 0;
    __syncthreads();
    for (int64_t w0 = s; w0 < e; w0 += SBP_CAP)
        sb_pack(sm, x, out, w0, static_cast<int>(e - w0 < SBP_CAP ? e - w0 : SBP_CAP), true, w0 == s, 0, 0, 0, 0);
}

static vkc_status scan_by_add_f64(vkc_ctx *ctx, const vkc_value *args, int, vkc_value *out) {
    vkc_status st;
    if (!array_arg(ctx, args[0], VKC_F64, &st) || !array_arg(ctx, args[1], VKC_BOOL, &st)) return st;
    const vkc_array *xa = args[0].array, *sa = args[1].array;
    const int64_t n = xa->len;
    if (sa->len != n)
        return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(n) + " vs " + std::to_string(sa->len));
    // Segment heads are counted and offset in u32 (the argsort's count scan).
    if (n >= (int64_t(1) << 32))
        return fail(ctx, VKC_USAGE, "scan_by of " + std::to_string(n) + " rows: at most 2^32 - 1 rows per call");
    vkc_array *o;
    if ((st = new_array(ctx, VKC_F64, n, false, &o))) return st;
    if (n == 0) {
        out->kind = VKC_VALUE_ARRAY;
        out->array = o;
        return VKC_OK;
    }
    const auto *x = static_cast<const unsigned long long *>(xa->data());
    const auto *starts = static_cast<const unsigned char *>(sa->data());
    auto *ov = static_cast<unsigned long long *>(o->data());
    const int64_t tiles = (n + SB_TILE - 1) / SB_TILE;
    const int64_t sum_words = scan_counts_sum_words(tiles);
    const int64_t max_long = n / (SB_SHORT + 1) + 1;
    // One i64 work array: counts and offsets (u32, tiles each), the scan's sums, the heads, the
    // long-segment list.
    const int64_t w_counts = (tiles + 1) / 2, w_sums = (sum_words + 1) / 2;
    vkc_array *work;
    if ((st = new_array(ctx, VKC_I64, 2 * w_counts + w_sums + n + 1 + 2 * max_long, false, &work))) {
        vkc_array_release(o);
        return st;
    }
    auto *w = static_cast<long long *>(work->data());
    auto *counts = reinterpret_cast<unsigned *>(w);
    auto *offs = reinterpret_cast<unsigned *>(w + w_counts);
    auto *sums = reinterpret_cast<unsigned *>(w + 2 * w_counts);
    long long *heads = w + 2 * w_counts + w_sums;
    auto *longs = reinterpret_cast<unsigned long long *>(heads + n);
    auto done = [&](vkc_status s2) {
        vkc_array_release(work);
        if (s2) {
            vkc_array_release(o);
            return s2;
        }
        out->kind = VKC_VALUE_ARRAY;
        out->array = o;
        return VKC_OK;
    };
    // CUDA errors release the arrays as well (done).
    auto cuda = [&](cudaError_t e, const char *what) { return e == cudaSuccess ? VKC_OK : cuda_fail(ctx, e, what); };
    if ((st = cuda(cudaMemsetAsync(longs, 0, sizeof(unsigned long long), ctx->stream), "cudaMemsetAsync")))
        return done(st);
    sb_count_kernel<<<static_cast<unsigned>(tiles), SB_TILE / 16, 0, ctx->stream>>>(starts, n, counts);
    if ((st = launched(ctx, "sb_count"))) return done(st);
    scan_counts(ctx, counts, tiles, sums, offs);
    sb_list_kernel<<<static_cast<unsigned>(tiles), SB_TILE / 16, 0, ctx->stream>>>(starts, n, offs, heads);
    if ((st = launched(ctx, "sb_list"))) return done(st);
    static std::atomic<unsigned long long> configured{0};
    once_per_device(configured, ctx->device, [] {
        cudaFuncSetAttribute(sb_pack_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sizeof(SbSmem)));
        cudaFuncSetAttribute(sb_long_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sizeof(SbSmem)));
    });
    sb_pack_kernel<<<static_cast<unsigned>(tiles), SBP_THREADS, sizeof(SbSmem), ctx->stream>>>(
        x, n, heads, offs, counts, static_cast<int>(tiles), ov, longs);
    if ((st = launched(ctx, "sb_pack"))) return done(st);
    unsigned long long nlong = 0;
    if ((st = cuda(cudaMemcpyAsync(&nlong, longs, sizeof nlong, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync")) ||
        (st = cuda(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize")))
        return done(st);
    if (nlong > 0) {
        std::vector<unsigned long long> list(2 * nlong);
        if ((st = cuda(cudaMemcpyAsync(list.data(), longs + 1, list.size() * sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync")) ||
            (st = cuda(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize")))
            return done(st);
        // One tiled scan per segment costs about 140 us of launches and waits plus 11 ps a row,
        // one after another; a block per segment in windows about 5 ns a row, all segments side
        // by side (figures measured at 2^27 rows). The cheaper of the two takes them all.
        unsigned long long longest = 0, rows = 0;
        for (unsigned long long k = 0; k < nlong; ++k) {
            longest = std::max(longest, list[2 * k + 1]);
            rows += list[2 * k + 1];
        }
        if (static_cast<double>(nlong) * 140e-6 + static_cast<double>(rows) * 11e-12 > static_cast<double>(longest) * 5e-9) {
            sb_long_kernel<<<static_cast<unsigned>(nlong), SBP_THREADS, sizeof(SbSmem), ctx->stream>>>(x, longs + 1, ov);
            st = launched(ctx, "sb_long");
        } else {
            for (unsigned long long k = 0; k < nlong && !st; ++k)
                st = canon_scan_rows(ctx, x + list[2 * k], static_cast<int64_t>(list[2 * k + 1]), ov + list[2 * k]);
        }
    }
    return done(st);
}

template <int OP, int CMP> static ReducerImpl *make_canon(vkc_ctx *ctx) {
    auto *r = new CanonReducer;
    r->op = OP;
    r->cmp = CMP;
    if (r->alloc(ctx, sizeof(CanonState))) {
        delete r;
        return nullptr;
    }
    return r;
}

void register_canon(std::vector<KernelDef> &t) {
    InSpec xa{IN_ARRAY, VKC_F64}, xs{IN_SCALAR, VKC_F64};
    KernelDef d{"reduce_add_f64", VKC_REDUCTION, {xa}, false, VKC_F64, 8};
    d.red = make_canon<ROW_SUM, -1>;
    t.push_back(d);
    d = KernelDef{"dot_f64", VKC_REDUCTION, {xa, xa}, false, VKC_F64, 16};
    d.red = make_canon<ROW_DOT, -1>;
    t.push_back(d);
    d = KernelDef{"sumsq_f64", VKC_REDUCTION, {xa}, false, VKC_F64, 8};
    d.red = make_canon<ROW_SUMSQ, -1>;
    t.push_back(d);
    static const char *names[6] = {"eq", "ne", "lt", "le", "gt", "ge"};
    ReducerMake makes[6] = {make_canon<ROW_CONDSUM, 0>, make_canon<ROW_CONDSUM, 1>,
                            make_canon<ROW_CONDSUM, 2>, make_canon<ROW_CONDSUM, 3>,
                            make_canon<ROW_CONDSUM, 4>, make_canon<ROW_CONDSUM, 5>};
    for (int c = 0; c < 6; ++c) {
        d = KernelDef{std::string("condsum_") + names[c] + "_f64", VKC_REDUCTION, {xa, xs, xs}, false,
                      VKC_F64, 8};
        d.red = makes[c];
        t.push_back(d);
    }
    // Float scans (an extension: the tier-2 notes' candidate order), whole entries.
    d = KernelDef{"scan_add_f64", VKC_WHOLE, {xa}, true, VKC_F64, 16};
    d.whole = scan_add_f64;
    t.push_back(d);
    d = KernelDef{"scan_by_add_f64", VKC_WHOLE, {xa, InSpec{IN_ARRAY, VKC_BOOL}}, true, VKC_F64, 17};
    d.whole = scan_by_add_f64;
    t.push_back(d);
}

}  // namespace vkc

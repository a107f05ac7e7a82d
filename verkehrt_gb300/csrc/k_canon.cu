// The canonical f64 sums: reduce_add_f64, dot_f64, sumsq_f64 and condsum_<cmp>_f64, bit-exact
// to the reference's canonical order at every length.
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
//  * Each 8192-row tile (512 blocks of 16 rows) computes, per lane and per 256-row segment,
//    the transfer functions for the one or two binades its running sum can be in. The binade
//    comes from an approximate prefix of the lane sums found by a first decoupled lookback
//    over the tiles (float sums, with a 2^-12 relative margin).
//  * A second decoupled lookback composes the predecessors' tile transfer functions until
//    it reaches a published exact lane state; the tile then walks its segments from its exact
//    start, applying each transfer function whose binade and bound check out, and adding the
//    rows of any other segment one by one with IEEE f64 adds (the reference's own operation).
//    Negative, infinite or NaN rows, the first rows of a lane and binade crossings take this
//    sequential path, so the result is the reference's in every case.
//
// All of the per-row work is integer arithmetic: GB300 executes FP64 adds at about 1/66 of
// its integer op rate, so an FP64 tree would be compute-bound well below the HBM roofline.
#include <climits>
#include <cmath>

#include "reduce_common.h"

namespace vkc {

constexpr int CT_THREADS = 256;
constexpr int CT_SEGS = 32;        // segments per tile
constexpr int CT_SEG_BLOCKS = 16;  // 16-row blocks per segment
constexpr int CT_BLOCKS = CT_SEGS * CT_SEG_BLOCKS;  // 512 blocks = 8192 rows per tile
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

// a, then b.
__device__ __forceinline__ TF compose(TF a, TF b) {
    TF r;
    r.d0 = sat_add(a.d0, (a.d0 & 1) ? b.d1 : b.d0);
    r.d1 = sat_add(a.d1, (a.d1 & 1) ? b.d0 : b.d1);
    return r;
}

// Applies f (valid in binade E) to the lane state with bits s. Fails when s is not a
// positive normal in binade E or when the result would leave the binade.
__device__ __forceinline__ bool apply(unsigned long long s, int E, TF f, unsigned long long *out) {
    unsigned long long ef = static_cast<unsigned long long>(E + 1023);
    if ((s >> 52) != ef) return false;
    unsigned long long S = (s & MANT) | ONE52;
    unsigned long long S2 = S + ((S & 1) ? f.d1 : f.d0);
    if (S2 >= (ONE52 << 1)) return false;
    *out = (ef << 52) | (S2 & MANT);
    return true;
}

// The transfer function of 16 row values in binade E (KE = 1023 + E >= 64). Returns false
// when a row is negative, infinite, NaN or not below 2^E (k < 1), where the integer step does
// not hold. For x = M * 2^(ex-1075), x/u = M / 2^k with k = KE - ex, and
// RNE(x/u) = (M + 2^(k-1)) >> k unless M mod 2^k is exactly 2^(k-1) (a tie).
__device__ __forceinline__ bool seg_tf(const unsigned long long (&v)[CT_SEG_BLOCKS][2], int h,
                                       int KE, TF *out) {
    unsigned long long D = 0;
    int kmin = 64;
    bool tie = false;
#pragma unroll
    for (int i = 0; i < CT_SEG_BLOCKS; ++i) {
        unsigned long long b = v[i][h];
        int ex = static_cast<int>(b >> 52);  // the sign bit makes negative rows fail k >= 1
        int k = KE - ex;
        kmin = min(kmin, k);
        k = min(max(k, 1), 63);  // zero and subnormal rows have k >= 64: increment 0, no tie
        unsigned long long M = (b & MANT) | ONE52;
        unsigned long long w = M + (1ull << (k - 1));
        D += w >> k;
        tie |= (w << (64 - k)) == 0;
    }
    if (kmin < 1) return false;
    if (!tie) {
        *out = TF{D, D};
        return true;
    }
    // Ties: both parities, in row order. A tie rounds S + floor(x/u) + 1/2 to the even
    // neighbour, so the increment is floor(x/u) plus the parity of S + floor(x/u).
    unsigned long long d0 = 0, d1 = 0;
    for (int i = 0; i < CT_SEG_BLOCKS; ++i) {
        unsigned long long b = v[i][h];
        int k = min(max(KE - static_cast<int>(b >> 52), 1), 63);
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

// Lookback records of one launch, in the context scratch arena.
struct CanonScratch {
    unsigned *flag1;           // approx: epoch<<2 | 1 aggregate, 2 inclusive
    unsigned *flag2;           // exact
    double *agg1, *inc1;       // [tiles][16]
    unsigned long long *agg2;  // [tiles][16][3]: E+1024 (0 = invalid), d0, d1
    unsigned long long *inc2;  // [tiles][16] lane state bits
};

// Reducer state on the device.
struct CanonState {
    unsigned long long lanes[16];
    unsigned long long tail[16];
    unsigned long long result;
};

template <int OP, bool ALIGNED>
__global__ void __launch_bounds__(CT_THREADS, 2)
canon_kernel(RowArgs args, int64_t nb, int tiles, CanonScratch sc, unsigned epoch,
             CanonState *state, unsigned *counters, DevStatus *status) {
    extern __shared__ unsigned long long s_vals[];  // [512 blocks][16 lanes], staged on demand
    __shared__ float s_apx[CT_SEGS][16];
    __shared__ int s_E[16][2];
    __shared__ TF s_tf[2][CT_SEGS][16];
    __shared__ unsigned char s_ok[2][CT_SEGS][16];
    __shared__ unsigned long long s_start[16];
    __shared__ int s_stage;
    __shared__ unsigned s_tile;

    const int t = threadIdx.x;
    const int lp = t & 7, seg = t >> 3;
    if (t == 0) {
        s_tile = atomicAdd(&counters[0], 1u);
        s_stage = 0;
    }
    __syncthreads();
    const int tile = static_cast<int>(s_tile);
    const int64_t blk0 = static_cast<int64_t>(tile) * CT_BLOCKS;

    // 1. Load the segment's rows (two lanes per thread) and compute the row values.
    unsigned long long v[CT_SEG_BLOCKS][2];
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
            // Past the last block: +0.0 leaves every lane state unchanged (a lane is never -0).
            v[i][0] = 0;
            v[i][1] = 0;
        }
    }

    // 2. Approximate lane sums of the tile.
    {
        float a0 = 0.f, a1 = 0.f;
#pragma unroll
        for (int i = 0; i < CT_SEG_BLOCKS; ++i) {
            a0 += approx_f32(v[i][0]);
            a1 += approx_f32(v[i][1]);
        }
        s_apx[seg][2 * lp] = a0;
        s_apx[seg][2 * lp + 1] = a1;
    }
    __syncthreads();

    // 3. Lookback 1 (approximate prefix), one thread per lane in warp 0.
    if (t < 16) {
        double A = 0;
        for (int s = 0; s < CT_SEGS; ++s) A += static_cast<double>(s_apx[s][t]);
        sc.agg1[tile * 16 + t] = A;
        __threadfence();
        __syncwarp(0xffffu);
        if (t == 0) st_release(&sc.flag1[tile], (epoch << 2) | 1u);
        double excl = 0;
        bool found = false;
        for (int tp = tile - 1; tp >= 0 && !found; --tp) {
            unsigned f = 0, it = 0;
            while (((f = ld_acquire(&sc.flag1[tp])) >> 2) != epoch) {
                if (++it > SPIN_LIMIT) {
                    set_timeout(status);
                    found = true;
                    break;
                }
                backoff(it);
            }
            if (found) break;
            if ((f & 3u) == 2u) {
                excl += sc.inc1[tp * 16 + t];
                found = true;
            } else {
                excl += sc.agg1[tp * 16 + t];
            }
        }
        if (!found) excl += as_f64(state->lanes[t]);
        sc.inc1[tile * 16 + t] = excl + A;
        __threadfence();
        __syncwarp(0xffffu);
        if (t == 0) st_release(&sc.flag1[tile], (epoch << 2) | 2u);
        // Candidate binades: the range [start, end] widened by 2^-12 on each side.
        double lo = excl < excl + A ? excl : excl + A;
        double hi = excl < excl + A ? excl + A : excl;
        int elo = binade(lo * (1.0 - 0x1p-12)), ehi = binade(hi * (1.0 + 0x1p-12));
        int e0 = NO_E, e1 = NO_E;
        if (elo != NO_E && ehi != NO_E && elo >= -959) {
            if (ehi == elo) e0 = elo;
            else if (ehi == elo + 1) {
                e0 = elo;
                e1 = ehi;
            }
        }
        s_E[t][0] = e0;
        s_E[t][1] = e1;
    }
    __syncthreads();

    // 4. Segment transfer functions for each candidate binade.
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int lane = 2 * lp + h;
        for (int c = 0; c < 2; ++c) {
            int E = s_E[lane][c];
            TF f{0, 0};
            bool ok = E != NO_E && seg_tf(v, h, 1023 + E, &f);
            s_tf[c][seg][lane] = f;
            s_ok[c][seg][lane] = ok;
        }
    }
    __syncthreads();

    // 5. Publish the tile's transfer function per lane (single-binade lanes only), then
    //    lookback 2 for the exact start state.
    TF tile_tf{0, 0};
    int tile_E = NO_E;
    if (t < 16) {
        if (s_E[t][0] != NO_E && s_E[t][1] == NO_E) {
            bool ok = true;
            for (int s = 0; s < CT_SEGS; ++s) {
                ok = ok && s_ok[0][s][t];
                tile_tf = compose(tile_tf, s_tf[0][s][t]);
            }
            if (ok) tile_E = s_E[t][0];
        }
        unsigned long long *rec = sc.agg2 + (static_cast<int64_t>(tile) * 16 + t) * 3;
        rec[0] = tile_E == NO_E ? 0ull : static_cast<unsigned long long>(tile_E + 1024);
        rec[1] = tile_tf.d0;
        rec[2] = tile_tf.d1;
        __threadfence();
        __syncwarp(0xffffu);
        if (t == 0) st_release(&sc.flag2[tile], (epoch << 2) | 1u);

        // Walk back over aggregates of one binade to the nearest exact state.
        TF acc{0, 0};
        int accE = NO_E;
        bool have_acc = false, done = false, timed_out = false;
        unsigned long long base = 0, start = 0;
        for (int tp = tile - 1; tp >= 0 && !done; --tp) {
            unsigned f = 0, it = 0;
            for (;;) {
                f = ld_acquire(&sc.flag2[tp]);
                if ((f >> 2) == epoch) {
                    if ((f & 3u) == 2u) break;
                    const unsigned long long *r = sc.agg2 + (static_cast<int64_t>(tp) * 16 + t) * 3;
                    int e = r[0] ? static_cast<int>(r[0]) - 1024 : NO_E;
                    if (e != NO_E && (!have_acc || e == accE)) break;
                }
                // An unusable aggregate: wait for that tile's exact state.
                if (++it > SPIN_LIMIT) {
                    set_timeout(status);
                    timed_out = true;
                    break;
                }
                backoff(it);
            }
            if (timed_out) break;
            if ((f & 3u) == 2u) {
                base = sc.inc2[tp * 16 + t];
                done = true;
            } else {
                const unsigned long long *r = sc.agg2 + (static_cast<int64_t>(tp) * 16 + t) * 3;
                TF g{r[1], r[2]};
                accE = static_cast<int>(r[0]) - 1024;
                acc = have_acc ? compose(g, acc) : g;
                have_acc = true;
            }
        }
        if (!done) base = state->lanes[t];
        start = base;
        if (have_acc && !timed_out && !apply(base, accE, acc, &start)) {
            // The composed aggregates do not hold from that state: wait for the previous
            // tile's exact state.
            unsigned f = 0, it = 0;
            while ((((f = ld_acquire(&sc.flag2[tile - 1])) >> 2) != epoch) || (f & 3u) != 2u) {
                if (++it > SPIN_LIMIT) {
                    set_timeout(status);
                    break;
                }
                backoff(it);
            }
            start = sc.inc2[(tile - 1) * 16 + t];
        }
        s_start[t] = start;
        // Stage the rows when the tile's own transfer function does not carry the lane.
        unsigned long long end;
        if (!(tile_E != NO_E && apply(start, tile_E, tile_tf, &end))) s_stage = 1;
    }
    __syncthreads();
    if (s_stage) {
#pragma unroll
        for (int i = 0; i < CT_SEG_BLOCKS; ++i)
            *reinterpret_cast<ulonglong2 *>(&s_vals[(seg * CT_SEG_BLOCKS + i) * 16 + 2 * lp]) =
                make_ulonglong2(v[i][0], v[i][1]);
    }
    __syncthreads();

    // 6. Walk the lane's segments from the exact start.
    if (t < 16) {
        unsigned long long s = s_start[t], end;
        if (tile_E != NO_E && apply(s, tile_E, tile_tf, &end)) {
            s = end;
        } else {
            for (int sg = 0; sg < CT_SEGS; ++sg) {
                bool ok = false;
                for (int c = 0; c < 2 && !ok; ++c)
                    if (s_E[t][c] != NO_E && s_ok[c][sg][t])
                        ok = apply(s, s_E[t][c], s_tf[c][sg][t], &s);
                if (!ok) {
                    double d = as_f64(s);
                    for (int i = 0; i < CT_SEG_BLOCKS; ++i)
                        d = __dadd_rn(d, as_f64(s_vals[(sg * CT_SEG_BLOCKS + i) * 16 + t]));
                    s = as_bits(d);
                }
            }
        }
        sc.inc2[tile * 16 + t] = s;
        __threadfence();
        __syncwarp(0xffffu);
        if (t == 0) st_release(&sc.flag2[tile], (epoch << 2) | 2u);
    }

    // The block that finishes last stores the end states (no block reads the start states
    // any more) and resets the ticket for the next launch.
    __shared__ int s_last;
    if (t == 0) {
        __threadfence();
        unsigned prev = atomicAdd(&counters[1], 1u);
        s_last = prev == static_cast<unsigned>(tiles) - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        if (t < 16) state->lanes[t] = ld_relaxed64(&sc.inc2[(tiles - 1) * 16 + t]);
        if (t == 0) {
            counters[0] = 0;
            counters[1] = 0;
        }
    }
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

template <int OP, bool ALIGNED>
static void launch_canon(vkc_ctx *ctx, const RowArgs &a, int64_t nb, int tiles, CanonScratch sc,
                         unsigned epoch, CanonState *state) {
    const size_t smem = sizeof(unsigned long long) * CT_BLOCKS * 16;
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(canon_kernel<OP, ALIGNED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem));
        configured = true;
    }
    canon_kernel<OP, ALIGNED><<<tiles, CT_THREADS, smem, ctx->stream>>>(a, nb, tiles, sc, epoch, state,
                                                                       ctx->counters, ctx->status);
}

// The canonical reducer of one row operation.
struct CanonReducer : DevReducer {
    int op;
    int cmp = -1;
    int tail_len = 0;

    vkc_status update(vkc_ctx *ctx, const Arg *args, int nargs) override {
        vkc_status st;
        RowArgs a{};
        int64_t n = 0;
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
        n = args[0].len();
        // reduce.rs:297-303: rows may only follow whole blocks.
        if (tail_len != 0) return fail(ctx, VKC_RUNTIME, "canonical update after a partial block");
        int64_t nb = n / 16;
        int rest = static_cast<int>(n % 16);
        auto *cs = static_cast<CanonState *>(state);
        if (nb > 0) {
            int64_t tiles64 = (nb + CT_BLOCKS - 1) / CT_BLOCKS;
            if (tiles64 > INT_MAX / 2) return fail(ctx, VKC_USAGE, "array too long for one update");
            int tiles = static_cast<int>(tiles64);
            size_t t16 = static_cast<size_t>(tiles) * 16;
            size_t off_inc1 = t16 * 8;
            size_t off_agg2 = off_inc1 + t16 * 8;
            size_t off_inc2 = off_agg2 + t16 * 24;
            size_t total = off_inc2 + t16 * 8;
            void *p;
            unsigned *flags;
            if ((st = scratch(ctx, total, &p))) return st;
            if ((st = flag_arena(ctx, static_cast<size_t>(tiles) * 2, &flags))) return st;
            char *base = static_cast<char *>(p);
            CanonScratch sc{flags, flags + tiles,
                            reinterpret_cast<double *>(base), reinterpret_cast<double *>(base + off_inc1),
                            reinterpret_cast<unsigned long long *>(base + off_agg2),
                            reinterpret_cast<unsigned long long *>(base + off_inc2)};
            unsigned epoch = next_epoch(ctx);
            bool aligned = (reinterpret_cast<uintptr_t>(a.x) & 15) == 0 &&
                           (op != ROW_DOT || (reinterpret_cast<uintptr_t>(a.y) & 15) == 0);
#define CANON_CASE(OPV)                                                              \
    case OPV:                                                                        \
        if (aligned) launch_canon<OPV, true>(ctx, a, nb, tiles, sc, epoch, cs);      \
        else launch_canon<OPV, false>(ctx, a, nb, tiles, sc, epoch, cs);             \
        break;
            switch (op) {
                CANON_CASE(ROW_SUM)
                CANON_CASE(ROW_DOT)
                CANON_CASE(ROW_SUMSQ)
                CANON_CASE(ROW_CONDSUM)
            }
#undef CANON_CASE
            if ((st = launched(ctx, "canon"))) return st;
        }
        if (rest > 0) {
            int64_t first = nb * 16;
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
        DevStatus ds;
        if ((st = read_status(ctx, &ds))) return st;
        out->type = VKC_F64;
        return download(ctx, &out->bits, 8, offsetof(CanonState, result));
    }
};

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
}

}  // namespace vkc

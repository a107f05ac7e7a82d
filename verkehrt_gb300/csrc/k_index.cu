// Index kernels: gather_T, histogram, reduce_into_add_i64 (src/kernels/scalar/index.rs:31-155,
// :194-222).
//
// The reference checks every index before it writes a row and reports the first offending
// value in index order (first_out_of_range, index.rs:102-111). Here the check is fused into
// the kernel: each offending row does an atomicMin of its row number into the status word,
// and the host reports the value at that row and discards the output.
#include "reduce_common.h"

namespace vkc {

int64_t scan_counts_sum_words(int64_t m);
void scan_counts(vkc_ctx *ctx, const unsigned *c, int64_t m, unsigned *sums, unsigned *out);

// ------------------------------------------------------------------ gather

template <int W> struct GWord;
template <> struct GWord<8> { using T = unsigned long long; };
template <> struct GWord<4> { using T = unsigned; };
template <> struct GWord<1> { using T = unsigned char; };

// R rows per thread (the autotuner's gather_rows_per_thread) over a grid that covers the rows
// once: random reads are bound by the number of DRAM sectors in flight across the whole GPU,
// which the largest grid maximizes (measured on GB300: 50 G random 8-byte reads/s with one
// row per thread, against 44 G for grid-stride loops). Row r of thread g is g + r * (threads
// of the grid), so each load of the R is coalesced across the warp; all R index loads, then
// all R source loads, are in flight together.
template <int W, int R>
__global__ void __launch_bounds__(256) gather_kernel(const typename GWord<W>::T *__restrict__ src, uint64_t nsrc,
                                                     const long long *__restrict__ idx, int64_t n,
                                                     typename GWord<W>::T *__restrict__ out, DevStatus *status) {
    const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t span = static_cast<int64_t>(gridDim.x) * blockDim.x;
    long long k[R];
#pragma unroll
    for (int r = 0; r < R; ++r) k[r] = g + r * span < n ? __ldcs(idx + g + r * span) : 0;
    typename GWord<W>::T v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = (g + r * span < n && static_cast<uint64_t>(k[r]) < nsrc) ? __ldg(src + k[r]) : 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int64_t i = g + r * span;
        if (i >= n) break;
        if (static_cast<uint64_t>(k[r]) < nsrc) out[i] = v[r];
        else atomicMin(&status->first_bad, static_cast<unsigned long long>(i));
    }
}

template <int W>
static void launch_gather(vkc_ctx *ctx, int rows, int64_t n, const typename GWord<W>::T *src, uint64_t nsrc,
                          const long long *idx, typename GWord<W>::T *out) {
    const int grid = static_cast<int>((n + 256 * rows - 1) / (256 * rows));
    switch (rows) {
    case 2: gather_kernel<W, 2><<<grid, 256, 0, ctx->stream>>>(src, nsrc, idx, n, out, ctx->status); break;
    case 4: gather_kernel<W, 4><<<grid, 256, 0, ctx->stream>>>(src, nsrc, idx, n, out, ctx->status); break;
    default: gather_kernel<W, 1><<<grid, 256, 0, ctx->stream>>>(src, nsrc, idx, n, out, ctx->status); break;
    }
}

// ------------------------------------------------------------------ partitioned gather
//
// Random 8-byte reads from a source far larger than L2 each cost a DRAM burst (about 97 DRAM
// bytes per row on GB300, against 24 algorithmic). For such sources the gather runs as four
// passes over tiles of GP_TILE index rows, so that the source is read one region at a time
// while that region sits in L2, and every other access is a coalesced run:
//   count      per tile, the rows that fall in each of the GP_NB source regions (and the bounds
//              check: an offending row is not counted and records its row number);
//   partition  after one exclusive scan of the counts (region-major), each row's offset within
//              its region goes to its tile's run of `part` in that region, and the row's slot in
//              the tile's region-sorted order goes to `loc`;
//   region     positions in region order read src[region base + part[p]] into vals[p]; the
//              blocks in flight cover one or two regions, whose lines stay in L2;
//   restore    each tile gathers its runs of vals into shared memory in region-sorted order and
//              writes out[i] = staged[loc[i]] in row order.
// About 60 DRAM bytes per row, nearly all in runs.
constexpr int GP_THREADS = 256, GP_ITEMS = 16, GP_TILE = GP_THREADS * GP_ITEMS;
constexpr int GP_NB = 64;  // source regions

// Warp 0: the exclusive prefix of GP_NB counts get(b) into s_start[0 .. GP_NB - 1], and their
// total into s_start[GP_NB].
template <class Get> __device__ __forceinline__ void gp_starts(Get get, unsigned *s_start) {
    const int lane = threadIdx.x & 31;
    unsigned run = 0;
#pragma unroll
    for (int b0 = 0; b0 < GP_NB; b0 += 32) {
        const unsigned c = get(b0 + lane);
        unsigned x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        s_start[b0 + lane] = run + x - c;
        run += __shfl_sync(FULL, x, 31);
    }
    if (lane == 0) s_start[GP_NB] = run;
}

// The last b with s_start[b] <= v (s_start[0] = 0 <= v < s_start[GP_NB]).
__device__ __forceinline__ int gp_region_of(const unsigned *s_start, unsigned v) {
    int lo = 0, hi = GP_NB;
#pragma unroll
    for (int it = 0; it < 6; ++it) {  // GP_NB = 2^6
        const int mid = (lo + hi) >> 1;
        if (s_start[mid] <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(GP_THREADS, 4) gp_count_kernel(const long long *__restrict__ idx, int64_t n, uint64_t nsrc,
                                                              int rb, int tiles, unsigned *__restrict__ counts,
                                                              DevStatus *status) {
    __shared__ unsigned h[GP_NB];
    if (threadIdx.x < GP_NB) h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = static_cast<int64_t>(blockIdx.x) * GP_TILE;
    // All of a thread's loads are issued before its first atomic (the atomics keep the order).
    unsigned long long k[GP_ITEMS];
#pragma unroll
    for (int j = 0; j < GP_ITEMS; ++j) {
        const int64_t r = base + j * GP_THREADS + threadIdx.x;
        k[j] = r < n ? static_cast<unsigned long long>(__ldcs(idx + r)) : 0ull;
    }
#pragma unroll
    for (int j = 0; j < GP_ITEMS; ++j) {
        const int64_t r = base + j * GP_THREADS + threadIdx.x;
        if (r < n) {
            if (k[j] < nsrc) atomicAdd(&h[static_cast<unsigned>(k[j] >> rb)], 1u);
            else atomicMin(&status->first_bad, static_cast<unsigned long long>(r));
        }
    }
    __syncthreads();
    if (threadIdx.x < GP_NB) counts[static_cast<int64_t>(threadIdx.x) * tiles + blockIdx.x] = h[threadIdx.x];
}

// PACK (regions of at most 2^26 rows): a row's region rides in the top 6 bits of its staged
// offset, so no byte array of regions is written and read back.
template <bool PACK>
__global__ void __launch_bounds__(GP_THREADS, 4) gp_partition_kernel(const long long *__restrict__ idx, int64_t n,
                                                                  uint64_t nsrc, int rb, int tiles,
                                                                  const unsigned *__restrict__ toffs,
                                                                  unsigned *__restrict__ part,
                                                                  unsigned short *__restrict__ loc) {
    __shared__ unsigned s_cnt[GP_NB], s_start[GP_NB + 1], s_goff[GP_NB];
    __shared__ unsigned s_part[GP_TILE];
    __shared__ unsigned char s_reg[PACK ? 1 : GP_TILE];
    if (threadIdx.x < GP_NB) {
        s_cnt[threadIdx.x] = 0;
        s_goff[threadIdx.x] = toffs[static_cast<int64_t>(blockIdx.x) * GP_NB + threadIdx.x];
    }
    __syncthreads();
    const int64_t base = static_cast<int64_t>(blockIdx.x) * GP_TILE;
    const unsigned long long mask = (1ull << rb) - 1;
    // Per row: its offset in its region, and its region (bits 16 and up) with its slot among
    // the tile's rows of that region (the low 16 bits; GP_TILE <= 2^16), or ~0u for an
    // offending row or one past the end (kept in 32-bit words: fewer registers, more blocks).
    unsigned off[GP_ITEMS], rk[GP_ITEMS];
#pragma unroll
    for (int j = 0; j < GP_ITEMS; ++j) {
        const int64_t r = base + j * GP_THREADS + threadIdx.x;
        const unsigned long long k = r < n ? static_cast<unsigned long long>(__ldcs(idx + r)) : ~0ull;
        off[j] = static_cast<unsigned>(k & mask);
        rk[j] = k < nsrc ? static_cast<unsigned>(k >> rb) << 16 : ~0u;
    }
    // Slots within the tile's region runs, in any order: the output does not depend on it.
#pragma unroll
    for (int j = 0; j < GP_ITEMS; ++j)
        if (rk[j] != ~0u) rk[j] |= atomicAdd(&s_cnt[rk[j] >> 16], 1u);
    __syncthreads();
    if (threadIdx.x < 32) gp_starts([&](int b) { return s_cnt[b]; }, s_start);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < GP_ITEMS; ++j) {
        const int64_t r = base + j * GP_THREADS + threadIdx.x;
        if (r >= n) continue;
        if (rk[j] != ~0u) {
            const unsigned b = rk[j] >> 16;
            const unsigned l = s_start[b] + (rk[j] & 0xffffu);
            loc[r] = static_cast<unsigned short>(l);
            if (PACK) {
                s_part[l] = off[j] | (b << 26);
            } else {
                s_part[l] = off[j];
                s_reg[l] = static_cast<unsigned char>(b);
            }
        } else {
            loc[r] = 0;  // the call fails; the row's output is never read
        }
    }
    __syncthreads();
    const int rows = static_cast<int>(s_start[GP_NB]);
    for (int l = threadIdx.x; l < rows; l += GP_THREADS) {
        const unsigned v = s_part[l];
        const unsigned b = PACK ? v >> 26 : s_reg[l];
        part[s_goff[b] + static_cast<unsigned>(l) - s_start[b]] = PACK ? v & ((1u << 26) - 1) : v;
    }
}

// The counts and offsets of every (region, tile), region-major as the scan needs them, copied
// tile-major (tile t's 64 values in one 256-byte run) for the passes that read one tile's.
__global__ void __launch_bounds__(256) gp_tables_kernel(const unsigned *__restrict__ counts,
                                                        const unsigned *__restrict__ offs, int tiles,
                                                        unsigned *__restrict__ tcounts, unsigned *__restrict__ toffs) {
    __shared__ unsigned s_c[GP_NB][GP_NB + 1], s_o[GP_NB][GP_NB + 1];
    const int t0 = blockIdx.x * GP_NB;
    for (int i = threadIdx.x; i < GP_NB * GP_NB; i += 256) {
        const int b = i / GP_NB, tt = i % GP_NB;
        if (t0 + tt < tiles) {
            s_c[b][tt] = counts[static_cast<int64_t>(b) * tiles + t0 + tt];
            s_o[b][tt] = offs[static_cast<int64_t>(b) * tiles + t0 + tt];
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < GP_NB * GP_NB; i += 256) {
        const int tt = i / GP_NB, b = i % GP_NB;
        if (t0 + tt < tiles) {
            tcounts[static_cast<int64_t>(t0 + tt) * GP_NB + b] = s_c[b][tt];
            toffs[static_cast<int64_t>(t0 + tt) * GP_NB + b] = s_o[b][tt];
        }
    }
}

__global__ void __launch_bounds__(GP_THREADS, 6) gp_region_kernel(const unsigned long long *__restrict__ src,
                                                               const unsigned *__restrict__ part,
                                                               const unsigned *__restrict__ counts,
                                                               const unsigned *__restrict__ offs, int tiles, int rb,
                                                               unsigned long long *__restrict__ vals) {
    __shared__ unsigned s_start[GP_NB + 1];
    const int64_t last = static_cast<int64_t>(GP_NB) * tiles - 1;
    // Region b's positions start at the offset of (b, tile 0); the last offset plus its count
    // is the number of rows in range.
    if (threadIdx.x <= GP_NB)
        s_start[threadIdx.x] = threadIdx.x < GP_NB ? offs[static_cast<int64_t>(threadIdx.x) * tiles] : offs[last] + counts[last];
    __syncthreads();
    const unsigned total = s_start[GP_NB];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * GP_TILE;
    if (base >= total) return;
    // A thread's positions rise, so its region only moves forward from the first one's. In
    // each quarter the offsets are loaded first, then the quarter's source reads are in flight
    // together; the source reads skip L1 (each touches one sector of a line that no other read
    // of this block is likely to use: the same reads as cp.async into shared memory, which
    // allocates in L1, took 886 us against 310 at 2^26).
    int b = gp_region_of(s_start, static_cast<unsigned>(base + threadIdx.x < total ? base + threadIdx.x : total - 1));
    // Four quarters of GP_ITEMS / 4 rows: fewer registers, six blocks an SM.
    constexpr int H = GP_ITEMS / 4;
#pragma unroll 1
    for (int h = 0; h < GP_ITEMS / H; ++h) {
        unsigned o[H];
#pragma unroll
        for (int j = 0; j < H; ++j) {
            const int64_t p = base + (h * H + j) * GP_THREADS + threadIdx.x;
            o[j] = p < total ? __ldcs(part + p) : 0u;
        }
        unsigned long long v[H];
#pragma unroll
        for (int j = 0; j < H; ++j) {
            const int64_t p = base + (h * H + j) * GP_THREADS + threadIdx.x;
            if (p < total) {
                while (static_cast<unsigned>(p) >= s_start[b + 1]) ++b;
                v[j] = __ldcg(src + (static_cast<int64_t>(b) << rb) + o[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < H; ++j) {
            const int64_t p = base + (h * H + j) * GP_THREADS + threadIdx.x;
            if (p < total) __stcs(vals + p, v[j]);
        }
    }
}

__global__ void __launch_bounds__(GP_THREADS, 6) gp_restore_kernel(const unsigned long long *__restrict__ vals,
                                                                const unsigned short *__restrict__ loc,
                                                                const unsigned *__restrict__ tcounts,
                                                                const unsigned *__restrict__ toffs, int64_t n,
                                                                unsigned long long *__restrict__ out) {
    __shared__ unsigned s_start[GP_NB + 1], s_goff[GP_NB];
    __shared__ unsigned long long s_vals[GP_TILE];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * GP_TILE;
    // The rows' slots first (two to a register): their loads overlap the tables' and the runs'.
    unsigned lp[GP_ITEMS / 2];
#pragma unroll
    for (int j = 0; j < GP_ITEMS; ++j) {
        const int64_t r = base + j * GP_THREADS + threadIdx.x;
        const unsigned lv = r < n ? static_cast<unsigned>(__ldcs(loc + r)) : 0u;
        lp[j / 2] = (j & 1) ? (lp[j / 2] | (lv << 16)) : lv;
    }
    const unsigned *tc = tcounts + static_cast<int64_t>(blockIdx.x) * GP_NB;
    if (threadIdx.x < 32) gp_starts([&](int b) { return tc[b]; }, s_start);
    if (threadIdx.x < GP_NB) s_goff[threadIdx.x] = toffs[static_cast<int64_t>(blockIdx.x) * GP_NB + threadIdx.x];
    __syncthreads();
    const int rows = static_cast<int>(s_start[GP_NB]);
    // The runs straight into shared memory (cp.async: every copy in flight, no registers held).
#pragma unroll
    for (int j = 0; j < GP_ITEMS; ++j) {
        const unsigned l = threadIdx.x + j * GP_THREADS;
        if (l < static_cast<unsigned>(rows)) {
            const int b = gp_region_of(s_start, l);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(static_cast<unsigned>(__cvta_generic_to_shared(&s_vals[l]))),
                         "l"(vals + s_goff[b] + l - s_start[b])
                         : "memory");
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
#pragma unroll
    for (int j = 0; j < GP_ITEMS; ++j) {
        const int64_t r = base + j * GP_THREADS + threadIdx.x;
        if (r < n) out[r] = s_vals[(lp[j / 2] >> (16 * (j & 1))) & 0xffffu];
    }
}

// The partitioned path pays when the source is well beyond L2 (2^26 rows, 512 MiB; at 2^25
// rows the one-pass gather still hits L2 often enough) and the index rows are at least half
// the source rows, so that each region line fetched into L2 is read about twice (with fewer,
// the one-pass gather moves fewer DRAM bytes). Measured on GB300 at n = 2^28 index rows into
// 2^28 source rows: 68 G rows/s against 45 G. Positions are u32: fewer than 2^32 index rows.
static bool gather_partitions(uint64_t nsrc, int64_t n) {
    return nsrc >= (uint64_t(1) << 26) && nsrc <= (uint64_t(1) << 38) && n >= (int64_t(1) << 22) &&
           2 * static_cast<uint64_t>(n) >= nsrc && n < (int64_t(1) << 32);
}

static vkc_status gather_partitioned(vkc_ctx *ctx, const unsigned long long *src, uint64_t nsrc, const long long *idx,
                                     int64_t n, unsigned long long *out) {
    int lg = 0;
    while ((uint64_t(1) << lg) < nsrc) ++lg;
    const int rb = lg - 6;  // GP_NB = 2^6 regions of 2^rb rows
    const int tiles = static_cast<int>((n + GP_TILE - 1) / GP_TILE);
    const int64_t m = static_cast<int64_t>(GP_NB) * tiles;
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t o_offs = up(m * 4), o_tc = o_offs + up(m * 4), o_to = o_tc + up(m * 4), o_sums = o_to + up(m * 4);
    const size_t o_part = o_sums + up(scan_counts_sum_words(m) * 4), o_loc = o_part + up(n * 4);
    const size_t o_vals = o_loc + up(n * 2), total = o_vals + n * 8;
    void *p;
    vkc_status st = scratch(ctx, total, &p);
    if (st) return st;
    char *b = static_cast<char *>(p);
    auto *counts = reinterpret_cast<unsigned *>(b);
    auto *offs = reinterpret_cast<unsigned *>(b + o_offs);
    auto *tcounts = reinterpret_cast<unsigned *>(b + o_tc);
    auto *toffs = reinterpret_cast<unsigned *>(b + o_to);
    auto *part = reinterpret_cast<unsigned *>(b + o_part);
    auto *loc = reinterpret_cast<unsigned short *>(b + o_loc);
    auto *vals = reinterpret_cast<unsigned long long *>(b + o_vals);
    gp_count_kernel<<<tiles, GP_THREADS, 0, ctx->stream>>>(idx, n, nsrc, rb, tiles, counts, ctx->status);
    scan_counts(ctx, counts, m, reinterpret_cast<unsigned *>(b + o_sums), offs);
    gp_tables_kernel<<<(tiles + GP_NB - 1) / GP_NB, 256, 0, ctx->stream>>>(counts, offs, tiles, tcounts, toffs);
    if (rb <= 26)
        gp_partition_kernel<true><<<tiles, GP_THREADS, 0, ctx->stream>>>(idx, n, nsrc, rb, tiles, toffs, part, loc);
    else
        gp_partition_kernel<false><<<tiles, GP_THREADS, 0, ctx->stream>>>(idx, n, nsrc, rb, tiles, toffs, part, loc);
    gp_region_kernel<<<tiles, GP_THREADS, 0, ctx->stream>>>(src, part, counts, offs, tiles, rb, vals);
    gp_restore_kernel<<<tiles, GP_THREADS, 0, ctx->stream>>>(vals, loc, tcounts, toffs, n, out);
    return launched(ctx, "gather_partitioned");
}

// Reads the value at `row` of an i64 device array.
static vkc_status read_i64(vkc_ctx *ctx, const void *base, uint64_t row, int64_t *out) {
    void *h;
    vkc_status st = pinned(ctx, 8, &h);
    if (st) return st;
    VKC_CUDA(ctx, cudaMemcpyAsync(h, static_cast<const long long *>(base) + row, 8, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *out = *static_cast<long long *>(h);
    return VKC_OK;
}

// index.rs:40-73 (Gather::checked, run).
template <vkc_type T> static vkc_status gather(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
    if (!array_arg(ctx, args[0], T, &st) || !array_arg(ctx, args[1], VKC_I64, &st)) return st;
    const vkc_array *xs = args[0].array, *ix = args[1].array;
    int64_t n = ix->len;
    vkc_array *o;
    if ((st = new_array(ctx, T, n, false, &o))) return st;
    if (n > 0) {
        const int64_t g64 = (n + 255) / 256;
        if (g64 > INT32_MAX) {
            vkc_array_release(o);
            return fail(ctx, VKC_USAGE, "gather of more than 2^39 rows");
        }
        const int rows = tune(ctx, TK_GATHER_ROWS, n);
        const auto *idx = static_cast<const long long *>(ix->data());
        if (type_width(T) == 8 && gather_partitions(static_cast<uint64_t>(xs->len), n)) {
            st = gather_partitioned(ctx, static_cast<const unsigned long long *>(xs->data()), xs->len, idx, n,
                                    static_cast<unsigned long long *>(o->data()));
        } else {
            switch (type_width(T)) {
            case 8: launch_gather<8>(ctx, rows, n, static_cast<const unsigned long long *>(xs->data()), xs->len, idx, static_cast<unsigned long long *>(o->data())); break;
            case 4: launch_gather<4>(ctx, rows, n, static_cast<const unsigned *>(xs->data()), xs->len, idx, static_cast<unsigned *>(o->data())); break;
            default: launch_gather<1>(ctx, rows, n, static_cast<const unsigned char *>(xs->data()), xs->len, idx, static_cast<unsigned char *>(o->data())); break;
            }
            st = launched(ctx, "gather");
        }
        if (st) {
            vkc_array_release(o);
            return st;
        }
        DevStatus ds;
        if ((st = read_status(ctx, &ds))) {
            vkc_array_release(o);
            return st;
        }
        if (ds.first_bad != ~0ull) {
            vkc_array_release(o);
            int64_t v;
            if ((st = read_i64(ctx, ix->data(), ds.first_bad, &v))) return st;
            return fail(ctx, VKC_RUNTIME, "gather index " + std::to_string(v) + " out of range for length " +
                                              std::to_string(static_cast<uint64_t>(xs->len)));
        }
    }
    out->kind = VKC_VALUE_ARRAY;
    out->array = o;
    return VKC_OK;
}

// ------------------------------------------------------------------ histogram, reduce_into

// Bounds only: the first key outside [0, nb).
__global__ void __launch_bounds__(256) keys_check_kernel(const long long *__restrict__ keys, int64_t n,
                                                         uint64_t nb, DevStatus *status) {
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    unsigned long long bad = ~0ull;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        if (static_cast<uint64_t>(__ldcs(keys + i)) >= nb && static_cast<unsigned long long>(i) < bad)
            bad = static_cast<unsigned long long>(i);
    if (bad != ~0ull) atomicMin(&status->first_bad, bad);
}

// Per-bucket wrapping sums (vals) or counts (vals == nullptr). Every warp walks chunks of
// BK_ITEMS groups of 32 consecutive rows (one coalesced load per group and array, all groups of
// a chunk loaded before any is added). Within a group, runs of equal keys in consecutive lanes
// are summed by a segmented warp scan, so only the lane that ends a run adds it to a bucket; the
// run that ends a group is carried into the next group while the key stays the same. Sorted
// keys (run numbers, sorted group keys) thus cost about one addition per run instead of one per
// row, which removes the contention of long runs on one bucket. Buckets below SMEM_BINS are
// added in shared memory per block and to the output once per block; the others go to global
// atomics. Small keys are where random contention is: group ids number groups by first
// occurrence, so frequent groups get small ids (under a Zipf(1.1) key distribution the first
// 4096 ids hold about three quarters of the rows).
constexpr int SMEM_BINS = 4096;
constexpr int BK_ITEMS = 8;  // groups of 32 rows per warp chunk, all loaded before use

template <bool COUNT>
__global__ void __launch_bounds__(256) bucket_kernel(const long long *__restrict__ keys,
                                                     const unsigned long long *__restrict__ vals, int64_t n,
                                                     uint64_t nb, unsigned long long *__restrict__ out,
                                                     DevStatus *status) {
    __shared__ unsigned long long bins[SMEM_BINS];
    const int sb = nb < static_cast<uint64_t>(SMEM_BINS) ? static_cast<int>(nb) : SMEM_BINS;
    for (int b = threadIdx.x; b < sb; b += blockDim.x) bins[b] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
    const int64_t chunk_rows = 32 * BK_ITEMS;
    const int64_t chunks = (n + chunk_rows - 1) / chunk_rows;
    const unsigned below = (1u << lane) - 1u;
    auto add = [&](long long k, unsigned long long v) {
        if (k < SMEM_BINS) atomicAdd(&bins[k], v);
        else atomicAdd(out + k, v);
    };
    constexpr long long NONE = -1;  // a lane with no row in range: never added
    unsigned long long bad = ~0ull;
    long long ckey = NONE;  // the carried run (the same in every lane)
    unsigned long long csum = 0;
    for (int64_t c = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); c < chunks;
         c += warps) {
        const int64_t base = c * chunk_rows + lane;
        long long k[BK_ITEMS];
        unsigned long long v[BK_ITEMS];
#pragma unroll
        for (int r = 0; r < BK_ITEMS; ++r) {
            const int64_t i = base + 32 * r;
            k[r] = i < n ? __ldcs(keys + i) : NONE;
            v[r] = (!COUNT && i < n) ? __ldcs(vals + i) : 1ull;
        }
#pragma unroll
        for (int r = 0; r < BK_ITEMS; ++r) {
            const int64_t i = base + 32 * r;
            long long key = k[r];
            if (i < n && static_cast<uint64_t>(key) >= nb) {
                if (static_cast<unsigned long long>(i) < bad) bad = static_cast<unsigned long long>(i);
                key = NONE;
            }
            unsigned long long x = key == NONE ? 0ull : v[r];
            // Runs of equal keys: a lane heads a run when its key differs from the lane before.
            const long long up = __shfl_up_sync(FULL, key, 1);
            const bool head = lane == 0 || up != key;
            const unsigned heads = __ballot_sync(FULL, head);
            const int start = 31 - __clz(heads & (below | (1u << lane)));  // this run's first lane
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long t = __shfl_up_sync(FULL, x, o);
                if (lane - o >= start) x += t;
            }
            const bool tail = lane == 31 || ((heads >> (lane + 1)) & 1u);
            // Runs of the carried key join the carry; the run ending at lane 31 becomes the next
            // carry; every other run is added now.
            const unsigned long long join = warp_sum(tail && key == ckey ? x : 0ull);
            csum += join;
            const long long k31 = __shfl_sync(FULL, key, 31);
            const unsigned long long x31 = __shfl_sync(FULL, x, 31);
            if (tail && lane != 31 && key != ckey && key != NONE) add(key, x);
            if (k31 != ckey) {
                if (lane == 0 && ckey != NONE) add(ckey, csum);
                ckey = k31;
                csum = x31;
            }
        }
    }
    if (lane == 0 && ckey != NONE) add(ckey, csum);
    if (bad != ~0ull) atomicMin(&status->first_bad, bad);
    __syncthreads();
    for (int b = threadIdx.x; b < sb; b += blockDim.x)
        if (bins[b]) atomicAdd(out + b, bins[b]);
}

// The reference's error for the first key outside [0, nb) (checked_keys, index.rs:116-130):
// *found and VKC_RUNTIME with the message, or VKC_OK when every key is in range.
vkc_status bucket_key_error(vkc_ctx *ctx, const long long *k, int64_t n, int64_t nb, bool *found) {
    *found = false;
    if (n == 0) return VKC_OK;
    int grid = stream_grid(ctx, n, 256, 8, 4096);
    keys_check_kernel<<<grid, 256, 0, ctx->stream>>>(k, n, static_cast<uint64_t>(nb), ctx->status);
    vkc_status s2 = launched(ctx, "keys_check");
    if (s2) return s2;
    DevStatus ds;
    if ((s2 = read_status(ctx, &ds))) return s2;
    if (ds.first_bad == ~0ull) return VKC_OK;
    int64_t v;
    if ((s2 = read_i64(ctx, k, ds.first_bad, &v))) return s2;
    *found = true;
    return fail(ctx, VKC_RUNTIME, "bucket key " + std::to_string(v) + " out of range for " +
                                      std::to_string(nb) + " buckets");
}

// index.rs:116-130 (checked_keys) then the result allocation (value.rs:285-307). The key check
// precedes allocation errors; a length mismatch of reduce_into follows it (index.rs:203-210).
static vkc_status run_buckets(vkc_ctx *ctx, const vkc_array *keys, const vkc_array *vals, int64_t nb,
                              vkc_value *out) {
    vkc_status st;
    if (nb < 0) return fail(ctx, VKC_RUNTIME, "negative bucket count " + std::to_string(nb));
    int64_t n = keys->len;
    const auto *k = static_cast<const long long *>(keys->data());
    auto key_error = [&](bool *found) -> vkc_status { return bucket_key_error(ctx, k, n, nb, found); };
    bool found;
    if (vals && vals->len != n) {
        if ((st = key_error(&found))) return st;
        return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(n) + " keys for " +
                                          std::to_string(vals->len) + " values");
    }
    vkc_array *o;
    st = new_array(ctx, VKC_I64, nb, true, &o);
    if (st) {
        std::string msg = ctx->err;
        vkc_status kst = key_error(&found);
        if (kst) return kst;
        return fail(ctx, st, msg);
    }
    if (n > 0) {
        // Every block adds its shared bins to the output once: at most 8 blocks per SM, and at
        // least 8192 rows per block.
        int grid = stream_grid(ctx, n, 256, 8, 8192);
        auto *ov = static_cast<unsigned long long *>(o->data());
        const auto *vv = vals ? static_cast<const unsigned long long *>(vals->data()) : nullptr;
        if (!vals) bucket_kernel<true><<<grid, 256, 0, ctx->stream>>>(k, vv, n, nb, ov, ctx->status);
        else bucket_kernel<false><<<grid, 256, 0, ctx->stream>>>(k, vv, n, nb, ov, ctx->status);
        if ((st = launched(ctx, "buckets"))) {
            vkc_array_release(o);
            return st;
        }
        DevStatus ds;
        if ((st = read_status(ctx, &ds))) {
            vkc_array_release(o);
            return st;
        }
        if (ds.first_bad != ~0ull) {
            vkc_array_release(o);
            int64_t v;
            if ((st = read_i64(ctx, k, ds.first_bad, &v))) return st;
            return fail(ctx, VKC_RUNTIME, "bucket key " + std::to_string(v) + " out of range for " +
                                              std::to_string(nb) + " buckets");
        }
    }
    out->kind = VKC_VALUE_ARRAY;
    out->array = o;
    return VKC_OK;
}

// index.rs:138-155 (Histogram).
static vkc_status histogram(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
    int64_t nb;
    if (!array_arg(ctx, args[0], VKC_I64, &st) || !i64_arg(ctx, args[1], &nb, &st)) return st;
    return run_buckets(ctx, args[0].array, nullptr, nb, out);
}

// index.rs:194-222 (ReduceInto with ScanSum<i64>): values kinds first, then checked_keys.
static vkc_status reduce_into_add(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 3) return fail(ctx, VKC_RUNTIME, arity_error(3, nargs));
    if (!array_arg(ctx, args[1], VKC_I64, &st)) return st;
    int64_t nb;
    if (!array_arg(ctx, args[0], VKC_I64, &st) || !i64_arg(ctx, args[2], &nb, &st)) return st;
    return run_buckets(ctx, args[0].array, args[1].array, nb, out);
}

void register_index(std::vector<KernelDef> &t) {
    struct G { vkc_type t; WholeFn f; };
    const G gs[] = {{VKC_F64, gather<VKC_F64>}, {VKC_F32, gather<VKC_F32>}, {VKC_I64, gather<VKC_I64>},
                    {VKC_U64, gather<VKC_U64>}, {VKC_I32, gather<VKC_I32>}, {VKC_U8, gather<VKC_U8>},
                    {VKC_BOOL, gather<VKC_BOOL>}};
    for (const G &g : gs) {
        // index.rs:255-270: cost 8 + 2 widths.
        KernelDef d{std::string("gather_") + type_name(g.t), VKC_WHOLE,
                    {InSpec{IN_ARRAY, g.t}, InSpec{IN_ARRAY, VKC_I64}}, true, g.t,
                    static_cast<uint64_t>(8 + 2 * type_width(g.t))};
        d.whole = g.f;
        t.push_back(d);
    }
    InSpec ia{IN_ARRAY, VKC_I64}, is{IN_SCALAR, VKC_I64};
    KernelDef d{"histogram", VKC_WHOLE, {ia, is}, true, VKC_I64, 24};
    d.whole = histogram;
    t.push_back(d);
    d = KernelDef{"reduce_into_add_i64", VKC_WHOLE, {ia, ia, is}, true, VKC_I64, 32};
    d.whole = reduce_into_add;
    t.push_back(d);
}

}  // namespace vkc

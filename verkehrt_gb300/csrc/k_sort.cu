// argsort_i64: the stable ascending positions of the rows (src/kernels/scalar/index.rs:159-173,
// src/kernels/scalar/index/radix.rs:126-259).
//
// LSD radix sort over the 8-bit digits of the sign-flipped image (radix.rs:58-61) of
// (key, position) pairs, as the reference does, restated for the GPU:
//  * one histogram kernel counts all 8 digits in one read (radix.rs:199-202);
//  * a digit that is equal in every row leaves the order unchanged and its pass is skipped
//    (radix.rs:203-211);
//  * each remaining digit is one reduce-then-scan pass over tiles of 256 x radix_items rows (the
//    autotuner's table: 2048, 3072 or 4096 rows by size): `up` counts each
//    tile's digits into a digit-major table, one exclusive scan of that table gives every
//    (digit, tile) its first output row, and `down` ranks the tile's rows stably by digit
//    (a ballot per digit bit, in row order) and scatters them. The first pass reads the keys, the
//    last writes the positions as i64. (A single-pass lookback per digit was slower here: the
//    lookback of 256 digits per tile advances a few tiles per L2 round trip. A persistent
//    `down` whose next tile arrives by TMA while it ranks the current one was no faster
//    either: the pass is bound by instruction issue, about 3.8 warp instructions per row.)
// Stability makes the output the reference's; inputs of at most 2048 rows are sorted in one
// block by comparison (as the reference does below 1024 rows, radix.rs:140-151), inputs of at
// most 8192 rows by the same radix passes inside one block.
#include <algorithm>

#include "lookback.cuh"
#include "reduce_common.h"

namespace vkc {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RADIX = 256;

// Rows per thread of a pass (the autotuner's radix_items: 8, 12 or 16; even, as ranks are
// packed in pairs), the tile, and the resident blocks per SM that the down kernel's registers
// allow (the best of a sweep over 3-6 per shape).
template <int ITEMS> struct RsShape {
    static_assert(ITEMS % 2 == 0, "ranks are packed two per word");
    static constexpr int TILE = RS_THREADS * ITEMS;
    static constexpr int MIN_BLOCKS = ITEMS >= 16 ? 3 : (ITEMS >= 12 ? 4 : 5);
    // Dynamic shared memory of the down kernel: the tile's images and positions sorted by digit.
    static constexpr size_t DOWN_SMEM = (sizeof(unsigned long long) + sizeof(unsigned)) * TILE;
};
constexpr int RS_MIN_TILE = RS_THREADS * 8;

__device__ __forceinline__ unsigned long long image_of(long long k) {
    return static_cast<unsigned long long>(k) ^ 0x8000000000000000ull;
}

// Counts every digit of every row into hist[8][256]. (One atomic per warp for a digit all 32
// rows share, found by warp votes, was slower: shared-memory atomics on one address are cheap
// here, the votes are not.)
__global__ void __launch_bounds__(256) rs_hist_kernel(const long long *__restrict__ keys, int64_t n,
                                                      unsigned *__restrict__ hist) {
    __shared__ unsigned h[8][RADIX];
    for (int i = threadIdx.x; i < 8 * RADIX; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    // Eight rows a thread per loop pass, all loaded before the first atomic (the atomics keep the
    // program's order, so a load after one would wait for it).
    constexpr int R = 8;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i0 = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i0 < n; i0 += R * stride) {
        unsigned long long k[R];
#pragma unroll
        for (int j = 0; j < R; ++j) k[j] = i0 + j * stride < n ? image_of(__ldcs(keys + i0 + j * stride)) : 0ull;
#pragma unroll
        for (int j = 0; j < R; ++j)
            if (i0 + j * stride < n)
#pragma unroll
                for (int p = 0; p < 8; ++p) atomicAdd(&h[p][(k[j] >> (8 * p)) & 0xff], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 8 * RADIX; i += blockDim.x) {
        unsigned v = (&h[0][0])[i];
        if (v) atomicAdd(hist + i, v);
    }
}

// Up: the digit counts of every tile, digit-major: counts[d * tiles + tile]. Shared-memory
// atomics into one histogram per warp (the order of the increments does not matter here).
template <int RS_ITEMS, bool FIRST, class IMG>
__global__ void __launch_bounds__(RS_THREADS) rs_up_kernel(const long long *__restrict__ keys_in,
                                                           const IMG *__restrict__ img_in, int64_t n,
                                                           int shift, int tiles, unsigned *__restrict__ counts) {
    constexpr int RS_TILE = RsShape<RS_ITEMS>::TILE;
    __shared__ unsigned s_cnt[RS_WARPS][RADIX];
    const int tile = blockIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < RS_WARPS * RADIX; i += RS_THREADS) (&s_cnt[0][0])[i] = 0;
    __syncthreads();
    const int64_t base = static_cast<int64_t>(tile) * RS_TILE + static_cast<int64_t>(w) * (32 * RS_ITEMS);
    if (base + 32 * RS_ITEMS <= n) {
        IMG img[RS_ITEMS];
#pragma unroll
        for (int j = 0; j < RS_ITEMS; ++j) {
            const int64_t r = base + j * 32 + lane;
            img[j] = FIRST ? static_cast<IMG>(image_of(__ldcs(keys_in + r))) : __ldcs(img_in + r);
        }
#pragma unroll
        for (int j = 0; j < RS_ITEMS; ++j) atomicAdd(&s_cnt[w][static_cast<unsigned>(img[j] >> shift) & 0xffu], 1u);
    } else {
        for (int j = 0; j < RS_ITEMS; ++j) {
            const int64_t r = base + j * 32 + lane;
            if (r < n) {
                const IMG im = FIRST ? static_cast<IMG>(image_of(__ldcs(keys_in + r))) : __ldcs(img_in + r);
                atomicAdd(&s_cnt[w][static_cast<unsigned>(im >> shift) & 0xffu], 1u);
            }
        }
    }
    __syncthreads();
    const int d = threadIdx.x;  // RS_THREADS == RADIX
    unsigned total = 0;
#pragma unroll
    for (int ww = 0; ww < RS_WARPS; ++ww) total += s_cnt[ww][d];
    counts[static_cast<int64_t>(d) * tiles + tile] = total;
}

// The lanes of the warp whose 8-bit digit equals this lane's, among the lanes of `valid`: one
// ballot per digit bit, each lane keeping the lanes that agree with it on that bit.
__device__ __forceinline__ unsigned digit_peers(unsigned d, unsigned valid) {
    unsigned m = valid;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const unsigned bit = (d >> b) & 1u;
        const unsigned v = __ballot_sync(FULL, bit);
        m &= ~(v ^ (0u - bit));  // keep the lanes whose bit b equals this lane's
    }
    return m;
}

// Exclusive scan of `m` u32 counts (n < 2^32, so sums fit) in SCAN_CHUNK-element blocks:
// block sums, one block scanning the sums, then each block scanning its chunk from its base.
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;

__global__ void __launch_bounds__(SCAN_THREADS) rs_scan_sums(const unsigned *__restrict__ c, int64_t m,
                                                              unsigned *__restrict__ sums) {
    const int64_t b0 = static_cast<int64_t>(blockIdx.x) * SCAN_CHUNK;
    unsigned t = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        const int64_t i = b0 + j * SCAN_THREADS + threadIdx.x;
        if (i < m) t += c[i];
    }
    unsigned total;
    block_exclusive_sum<unsigned>(t, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// One block: exclusive scan of `k` block sums in place.
__global__ void __launch_bounds__(1024) rs_scan_top(unsigned *sums, int k) {
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < k; b0 += 1024) {
        const int i = b0 + threadIdx.x;
        const unsigned v = i < k ? sums[i] : 0u;
        unsigned total;
        const unsigned ex = block_exclusive_sum<unsigned>(v, &total);
        if (i < k) sums[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) rs_scan_apply(const unsigned *__restrict__ c, int64_t m,
                                                               const unsigned *__restrict__ sums,
                                                               unsigned *__restrict__ out) {
    // Thread t holds the chunk's rows t*SCAN_ITEMS .. +SCAN_ITEMS-1 (contiguous), so a block
    // exclusive sum of the thread totals orders them.
    const int64_t b0 = static_cast<int64_t>(blockIdx.x) * SCAN_CHUNK + static_cast<int64_t>(threadIdx.x) * SCAN_ITEMS;
    unsigned v[SCAN_ITEMS], t = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        v[j] = b0 + j < m ? c[b0 + j] : 0u;
        t += v[j];
    }
    unsigned total;
    unsigned run = sums[blockIdx.x] + block_exclusive_sum<unsigned>(t, &total);
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        if (b0 + j < m) out[b0 + j] = run;
        run += v[j];
    }
}

// Exclusive scan of m u32 counts into out, with sum_words(m) words of scratch in `sums`
// (used by the partitioned gather as well as the passes below).
int64_t scan_counts_sum_words(int64_t m) { return (m + SCAN_CHUNK - 1) / SCAN_CHUNK; }
void scan_counts(vkc_ctx *ctx, const unsigned *c, int64_t m, unsigned *sums, unsigned *out) {
    const int chunks = static_cast<int>(scan_counts_sum_words(m));
    rs_scan_sums<<<chunks, SCAN_THREADS, 0, ctx->stream>>>(c, m, sums);
    rs_scan_top<<<1, 1024, 0, ctx->stream>>>(sums, chunks);
    rs_scan_apply<<<chunks, SCAN_THREADS, 0, ctx->stream>>>(c, m, sums, out);
}

// Down: one pass over digit `shift` with the tile's first output row per digit in
// offsets[d * tiles + tile]. FIRST reads the i64 keys (positions are the row numbers); LAST
// writes only the positions, as i64. IMG is the key image carried between passes: 64 bits, or
// its low 32 bits when every active digit lies there.
// The body of a down tile; WHOLE when every row of the tile is below n (all but the last
// tile), which drops the per-row bounds checks.
template <int RS_ITEMS, bool FIRST, bool LAST, class IMG, bool WHOLE>
__device__ __forceinline__ void rs_down_tile(const long long *__restrict__ keys_in, const IMG *__restrict__ img_in,
                                             const unsigned *__restrict__ pos_in, IMG *__restrict__ img_out,
                                             unsigned *__restrict__ pos_out, long long *__restrict__ out, int64_t n,
                                             int shift, int tile, unsigned short (*s_wcnt)[RADIX],
                                             unsigned *s_tile_excl, unsigned *s_dstart, unsigned char *smem) {
    constexpr int RS_TILE = RsShape<RS_ITEMS>::TILE;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // Rows of this warp: warp-striped, row = base + j*32 + lane, so (j, lane) is row order.
    const int64_t base = static_cast<int64_t>(tile) * RS_TILE + static_cast<int64_t>(w) * (32 * RS_ITEMS);
    IMG img[RS_ITEMS];
    unsigned pos[RS_ITEMS];
    unsigned rank2[RS_ITEMS / 2];  // two 16-bit ranks per word
    const unsigned lt = (1u << lane) - 1;
#pragma unroll
    for (int j = 0; j < RS_ITEMS; ++j) {
        const int64_t r = base + j * 32 + lane;
        const bool in = WHOLE || r < n;
        if (FIRST) {
            img[j] = in ? static_cast<IMG>(image_of(__ldcs(keys_in + r))) : static_cast<IMG>(~0ull);
            pos[j] = 0u;  // the row number, recomputed when stored
        } else {
            img[j] = in ? __ldcs(img_in + r) : static_cast<IMG>(~0ull);
            pos[j] = in ? __ldcs(pos_in + r) : 0u;
        }
    }
#pragma unroll
    for (int j = 0; j < RS_ITEMS; ++j) {
        const bool in = WHOLE || base + j * 32 + lane < n;
        const unsigned d = static_cast<unsigned>(img[j] >> shift) & 0xffu;
        // Rank among this warp's earlier rows with the same digit.
        const unsigned peers = digit_peers(d, WHOLE ? FULL : __ballot_sync(FULL, in));
        const unsigned short before = s_wcnt[w][d];
        __syncwarp();
        if (in) {
            const unsigned rk = before + __popc(peers & lt);
            rank2[j / 2] = (j & 1) ? (rank2[j / 2] | (rk << 16)) : rk;
            if ((peers & lt) == 0) s_wcnt[w][d] = static_cast<unsigned short>(before + __popc(peers));
        }
        __syncwarp();
    }
    __syncthreads();
    // Per digit: exclusive offsets of the warps within the digit, and the digit's first row in
    // the tile sorted by digit.
    {
        const int d = threadIdx.x;
        unsigned total = 0;
#pragma unroll
        for (int ww = 0; ww < RS_WARPS; ++ww) {
            const unsigned c = s_wcnt[ww][d];
            s_wcnt[ww][d] = static_cast<unsigned short>(total);
            total += c;
        }
        unsigned tile_total;
        const unsigned start = block_exclusive_sum<unsigned>(total, &tile_total);
        s_dstart[d] = start;
        s_tile_excl[d] -= start;  // from here: the output row of sorted-tile row l is s_tile_excl[d] + l
    }
    __syncthreads();
    // The tile sorted by digit (stable) in shared memory, then written out with consecutive
    // threads on consecutive rows of each digit's run, so the stores coalesce.
    IMG *s_img = reinterpret_cast<IMG *>(smem);
    unsigned *s_pos = reinterpret_cast<unsigned *>(smem + sizeof(IMG) * RS_TILE);
#pragma unroll
    for (int j = 0; j < RS_ITEMS; ++j) {
        if (WHOLE || base + j * 32 + lane < n) {
            const unsigned d = static_cast<unsigned>(img[j] >> shift) & 0xffu;
            const unsigned l = s_dstart[d] + s_wcnt[w][d] + ((rank2[j / 2] >> (16 * (j & 1))) & 0xffffu);
            s_img[l] = img[j];
            s_pos[l] = FIRST ? static_cast<unsigned>(base + j * 32 + lane) : pos[j];
        }
    }
    __syncthreads();
    auto put = [&](int l) {
        const IMG im = s_img[l];
        const unsigned d = static_cast<unsigned>(im >> shift) & 0xffu;
        const unsigned dst = s_tile_excl[d] + static_cast<unsigned>(l);
        if (LAST) {
            out[dst] = static_cast<long long>(s_pos[l]);
        } else {
            img_out[dst] = im;
            pos_out[dst] = s_pos[l];
        }
    };
    if (WHOLE) {
#pragma unroll
        for (int i = 0; i < RS_ITEMS; ++i) put(static_cast<int>(threadIdx.x) + i * RS_THREADS);
    } else {
        const int rows = static_cast<int>(n - static_cast<int64_t>(tile) * RS_TILE);
        for (int l = threadIdx.x; l < rows; l += RS_THREADS) put(l);
    }
}

template <int RS_ITEMS, bool FIRST, bool LAST, class IMG>
__global__ void __launch_bounds__(RS_THREADS, RsShape<RS_ITEMS>::MIN_BLOCKS) rs_down_kernel(
    const long long *__restrict__ keys_in, const IMG *__restrict__ img_in,
    const unsigned *__restrict__ pos_in, IMG *__restrict__ img_out,
    unsigned *__restrict__ pos_out, long long *__restrict__ out, int64_t n, int shift, int tiles,
    const unsigned *__restrict__ offsets) {
    constexpr int RS_TILE = RsShape<RS_ITEMS>::TILE;
    __shared__ unsigned short s_wcnt[RS_WARPS][RADIX];  // per-warp digit counts, then offsets
    __shared__ unsigned s_tile_excl[RADIX];             // the digit's first output row
    __shared__ unsigned s_dstart[RADIX];                // the digit's first row in the sorted tile
    extern __shared__ __align__(16) unsigned char rs_smem[];
    const int tile = blockIdx.x;
    for (int i = threadIdx.x; i < RS_WARPS * RADIX; i += RS_THREADS) (&s_wcnt[0][0])[i] = 0;
    s_tile_excl[threadIdx.x] = offsets[static_cast<int64_t>(threadIdx.x) * tiles + tile];  // RS_THREADS == RADIX
    __syncthreads();
    if (static_cast<int64_t>(tile + 1) * RS_TILE <= n)
        rs_down_tile<RS_ITEMS, FIRST, LAST, IMG, true>(keys_in, img_in, pos_in, img_out, pos_out, out, n, shift, tile,
                                                       s_wcnt, s_tile_excl, s_dstart, rs_smem);
    else
        rs_down_tile<RS_ITEMS, FIRST, LAST, IMG, false>(keys_in, img_in, pos_in, img_out, pos_out, out, n, shift, tile,
                                                        s_wcnt, s_tile_excl, s_dstart, rs_smem);
}

// Launches of one pass's kernels for the tuned shape.
template <bool FIRST, class IMG>
static void launch_up(vkc_ctx *ctx, int items, int tiles, const long long *keys, const IMG *img, int64_t n, int shift,
                      unsigned *counts) {
    switch (items) {
    case 8: rs_up_kernel<8, FIRST, IMG><<<tiles, RS_THREADS, 0, ctx->stream>>>(keys, img, n, shift, tiles, counts); break;
    case 16: rs_up_kernel<16, FIRST, IMG><<<tiles, RS_THREADS, 0, ctx->stream>>>(keys, img, n, shift, tiles, counts); break;
    default: rs_up_kernel<12, FIRST, IMG><<<tiles, RS_THREADS, 0, ctx->stream>>>(keys, img, n, shift, tiles, counts); break;
    }
}

template <int ITEMS, bool FIRST, bool LAST, class IMG> static void set_down_smem() {
    cudaFuncSetAttribute(rs_down_kernel<ITEMS, FIRST, LAST, IMG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(RsShape<ITEMS>::DOWN_SMEM));
}

template <bool FIRST, bool LAST, class IMG>
static void launch_down(vkc_ctx *ctx, int items, int tiles, const long long *keys, const IMG *img_in,
                        const unsigned *pos_in, IMG *img_out, unsigned *pos_out, long long *out, int64_t n, int shift,
                        const unsigned *offs) {
    static std::atomic<unsigned long long> configured{0};
    once_per_device(configured, ctx->device, [] {
        set_down_smem<8, FIRST, LAST, IMG>();
        set_down_smem<12, FIRST, LAST, IMG>();
        set_down_smem<16, FIRST, LAST, IMG>();
    });
#define RS_DOWN(I)                                                                                             \
    rs_down_kernel<I, FIRST, LAST, IMG><<<tiles, RS_THREADS, (sizeof(IMG) + sizeof(unsigned)) * RsShape<I>::TILE, \
                                          ctx->stream>>>(keys, img_in, pos_in, img_out, pos_out, out, n, shift, tiles, offs)
    switch (items) {
    case 8: RS_DOWN(8); break;
    case 16: RS_DOWN(16); break;
    default: RS_DOWN(12); break;
    }
#undef RS_DOWN
}

__global__ void rs_iota_kernel(long long *out, int64_t n) {
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) out[i] = i;
}

// Short inputs (the reference sorts up to 1024 rows by comparison, radix.rs:140-151): one
// block sorts (image, position) pairs in shared memory with a bitonic network. The pairs are
// distinct, so the order is total and the result is the stable order; padding pairs (all-ones
// image, position >= n) sort after every row.
constexpr int SMALL_SORT = 2048;

__global__ void __launch_bounds__(1024) small_argsort_kernel(const long long *__restrict__ keys, int n,
                                                              long long *__restrict__ out) {
    __shared__ unsigned long long s_img[SMALL_SORT];
    __shared__ unsigned s_pos[SMALL_SORT];
    int p = 1;
    while (p < n) p <<= 1;
    for (int i = threadIdx.x; i < p; i += blockDim.x) {
        s_img[i] = i < n ? image_of(keys[i]) : ~0ull;
        s_pos[i] = static_cast<unsigned>(i);
    }
    __syncthreads();
    for (int k = 2; k <= p; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < p; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const unsigned long long a = s_img[i], b = s_img[l];
                    const unsigned pa = s_pos[i], pb = s_pos[l];
                    const bool greater = a > b || (a == b && pa > pb);
                    if (greater == ((i & k) == 0)) {
                        s_img[i] = b;
                        s_img[l] = a;
                        s_pos[i] = pb;
                        s_pos[l] = pa;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = static_cast<long long>(s_pos[i]);
}

// Inputs of at most MID_SORT rows: one block of 1024 threads sorts (image, position) pairs in
// shared memory by the LSD passes of the active digits (the digits not equal in every row,
// found by a block-wide AND and OR of the images), each pass ranked stably as the down pass
// does (per warp, a ballot per digit bit; warp w holds rows 256w .. 256w + 255), one launch and
// no host synchronisation.
constexpr int MID_SORT = 8192;
constexpr int MID_THREADS = 1024, MID_ITEMS = MID_SORT / MID_THREADS, MID_WARPS = MID_THREADS / 32;
struct MidSmem {
    unsigned long long img[2][MID_SORT];
    unsigned short pos[2][MID_SORT];
    unsigned short wcnt[MID_WARPS][RADIX];  // per-warp digit counts, then offsets within the digit
    unsigned dstart[RADIX];                 // the digit's first row
    unsigned long long all_and[MID_WARPS], all_or[MID_WARPS];
};

__global__ void __launch_bounds__(MID_THREADS) mid_argsort_kernel(const long long *__restrict__ keys, int n,
                                                                   long long *__restrict__ out) {
    extern __shared__ __align__(16) unsigned char mid_smem[];
    MidSmem &sm = *reinterpret_cast<MidSmem *>(mid_smem);
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    unsigned long long a = ~0ull, o = 0;
    for (int i = t; i < n; i += MID_THREADS) {
        const unsigned long long im = image_of(keys[i]);
        sm.img[0][i] = im;
        sm.pos[0][i] = static_cast<unsigned short>(i);
        a &= im;
        o |= im;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        a &= __shfl_xor_sync(FULL, a, off);
        o |= __shfl_xor_sync(FULL, o, off);
    }
    if (lane == 0) {
        sm.all_and[w] = a;
        sm.all_or[w] = o;
    }
    __syncthreads();
    a = ~0ull;
    o = 0;
#pragma unroll 4
    for (int k = 0; k < MID_WARPS; ++k) {
        a &= sm.all_and[k];
        o |= sm.all_or[k];
    }
    const unsigned long long varies = a ^ o;  // bits that differ between rows
    int cur = 0;
    const unsigned lt = (1u << lane) - 1;
    for (int shift = 0; shift < 64; shift += 8) {
        if (((varies >> shift) & 0xffu) == 0) continue;  // a constant digit leaves the order as it is
        for (int i = t; i < MID_WARPS * RADIX; i += MID_THREADS) (&sm.wcnt[0][0])[i] = 0;
        __syncthreads();
        unsigned long long img[MID_ITEMS];
        unsigned short pos[MID_ITEMS];
        unsigned rank2[MID_ITEMS / 2];
        const int base = w * (32 * MID_ITEMS);
#pragma unroll
        for (int j = 0; j < MID_ITEMS; ++j) {
            const int r = base + j * 32 + lane;
            img[j] = r < n ? sm.img[cur][r] : ~0ull;
            pos[j] = r < n ? sm.pos[cur][r] : 0;
        }
#pragma unroll
        for (int j = 0; j < MID_ITEMS; ++j) {
            const bool in = base + j * 32 + lane < n;
            const unsigned d = static_cast<unsigned>(img[j] >> shift) & 0xffu;
            const unsigned peers = digit_peers(d, __ballot_sync(FULL, in));
            const unsigned short before = sm.wcnt[w][d];
            __syncwarp();
            if (in) {
                const unsigned rk = before + __popc(peers & lt);
                rank2[j / 2] = (j & 1) ? (rank2[j / 2] | (rk << 16)) : rk;
                if ((peers & lt) == 0) sm.wcnt[w][d] = static_cast<unsigned short>(before + __popc(peers));
            }
            __syncwarp();
        }
        __syncthreads();
        // Per digit: the warps' offsets within it (threads 0..255), then the digits' first rows
        // (warp 0, eight digits a lane).
        unsigned total = 0;
        if (t < RADIX) {
#pragma unroll 4
            for (int ww = 0; ww < MID_WARPS; ++ww) {
                const unsigned c = sm.wcnt[ww][t];
                sm.wcnt[ww][t] = static_cast<unsigned short>(total);
                total += c;
            }
            sm.dstart[t] = total;
        }
        __syncthreads();
        if (t < 32) {
            unsigned v[8], run = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                v[k] = sm.dstart[8 * t + k];
                run += v[k];
            }
            unsigned x = run;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned y = __shfl_up_sync(FULL, x, off);
                if (lane >= off) x += y;
            }
            unsigned ex = x - run;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                sm.dstart[8 * t + k] = ex;
                ex += v[k];
            }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < MID_ITEMS; ++j) {
            if (base + j * 32 + lane < n) {
                const unsigned d = static_cast<unsigned>(img[j] >> shift) & 0xffu;
                const unsigned l = sm.dstart[d] + sm.wcnt[w][d] + ((rank2[j / 2] >> (16 * (j & 1))) & 0xffffu);
                sm.img[cur ^ 1][l] = img[j];
                sm.pos[cur ^ 1][l] = pos[j];
            }
        }
        __syncthreads();
        cur ^= 1;
    }
    for (int i = t; i < n; i += MID_THREADS) out[i] = static_cast<long long>(sm.pos[cur][i]);
}

// The active-digit passes of argsort over (image, position) ping-pong buffers of image type IMG.
template <class IMG>
static vkc_status radix_argsort_passes(vkc_ctx *ctx, int items, int tiles, int64_t m, int chunks, const long long *keys,
                                       void *const img_v[2], unsigned *const pos[2], unsigned *counts, unsigned *offs,
                                       unsigned *sums, long long *oo, int64_t n, const int *active, int passes) {
    IMG *img[2] = {static_cast<IMG *>(img_v[0]), static_cast<IMG *>(img_v[1])};
    int cur = 0;
    for (int a = 0; a < passes; ++a) {
        const bool fst = a == 0, lst = a == passes - 1;
        const int shift = 8 * active[a];
        const int src = cur, dst = passes > 2 ? 1 - cur : 0;
        if (fst) launch_up<true, IMG>(ctx, items, tiles, keys, nullptr, n, shift, counts);
        else launch_up<false, IMG>(ctx, items, tiles, nullptr, img[src], n, shift, counts);
        rs_scan_sums<<<chunks, SCAN_THREADS, 0, ctx->stream>>>(counts, m, sums);
        rs_scan_top<<<1, 1024, 0, ctx->stream>>>(sums, chunks);
        rs_scan_apply<<<chunks, SCAN_THREADS, 0, ctx->stream>>>(counts, m, sums, offs);
        if (fst && lst)
            launch_down<true, true, IMG>(ctx, items, tiles, keys, nullptr, nullptr, nullptr, nullptr, oo, n, shift, offs);
        else if (fst)
            launch_down<true, false, IMG>(ctx, items, tiles, keys, nullptr, nullptr, img[0], pos[0], nullptr, n, shift, offs);
        else if (lst)
            launch_down<false, true, IMG>(ctx, items, tiles, nullptr, img[src], pos[src], nullptr, nullptr, oo, n, shift, offs);
        else
            launch_down<false, false, IMG>(ctx, items, tiles, nullptr, img[src], pos[src], img[dst], pos[dst], nullptr, n,
                                           shift, offs);
        vkc_status st = launched(ctx, "rs_pass");
        if (st) return st;
        if (fst) cur = 0;
        else if (!lst) cur = dst;
    }
    return VKC_OK;
}

// index.rs:159-173 (ArgSort::run).
static vkc_status argsort_i64(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 1) return fail(ctx, VKC_RUNTIME, arity_error(1, nargs));
    if (!array_arg(ctx, args[0], VKC_I64, &st)) return st;
    const vkc_array *xs = args[0].array;
    int64_t n = xs->len;
    if (n >= (int64_t(1) << 32))
        return fail(ctx, VKC_USAGE, "argsort of " + std::to_string(n) + " rows: at most 2^32 - 1 rows per call");
    vkc_array *o;
    if ((st = new_array(ctx, VKC_I64, n, false, &o))) return st;
    auto release = [&](vkc_status s) {
        vkc_array_release(o);
        return s;
    };
    if (n == 0) {
        out->kind = VKC_VALUE_ARRAY;
        out->array = o;
        return VKC_OK;
    }
    const auto *keys = static_cast<const long long *>(xs->data());
    if (n <= SMALL_SORT) {
        small_argsort_kernel<<<1, 1024, 0, ctx->stream>>>(keys, static_cast<int>(n), static_cast<long long *>(o->data()));
        if ((st = launched(ctx, "small_argsort"))) return release(st);
        out->kind = VKC_VALUE_ARRAY;
        out->array = o;
        return VKC_OK;
    }
    if (n <= MID_SORT) {
        static std::atomic<unsigned long long> configured{0};
        once_per_device(configured, ctx->device, [] {
            cudaFuncSetAttribute(mid_argsort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(sizeof(MidSmem)));
        });
        mid_argsort_kernel<<<1, MID_THREADS, sizeof(MidSmem), ctx->stream>>>(keys, static_cast<int>(n),
                                                                              static_cast<long long *>(o->data()));
        if ((st = launched(ctx, "mid_argsort"))) return release(st);
        out->kind = VKC_VALUE_ARRAY;
        out->array = o;
        return VKC_OK;
    }
    // Histogram of every digit.
    void *p;
    if ((st = scratch(ctx, 8 * RADIX * sizeof(unsigned), &p))) return release(st);
    auto *hist = static_cast<unsigned *>(p);
    VKC_CUDA(ctx, cudaMemsetAsync(hist, 0, 8 * RADIX * sizeof(unsigned), ctx->stream));
    rs_hist_kernel<<<stream_grid(ctx, n, 256, 6, 16384), 256, 0, ctx->stream>>>(keys, n, hist);
    if ((st = launched(ctx, "rs_hist"))) return release(st);
    void *h;
    if ((st = pinned(ctx, 2 * 8 * RADIX * sizeof(unsigned) + 16, &h))) return release(st);
    auto *hh = static_cast<unsigned *>(h);
    auto *first = reinterpret_cast<long long *>(hh + 2 * 8 * RADIX);
    VKC_CUDA(ctx, cudaMemcpyAsync(hh, hist, 8 * RADIX * sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    VKC_CUDA(ctx, cudaMemcpyAsync(first, keys, 8, cudaMemcpyDeviceToHost, ctx->stream));
    VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // Active digits (radix.rs:203-211): a digit whose bucket of the first row holds every row.
    unsigned long long first_img = static_cast<unsigned long long>(*first) ^ 0x8000000000000000ull;
    int active[8], passes = 0;
    for (int pss = 0; pss < 8; ++pss) {
        unsigned fd = static_cast<unsigned>(first_img >> (8 * pss)) & 0xffu;
        if (hh[pss * RADIX + fd] != static_cast<unsigned>(n)) active[passes++] = pss;
    }
    auto *oo = static_cast<long long *>(o->data());
    if (passes == 0) {
        rs_iota_kernel<<<stream_grid(ctx, n, 256, 8, 2048), 256, 0, ctx->stream>>>(oo, n);
        if ((st = launched(ctx, "rs_iota"))) return release(st);
        out->kind = VKC_VALUE_ARRAY;
        out->array = o;
        return VKC_OK;
    }
    // Ping-pong buffers of (image, position), as radix.rs:224-232.
    vkc_array *ia = nullptr, *ib = nullptr, *pa = nullptr, *pb = nullptr, *ca = nullptr, *oa = nullptr,
              *sa = nullptr;
    auto cleanup = [&]() {
        for (vkc_array *a : {ia, ib, pa, pb, ca, oa, sa})
            if (a) vkc_array_release(a);
    };
    // When every active digit lies in the low 32 bits, rows with equal high halves differ only
    // there, so the passes carry the image's low 32 bits: 16 bytes a row per pass, not 24.
    const bool narrow = active[passes - 1] < 4;
    const vkc_type img_type = narrow ? VKC_I32 : VKC_U64;
    if (passes > 1) {
        if ((st = new_array(ctx, img_type, n, false, &ia)) || (st = new_array(ctx, VKC_I32, n, false, &pa))) {
            cleanup();
            return release(fail(ctx, VKC_ALLOC, "cannot allocate argsort scratch for " + std::to_string(n) + " rows"));
        }
        if (passes > 2 && ((st = new_array(ctx, img_type, n, false, &ib)) || (st = new_array(ctx, VKC_I32, n, false, &pb)))) {
            cleanup();
            return release(fail(ctx, VKC_ALLOC, "cannot allocate argsort scratch for " + std::to_string(n) + " rows"));
        }
    }
    // Digit-major tile counts, their exclusive scan, and the scan's block sums.
    const int items = tune(ctx, TK_RADIX_ITEMS, n);
    const int64_t tile_rows = static_cast<int64_t>(RS_THREADS) * items;
    const int tiles = static_cast<int>((n + tile_rows - 1) / tile_rows);
    const int64_t m = static_cast<int64_t>(RADIX) * tiles;
    const int chunks = static_cast<int>((m + SCAN_CHUNK - 1) / SCAN_CHUNK);
    if ((st = new_array(ctx, VKC_I32, m, false, &ca)) || (st = new_array(ctx, VKC_I32, m, false, &oa)) ||
        (st = new_array(ctx, VKC_I32, chunks, false, &sa))) {
        cleanup();
        return release(fail(ctx, VKC_ALLOC, "cannot allocate argsort scratch for " + std::to_string(n) + " rows"));
    }
    auto *counts = static_cast<unsigned *>(ca->data());
    auto *offs = static_cast<unsigned *>(oa->data());
    auto *sums = static_cast<unsigned *>(sa->data());
    void *img[2] = {ia ? ia->data() : nullptr, ib ? ib->data() : nullptr};
    unsigned *pos[2] = {pa ? static_cast<unsigned *>(pa->data()) : nullptr,
                        pb ? static_cast<unsigned *>(pb->data()) : nullptr};
    const vkc_status pst = narrow ? radix_argsort_passes<unsigned>(ctx, items, tiles, m, chunks, keys, img, pos, counts,
                                                                    offs, sums, oo, n, active, passes)
                                  : radix_argsort_passes<unsigned long long>(ctx, items, tiles, m, chunks, keys, img, pos,
                                                                             counts, offs, sums, oo, n, active, passes);
    if (pst) {
        cleanup();
        return release(pst);
    }
    DevStatus ds;
    st = read_status(ctx, &ds);
    cleanup();
    if (st) return release(st);
    out->kind = VKC_VALUE_ARRAY;
    out->array = o;
    return VKC_OK;
}

// Stable LSD passes over (image, position) pairs that are already in img[0] / pos[0], one per
// entry of `shifts`, ping-ponging between the two buffers; *which gets the buffer that holds
// the result. counts and offs hold radix_pairs_scratch's words and sums
// ceil(that / SCAN_CHUNK). Enqueue only: no host synchronisation and no allocation.
vkc_status radix_pairs(vkc_ctx *ctx, unsigned long long *img[2], unsigned *pos[2], int64_t n, const int *shifts,
                       int npasses, unsigned *counts, unsigned *offs, unsigned *sums, int *which) {
    vkc_status st;
    const int items = tune(ctx, TK_RADIX_ITEMS, n);
    const int64_t tile_rows = static_cast<int64_t>(RS_THREADS) * items;
    const int tiles = static_cast<int>((n + tile_rows - 1) / tile_rows);
    const int64_t m = static_cast<int64_t>(RADIX) * tiles;
    const int chunks = static_cast<int>((m + SCAN_CHUNK - 1) / SCAN_CHUNK);
    int cur = 0;
    for (int a = 0; a < npasses; ++a) {
        const int shift = shifts[a];
        launch_up<false, unsigned long long>(ctx, items, tiles, nullptr, img[cur], n, shift, counts);
        rs_scan_sums<<<chunks, SCAN_THREADS, 0, ctx->stream>>>(counts, m, sums);
        rs_scan_top<<<1, 1024, 0, ctx->stream>>>(sums, chunks);
        rs_scan_apply<<<chunks, SCAN_THREADS, 0, ctx->stream>>>(counts, m, sums, offs);
        launch_down<false, false, unsigned long long>(ctx, items, tiles, nullptr, img[cur], pos[cur], img[1 - cur], pos[1 - cur], nullptr, n,
                                  shift, offs);
        if ((st = launched(ctx, "radix_pairs"))) return st;
        cur = 1 - cur;
    }
    *which = cur;
    return VKC_OK;
}

// Words of the radix_pairs scratch for n rows: counts/offs each, and sums (for the smallest
// tile, so any tuned shape fits).
void radix_pairs_scratch(int64_t n, int64_t *count_words, int64_t *sum_words) {
    const int64_t tiles = (n + RS_MIN_TILE - 1) / RS_MIN_TILE;
    *count_words = static_cast<int64_t>(RADIX) * tiles;
    *sum_words = (*count_words + SCAN_CHUNK - 1) / SCAN_CHUNK;
}

void register_sort(std::vector<KernelDef> &t) {
    // index.rs:241-255: cost = key width + 8.
    KernelDef d{"argsort_i64", VKC_WHOLE, {InSpec{IN_ARRAY, VKC_I64}}, true, VKC_I64, 16};
    d.whole = argsort_i64;
    t.push_back(d);
}

}  // namespace vkc

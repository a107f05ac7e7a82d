// argsort_i64: the stable ascending positions of the rows (src/kernels/scalar/index.rs:159-173,
// src/kernels/scalar/index/radix.rs:126-259).
//
// LSD radix sort over the 8-bit digits of the sign-flipped image (radix.rs:58-61) of
// (key, position) pairs, as the reference does, restated for the GPU:
//  * one histogram kernel counts all 8 digits in one read (radix.rs:199-202);
//  * a digit that is equal in every row leaves the order unchanged and its pass is skipped
//    (radix.rs:203-211);
//  * each remaining digit is one "onesweep" pass: a 4096-row tile ranks its rows stably by
//    digit (warp match + ballot in row order), finds each digit's offset among the earlier
//    tiles with a decoupled lookback per digit, and scatters. The first pass reads the keys,
//    the last writes the positions as i64.
// Stability makes the output the reference's, which the comparison sort of short inputs
// (radix.rs:140-151) also gives, so one path serves every length.
#include <algorithm>

#include "lookback.cuh"
#include "reduce_common.h"

namespace vkc {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RADIX = 256;

__device__ __forceinline__ unsigned long long image_of(long long k) {
    return static_cast<unsigned long long>(k) ^ 0x8000000000000000ull;
}

// Counts every digit of every row into hist[8][256].
__global__ void __launch_bounds__(256) rs_hist_kernel(const long long *__restrict__ keys, int64_t n,
                                                      unsigned *__restrict__ hist) {
    __shared__ unsigned h[8][RADIX];
    for (int i = threadIdx.x; i < 8 * RADIX; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        unsigned long long k = image_of(__ldcs(keys + i));
#pragma unroll
        for (int p = 0; p < 8; ++p) atomicAdd(&h[p][(k >> (8 * p)) & 0xff], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 8 * RADIX; i += blockDim.x) {
        unsigned v = (&h[0][0])[i];
        if (v) atomicAdd(hist + i, v);
    }
}

// Lookback word of one (tile, digit): epoch << 34 | state << 32 | count (n < 2^32).
__device__ __forceinline__ unsigned long long rs_word(unsigned epoch, unsigned state, unsigned count) {
    return (static_cast<unsigned long long>(epoch) << 34) | (static_cast<unsigned long long>(state) << 32) | count;
}

// One pass over digit `shift`. FIRST reads the i64 keys (positions are the row numbers);
// LAST writes only the positions, as i64.
template <bool FIRST, bool LAST>
__global__ void __launch_bounds__(RS_THREADS) rs_pass_kernel(
    const long long *__restrict__ keys_in, const unsigned long long *__restrict__ img_in,
    const unsigned *__restrict__ pos_in, unsigned long long *__restrict__ img_out,
    unsigned *__restrict__ pos_out, long long *__restrict__ out, int64_t n, int shift,
    const unsigned *__restrict__ bucket_base, unsigned long long *status, int tiles, unsigned epoch,
    unsigned *counters, DevStatus *st) {
    __shared__ unsigned short s_wcnt[RS_WARPS][RADIX];  // per-warp digit counts, then offsets
    __shared__ unsigned s_tile_excl[RADIX];
    const int tile = take_ticket(counters);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < RS_WARPS * RADIX; i += RS_THREADS) (&s_wcnt[0][0])[i] = 0;
    __syncthreads();

    // Rows of this warp: warp-striped, row = base + j*32 + lane, so (j, lane) is row order.
    const int64_t base = static_cast<int64_t>(tile) * RS_TILE + static_cast<int64_t>(w) * (32 * RS_ITEMS);
    unsigned long long img[RS_ITEMS];
    unsigned pos[RS_ITEMS];
    unsigned short rank[RS_ITEMS];
    unsigned char dig[RS_ITEMS];
    const unsigned lt = (1u << lane) - 1;
#pragma unroll
    for (int j = 0; j < RS_ITEMS; ++j) {
        int64_t r = base + j * 32 + lane;
        bool in = r < n;
        if (FIRST) {
            img[j] = in ? image_of(__ldcs(keys_in + r)) : ~0ull;
            pos[j] = static_cast<unsigned>(r);
        } else {
            img[j] = in ? __ldcs(img_in + r) : ~0ull;
            pos[j] = in ? __ldcs(pos_in + r) : 0u;
        }
        unsigned d = static_cast<unsigned>(img[j] >> shift) & 0xffu;
        dig[j] = static_cast<unsigned char>(d);
        // Rank among this warp's earlier rows with the same digit.
        unsigned active = __ballot_sync(FULL, in);
        unsigned peers = __match_any_sync(FULL, in ? d : 0x100u + lane) & active;
        unsigned short before = s_wcnt[w][d];
        __syncwarp();
        if (in) {
            rank[j] = static_cast<unsigned short>(before + __popc(peers & lt));
            if ((peers & lt) == 0) s_wcnt[w][d] = static_cast<unsigned short>(before + __popc(peers));
        }
        __syncwarp();
    }
    __syncthreads();
    // Per digit: tile count, per-warp exclusive offsets, and the lookback over earlier tiles.
    {
        const int d = threadIdx.x;  // RS_THREADS == RADIX
        unsigned total = 0;
#pragma unroll
        for (int ww = 0; ww < RS_WARPS; ++ww) {
            unsigned c = s_wcnt[ww][d];
            s_wcnt[ww][d] = static_cast<unsigned short>(total);
            total += c;
        }
        unsigned long long *my = status + static_cast<int64_t>(tile) * RADIX + d;
        st_release64(my, rs_word(epoch, 1, total));
        unsigned excl = 0;
        for (int tp = tile - 1; tp >= 0; --tp) {
            unsigned long long v;
            unsigned it = 0;
            while (((v = ld_acquire64(status + static_cast<int64_t>(tp) * RADIX + d)) >> 34) != epoch) {
                if (++it > SPIN_LIMIT) {
                    set_timeout(st);
                    break;
                }
                backoff(it);
            }
            if ((v >> 34) != epoch) break;
            excl += static_cast<unsigned>(v);
            if (((v >> 32) & 3u) == 2u) break;
        }
        st_release64(my, rs_word(epoch, 2, excl + total));
        s_tile_excl[d] = bucket_base[d] + excl;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < RS_ITEMS; ++j) {
        int64_t r = base + j * 32 + lane;
        if (r < n) {
            unsigned d = dig[j];
            unsigned dst = s_tile_excl[d] + s_wcnt[w][d] + rank[j];
            if (LAST) {
                out[dst] = static_cast<long long>(pos[j]);
            } else {
                img_out[dst] = img[j];
                pos_out[dst] = pos[j];
            }
        }
    }
    release_ticket(counters, tiles);
}

__global__ void rs_iota_kernel(long long *out, int64_t n) {
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) out[i] = i;
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
    // Histogram of every digit.
    void *p;
    if ((st = scratch(ctx, 8 * RADIX * sizeof(unsigned) * 2, &p))) return release(st);
    auto *hist = static_cast<unsigned *>(p);
    auto *bases = hist + 8 * RADIX;
    VKC_CUDA(ctx, cudaMemsetAsync(hist, 0, 8 * RADIX * sizeof(unsigned), ctx->stream));
    rs_hist_kernel<<<stream_grid(ctx, n, 256, 4, 16384), 256, 0, ctx->stream>>>(keys, n, hist);
    if ((st = launched(ctx, "rs_hist"))) return release(st);
    void *h;
    if ((st = pinned(ctx, 2 * 8 * RADIX * sizeof(unsigned) + 16, &h))) return release(st);
    auto *hh = static_cast<unsigned *>(h);
    auto *first = reinterpret_cast<long long *>(hh + 2 * 8 * RADIX);
    VKC_CUDA(ctx, cudaMemcpyAsync(hh, hist, 8 * RADIX * sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    VKC_CUDA(ctx, cudaMemcpyAsync(first, keys, 8, cudaMemcpyDeviceToHost, ctx->stream));
    VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // Active digits (radix.rs:203-211) and each pass's exclusive bucket offsets.
    unsigned long long first_img = static_cast<unsigned long long>(*first) ^ 0x8000000000000000ull;
    int active[8], passes = 0;
    unsigned *hb = hh + 8 * RADIX;
    for (int pss = 0; pss < 8; ++pss) {
        unsigned fd = static_cast<unsigned>(first_img >> (8 * pss)) & 0xffu;
        if (hh[pss * RADIX + fd] != static_cast<unsigned>(n)) {
            unsigned sum = 0;
            for (int d = 0; d < RADIX; ++d) {
                hb[passes * RADIX + d] = sum;
                sum += hh[pss * RADIX + d];
            }
            active[passes++] = pss;
        }
    }
    auto *oo = static_cast<long long *>(o->data());
    if (passes == 0) {
        rs_iota_kernel<<<stream_grid(ctx, n, 256, 8, 2048), 256, 0, ctx->stream>>>(oo, n);
        if ((st = launched(ctx, "rs_iota"))) return release(st);
        out->kind = VKC_VALUE_ARRAY;
        out->array = o;
        return VKC_OK;
    }
    VKC_CUDA(ctx, cudaMemcpyAsync(bases, hb, static_cast<size_t>(passes) * RADIX * sizeof(unsigned),
                                  cudaMemcpyHostToDevice, ctx->stream));
    // Ping-pong buffers of (image, position), as radix.rs:224-232.
    vkc_array *ia = nullptr, *ib = nullptr, *pa = nullptr, *pb = nullptr;
    auto cleanup = [&]() {
        for (vkc_array *a : {ia, ib, pa, pb})
            if (a) vkc_array_release(a);
    };
    if (passes > 1) {
        if ((st = new_array(ctx, VKC_U64, n, false, &ia)) || (st = new_array(ctx, VKC_I32, n, false, &pa))) {
            cleanup();
            return release(fail(ctx, VKC_ALLOC, "cannot allocate argsort scratch for " + std::to_string(n) + " rows"));
        }
        if (passes > 2 && ((st = new_array(ctx, VKC_U64, n, false, &ib)) || (st = new_array(ctx, VKC_I32, n, false, &pb)))) {
            cleanup();
            return release(fail(ctx, VKC_ALLOC, "cannot allocate argsort scratch for " + std::to_string(n) + " rows"));
        }
    }
    int tiles = static_cast<int>((n + RS_TILE - 1) / RS_TILE);
    unsigned *flags;
    if ((st = flag_arena(ctx, static_cast<size_t>(tiles) * RADIX * 2, &flags))) {
        cleanup();
        return release(st);
    }
    auto *status = reinterpret_cast<unsigned long long *>(flags);
    unsigned long long *img[2] = {ia ? static_cast<unsigned long long *>(ia->data()) : nullptr,
                                  ib ? static_cast<unsigned long long *>(ib->data()) : nullptr};
    unsigned *pos[2] = {pa ? static_cast<unsigned *>(pa->data()) : nullptr,
                        pb ? static_cast<unsigned *>(pb->data()) : nullptr};
    int cur = 0;
    for (int a = 0; a < passes; ++a) {
        bool fst = a == 0, lst = a == passes - 1;
        int shift = 8 * active[a];
        unsigned epoch = next_epoch(ctx);
        const unsigned *bb = bases + a * RADIX;
        int src = cur, dst = passes > 2 ? 1 - cur : 0;
        if (fst && lst)
            rs_pass_kernel<true, true><<<tiles, RS_THREADS, 0, ctx->stream>>>(keys, nullptr, nullptr, nullptr, nullptr, oo, n, shift, bb, status, tiles, epoch, ctx->counters, ctx->status);
        else if (fst)
            rs_pass_kernel<true, false><<<tiles, RS_THREADS, 0, ctx->stream>>>(keys, nullptr, nullptr, img[0], pos[0], nullptr, n, shift, bb, status, tiles, epoch, ctx->counters, ctx->status);
        else if (lst)
            rs_pass_kernel<false, true><<<tiles, RS_THREADS, 0, ctx->stream>>>(nullptr, img[src], pos[src], nullptr, nullptr, oo, n, shift, bb, status, tiles, epoch, ctx->counters, ctx->status);
        else
            rs_pass_kernel<false, false><<<tiles, RS_THREADS, 0, ctx->stream>>>(nullptr, img[src], pos[src], img[dst], pos[dst], nullptr, n, shift, bb, status, tiles, epoch, ctx->counters, ctx->status);
        if ((st = launched(ctx, "rs_pass"))) {
            cleanup();
            return release(st);
        }
        if (fst) cur = 0;
        else if (!lst) cur = dst;
    }
    DevStatus ds;
    st = read_status(ctx, &ds);
    cleanup();
    if (st) return release(st);
    out->kind = VKC_VALUE_ARRAY;
    out->array = o;
    return VKC_OK;
}

void register_sort(std::vector<KernelDef> &t) {
    // index.rs:241-255: cost = key width + 8.
    KernelDef d{"argsort_i64", VKC_WHOLE, {InSpec{IN_ARRAY, VKC_I64}}, true, VKC_I64, 16};
    d.whole = argsort_i64;
    t.push_back(d);
}

}  // namespace vkc

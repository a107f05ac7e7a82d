// Batched execution of one planned statement over many arrays, and CUDA graphs of statement
// sequences: the device side of the reference executor's per-array loop (src/exec.rs:162-231,
// Strategy :77-91), which runs a statement once per array and so pays every kernel launch and
// host round trip once per array.
//
// A batch is a table of arrays in device memory (pointer, rows, first row in the batch's
// concatenation, index), ordered largest first so that the persistent kernels' tickets hand out
// the long arrays early. The batch entries only enqueue work on the context's stream: no host
// synchronisation, and no allocation once a batch's scratch exists, so a sequence of them can
// be captured in a CUDA graph (vkc_graph_begin / vkc_graph_end) and replayed.
//
//  * filter -> sum (vkc_batch_filter_sum_f64): one persistent kernel; a block takes an array,
//    counts its survivors, then compacts them in row order chunk by chunk and feeds them to the
//    reference's 16 lanes (lane j takes survivors j, j+16, ... below the last whole block of 16,
//    with IEEE adds in that order), combines the lanes +8, +4, +2, +1 and adds the tail
//    (src/kernels/scalar/reduce.rs:45-91): the bits of filter then reduce_add_f64.
//  * argsort (vkc_batch_argsort_i64): the keys of every array, as their sign-flipped images, are
//    copied into one run with their positions in the run; stable radix passes over the key
//    digits given (all eight when none are), then over the digits of the array index, sort the
//    run by (array, key); each array's positions are written to its output relative to its first
//    row. Stability makes every output the array's own argsort.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <type_traits>
#include <vector>

#include "lookback.cuh"
#include "reduce_common.h"

namespace vkc {

vkc_status radix_pairs(vkc_ctx *ctx, unsigned long long *img[2], unsigned *pos[2], int64_t n, const int *shifts,
                       int npasses, unsigned *counts, unsigned *offs, unsigned *sums, int *which);
void radix_pairs_scratch(int64_t n, int64_t *count_words, int64_t *sum_words);

struct BSeg {
    const void *ptr;
    int64_t n;
    int64_t base;   // first row of the array in the batch's concatenation (in index order)
    int64_t index;  // position of the array in the caller's list
};

}  // namespace vkc

struct vkc_batch {
    vkc_ctx *ctx = nullptr;
    vkc_type type = VKC_F64;
    std::vector<vkc_array *> arrays;  // retained, caller's order
    std::vector<vkc::BSeg> host;      // largest first
    int64_t total = 0;
    vkc::DeviceMem table;             // BSeg[n] on the device, largest first
    vkc::DeviceMem bases;             // int64 first rows [n + 1], index order (for the argsort)
    vkc::DeviceMem outs;              // argsort output pointers [n], index order
    vkc::DeviceMem chunks;            // int64 [n + 1]: first concat chunk of each array, table order
    // Argsort scratch, made on first use.
    std::vector<vkc_array *> scratch;
    unsigned long long *img[2] = {nullptr, nullptr};
    unsigned *pos[2] = {nullptr, nullptr};
    unsigned *counts = nullptr, *offs = nullptr, *sums = nullptr;
    const vkc_batch *out_batch = nullptr;  // the batch whose pointers `outs` holds
};

namespace vkc {

// ------------------------------------------------------------------ filter -> sum

constexpr int BF_THREADS = 256;
constexpr int BF_ROWS = 8;                        // rows per thread per chunk (contiguous)
constexpr int BF_CHUNK = BF_THREADS * BF_ROWS;    // 2048 rows

template <bool POS>
__global__ void __launch_bounds__(BF_THREADS) batch_filter_sum_kernel(const BSeg *__restrict__ segs, int nseg,
                                                                     CmpRange r, unsigned long long *sums,
                                                                     unsigned *ticket) {
    __shared__ double s_keep[BF_CHUNK];  // the chunk's survivors in row order
    __shared__ double s_tail[16];
    __shared__ int s_seg;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    for (;;) {
        if (t == 0) s_seg = static_cast<int>(atomicAdd(ticket, 1u));
        __syncthreads();
        const int sg = s_seg;
        if (sg >= nseg) break;
        const BSeg seg = segs[sg];
        const auto *x = static_cast<const unsigned long long *>(seg.ptr);
        // Survivors of the whole array.
        unsigned long long kc = 0;
        for (int64_t i = t; i < seg.n; i += BF_THREADS) kc += in_range_t<POS>(r, __ldg(x + i));
        unsigned long long k;
        block_exclusive_sum<unsigned long long>(kc, &k);
        const unsigned long long b = k - k % 16;  // survivors in whole blocks of 16
        double acc = 0.0;                         // lane t (t < 16) of the canonical order
        unsigned long long c0 = 0;                // survivors before the chunk
        for (int64_t r0 = 0; r0 < seg.n; r0 += BF_CHUNK) {
            const int64_t i0 = r0 + static_cast<int64_t>(t) * BF_ROWS;
            unsigned long long v[BF_ROWS];
            unsigned keep = 0;
#pragma unroll
            for (int j = 0; j < BF_ROWS; ++j) {
                v[j] = i0 + j < seg.n ? __ldg(x + i0 + j) : 0ull;
                if (i0 + j < seg.n && in_range_t<POS>(r, v[j])) keep |= 1u << j;
            }
            unsigned chunk;
            unsigned at = block_exclusive_sum<unsigned>(__popc(keep), &chunk);
#pragma unroll
            for (int j = 0; j < BF_ROWS; ++j)
                if ((keep >> j) & 1u) s_keep[at++] = __longlong_as_double(static_cast<long long>(v[j]));
            __syncthreads();
            if (t < 16) {
                // Lane t takes the chunk's survivors whose index in the array is t mod 16.
                unsigned idx = static_cast<unsigned>((16 + t - static_cast<int>(c0 % 16)) % 16);
                for (; idx < chunk && c0 + idx < b; idx += 16) acc = __dadd_rn(acc, s_keep[idx]);
            } else if (t == 32) {
                // Survivors at or past b are the tail, added to lane 0 at the end in order.
                for (unsigned idx = 0; idx < chunk; ++idx)
                    if (c0 + idx >= b) s_tail[c0 + idx - b] = s_keep[idx];
            }
            c0 += chunk;
            __syncthreads();
        }
        if (w == 0) {
            // +8, +4, +2, +1 (lane j adds lane j + step), then the tail into lane 0.
#pragma unroll
            for (int step = 8; step > 0; step >>= 1) {
                const double other = __shfl_down_sync(FULL, acc, step);
                if (lane < step) acc = __dadd_rn(acc, other);
            }
            if (lane == 0) {
                for (unsigned j = 0; j < k - b; ++j) acc = __dadd_rn(acc, s_tail[j]);
                sums[seg.index] = static_cast<unsigned long long>(__double_as_longlong(acc));
            }
        }
        __syncthreads();
    }
    // The last block resets the ticket for the next launch.
    __syncthreads();
    if (t == 0) {
        const unsigned prev = atomicAdd(ticket + 1, 1u);
        if (prev == gridDim.x - 1) {
            ticket[0] = 0;
            ticket[1] = 0;
        }
    }
}

// Counts of rows with x <cmp> c per array (length of filter), one block per array.
template <bool POS>
__global__ void __launch_bounds__(BF_THREADS) batch_count_kernel(const BSeg *__restrict__ segs, int nseg, CmpRange r,
                                                                long long *counts, unsigned *ticket) {
    __shared__ int s_seg;
    const int t = threadIdx.x;
    for (;;) {
        if (t == 0) s_seg = static_cast<int>(atomicAdd(ticket, 1u));
        __syncthreads();
        const int sg = s_seg;
        if (sg >= nseg) break;
        const BSeg seg = segs[sg];
        const auto *x = static_cast<const unsigned long long *>(seg.ptr);
        unsigned long long kc = 0;
        for (int64_t i = t; i < seg.n; i += BF_THREADS) kc += in_range_t<POS>(r, __ldg(x + i));
        unsigned long long k;
        block_exclusive_sum<unsigned long long>(kc, &k);
        if (t == 0) counts[seg.index] = static_cast<long long>(k);
        __syncthreads();
    }
    __syncthreads();
    if (t == 0) {
        const unsigned prev = atomicAdd(ticket + 1, 1u);
        if (prev == gridDim.x - 1) {
            ticket[0] = 0;
            ticket[1] = 0;
        }
    }
}

// dot_f64 per pair of arrays (x from xs, y from ys, same index and length), one block per pair:
// lane j (thread j < 16) adds fl(x*y) of rows j, j+16, ... below the last whole block of 16 in
// order, the lanes combine +8, +4, +2, +1, and the tail rows are added to lane 0 in order
// (src/kernels/scalar/fused.rs:73-106 with reduce.rs:45-91). The other threads stage the rows
// into shared memory ahead of the lanes. Meant for short arrays: a lane's chain is n/16 adds.
constexpr int BD_CHUNK = 4096;

__global__ void __launch_bounds__(BF_THREADS) batch_dot_kernel(const BSeg *__restrict__ xs, const BSeg *__restrict__ ys,
                                                              int nseg, unsigned long long *sums, unsigned *ticket) {
    __shared__ double s_p[BD_CHUNK];  // the chunk's products fl(x*y)
    __shared__ int s_seg;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    for (;;) {
        if (t == 0) s_seg = static_cast<int>(atomicAdd(ticket, 1u));
        __syncthreads();
        const int sg = s_seg;
        if (sg >= nseg) break;
        const BSeg sx = xs[sg];
        const BSeg sy = ys[sg];
        const auto *x = static_cast<const double *>(sx.ptr);
        const auto *y = static_cast<const double *>(sy.ptr);
        const int64_t n = sx.n, b = n - n % 16;
        double acc = 0.0;
        for (int64_t r0 = 0; r0 < n; r0 += BD_CHUNK) {
            const int rows = static_cast<int>(n - r0 < BD_CHUNK ? n - r0 : BD_CHUNK);
            for (int i = t; i < rows; i += BF_THREADS) s_p[i] = __dmul_rn(__ldg(x + r0 + i), __ldg(y + r0 + i));
            __syncthreads();
            if (t < 16) {
                // r0 is a multiple of 16, so row r0 + i belongs to lane i mod 16.
                for (int i = t; i < rows && r0 + i < b; i += 16) acc = __dadd_rn(acc, s_p[i]);
            }
            __syncthreads();
        }
        if (w == 0) {
#pragma unroll
            for (int step = 8; step > 0; step >>= 1) {
                const double other = __shfl_down_sync(FULL, acc, step);
                if (lane < step) acc = __dadd_rn(acc, other);
            }
            if (lane == 0) {
                for (int64_t i = b; i < n; ++i) acc = __dadd_rn(acc, __dmul_rn(__ldg(x + i), __ldg(y + i)));
                sums[sx.index] = static_cast<unsigned long long>(__double_as_longlong(acc));
            }
        }
        __syncthreads();
    }
    __syncthreads();
    if (t == 0) {
        const unsigned prev = atomicAdd(ticket + 1, 1u);
        if (prev == gridDim.x - 1) {
            ticket[0] = 0;
            ticket[1] = 0;
        }
    }
}

// ------------------------------------------------------------------ argsort

// Images and positions of every array, in index order (array i at rows bases[i]..).
__global__ void __launch_bounds__(256) batch_keys_kernel(const BSeg *__restrict__ segs, int nseg,
                                                         unsigned long long *__restrict__ img,
                                                         unsigned *__restrict__ pos) {
    for (int sg = blockIdx.y; sg < nseg; sg += gridDim.y) {
        const BSeg seg = segs[sg];
        const auto *k = static_cast<const long long *>(seg.ptr);
        for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < seg.n;
             i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
            img[seg.base + i] = static_cast<unsigned long long>(__ldg(k + i)) ^ 0x8000000000000000ull;
            pos[seg.base + i] = static_cast<unsigned>(seg.base + i);
        }
    }
}

// Replaces every image by the index of the array its position belongs to (bases[nseg] = total).
__global__ void __launch_bounds__(256) batch_owner_kernel(const int64_t *__restrict__ bases, int nseg,
                                                          const unsigned *__restrict__ pos,
                                                          unsigned long long *__restrict__ img, int64_t total) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t p = pos[i];
        int lo = 0, hi = nseg - 1;  // the last array whose first row is <= p (arrays may be empty)
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (bases[mid] <= p) lo = mid;
            else hi = mid - 1;
        }
        img[i] = static_cast<unsigned long long>(lo);
    }
}

// Row i of the sorted run belongs to the array whose rows cover i; its position relative to that
// array's first row goes to that array's output at i - first row.
__global__ void __launch_bounds__(256) batch_split_kernel(const int64_t *__restrict__ bases, int nseg,
                                                          const unsigned *__restrict__ pos,
                                                          long long *const *__restrict__ outs, int64_t total) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int lo = 0, hi = nseg - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (bases[mid] <= i) lo = mid;
            else hi = mid - 1;
        }
        outs[lo][i - bases[lo]] = static_cast<long long>(pos[i]) - bases[lo];
    }
}

// ------------------------------------------------------------------ concatenation

// Batched statements whose kernel has no batched form (group_id, reduce_into, scans) run once
// over the concatenation of the batch's arrays, with an index column naming each row's array:
// a segmented statement keyed by that column gives every array's own result. One block per
// 8192-row chunk of one array (chunks[] gives each array's first chunk, table order).
constexpr int BC_ROWS = 8192;

template <int W>
__global__ void __launch_bounds__(256) batch_concat_kernel(const BSeg *__restrict__ segs, int nseg,
                                                           const int64_t *__restrict__ chunks, void *rows,
                                                           long long *index) {
    using U = typename std::conditional<W == 8, unsigned long long,
                                        typename std::conditional<W == 4, unsigned, unsigned char>::type>::type;
    const int64_t c = blockIdx.x;
    int lo = 0, hi = nseg - 1;  // the last array whose first chunk is <= c (no chunk: empty array)
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (chunks[mid] <= c) lo = mid;
        else hi = mid - 1;
    }
    const BSeg seg = segs[lo];
    const int64_t r0 = (c - chunks[lo]) * BC_ROWS;
    const int64_t r1 = min(seg.n, r0 + BC_ROWS);
    const U *src = static_cast<const U *>(seg.ptr);
    U *dst = static_cast<U *>(rows) + seg.base;
#pragma unroll 8
    for (int64_t r = r0 + threadIdx.x; r < r1; r += 256) {
        dst[r] = __ldcs(src + r);
        if (index) index[seg.base + r] = seg.index;
    }
}

static bool capturing(vkc_ctx *ctx) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return cs != cudaStreamCaptureStatusNone;
}

}  // namespace vkc

using namespace vkc;

extern "C" VKC_API vkc_status vkc_batch_new(vkc_ctx *ctx, int n, vkc_array *const *arrays, vkc_batch **out) {
    if (!ctx || !out || n < 0 || (n > 0 && !arrays)) return VKC_USAGE;
    *out = nullptr;
    if (capturing(ctx)) return fail(ctx, VKC_USAGE, "vkc_batch_new during a stream capture");
    auto *b = new vkc_batch;
    b->ctx = ctx;
    b->type = n > 0 ? arrays[0]->type : VKC_F64;
    std::vector<int64_t> base(static_cast<size_t>(n) + 1, 0);
    for (int i = 0; i < n; ++i) {
        if (!arrays[i] || arrays[i]->type != b->type) {
            delete b;
            return fail(ctx, VKC_RUNTIME, "batch arrays must share one element type");
        }
        base[i + 1] = base[i] + arrays[i]->len;
    }
    b->total = base[n];
    for (int i = 0; i < n; ++i) {
        vkc_array_retain(arrays[i]);
        await_write(ctx, arrays[i]);  // batches are read and written on the context stream
        b->arrays.push_back(arrays[i]);
        b->host.push_back(BSeg{arrays[i]->data(), arrays[i]->len, base[i], i});
    }
    std::stable_sort(b->host.begin(), b->host.end(), [](const BSeg &a, const BSeg &c) { return a.n > c.n; });
    auto upload = [&](DeviceMem &m, const void *src, size_t bytes) -> vkc_status {
        if (!bytes) return VKC_OK;
        void *p = nullptr;
        VKC_CUDA(ctx, cudaMallocAsync(&p, bytes, ctx->stream));
        m.ptr = p;
        m.box = ctx->box;
        void *h;
        vkc_status st = pinned(ctx, bytes, &h);
        if (st) return st;
        VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        memcpy(h, src, bytes);
        VKC_CUDA(ctx, cudaMemcpyAsync(p, h, bytes, cudaMemcpyHostToDevice, ctx->stream));
        VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return VKC_OK;
    };
    std::vector<int64_t> chunk(static_cast<size_t>(n) + 1, 0);
    for (int i = 0; i < n; ++i) chunk[i + 1] = chunk[i] + (b->host[i].n + BC_ROWS - 1) / BC_ROWS;
    vkc_status st = upload(b->table, b->host.data(), sizeof(BSeg) * b->host.size());
    if (!st) st = upload(b->bases, base.data(), sizeof(int64_t) * base.size());
    if (!st) st = upload(b->chunks, chunk.data(), sizeof(int64_t) * chunk.size());
    if (st) {
        vkc_batch_free(b);
        return st;
    }
    *out = b;
    return VKC_OK;
}

extern "C" VKC_API void vkc_batch_free(vkc_batch *b) {
    if (!b) return;
    for (vkc_array *a : b->arrays) vkc_array_release(a);
    for (vkc_array *a : b->scratch) vkc_array_release(a);
    delete b;
}

extern "C" VKC_API int vkc_batch_len(const vkc_batch *b) { return b ? static_cast<int>(b->arrays.size()) : 0; }

extern "C" VKC_API vkc_status vkc_batch_filter_sum_f64(vkc_ctx *ctx, vkc_batch *b, int cmp, double c,
                                                       vkc_array *sums) {
    if (!ctx || !b || !sums) return VKC_USAGE;
    if (b->type != VKC_F64) return fail(ctx, VKC_RUNTIME, "batch filter_sum: expected f64[] arrays");
    if (cmp < 0 || cmp > 5) return fail(ctx, VKC_USAGE, "batch filter_sum: comparison 0..5 (eq ne lt le gt ge)");
    const int n = static_cast<int>(b->host.size());
    if (sums->type != VKC_F64 || sums->len != n)
        return fail(ctx, VKC_RUNTIME, "batch filter_sum: the result array must be f64[" + std::to_string(n) + "]");
    if (n == 0) return VKC_OK;
    const CmpRange r = cmp_range(cmp, c);
    const int grid = std::min(n, ctx->sms * 8);
    await_write(ctx, sums);
    auto *out = static_cast<unsigned long long *>(sums->data());
    const auto *tab = static_cast<const BSeg *>(b->table.ptr);
    unsigned *ticket = ctx->counters + 4;  // two words, zero between launches
    if (pos_range(r)) batch_filter_sum_kernel<true><<<grid, BF_THREADS, 0, ctx->stream>>>(tab, n, r, out, ticket);
    else batch_filter_sum_kernel<false><<<grid, BF_THREADS, 0, ctx->stream>>>(tab, n, r, out, ticket);
    return launched(ctx, "batch_filter_sum");
}

extern "C" VKC_API vkc_status vkc_batch_count_f64(vkc_ctx *ctx, vkc_batch *b, int cmp, double c, vkc_array *counts) {
    if (!ctx || !b || !counts) return VKC_USAGE;
    if (b->type != VKC_F64) return fail(ctx, VKC_RUNTIME, "batch count: expected f64[] arrays");
    if (cmp < 0 || cmp > 5) return fail(ctx, VKC_USAGE, "batch count: comparison 0..5 (eq ne lt le gt ge)");
    const int n = static_cast<int>(b->host.size());
    if (counts->type != VKC_I64 || counts->len != n)
        return fail(ctx, VKC_RUNTIME, "batch count: the result array must be i64[" + std::to_string(n) + "]");
    if (n == 0) return VKC_OK;
    const CmpRange r = cmp_range(cmp, c);
    const int grid = std::min(n, ctx->sms * 8);
    await_write(ctx, counts);
    auto *out = static_cast<long long *>(counts->data());
    const auto *tab = static_cast<const BSeg *>(b->table.ptr);
    if (pos_range(r)) batch_count_kernel<true><<<grid, BF_THREADS, 0, ctx->stream>>>(tab, n, r, out, ctx->counters + 4);
    else batch_count_kernel<false><<<grid, BF_THREADS, 0, ctx->stream>>>(tab, n, r, out, ctx->counters + 4);
    return launched(ctx, "batch_count");
}

extern "C" VKC_API vkc_status vkc_batch_dot_f64(vkc_ctx *ctx, vkc_batch *xs, vkc_batch *ys, vkc_array *sums) {
    if (!ctx || !xs || !ys || !sums) return VKC_USAGE;
    if (xs->type != VKC_F64 || ys->type != VKC_F64) return fail(ctx, VKC_RUNTIME, "batch dot: expected f64[] arrays");
    const int n = static_cast<int>(xs->host.size());
    if (static_cast<int>(ys->host.size()) != n) return fail(ctx, VKC_RUNTIME, "batch dot: batches of different sizes");
    // Both tables are largest first with ties kept in index order, so equal lengths pair up.
    for (int i = 0; i < n; ++i)
        if (xs->arrays[i]->len != ys->arrays[i]->len)
            return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(xs->arrays[i]->len) + " vs " +
                                              std::to_string(ys->arrays[i]->len));
    if (sums->type != VKC_F64 || sums->len != n)
        return fail(ctx, VKC_RUNTIME, "batch dot: the result array must be f64[" + std::to_string(n) + "]");
    if (n == 0) return VKC_OK;
    const int grid = std::min(n, ctx->sms * 8);
    await_write(ctx, sums);
    batch_dot_kernel<<<grid, BF_THREADS, 0, ctx->stream>>>(static_cast<const BSeg *>(xs->table.ptr),
                                                           static_cast<const BSeg *>(ys->table.ptr), n,
                                                           static_cast<unsigned long long *>(sums->data()),
                                                           ctx->counters + 4);
    return launched(ctx, "batch_dot");
}

extern "C" VKC_API vkc_status vkc_batch_argsort_i64(vkc_ctx *ctx, vkc_batch *keys, const vkc_batch *outs,
                                                    unsigned key_digits) {
    if (!ctx || !keys || !outs) return VKC_USAGE;
    if (keys->type != VKC_I64) return fail(ctx, VKC_RUNTIME, "batch argsort: expected i64[] keys");
    const int n = static_cast<int>(keys->arrays.size());
    if (outs->type != VKC_I64 || static_cast<int>(outs->arrays.size()) != n)
        return fail(ctx, VKC_RUNTIME, "batch argsort: outputs must be " + std::to_string(n) + " i64[] arrays");
    for (int i = 0; i < n; ++i)
        if (outs->arrays[i]->len != keys->arrays[i]->len)
            return fail(ctx, VKC_RUNTIME, "batch argsort: output " + std::to_string(i) + " has the wrong length");
    const int64_t total = keys->total;
    if (n == 0 || total == 0) return VKC_OK;
    for (int i = 0; i < n; ++i) await_write(ctx, outs->arrays[i]);
    if (total >= (int64_t(1) << 32)) return fail(ctx, VKC_USAGE, "batch argsort of 2^32 rows or more");
    const bool cap = capturing(ctx);
    // Scratch (first use only, never during a capture).
    if (keys->scratch.empty() || keys->out_batch != outs) {
        if (cap) return fail(ctx, VKC_USAGE, "batch argsort: make its first call before capturing");
        vkc_status st;
        for (vkc_array *a : keys->scratch) vkc_array_release(a);
        keys->scratch.clear();
        int64_t cw, sw;
        radix_pairs_scratch(total, &cw, &sw);
        vkc_array *a[7];
        const vkc_type ty[7] = {VKC_U64, VKC_U64, VKC_I32, VKC_I32, VKC_I32, VKC_I32, VKC_I32};
        const int64_t len[7] = {total, total, total, total, cw, cw, sw};
        for (int i = 0; i < 7; ++i) {
            if ((st = new_array(ctx, ty[i], len[i], false, &a[i]))) return st;
            keys->scratch.push_back(a[i]);
        }
        keys->img[0] = static_cast<unsigned long long *>(a[0]->data());
        keys->img[1] = static_cast<unsigned long long *>(a[1]->data());
        keys->pos[0] = static_cast<unsigned *>(a[2]->data());
        keys->pos[1] = static_cast<unsigned *>(a[3]->data());
        keys->counts = static_cast<unsigned *>(a[4]->data());
        keys->offs = static_cast<unsigned *>(a[5]->data());
        keys->sums = static_cast<unsigned *>(a[6]->data());
        std::vector<long long *> optr(n);
        for (int i = 0; i < n; ++i) optr[i] = static_cast<long long *>(outs->arrays[i]->data());
        void *p = nullptr;
        VKC_CUDA(ctx, cudaMallocAsync(&p, sizeof(long long *) * n, ctx->stream));
        keys->outs.ptr = p;
        keys->outs.box = ctx->box;
        void *h;
        if ((st = pinned(ctx, sizeof(long long *) * n, &h))) return st;
        VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        memcpy(h, optr.data(), sizeof(long long *) * n);
        VKC_CUDA(ctx, cudaMemcpyAsync(p, h, sizeof(long long *) * n, cudaMemcpyHostToDevice, ctx->stream));
        VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        keys->out_batch = outs;
    }
    const auto *tab = static_cast<const BSeg *>(keys->table.ptr);
    const auto *bases = static_cast<const int64_t *>(keys->bases.ptr);
    dim3 kg(std::max(1, std::min(64, static_cast<int>((total / n + 255) / 256))), std::min(n, 65535));
    batch_keys_kernel<<<kg, 256, 0, ctx->stream>>>(tab, n, keys->img[0], keys->pos[0]);
    vkc_status st = launched(ctx, "batch_keys");
    if (st) return st;
    // Key digits: given, or all eight.
    int shifts[8], np = 0;
    if (key_digits == 0) key_digits = 0xff;
    for (int d = 0; d < 8; ++d)
        if ((key_digits >> d) & 1u) shifts[np++] = 8 * d;
    int which = 0;
    if ((st = radix_pairs(ctx, keys->img, keys->pos, total, shifts, np, keys->counts, keys->offs, keys->sums, &which)))
        return st;
    // Then by array index (two 8-bit digits cover 65536 arrays).
    const int grid = stream_grid(ctx, total, 256, 8, 2048);
    batch_owner_kernel<<<grid, 256, 0, ctx->stream>>>(bases, n, keys->pos[which], keys->img[which], total);
    if ((st = launched(ctx, "batch_owner"))) return st;
    if (n > 65536) return fail(ctx, VKC_USAGE, "batch argsort of more than 65536 arrays");
    const int seg_shifts[2] = {0, 8};
    unsigned long long *img2[2] = {keys->img[which], keys->img[1 - which]};
    unsigned *pos2[2] = {keys->pos[which], keys->pos[1 - which]};
    int w2 = 0;
    if ((st = radix_pairs(ctx, img2, pos2, total, seg_shifts, n > 256 ? 2 : 1, keys->counts, keys->offs, keys->sums, &w2)))
        return st;
    batch_split_kernel<<<grid, 256, 0, ctx->stream>>>(bases, n, pos2[w2], static_cast<long long *const *>(keys->outs.ptr),
                                                     total);
    return launched(ctx, "batch_split");
}

extern "C" VKC_API vkc_status vkc_batch_concat(vkc_ctx *ctx, vkc_batch *b, vkc_array **rows, vkc_array **index) {
    if (!ctx || !b || !rows) return VKC_USAGE;
    *rows = nullptr;
    if (index) *index = nullptr;
    vkc_status st;
    vkc_array *r = nullptr, *ix = nullptr;
    if ((st = new_array(ctx, b->type, b->total, false, &r))) return st;
    if (index && (st = new_array(ctx, VKC_I64, b->total, false, &ix))) {
        vkc_array_release(r);
        return st;
    }
    const int n = static_cast<int>(b->host.size());
    int64_t nchunks = 0;
    for (const BSeg &g : b->host) nchunks += (g.n + BC_ROWS - 1) / BC_ROWS;
    if (nchunks > 0) {
        const auto *tab = static_cast<const BSeg *>(b->table.ptr);
        const auto *ch = static_cast<const int64_t *>(b->chunks.ptr);
        long long *ip = ix ? static_cast<long long *>(ix->data()) : nullptr;
        const dim3 grid(static_cast<unsigned>(nchunks));
        switch (type_width(b->type)) {
        case 8: batch_concat_kernel<8><<<grid, 256, 0, ctx->stream>>>(tab, n, ch, r->data(), ip); break;
        case 4: batch_concat_kernel<4><<<grid, 256, 0, ctx->stream>>>(tab, n, ch, r->data(), ip); break;
        default: batch_concat_kernel<1><<<grid, 256, 0, ctx->stream>>>(tab, n, ch, r->data(), ip); break;
        }
        if ((st = launched(ctx, "batch_concat"))) {
            vkc_array_release(r);
            vkc_array_release(ix);
            return st;
        }
    }
    *rows = r;
    if (index) *index = ix;
    return VKC_OK;
}

// ------------------------------------------------------------------ CUDA graphs

struct vkc_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" VKC_API vkc_status vkc_graph_begin(vkc_ctx *ctx) {
    if (!ctx) return VKC_USAGE;
    VKC_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    return VKC_OK;
}

extern "C" VKC_API vkc_status vkc_graph_end(vkc_ctx *ctx, vkc_graph **out) {
    if (!ctx || !out) return VKC_USAGE;
    *out = nullptr;
    auto *g = new vkc_graph;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g->graph);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (g->graph) cudaGraphDestroy(g->graph);
        delete g;
        return fail(ctx, VKC_DEVICE, std::string("graph capture failed: ") + cudaGetErrorString(e));
    }
    *out = g;
    return VKC_OK;
}

extern "C" VKC_API vkc_status vkc_graph_launch(vkc_ctx *ctx, vkc_graph *g) {
    if (!ctx || !g) return VKC_USAGE;
    VKC_CUDA(ctx, cudaGraphLaunch(g->exec, ctx->stream));
    return VKC_OK;
}

extern "C" VKC_API void vkc_graph_free(vkc_graph *g) {
    if (!g) return;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
}

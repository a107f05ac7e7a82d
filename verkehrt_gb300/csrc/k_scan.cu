// Scans: scan_add_i64 and scan_by_add_i64 (src/kernels/scalar/scan.rs:284-326), plus prev_i64
// (scan.rs:16-48).
//
// One pass with decoupled lookback over 8192-row tiles. scan_by uses the segmented operator
// on (starts-a-segment, sum): (f1, v1) then (f2, v2) = (f1 | f2, f2 ? v2 : v1 + v2). Row 0 of
// the array always starts a segment; a later update continues the segment of the previous
// one unless its first start byte says otherwise, as Scan::update does.
#include <cstring>
#include <mutex>

#include "lookback.cuh"
#include "reduce_common.h"

namespace vkc {

constexpr int SC_THREADS = 512;
constexpr int SC_ITEMS = 16;
constexpr int SC_TILE = SC_THREADS * SC_ITEMS;

// A segmented partial: `start` when a segment starts inside it, `sum` since the last start.
struct Seg {
    unsigned long long sum;
    unsigned long long start;
};

__device__ __forceinline__ Seg seg_op(Seg a, Seg b) {
    return Seg{b.start ? b.sum : a.sum + b.sum, a.start | b.start};
}

// The carried state of a scanner: the last output and whether any row was seen.
struct ScanState {
    unsigned long long last;
    unsigned long long seen;
};

__device__ __forceinline__ Seg shfl_down_v(Seg v, int o) {
    return Seg{__shfl_down_sync(FULL, v.sum, o), __shfl_down_sync(FULL, v.start, o)};
}
__device__ __forceinline__ Seg __shfl_sync_v(Seg v, int src) {
    return Seg{__shfl_sync(FULL, v.sum, src), __shfl_sync(FULL, v.start, src)};
}

// Per warp, 4 rows of 128 consecutive rows of the input: lane l holds rows 4l..4l+3 of each
// (one 32-byte load), so loads and stores are coalesced and row order is (row, lane, item).
constexpr int SC_VEC = 4;
constexpr int SC_ROWS = SC_ITEMS / SC_VEC;

template <bool BY, bool ALIGNED>
__global__ void __launch_bounds__(SC_THREADS, 2) scan_kernel(const unsigned long long *__restrict__ x,
                                                          const unsigned char *__restrict__ starts,
                                                          unsigned long long *__restrict__ out, int64_t n,
                                                          int tiles, LookbackTiles<Seg> lb, unsigned epoch,
                                                          ScanState *state, unsigned *counters,
                                                          DevStatus *status) {
    // The carried state is read once, before this block publishes anything; the block that
    // finishes last rewrites it, after every block has read it.
    const bool seen = state->seen != 0;
    const unsigned long long carried = state->last;
    constexpr int SLICE = 32 * SC_ITEMS;  // rows of one warp
    // Each warp stages its slice's partial results (sums since the slice start or the last
    // segment start) and whether a segment started at or before each row, so no row value
    // waits in registers while the block waits for its prefix.
    extern __shared__ __align__(16) unsigned char scan_smem[];
    unsigned long long *s_val = reinterpret_cast<unsigned long long *>(scan_smem);
    unsigned char *s_has = scan_smem + sizeof(unsigned long long) * SC_TILE;
    __shared__ Seg s_warp[SC_THREADS / 32];
    __shared__ Seg s_prefix;
    const int tile = take_ticket(counters);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t wbase = static_cast<int64_t>(tile) * SC_TILE + static_cast<int64_t>(w) * SLICE;

    // Every row's load is issued before any is used: the loads of a thread are all in flight.
    unsigned long long vv[SC_ROWS][SC_VEC];
    unsigned ff = 0;  // start flags, 4 bits per row
#pragma unroll
    for (int r = 0; r < SC_ROWS; ++r) {
        const int64_t i0 = wbase + r * (32 * SC_VEC) + lane * SC_VEC;
        if (ALIGNED && i0 + SC_VEC <= n) {
            ulonglong4_32a u = *reinterpret_cast<const ulonglong4_32a *>(x + i0);
            vv[r][0] = u.x;
            vv[r][1] = u.y;
            vv[r][2] = u.z;
            vv[r][3] = u.w;
            if (BY) {
                unsigned m = *reinterpret_cast<const unsigned *>(starts + i0);
#pragma unroll
                for (int k = 0; k < SC_VEC; ++k)
                    if ((m >> (8 * k)) & 0xffu) ff |= 1u << (r * SC_VEC + k);
            }
        } else {
#pragma unroll
            for (int k = 0; k < SC_VEC; ++k) {
                bool in = i0 + k < n;
                vv[r][k] = in ? x[i0 + k] : 0ull;
                if (BY && in && starts[i0 + k]) ff |= 1u << (r * SC_VEC + k);
            }
        }
    }
    Seg carry{0, 0};  // the warp slice so far
#pragma unroll
    for (int r = 0; r < SC_ROWS; ++r) {
        const int64_t i0 = wbase + r * (32 * SC_VEC) + lane * SC_VEC;
        unsigned long long v[SC_VEC];
#pragma unroll
        for (int k = 0; k < SC_VEC; ++k) v[k] = vv[r][k];
        unsigned f = (ff >> (r * SC_VEC)) & 0xfu;
        // Row 0 of the array starts a segment whatever its byte (scan.rs:300-308).
        if (i0 == 0 && !seen) f |= 1u;
        // Lane-local inclusive segmented scan of the 4 rows.
        Seg loc{0, 0};
#pragma unroll
        for (int k = 0; k < SC_VEC; ++k) {
            loc = seg_op(loc, Seg{v[k], (f >> k) & 1u});
            v[k] = loc.sum;
        }
        // Warp inclusive scan of the lane partials.
        Seg inc = loc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            Seg y{__shfl_up_sync(FULL, inc.sum, o), __shfl_up_sync(FULL, inc.start, o)};
            if (lane >= o) inc = seg_op(y, inc);
        }
        Seg ex{__shfl_up_sync(FULL, inc.sum, 1), __shfl_up_sync(FULL, inc.start, 1)};
        if (lane == 0) ex = Seg{0, 0};
        const Seg pre = seg_op(carry, ex);  // the warp slice before this lane's rows
        const unsigned first = f ? __ffs(f) - 1 : SC_VEC;
        const int j0 = w * SLICE + r * (32 * SC_VEC) + lane * SC_VEC;
        unsigned hasw = 0;
#pragma unroll
        for (int k = 0; k < SC_VEC; ++k) {
            if (static_cast<unsigned>(k) < first) v[k] += pre.sum;
            if (static_cast<unsigned>(k) >= first || pre.start) hasw |= 1u << (8 * k);
        }
        ulonglong4_32a sv;
        sv.x = v[0];
        sv.y = v[1];
        sv.z = v[2];
        sv.w = v[3];
        *reinterpret_cast<ulonglong4_32a *>(s_val + j0) = sv;
        *reinterpret_cast<unsigned *>(s_has + j0) = hasw;
        carry = seg_op(carry, __shfl_sync_v(inc, 31));
    }
    if (lane == 0) s_warp[w] = carry;
    __syncthreads();
    if (w == 0) {
        // Exclusive segmented scan over the warps, then the lookback over tiles.
        Seg c = lane < SC_THREADS / 32 ? s_warp[lane] : Seg{0, 0}, inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            Seg y{__shfl_up_sync(FULL, inc.sum, o), __shfl_up_sync(FULL, inc.start, o)};
            if (lane >= o) inc = seg_op(y, inc);
        }
        Seg ex{__shfl_up_sync(FULL, inc.sum, 1), __shfl_up_sync(FULL, inc.start, 1)};
        if (lane == 0) ex = Seg{0, 0};
        Seg tile_agg = __shfl_sync_v(inc, SC_THREADS / 32 - 1);
        Seg pre = warp_lookback<4, Seg>(lb, tile, tile_agg, Seg{carried, 0}, Seg{0, 0}, epoch, seg_op, status);
        if (lane < SC_THREADS / 32) s_warp[lane] = ex;
        if (lane == 0) s_prefix = pre;
    }
    __syncthreads();
    // Rows without a segment start before them in their warp slice add the slice's prefix.
    const unsigned long long before = seg_op(s_prefix, s_warp[w]).sum;
#pragma unroll
    for (int r = 0; r < SC_ROWS; ++r) {
        const int j0 = w * SLICE + r * (32 * SC_VEC) + lane * SC_VEC;
        const int64_t i0 = wbase + r * (32 * SC_VEC) + lane * SC_VEC;
        ulonglong4_32a u = *reinterpret_cast<const ulonglong4_32a *>(s_val + j0);
        const unsigned hasw = *reinterpret_cast<const unsigned *>(s_has + j0);
        if (!(hasw & 0xffu)) u.x += before;
        if (!(hasw & 0xff00u)) u.y += before;
        if (!(hasw & 0xff0000u)) u.z += before;
        if (!(hasw & 0xff000000u)) u.w += before;
        if (ALIGNED && i0 + SC_VEC <= n) {
            *reinterpret_cast<ulonglong4_32a *>(out + i0) = u;
        } else {
            unsigned long long e[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int k = 0; k < SC_VEC; ++k)
                if (i0 + k < n) out[i0 + k] = e[k];
        }
    }
    // The last row's output, the last tile's inclusive value, is the carried state.
    if (release_ticket_last(counters, tiles) && threadIdx.x == 0) {
        state->last = ld_relaxed64(&lb.inc[tiles - 1].sum);
        state->seen = 1;
    }
}

// Dynamic shared memory of scan_kernel: the staged rows and their start flags.
constexpr size_t SC_SMEM = (sizeof(unsigned long long) + 1) * SC_TILE;

template <bool BY, bool ALIGNED> static void scan_configure() {
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(scan_kernel<BY, ALIGNED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(SC_SMEM));
        configured = true;
    }
}

struct ScanImpl : ScannerImpl {
    bool by;
    ScanState *state = nullptr;
    DeviceMem mem;  // owns `state`
    // scan.rs:228-282 (tile_rows): arity, kinds, then destination rows.
    vkc_status update(vkc_ctx *ctx, const Arg *args, int nargs, vkc_array *out) override {
        vkc_status st;
        int want = by ? 2 : 1;
        if (nargs != want) return fail(ctx, VKC_RUNTIME, arity_error(want, nargs));
        if (!rows_arg(ctx, args[0], VKC_I64, &st)) return st;
        if (by && !rows_arg(ctx, args[1], VKC_BOOL, &st)) return st;
        if (out->type != VKC_I64) return fail(ctx, VKC_RUNTIME, "bad destination");
        int64_t n = args[0].len();
        if (out->len != n || (by && args[1].len() != n))
            return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(n) +
                                              " rows for a destination of " + std::to_string(out->len) +
                                              " rows");
        if (n == 0) return VKC_OK;
        int tiles = static_cast<int>((n + SC_TILE - 1) / SC_TILE);
        void *p;
        unsigned *flags;
        if ((st = scratch(ctx, 2 * sizeof(Seg) * static_cast<size_t>(tiles), &p))) return st;
        if ((st = flag_arena(ctx, static_cast<size_t>(tiles), &flags))) return st;
        Seg *vals = static_cast<Seg *>(p);
        LookbackTiles<Seg> lb{flags, vals, vals + tiles};
        unsigned epoch = next_epoch(ctx);
        const auto *x = args[0].ptr<unsigned long long>();
        const unsigned char *s = by ? args[1].ptr<unsigned char>() : nullptr;
        auto *o = static_cast<unsigned long long *>(out->data());
        bool aligned = (reinterpret_cast<uintptr_t>(x) & 31) == 0 && (reinterpret_cast<uintptr_t>(o) & 31) == 0 &&
                       (reinterpret_cast<uintptr_t>(s) & 3) == 0;
        if (by && aligned) scan_configure<true, true>(), scan_kernel<true, true><<<tiles, SC_THREADS, SC_SMEM, ctx->stream>>>(x, s, o, n, tiles, lb, epoch, state, ctx->counters, ctx->status);
        else if (by) scan_configure<true, false>(), scan_kernel<true, false><<<tiles, SC_THREADS, SC_SMEM, ctx->stream>>>(x, s, o, n, tiles, lb, epoch, state, ctx->counters, ctx->status);
        else if (aligned) scan_configure<false, true>(), scan_kernel<false, true><<<tiles, SC_THREADS, SC_SMEM, ctx->stream>>>(x, s, o, n, tiles, lb, epoch, state, ctx->counters, ctx->status);
        else scan_configure<false, false>(), scan_kernel<false, false><<<tiles, SC_THREADS, SC_SMEM, ctx->stream>>>(x, s, o, n, tiles, lb, epoch, state, ctx->counters, ctx->status);
        return launched(ctx, "scan");
    }
};

// A zeroed ScanState on the context's stream, owned by `mem`.
static bool alloc_scan_state(vkc_ctx *ctx, ScanState **state, DeviceMem *mem) {
    if (cudaMallocAsync(reinterpret_cast<void **>(state), sizeof(ScanState), ctx->stream) != cudaSuccess) {
        cudaGetLastError();
        *state = nullptr;
        return false;
    }
    mem->ptr = *state;
    mem->box = ctx->box;
    if (cudaMemsetAsync(*state, 0, sizeof(ScanState), ctx->stream) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return true;
}

template <bool BY> static ScannerImpl *make_scan(vkc_ctx *ctx) {
    auto *s = new ScanImpl;
    s->by = BY;
    if (!alloc_scan_state(ctx, &s->state, &s->mem)) {
        delete s;
        return nullptr;
    }
    return s;
}

// ------------------------------------------------------------------ prev

__global__ void prev_kernel(const unsigned long long *__restrict__ x, unsigned long long *__restrict__ out,
                            int64_t n, unsigned long long fill, const ScanState *state) {
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = i == 0 ? (state->seen ? state->last : fill) : __ldcs(x + i - 1);
}

__global__ void prev_carry(const unsigned long long *x, int64_t n, ScanState *state) {
    state->last = x[n - 1];
    state->seen = 1;
}

// scan.rs:16-48 (Prev): row 0 is the fill on the first update, else the previous update's
// last row.
struct PrevImpl : ScannerImpl {
    ScanState *state = nullptr;
    DeviceMem mem;  // owns `state`
    vkc_status update(vkc_ctx *ctx, const Arg *args, int nargs, vkc_array *out) override {
        vkc_status st;
        if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
        if (!rows_arg(ctx, args[0], VKC_I64, &st) || !splat_arg(ctx, args[1], VKC_I64, &st)) return st;
        int64_t n = args[0].len();
        if (out->len != n)
            return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(n) +
                                              " rows for a destination of " + std::to_string(out->len) +
                                              " rows");
        if (n == 0) return VKC_OK;
        const auto *x = args[0].ptr<unsigned long long>();
        int grid = stream_grid(ctx, n, 256, 8, 2048);
        prev_kernel<<<grid, 256, 0, ctx->stream>>>(x, static_cast<unsigned long long *>(out->data()), n,
                                                  args[1].s.bits, state);
        if ((st = launched(ctx, "prev"))) return st;
        prev_carry<<<1, 1, 0, ctx->stream>>>(x, n, state);
        return launched(ctx, "prev_carry");
    }
};

static ScannerImpl *make_prev(vkc_ctx *ctx) {
    auto *s = new PrevImpl;
    if (!alloc_scan_state(ctx, &s->state, &s->mem)) {
        delete s;
        return nullptr;
    }
    return s;
}

void register_scan(std::vector<KernelDef> &t) {
    InSpec ia{IN_ARRAY, VKC_I64};
    // scan.rs:336-352: cost = input + output width (+1 for the starts byte).
    KernelDef d{"scan_add_i64", VKC_SCAN, {ia}, true, VKC_I64, 16};
    d.scan = make_scan<false>;
    t.push_back(d);
    d = KernelDef{"scan_by_add_i64", VKC_SCAN, {ia, InSpec{IN_ARRAY, VKC_BOOL}}, true, VKC_I64, 17};
    d.scan = make_scan<true>;
    t.push_back(d);
    d = KernelDef{"prev_i64", VKC_SCAN, {ia, InSpec{IN_SCALAR, VKC_I64}}, true, VKC_I64, 16};
    d.scan = make_prev;
    t.push_back(d);
}

}  // namespace vkc

// ------------------------------------------------------------------ allocation-free scan_add_i64
//
// vkc_scan_add_i64_noalloc: scan_add_i64 for callers that cannot allocate device memory. An
// embedding host that hands this library only its own buffers (an interpreter's arena or a
// memory pool with a fixed budget), or a serving loop that must not take the allocator's lock
// or latency while it answers a request, cannot use the entries above, which take their
// lookback scratch from a context arena that grows with cudaMallocAsync. This entry needs no
// context and allocates nothing: the lookback records live in the file-scope array below, whose
// address is looked up once per device. Every call shares the array and finds it as the last
// call left it, so each call clears the words that must start at zero (the ticket counters,
// the tile flags, the carried state and the status). Calls that overlap on the GPU race on the
// array: issue them on one stream, or wait for one to finish before the next starts.
namespace vkc {

// Header (ticket counters, status, carried state), the tile flags, then the tile aggregates
// and inclusive prefixes. 1.13 MiB holds the 32,768 tiles of 2^28 rows.
constexpr int64_t NOALLOC_MAX_ROWS = int64_t(1) << 28;
constexpr int64_t NOALLOC_MAX_TILES = NOALLOC_MAX_ROWS / SC_TILE;
constexpr size_t NOALLOC_HEADER = 512;
constexpr size_t NOALLOC_FLAGS = NOALLOC_MAX_TILES * sizeof(unsigned);
constexpr size_t NOALLOC_BYTES = NOALLOC_HEADER + NOALLOC_FLAGS + 2 * NOALLOC_MAX_TILES * sizeof(Seg);

static __device__ __align__(256) unsigned char g_scan_scratch[NOALLOC_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
static std::mutex g_noalloc_mu;
static unsigned char *g_noalloc_ptr[NOALLOC_MAX_DEVICES];

static void noalloc_msg(char *err, size_t err_len, const std::string &msg) {
    if (err && err_len) {
        size_t k = msg.size() < err_len - 1 ? msg.size() : err_len - 1;
        memcpy(err, msg.data(), k);
        err[k] = 0;
    }
}

}  // namespace vkc

extern "C" vkc_status vkc_scan_add_i64_noalloc(int device, const int64_t *in, int64_t *out, int64_t n,
                                               void *stream, char *err, size_t err_len) {
    using namespace vkc;
    noalloc_msg(err, err_len, "");
    if (n < 0 || n > NOALLOC_MAX_ROWS) {
        noalloc_msg(err, err_len, "vkc_scan_add_i64_noalloc: " + std::to_string(n) +
                                      " rows is more than its maximum of 268435456 rows (2^28)");
        return VKC_USAGE;
    }
    if (device < 0 || device >= NOALLOC_MAX_DEVICES) {
        noalloc_msg(err, err_len, "vkc_scan_add_i64_noalloc: device " + std::to_string(device) +
                                      " is out of range");
        return VKC_USAGE;
    }
    if (n == 0) return VKC_OK;
    int prev = 0;
    if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        noalloc_msg(err, err_len, "vkc_scan_add_i64_noalloc: cannot make device " + std::to_string(device) +
                                      " current");
        return VKC_DEVICE;
    }
    auto done = [&](vkc_status st, const std::string &msg) {
        if (st != VKC_OK) noalloc_msg(err, err_len, msg);
        cudaSetDevice(prev);
        return st;
    };
    unsigned char *base;
    {
        // Set-up, once per device: the device address of the scratch array. On the first call on
        // a device this runs inside that call.
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[device]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_scan_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                return done(VKC_DEVICE, std::string("vkc_scan_add_i64_noalloc: cudaGetSymbolAddress failed: ") +
                                            cudaGetErrorString(e));
            }
            g_noalloc_ptr[device] = static_cast<unsigned char *>(p);
        }
        base = g_noalloc_ptr[device];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int tiles = static_cast<int>((n + SC_TILE - 1) / SC_TILE);
    unsigned *counters = reinterpret_cast<unsigned *>(base);
    DevStatus *status = reinterpret_cast<DevStatus *>(base + 256);
    ScanState *state = reinterpret_cast<ScanState *>(base + 256 + sizeof(DevStatus));
    unsigned *flags = reinterpret_cast<unsigned *>(base + NOALLOC_HEADER);
    Seg *agg = reinterpret_cast<Seg *>(base + NOALLOC_HEADER + NOALLOC_FLAGS);
    LookbackTiles<Seg> lb{flags, agg, agg + NOALLOC_MAX_TILES};
    // The header and the flags of this call's tiles start at zero; with clean flags one epoch
    // value serves every call.
    cudaError_t e = cudaMemsetAsync(base, 0, NOALLOC_HEADER, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, static_cast<size_t>(tiles) * sizeof(unsigned), s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return done(VKC_DEVICE, std::string("vkc_scan_add_i64_noalloc: ") + cudaGetErrorString(e));
    }
    const auto *x = reinterpret_cast<const unsigned long long *>(in);
    auto *o = reinterpret_cast<unsigned long long *>(out);
    bool aligned = (reinterpret_cast<uintptr_t>(x) & 31) == 0 && (reinterpret_cast<uintptr_t>(o) & 31) == 0;
    if (aligned) {
        scan_configure<false, true>();
        scan_kernel<false, true><<<tiles, SC_THREADS, SC_SMEM, s>>>(x, nullptr, o, n, tiles, lb, 1u, state, counters, status);
    } else {
        scan_configure<false, false>();
        scan_kernel<false, false><<<tiles, SC_THREADS, SC_SMEM, s>>>(x, nullptr, o, n, tiles, lb, 1u, state, counters, status);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return done(VKC_DEVICE, std::string("vkc_scan_add_i64_noalloc: ") + cudaGetErrorString(e));
    // Synchronous, like the other entries: read the status word into host memory.
    DevStatus hs{};
    e = cudaMemcpyAsync(&hs, status, sizeof hs, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return done(VKC_DEVICE, std::string("vkc_scan_add_i64_noalloc: ") + cudaGetErrorString(e));
    }
    if (hs.timeout) return done(VKC_TIMEOUT, "vkc_scan_add_i64_noalloc: a device-side wait gave up");
    return done(VKC_OK, "");
}

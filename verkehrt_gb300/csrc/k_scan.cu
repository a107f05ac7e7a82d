// Scans: scan_add_i64 and scan_by_add_i64 (src/kernels/scalar/scan.rs:284-326), plus prev_i64
// (scan.rs:16-48).
//
// One persistent pass (tilepass.cuh) over 8192-row tiles: a tile's aggregate is taken while it
// streams from HBM, the tile is read again from L2 and scanned into shared memory while the
// decoupled lookback finds its prefix, and the scanned rows are written with the prefix added. scan_by uses the segmented operator on
// (starts-a-segment, sum): (f1, v1) then (f2, v2) = (f1 | f2, f2 ? v2 : v1 + v2). Row 0 of the
// array always starts a segment; a later update continues the segment of the previous one
// unless its first start byte says otherwise, as Scan::update does.
#include <cstring>
#include <mutex>

#include "reduce_common.h"
#include "tilepass.cuh"

namespace vkc {

constexpr int SC_THREADS = 512;  // compute threads (+ 2 warps)
constexpr int SC_TILE = 8192;
constexpr int SC_SLICE = SC_TILE / (SC_THREADS / 32);  // rows per warp
constexpr int SC_WINDOW = 4;
constexpr int SC_SLOTS = 3;   // tile ring: 1 copy in flight
constexpr int SC_BLOCKS = 1;  // blocks per SM

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

__device__ __forceinline__ ulonglong2 ld_relaxed128(const ulonglong2 *p) {
    ulonglong2 v;
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed128(ulonglong2 *p, ulonglong2 v) {
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(v.x), "l"(v.y) : "memory");
}

// Lookback record of a Seg in two words, each carrying the epoch and the state: the start
// flag and the high half of the sum in one, the low half in the other. Each word is read or
// written whole, so a record read in the middle of its update from aggregate to inclusive
// shows two states and is polled again.
struct SegRec {
    using V = Seg;
    using W = ulonglong2;
    __device__ static V ident() { return Seg{0, 0}; }
    __device__ static V op(V a, V b) { return seg_op(a, b); }
    __device__ static W make(unsigned ep, unsigned state, V v) {
        const unsigned long long tag = (static_cast<unsigned long long>(ep & 0xffffffu) << 40) |
                                       (static_cast<unsigned long long>(state) << 38);
        return W{tag | ((v.start & 1ull) << 37) | (v.sum >> 32), tag | (v.sum & 0xffffffffull)};
    }
    __device__ static bool ready(W w, unsigned ep) {
        const unsigned long long e = ep & 0xffffffu;
        return (w.x >> 40) == e && (w.y >> 40) == e && ((w.x >> 38) & 3u) == ((w.y >> 38) & 3u);
    }
    __device__ static unsigned state(W w) { return static_cast<unsigned>(w.x >> 38) & 3u; }
    __device__ static V value(W w) {
        return Seg{((w.x & 0xffffffffull) << 32) | (w.y & 0xffffffffull), (w.x >> 37) & 1ull};
    }
    __device__ static W load(const W *p) { return ld_relaxed128(p); }
    __device__ static void store(W *p, W w) { st_relaxed128(p, w); }
    __device__ static V shfl_up(V v, int o) {
        return Seg{__shfl_up_sync(FULL, v.sum, o), __shfl_up_sync(FULL, v.start, o)};
    }
    __device__ static V shfl(V v, int src) { return Seg{__shfl_sync(FULL, v.sum, src), __shfl_sync(FULL, v.start, src)}; }
    __device__ static V shfl_down(V v, int o) {
        return Seg{__shfl_down_sync(FULL, v.sum, o), __shfl_down_sync(FULL, v.start, o)};
    }
};

// A scan as a tile pass. A slot holds the tile's values (scanned in place by the stage) and
// one byte per row: the start flags of scan_by as copied, then whether a segment starts at or
// before the row in its warp slice. A compute warp's slice is SC_SLICE consecutive rows, read in
// STEPS steps of 32 * VEC rows; in a step lane l holds rows VEC l .. VEC l + VEC - 1, so global
// stores are coalesced and row order is (step, lane, item). The plain scan takes two rows a lane
// (one 16-byte read of the slot a step, every bank once: with four rows a lane, 32 bytes apart,
// each read took two passes; 0.76 against 0.88 ms at 2^28); the segmented scan keeps four,
// whose fewer warp scans of (sum, start) pairs cost less than the bank passes (0.56 against
// 0.60 ms at 2^27). A tile that is not whole, or not aligned, is
// read from global memory instead of the slot.
template <bool BY> struct ScanPass {
    static constexpr int VEC = BY ? 4 : 2;  // rows per lane per step
    static constexpr int STEPS = SC_SLICE / (32 * VEC);
    static constexpr int THREADS = SC_THREADS;
    static constexpr int VAL_BYTES = 8 * SC_TILE;
    static constexpr int SLOT_BYTES = VAL_BYTES + SC_TILE;
    static constexpr int SLOTS = SC_SLOTS;
    using R = SegRec;
    using V = Seg;
    struct Staged {};

    const unsigned long long *x;
    const unsigned char *starts;
    unsigned long long *out;
    int64_t n;
    bool seen;     // an earlier update saw rows: row 0 continues its segment
    bool aligned;  // x, out (32 bytes) and starts (16 bytes) aligned: whole tiles go by TMA

    __device__ bool whole(int tile) const { return aligned && static_cast<int64_t>(tile + 1) * SC_TILE <= n; }
    __device__ unsigned bulk_bytes(int tile) const { return whole(tile) ? VAL_BYTES + (BY ? SC_TILE : 0) : 0u; }
    __device__ void load(int tile, unsigned char *slot, unsigned long long *bar) const {
        const int64_t r0 = static_cast<int64_t>(tile) * SC_TILE;
        bulk_load(slot, x + r0, VAL_BYTES, bar);
        if (BY) bulk_load(slot + VAL_BYTES, starts + r0, SC_TILE, bar);
    }

    // The rows of one step and their start flags (bit k: row 4l + k), from the slot or from
    // global memory. Row 0 of the array starts a segment whatever its byte (scan.rs:300-308).
    __device__ __forceinline__ void load_step(bool sm, const unsigned char *slot, int j, int64_t i0,
                                              unsigned long long (&v)[VEC], unsigned &f) const {
        f = 0;
        if (sm) {
            const ulonglong2 *p = reinterpret_cast<const ulonglong2 *>(reinterpret_cast<const unsigned long long *>(slot) + j);
#pragma unroll
            for (int c = 0; c < VEC / 2; ++c) {
                const ulonglong2 u = p[c];
                v[2 * c] = u.x;
                v[2 * c + 1] = u.y;
            }
            if (BY) {
                const unsigned m = VEC == 4 ? *reinterpret_cast<const unsigned *>(slot + VAL_BYTES + j)
                                            : *reinterpret_cast<const unsigned short *>(slot + VAL_BYTES + j);
#pragma unroll
                for (int k = 0; k < VEC; ++k)
                    if ((m >> (8 * k)) & 0xffu) f |= 1u << k;
            }
        } else {
#pragma unroll
            for (int k = 0; k < VEC; ++k) {
                const bool in = i0 + k < n;
                v[k] = in ? x[i0 + k] : 0ull;
                if (BY && in && starts[i0 + k]) f |= 1u << k;
            }
        }
        if (BY && i0 == 0 && !seen) f |= 1u;
    }

    // The slice aggregate: the sum of the rows from the slice's last segment start on (of all
    // rows when none starts), which needs no ordered combination across lanes.
    __device__ Seg count(int tile, unsigned char *slot) const {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const int64_t r0 = static_cast<int64_t>(tile) * SC_TILE;
        const bool sm = whole(tile);
        unsigned long long t = 0;
        unsigned last = 0;  // the last start in the slice, as a position in row order + 1 (0: none)
        unsigned long long v[STEPS][VEC];
        unsigned f[STEPS];
#pragma unroll
        for (int s = 0; s < STEPS; ++s) {
            const int j = w * SC_SLICE + s * (32 * VEC) + lane * VEC;
            load_step(sm, slot, j, r0 + j, v[s], f[s]);
        }
        if (!BY) {
#pragma unroll
            for (int s = 0; s < STEPS; ++s)
#pragma unroll
                for (int k = 0; k < VEC; ++k) t += v[s][k];
            return Seg{warp_sum(t), 0};
        }
#pragma unroll
        for (int s = 0; s < STEPS; ++s)
#pragma unroll
            for (int k = 0; k < VEC; ++k)
                if ((f[s] >> k) & 1u) last = (s * 32 + lane) * VEC + k + 1;
        last = __reduce_max_sync(FULL, last);
#pragma unroll
        for (int s = 0; s < STEPS; ++s)
#pragma unroll
            for (int k = 0; k < VEC; ++k)
                if (static_cast<unsigned>((s * 32 + lane) * VEC + k + 1) >= last) t += v[s][k];
        return Seg{warp_sum(t), last != 0};
    }

    // Scans the slice from its own start, in place in the slot, with the has-a-start bytes
    // over the start flags; a lane reads back only what it wrote itself.
    __device__ Staged stage(int tile, unsigned char *slot) const {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const int64_t r0 = static_cast<int64_t>(tile) * SC_TILE;
        const bool sm = whole(tile);
        if constexpr (!BY) {
            // Without segments: a plain wrapping add scan of the slice, in place.
            unsigned long long carry = 0;
#pragma unroll
            for (int s = 0; s < STEPS; ++s) {
                const int j = w * SC_SLICE + s * (32 * VEC) + lane * VEC;
                unsigned long long v[VEC];
                unsigned f;
                load_step(sm, slot, j, r0 + j, v, f);
#pragma unroll
                for (int k = 1; k < VEC; ++k) v[k] += v[k - 1];
                unsigned long long inc = v[VEC - 1];
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const unsigned long long y = __shfl_up_sync(FULL, inc, o);
                    if (lane >= o) inc += y;
                }
                const unsigned long long pre = carry + inc - v[VEC - 1];
                *reinterpret_cast<ulonglong2 *>(reinterpret_cast<unsigned long long *>(slot) + j) =
                    ulonglong2{v[0] + pre, v[1] + pre};
                carry += __shfl_sync(FULL, inc, 31);
            }
            return Staged{};
        }
        Seg carry{0, 0};  // the slice so far
#pragma unroll
        for (int s = 0; s < STEPS; ++s) {
            const int j = w * SC_SLICE + s * (32 * VEC) + lane * VEC;
            unsigned long long v[VEC];
            unsigned f;
            load_step(sm, slot, j, r0 + j, v, f);
            // Lane-local inclusive segmented scan of the 4 rows.
            Seg loc{0, 0};
#pragma unroll
            for (int k = 0; k < VEC; ++k) {
                loc = seg_op(loc, Seg{v[k], (f >> k) & 1u});
                v[k] = loc.sum;
            }
            const Seg inc = warp_inclusive<SegRec>(loc);
            Seg ex = SegRec::shfl_up(inc, 1);
            if (lane == 0) ex = Seg{0, 0};
            const Seg pre = seg_op(carry, ex);  // the slice before this lane's rows
            const unsigned first = f ? __ffs(f) - 1 : VEC;
            unsigned has = 0;
#pragma unroll
            for (int k = 0; k < VEC; ++k) {
                if (static_cast<unsigned>(k) < first) v[k] += pre.sum;
                if (static_cast<unsigned>(k) >= first || pre.start) has |= 1u << (8 * k);
            }
            ulonglong2 *p = reinterpret_cast<ulonglong2 *>(reinterpret_cast<unsigned long long *>(slot) + j);
#pragma unroll
            for (int c = 0; c < VEC / 2; ++c) p[c] = ulonglong2{v[2 * c], v[2 * c + 1]};
            if constexpr (VEC == 4) *reinterpret_cast<unsigned *>(slot + VAL_BYTES + j) = has;
            else *reinterpret_cast<unsigned short *>(slot + VAL_BYTES + j) = static_cast<unsigned short>(has);
            carry = seg_op(carry, SegRec::shfl(inc, 31));
        }
        return Staged{};
    }

    __device__ void flush(int tile, Seg pre, Staged, unsigned char *slot) const {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const int64_t r0 = static_cast<int64_t>(tile) * SC_TILE;
#pragma unroll
        for (int s = 0; s < STEPS; ++s) {
            const int j = w * SC_SLICE + s * (32 * VEC) + lane * VEC;
            const int64_t i0 = r0 + j;
            const ulonglong2 *p = reinterpret_cast<const ulonglong2 *>(reinterpret_cast<const unsigned long long *>(slot) + j);
            unsigned long long e[VEC];
#pragma unroll
            for (int c = 0; c < VEC / 2; ++c) {
                const ulonglong2 u = p[c];
                e[2 * c] = u.x;
                e[2 * c + 1] = u.y;
            }
            if constexpr (BY) {
                const unsigned has = VEC == 4 ? *reinterpret_cast<const unsigned *>(slot + VAL_BYTES + j)
                                              : *reinterpret_cast<const unsigned short *>(slot + VAL_BYTES + j);
#pragma unroll
                for (int k = 0; k < VEC; ++k)
                    if (!((has >> (8 * k)) & 0xffu)) e[k] += pre.sum;
            } else {
#pragma unroll
                for (int k = 0; k < VEC; ++k) e[k] += pre.sum;
            }
            if (aligned && i0 + VEC <= n) {
                if constexpr (VEC == 4) {
                    ulonglong4_32a u;
                    u.x = e[0];
                    u.y = e[1];
                    u.z = e[2];
                    u.w = e[3];
                    *reinterpret_cast<ulonglong4_32a *>(out + i0) = u;
                } else {
                    *reinterpret_cast<ulonglong2 *>(out + i0) = ulonglong2{e[0], e[1]};
                }
            } else {
#pragma unroll
                for (int k = 0; k < VEC; ++k)
                    if (i0 + k < n) out[i0 + k] = e[k];
            }
        }
    }

    __device__ void last_tile(Seg) const {}
};

template <bool BY>
__global__ void __launch_bounds__(SC_THREADS + 64, SC_BLOCKS) scan_kernel(const unsigned long long *__restrict__ x,
                                                                  const unsigned char *__restrict__ starts,
                                                                  unsigned long long *__restrict__ out, int64_t n,
                                                                  bool aligned, int tiles, ulonglong2 *recs,
                                                                  unsigned epoch, ScanState *state,
                                                                  unsigned *counters, DevStatus *status) {
    // The carried state is read once, before this block publishes anything; the block that
    // finishes last rewrites it, after every block has read it.
    const bool seen = state->seen != 0;
    const unsigned long long carried = state->last;
    ScanPass<BY> p{x, starts, out, n, seen, aligned};
    // The last row's output, the last tile's inclusive value, is the carried state.
    if (tile_pass<SC_WINDOW>(p, recs, tiles, epoch, counters, status, Seg{carried, 0}) && threadIdx.x == 0) {
        state->last = SegRec::value(ld_relaxed128(rec_at<SegRec>(recs, tiles - 1))).sum;
        state->seen = 1;
    }
}

// Launches a scan on `stream` with the tile records at `recs` (REC_STRIDE bytes per tile).
template <bool BY>
static void launch_scan(int device, int sms, cudaStream_t stream, const unsigned long long *x, const unsigned char *s,
                        unsigned long long *o, int64_t n, int tiles, ulonglong2 *recs, unsigned epoch,
                        ScanState *state, unsigned *counters, DevStatus *status) {
    const bool aligned = (reinterpret_cast<uintptr_t>(x) & 31) == 0 && (reinterpret_cast<uintptr_t>(o) & 31) == 0 &&
                         (reinterpret_cast<uintptr_t>(s) & 15) == 0;
    constexpr size_t smem = SC_SLOTS * ScanPass<BY>::SLOT_BYTES;
    static std::atomic<unsigned long long> configured{0};
    once_per_device(configured, device, [] {
        cudaFuncSetAttribute(scan_kernel<BY>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    });
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, scan_kernel<BY>, SC_THREADS + 64, smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    const long long g = static_cast<long long>(per_sm) * sms;
    const int grid = static_cast<int>(g < tiles ? g : tiles);
    scan_kernel<BY><<<grid, SC_THREADS + 64, smem, stream>>>(x, s, o, n, aligned, tiles, recs, epoch, state, counters,
                                                             status);
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
        const int tiles = static_cast<int>((n + SC_TILE - 1) / SC_TILE);
        ulonglong2 *recs;
        if ((st = rec_arena(ctx, tiles, &recs))) return st;
        const unsigned epoch = next_epoch(ctx);
        const auto *x = args[0].ptr<unsigned long long>();
        const unsigned char *s = by ? args[1].ptr<unsigned char>() : nullptr;
        auto *o = static_cast<unsigned long long *>(out->data());
        if (by) launch_scan<true>(ctx->device, ctx->sms, ctx->stream, x, s, o, n, tiles, recs, epoch, state, ctx->counters, ctx->status);
        else launch_scan<false>(ctx->device, ctx->sms, ctx->stream, x, s, o, n, tiles, recs, epoch, state, ctx->counters, ctx->status);
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
// the tile records, the carried state and the status). Calls that overlap on the GPU race on the
// array: issue them on one stream, or wait for one to finish before the next starts.
namespace vkc {

// Header (ticket counters, status, carried state), then one lookback record per tile, REC_STRIDE
// (128) bytes apart. 4 MiB and 512 bytes hold the 32,768 tiles of 2^28 rows.
constexpr int64_t NOALLOC_MAX_ROWS = int64_t(1) << 28;
constexpr int64_t NOALLOC_MAX_TILES = NOALLOC_MAX_ROWS / SC_TILE;
constexpr size_t NOALLOC_HEADER = 512;
constexpr size_t NOALLOC_BYTES = NOALLOC_HEADER + NOALLOC_MAX_TILES * REC_STRIDE;

static __device__ __align__(256) unsigned char g_scan_scratch[NOALLOC_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
static std::mutex g_noalloc_mu;
static unsigned char *g_noalloc_ptr[NOALLOC_MAX_DEVICES];
static int g_noalloc_sms[NOALLOC_MAX_DEVICES];

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
    if (!in || !out) {
        noalloc_msg(err, err_len, "vkc_scan_add_i64_noalloc: `in` and `out` must be device pointers, got NULL");
        return VKC_USAGE;
    }
    // Pointers the GPU cannot address as device memory of `device` (host memory, another
    // device's buffers) would fault the kernel: reject them before anything is launched.
    for (const void *p : {static_cast<const void *>(in), static_cast<const void *>(out)}) {
        cudaPointerAttributes at{};
        cudaError_t pe = cudaPointerGetAttributes(&at, p);
        if (pe != cudaSuccess) cudaGetLastError();
        bool ok = pe == cudaSuccess && (at.type == cudaMemoryTypeManaged ||
                                        (at.type == cudaMemoryTypeDevice && at.device == device));
        if (!ok) {
            noalloc_msg(err, err_len, "vkc_scan_add_i64_noalloc: `in` and `out` must be device or managed "
                                      "memory of device " + std::to_string(device));
            return VKC_USAGE;
        }
    }
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
    int sms;
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
            int sms = 0;
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
            if (e != cudaSuccess || sms < 1) {
                cudaGetLastError();
                return done(VKC_DEVICE, std::string("vkc_scan_add_i64_noalloc: cannot read the SM count: ") +
                                            cudaGetErrorString(e));
            }
            g_noalloc_sms[device] = sms;
            g_noalloc_ptr[device] = static_cast<unsigned char *>(p);
        }
        base = g_noalloc_ptr[device];
        sms = g_noalloc_sms[device];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int tiles = static_cast<int>((n + SC_TILE - 1) / SC_TILE);
    unsigned *counters = reinterpret_cast<unsigned *>(base);
    DevStatus *status = reinterpret_cast<DevStatus *>(base + 256);
    ScanState *state = reinterpret_cast<ScanState *>(base + 256 + sizeof(DevStatus));
    auto *recs = reinterpret_cast<ulonglong2 *>(base + NOALLOC_HEADER);
    // The header and the records of this call's tiles start at zero; with clean records one
    // epoch value serves every call.
    cudaError_t e = cudaMemsetAsync(base, 0, NOALLOC_HEADER, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(recs, 0, static_cast<size_t>(tiles) * REC_STRIDE, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return done(VKC_DEVICE, std::string("vkc_scan_add_i64_noalloc: ") + cudaGetErrorString(e));
    }
    launch_scan<false>(device, sms, s, reinterpret_cast<const unsigned long long *>(in), nullptr,
                       reinterpret_cast<unsigned long long *>(out), n, tiles, recs, 1u, state, counters, status);
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

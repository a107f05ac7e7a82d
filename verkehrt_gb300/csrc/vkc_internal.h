// Internal declarations shared by the runtime (runtime.cu) and the kernel families (k_*.cu).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/vkcuda.h"
#include "tuning.h"

namespace vkc {

// Bytes per row of each element type (src/value.rs:47-55, ScalarType::width).
inline int type_width(vkc_type t) {
    switch (t) {
    case VKC_F64: case VKC_I64: case VKC_U64: return 8;
    case VKC_F32: case VKC_I32: return 4;
    default: return 1;
    }
}

// ScalarType::name, src/value.rs:57-71.
inline const char *type_name(vkc_type t) {
    switch (t) {
    case VKC_F64: return "f64";
    case VKC_F32: return "f32";
    case VKC_I64: return "i64";
    case VKC_U64: return "u64";
    case VKC_I32: return "i32";
    case VKC_U8: return "u8";
    default: return "bool";
    }
}

// The context's own stream, shared by the context and every allocation freed on it, so the
// stream outlives the context while arrays, reducers or scanners of that context live on. It
// also caches freed array blocks by size class: every use of a block is ordered on this one
// stream, so a block freed by one statement can serve the next without a driver call or a new
// mapping of pages.
struct StreamBox {
    cudaStream_t stream = nullptr;
    int device = 0;
    std::multimap<size_t, void *> free_blocks;  // size class -> block
    size_t cached = 0;
    size_t limit = size_t(48) << 30;  // cached bytes at most (vkc_set_cache_limit)
    std::mutex mu;
    ~StreamBox();
    // A block of at least `bytes` (its class size in *cls), or nullptr.
    void *take(size_t bytes, size_t *cls);
    // Returns a block of class size `cls` to the cache (or frees it past the cache limit).
    void give(void *p, size_t cls);
    // Frees every cached block.
    void release_all();
};

// The size class of an allocation: 256-byte multiples below 1 MiB, then 2 MiB multiples.
inline size_t size_class(size_t bytes) {
    if (bytes < (size_t(1) << 20)) return (bytes + 255) & ~size_t(255);
    return (bytes + (size_t(2) << 20) - 1) & ~((size_t(2) << 20) - 1);
}

// A device allocation freed stream-ordered on its context's stream, whenever it goes.
struct DeviceMem {
    void *ptr = nullptr;
    std::shared_ptr<StreamBox> box;
    ~DeviceMem();
};

// A device allocation shared by an array and its views. Copies on the context's copy streams
// leave events here: `pending` until an upload has written the buffer, `reading` until an
// asynchronous download has read it. Work on the context stream waits for them when it first
// reads (pending) or writes (both) the buffer, and the buffer returns to the cache after them.
struct Buffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    std::shared_ptr<StreamBox> box;
    cudaEvent_t pending = nullptr;
    cudaEvent_t reading = nullptr;
    ~Buffer();
};

}  // namespace vkc

struct vkc_array {
    std::atomic<int> refs{1};
    std::shared_ptr<vkc::Buffer> buf;
    int64_t offset = 0;  // rows into buf
    int64_t len = 0;
    vkc_type type = VKC_F64;
    void *data() const {
        return buf && buf->ptr ? static_cast<char *>(buf->ptr) + offset * vkc::type_width(type)
                               : nullptr;
    }
};

// An asynchronous download in flight: the array it reads and the copy's completion event.
struct vkc_copy {
    vkc_array *array;
    cudaEvent_t done;
};

namespace vkc {

// Lookback and reduction scratch. One arena per context: kernels on the context stream run
// one after another, so consecutive launches may reuse it.
struct Scratch {
    void *ptr = nullptr;
    size_t bytes = 0;
};

// Device-side status word, written by kernels on a detected error (an out-of-range index, a
// wait that ran out). Positions are row indices of the offending input element.
struct DevStatus {
    unsigned long long first_bad;  // min offending row, ~0 when none
    unsigned int timeout;          // a bounded spin gave up
    unsigned int spin_limit;       // polls of a wait on another block (0: SPIN_LIMIT)
};

}  // namespace vkc

struct vkc_ctx {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    std::shared_ptr<vkc::StreamBox> box;  // owns own_stream
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    std::string err;
    uint64_t launches = 0;
    // Epoch tag of lookback flags: a flag word written by an earlier launch never matches.
    uint32_t epoch = 0;
    vkc::Scratch scratch;
    // Lookback flag words, written only as epoch<<2 | state, so a word from another launch
    // never reads as ready.
    vkc::Scratch flags;
    // Device status and the counters that last-block-done reductions reset on exit.
    vkc::DevStatus *status = nullptr;
    unsigned int *counters = nullptr;  // [0] ticket, [1] done; zero between launches
    // Pinned host copy of the status word (its own buffer: never shared with results).
    vkc::DevStatus *status_host = nullptr;
    // Pinned host staging for small results.
    void *pinned = nullptr;
    size_t pinned_bytes = 0;
    // Pinned chunk buffers of file ingestion (two of 32 MiB) and their copy events.
    void *io_buf = nullptr;
    cudaEvent_t io_ev[2] = {nullptr, nullptr};
    // Launch shapes per size class: the committed autotuner table, or overrides.
    vkc::Tuning tuning = vkc::tune_defaults();
    // Test hooks (vkc_tune_set "spin_limit" / "fail_alloc_after"): the polls a wait on another
    // block may take (0: the built-in limit), and the number of array allocations that succeed
    // before the next one reports failure (-1: none fails).
    unsigned spin_limit = 0;
    int64_t fail_alloc_after = -1;
    // Copy streams (made on first use): uploads of at least 1 MiB, and asynchronous downloads,
    // so that copies in both directions overlap each other and the kernels.
    cudaStream_t h2d = nullptr, d2h = nullptr;
};

namespace vkc {

constexpr int kCounterSlots = 64;

// Runs `setup` (per-device function attributes such as the dynamic shared memory limit) the
// first time a call site reaches it on a device. The bit is set after the setup, so a thread
// that finds it set knows the setup is done; racing threads may both run it, which is harmless.
template <class F> inline void once_per_device(std::atomic<unsigned long long> &seen, int device, F setup) {
    const unsigned long long bit = 1ull << (device & 63);
    if (seen.load(std::memory_order_acquire) & bit) return;
    setup();
    seen.fetch_or(bit, std::memory_order_release);
}

// The tuned value of knob k for a call over n rows.
inline int tune(const vkc_ctx *ctx, TuneKnob k, int64_t n) { return ctx->tuning.v[k][tune_class(n)]; }

// Status helpers. `fail` records the message and returns the status.
vkc_status fail(vkc_ctx *ctx, vkc_status st, const std::string &msg);
vkc_status cuda_fail(vkc_ctx *ctx, cudaError_t e, const char *what);
#define VKC_CUDA(ctx, call)                                          \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return ::vkc::cuda_fail(ctx, e_, #call); \
    } while (0)

// Scratch of at least `bytes`, 256-byte aligned. The pointer stays valid until the next call.
vkc_status scratch(vkc_ctx *ctx, size_t bytes, void **out);
// `count` epoch-tagged lookback flag words (see vkc_ctx::flags).
vkc_status flag_arena(vkc_ctx *ctx, size_t count, unsigned **out);
// Pinned host staging of at least `bytes`.
vkc_status pinned(vkc_ctx *ctx, size_t bytes, void **out);
// Next lookback epoch (1..2^24-1). Wraps by clearing the flag arena.
uint32_t next_epoch(vkc_ctx *ctx);
// Reads and clears the device status after the stream's work completes.
vkc_status read_status(vkc_ctx *ctx, DevStatus *out);
// Orders the context stream after the copies of an array's buffer: before it reads the array
// (an upload in flight), or writes it (an upload or an asynchronous download in flight).
void await_read(vkc_ctx *ctx, const vkc_array *a);
void await_write(vkc_ctx *ctx, const vkc_array *a);
void await_values(vkc_ctx *ctx, const vkc_value *args, int nargs);
// Checks a kernel launch and counts it.
vkc_status launched(vkc_ctx *ctx, const char *what);

// New array of `len` rows (uninitialised unless `zero`). Message texts follow
// src/value.rs:285-307.
vkc_status new_array(vkc_ctx *ctx, vkc_type t, int64_t len, bool zero, vkc_array **out);
// Shrinks an array's logical length (the allocation stays).
inline void set_len(vkc_array *a, int64_t len) { a->len = len; }

// Grid size for a streaming kernel: a multiple of the SM count, at most enough blocks to give
// every block `min_items` items.
int stream_grid(const vkc_ctx *ctx, int64_t items, int block, int per_sm, int64_t min_items);

}  // namespace vkc

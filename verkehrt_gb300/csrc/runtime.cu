// Context, arrays, scratch and the Dispatch mirror of the `cuda` ISA.
//
// vkc_call restates Dispatch::call (src/kernels/dispatch.rs:56-142) and prepare
// (:296-322); the tile entries restate Dispatch::reducer / scanner / elementwise_tile /
// select_tile (:156-265). Error texts are the reference's.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "registry.h"

namespace vkc {

StreamBox::~StreamBox() {
    if (stream) {
        int prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(device);
        for (auto &kv : free_blocks) cudaFreeAsync(kv.second, stream);
        free_blocks.clear();
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
        cudaSetDevice(prev);
    }
}

void *StreamBox::take(size_t bytes, size_t *cls) {
    *cls = size_class(bytes);
    std::lock_guard<std::mutex> lock(mu);
    // The smallest cached block of the class or up to a quarter larger.
    auto it = free_blocks.lower_bound(*cls);
    if (it == free_blocks.end() || it->first > *cls + *cls / 4) return nullptr;
    void *p = it->second;
    *cls = it->first;
    cached -= it->first;
    free_blocks.erase(it);
    return p;
}

void StreamBox::release_all() {
    std::lock_guard<std::mutex> lock(mu);
    for (auto &kv : free_blocks) cudaFreeAsync(kv.second, stream);
    free_blocks.clear();
    cached = 0;
}

void StreamBox::give(void *p, size_t cls) {
    {
        std::lock_guard<std::mutex> lock(mu);
        if (cached + cls <= limit) {
            free_blocks.emplace(cls, p);
            cached += cls;
            return;
        }
    }
    cudaFreeAsync(p, stream);
}

DeviceMem::~DeviceMem() {
    if (ptr && box) cudaFreeAsync(ptr, box->stream);
}

Buffer::~Buffer() {
    // The cached block is reused in the order of the box's stream: after the copies.
    for (cudaEvent_t *e : {&pending, &reading})
        if (*e) {
            if (box) cudaStreamWaitEvent(box->stream, *e, 0);
            cudaEventDestroy(*e);
        }
    if (ptr && box) box->give(ptr, bytes);
}

// Makes `stream` wait for *e (once), then drops the event. Under graph capture an event from
// outside the capture cannot be waited on by the stream, so the host waits for it instead.
static bool stream_capturing(cudaStream_t stream);
// A host wait for an event, allowed during this thread's stream capture.
static void host_wait(cudaEvent_t e) {
    cudaStreamCaptureMode mode = cudaStreamCaptureModeRelaxed;
    cudaThreadExchangeStreamCaptureMode(&mode);
    cudaEventSynchronize(e);
    cudaThreadExchangeStreamCaptureMode(&mode);
}
static void take_event(cudaStream_t stream, cudaEvent_t *e) {
    if (!*e) return;
    if (stream_capturing(stream))
        host_wait(*e);
    else
        cudaStreamWaitEvent(stream, *e, 0);
    cudaEventDestroy(*e);
    *e = nullptr;
}

void await_read(vkc_ctx *ctx, const vkc_array *a) {
    if (a && a->buf) take_event(ctx->stream, &a->buf->pending);
}

void await_write(vkc_ctx *ctx, const vkc_array *a) {
    if (!a || !a->buf) return;
    take_event(ctx->stream, &a->buf->pending);
    take_event(ctx->stream, &a->buf->reading);
}

void await_values(vkc_ctx *ctx, const vkc_value *args, int nargs) {
    for (int i = 0; i < nargs; ++i)
        if (args[i].kind == VKC_VALUE_ARRAY && args[i].array) await_read(ctx, args[i].array);
}

static bool stream_capturing(cudaStream_t stream) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

// The copy streams, made on first use.
static vkc_status copy_streams(vkc_ctx *ctx) {
    if (!ctx->h2d) VKC_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->h2d, cudaStreamNonBlocking));
    if (!ctx->d2h) VKC_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->d2h, cudaStreamNonBlocking));
    return VKC_OK;
}

// An event recorded on `stream` now.
static vkc_status mark(vkc_ctx *ctx, cudaStream_t stream, cudaEvent_t *e) {
    VKC_CUDA(ctx, cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    VKC_CUDA(ctx, cudaEventRecord(*e, stream));
    return VKC_OK;
}

vkc_status fail(vkc_ctx *ctx, vkc_status st, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return st;
}

vkc_status cuda_fail(vkc_ctx *ctx, cudaError_t e, const char *what) {
    char buf[512];
    snprintf(buf, sizeof buf, "CUDA error %s (%s) in %s", cudaGetErrorName(e),
             cudaGetErrorString(e), what);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(ctx, VKC_ALLOC, buf);
    }
    return fail(ctx, VKC_DEVICE, buf);
}

// Arenas are freed and made again when they grow, which a captured graph could not replay: a
// capture fails instead (growing needs a call of the same size outside the capture first).
static const char *const GROW_IN_CAPTURE =
    "the scratch arena would grow during a capture: make the call once before capturing";

vkc_status scratch(vkc_ctx *ctx, size_t bytes, void **out) {
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes > ctx->scratch.bytes) {
        if (stream_capturing(ctx->stream)) return fail(ctx, VKC_USAGE, GROW_IN_CAPTURE);
        if (ctx->scratch.ptr) VKC_CUDA(ctx, cudaFreeAsync(ctx->scratch.ptr, ctx->stream));
        ctx->scratch.ptr = nullptr;
        ctx->scratch.bytes = 0;
        size_t want = bytes < (size_t(1) << 20) ? (size_t(1) << 20) : bytes + bytes / 4;
        VKC_CUDA(ctx, cudaMallocAsync(&ctx->scratch.ptr, want, ctx->stream));
        ctx->scratch.bytes = want;
    }
    *out = ctx->scratch.ptr;
    return VKC_OK;
}

vkc_status flag_arena(vkc_ctx *ctx, size_t count, unsigned **out) {
    size_t bytes = (count * sizeof(unsigned) + 255) & ~size_t(255);
    if (bytes > ctx->flags.bytes) {
        if (stream_capturing(ctx->stream)) return fail(ctx, VKC_USAGE, GROW_IN_CAPTURE);
        if (ctx->flags.ptr) VKC_CUDA(ctx, cudaFreeAsync(ctx->flags.ptr, ctx->stream));
        ctx->flags.ptr = nullptr;
        ctx->flags.bytes = 0;
        size_t want = bytes < (size_t(1) << 16) ? (size_t(1) << 16) : bytes + bytes / 4;
        VKC_CUDA(ctx, cudaMallocAsync(&ctx->flags.ptr, want, ctx->stream));
        VKC_CUDA(ctx, cudaMemsetAsync(ctx->flags.ptr, 0, want, ctx->stream));
        ctx->flags.bytes = want;
    }
    *out = static_cast<unsigned *>(ctx->flags.ptr);
    return VKC_OK;
}

vkc_status pinned(vkc_ctx *ctx, size_t bytes, void **out) {
    if (bytes > ctx->pinned_bytes) {
        if (ctx->pinned) {
            VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            cudaFreeHost(ctx->pinned);
        }
        ctx->pinned = nullptr;
        ctx->pinned_bytes = 0;
        size_t want = bytes < 4096 ? 4096 : bytes;
        VKC_CUDA(ctx, cudaMallocHost(&ctx->pinned, want));
        ctx->pinned_bytes = want;
    }
    *out = ctx->pinned;
    return VKC_OK;
}

uint32_t next_epoch(vkc_ctx *ctx) {
    // 24 bits: packed lookback words keep the epoch in their top 24 bits.
    ctx->epoch = (ctx->epoch + 1) & 0xffffffu;
    if (ctx->epoch == 0) {
        if (ctx->flags.ptr)
            cudaMemsetAsync(ctx->flags.ptr, 0, ctx->flags.bytes, ctx->stream);
        ctx->epoch = 1;
    }
    return ctx->epoch;
}

vkc_status read_status(vkc_ctx *ctx, DevStatus *out) {
    VKC_CUDA(ctx, cudaMemcpyAsync(ctx->status_host, ctx->status, sizeof(DevStatus),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    memcpy(out, ctx->status_host, sizeof(DevStatus));
    if (out->first_bad != ~0ull || out->timeout) {
        DevStatus clean{~0ull, 0, ctx->spin_limit};
        VKC_CUDA(ctx, cudaMemcpyAsync(ctx->status, &clean, sizeof clean, cudaMemcpyHostToDevice,
                                      ctx->stream));
        VKC_CUDA(ctx, cudaMemsetAsync(ctx->counters, 0, kCounterSlots * sizeof(unsigned),
                                      ctx->stream));
        VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    if (out->timeout) return fail(ctx, VKC_TIMEOUT, "a device-side wait gave up");
    return VKC_OK;
}

vkc_status launched(vkc_ctx *ctx, const char *what) {
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, what);
    return VKC_OK;
}

vkc_status new_array(vkc_ctx *ctx, vkc_type t, int64_t len, bool zero, vkc_array **out) {
    *out = nullptr;
    uint64_t w = static_cast<uint64_t>(type_width(t));
    // value.rs:285-289 (Array::byte_size): the size must fit in isize.
    if (len < 0 || static_cast<uint64_t>(len) > static_cast<uint64_t>(INT64_MAX) / w)
        return fail(ctx, VKC_RUNTIME, "array of " + std::to_string(static_cast<uint64_t>(len)) +
                                          " elements is too large");
    size_t bytes = static_cast<size_t>(len) * w;
    if (ctx->fail_alloc_after >= 0 && ctx->fail_alloc_after-- == 0)  // test hook: an injected failure
        return fail(ctx, VKC_ALLOC, "cannot allocate an array of " + std::to_string(len) + " elements");
    auto buf = std::make_shared<Buffer>();
    buf->box = ctx->box;
    if (bytes) {
        // Whole size classes, so vector kernels may read the last 16 bytes of any allocation.
        size_t cls = 0;
        buf->ptr = ctx->box->take(bytes, &cls);
        if (!buf->ptr) {
            cudaError_t e = cudaMallocAsync(&buf->ptr, cls, ctx->stream);
            if (e != cudaSuccess) {
                // Give the cached blocks back to the pool and try once more.
                cudaGetLastError();
                ctx->box->release_all();
                cudaStreamSynchronize(ctx->stream);
                e = cudaMallocAsync(&buf->ptr, cls, ctx->stream);
            }
            if (e != cudaSuccess) {
                cudaGetLastError();
                buf->ptr = nullptr;
                // value.rs:297-307 (try_zeroed).
                return fail(ctx, VKC_ALLOC,
                            "cannot allocate an array of " + std::to_string(len) + " elements");
            }
        }
        buf->bytes = cls;
        if (zero) VKC_CUDA(ctx, cudaMemsetAsync(buf->ptr, 0, cls, ctx->stream));
    }
    vkc_array *a = new vkc_array;
    a->buf = std::move(buf);
    a->offset = 0;
    a->len = len;
    a->type = t;
    *out = a;
    return VKC_OK;
}

int stream_grid(const vkc_ctx *ctx, int64_t items, int block, int per_sm, int64_t min_items) {
    int64_t full = static_cast<int64_t>(ctx->sms) * per_sm;
    int64_t want = (items + min_items - 1) / min_items;
    if (want < 1) want = 1;
    if (want < full) return static_cast<int>(want);
    (void)block;
    return static_cast<int>(full);
}

vkc_status Builder::reserve(int64_t more, void **at) {
    int w = type_width(type);
    if (len + more > cap) {
        int64_t ncap = cap * 2 > len + more ? cap * 2 : len + more;
        vkc_array *na;
        vkc_status st = new_array(ctx, type, ncap, false, &na);
        if (st) return st;
        if (len)
            VKC_CUDA(ctx, cudaMemcpyAsync(na->buf->ptr, buf->ptr, static_cast<size_t>(len) * w,
                                          cudaMemcpyDeviceToDevice, ctx->stream));
        buf = na->buf;
        cap = ncap;
        delete na;
    }
    *at = buf ? static_cast<char *>(buf->ptr) + static_cast<size_t>(len) * w : nullptr;
    return VKC_OK;
}

// ------------------------------------------------------------------ argument helpers

std::string arity_error(int want, int got) {
    return "expected " + std::to_string(want) + " arguments, got " + std::to_string(got);
}

std::string value_type_name(const Arg &a) {
    return a.rows ? std::string(type_name(a.a->type)) + "[]" : std::string(type_name(a.s.type));
}

std::string value_type_name(const vkc_value &v) {
    if (v.kind == VKC_VALUE_STR) return "str";
    return v.kind == VKC_VALUE_ARRAY ? std::string(type_name(v.array->type)) + "[]"
                                     : std::string(type_name(v.scalar.type));
}

bool rows_arg(vkc_ctx *ctx, const Arg &a, vkc_type t, vkc_status *st) {
    if (a.rows && a.a->type == t) return true;
    *st = fail(ctx, VKC_RUNTIME,
               std::string("expected ") + type_name(t) + "[], got " + value_type_name(a));
    return false;
}

bool splat_arg(vkc_ctx *ctx, const Arg &a, vkc_type t, vkc_status *st) {
    if (!a.rows && a.s.type == t) return true;
    *st = fail(ctx, VKC_RUNTIME,
               std::string("expected ") + type_name(t) + ", got " + value_type_name(a));
    return false;
}

bool array_arg(vkc_ctx *ctx, const vkc_value &v, vkc_type t, vkc_status *st) {
    if (v.kind == VKC_VALUE_ARRAY && v.array && v.array->type == t) return true;
    *st = fail(ctx, VKC_RUNTIME,
               std::string("expected ") + type_name(t) + "[], got " + value_type_name(v));
    return false;
}

bool i64_arg(vkc_ctx *ctx, const vkc_value &v, int64_t *out, vkc_status *st) {
    if (v.kind == VKC_VALUE_SCALAR && v.scalar.type == VKC_I64) {
        *out = static_cast<int64_t>(v.scalar.bits);
        return true;
    }
    *st = fail(ctx, VKC_RUNTIME, "expected i64, got " + value_type_name(v));
    return false;
}

// ------------------------------------------------------------------ registry

static const std::vector<KernelDef> &table() {
    static std::vector<KernelDef> t = [] {
        std::vector<KernelDef> v;
        register_construct(v);
        register_reduce(v);
        register_select(v);
        register_scan(v);
        register_index(v);
        register_sort(v);
        register_group(v);
        register_elementwise(v);
        register_io(v);
        register_reduce_into_f64(v);
        register_families(v);
        return v;
    }();
    return t;
}

static const KernelDef *def_of(int id) {
    const auto &t = table();
    if (id < 0 || id >= static_cast<int>(t.size())) return nullptr;
    return &t[static_cast<size_t>(id)];
}

const KernelDef *kernel_def(const char *name) {
    for (const KernelDef &d : table())
        if (d.name == name) return &d;
    return nullptr;
}

// kind_error, src/kernels/dispatch.rs:324-330.
static std::string kind_error(const InSpec &spec, const std::string &got) {
    switch (spec.kind) {
    case IN_STR: return "expected str, got " + got;
    case IN_ARRAY: return std::string("expected ") + type_name(spec.type) + "[], got " + got;
    case IN_SCALAR: return std::string("expected ") + type_name(spec.type) + ", got " + got;
    default:
        return std::string("expected ") + type_name(spec.type) + " or " + type_name(spec.type) +
               "[], got " + got;
    }
}

static bool spec_accepts(const InSpec &spec, const vkc_value &v) {
    if (v.kind == VKC_VALUE_STR || spec.kind == IN_STR) return v.kind == VKC_VALUE_STR && spec.kind == IN_STR;
    bool arr = v.kind == VKC_VALUE_ARRAY;
    vkc_type t = arr ? v.array->type : v.scalar.type;
    if (t != spec.type) return false;
    return spec.kind == IN_EITHER || (spec.kind == IN_ARRAY) == arr;
}

// prepare, src/kernels/dispatch.rs:296-322: argument kinds, then the common row count.
static vkc_status prepare(vkc_ctx *ctx, const KernelDef &d, const vkc_value *args, int nargs,
                          std::vector<Arg> *call, int64_t *rows) {
    if (static_cast<int>(d.inputs.size()) != nargs)
        return fail(ctx, VKC_USAGE, arity_error(static_cast<int>(d.inputs.size()), nargs));
    *rows = -1;
    call->clear();
    for (int i = 0; i < nargs; ++i) {
        const vkc_value &v = args[i];
        if (v.kind == VKC_VALUE_ARRAY && !v.array)
            return fail(ctx, VKC_USAGE, "null array handle");
        if (!spec_accepts(d.inputs[static_cast<size_t>(i)], v))
            return fail(ctx, VKC_USAGE, kind_error(d.inputs[static_cast<size_t>(i)],
                                                   value_type_name(v)));
        Arg a;
        a.rows = v.kind == VKC_VALUE_ARRAY;
        a.a = v.array;
        a.s = v.scalar;
        if (a.rows) {
            if (*rows >= 0 && *rows != a.a->len)
                return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(*rows) +
                                                  " vs " + std::to_string(a.a->len));
            *rows = a.a->len;
        }
        call->push_back(a);
    }
    return VKC_OK;
}

// KernelDef::accepts (src/kernels.rs:382-397): elementwise kernels with an Either operand need
// an array operand.
static bool needs_array(const KernelDef &d) {
    if (d.cls != VKC_ELEMENTWISE) return false;
    for (const auto &s : d.inputs)
        if (s.kind == IN_EITHER) return true;
    return false;
}

static vkc_status finish_builder(Builder &b, vkc_array **out) {
    vkc_array *a = new vkc_array;
    a->type = b.type;
    a->len = b.len;
    a->offset = 0;
    int w = type_width(b.type);
    // A selection reserves for every row of its input; keep at most a quarter of slack.
    if (b.buf && b.len * 4 < b.cap) {
        vkc_array *na;
        vkc_status st = new_array(b.ctx, b.type, b.len, false, &na);
        if (st) {
            delete a;
            return st;
        }
        if (b.len)
            VKC_CUDA(b.ctx, cudaMemcpyAsync(na->buf->ptr, b.buf->ptr, static_cast<size_t>(b.len) * w,
                                            cudaMemcpyDeviceToDevice, b.ctx->stream));
        a->buf = na->buf;
        delete na;
    } else {
        a->buf = b.buf ? b.buf : std::make_shared<Buffer>();
    }
    *out = a;
    return VKC_OK;
}

}  // namespace vkc

using namespace vkc;

struct vkc_reducer {
    vkc_ctx *ctx;
    ReducerImpl *impl;
};
struct vkc_scanner {
    vkc_ctx *ctx;
    ScannerImpl *impl;
};
struct vkc_builder {
    Builder b;
};

extern "C" {

vkc_status vkc_open(int device, vkc_ctx **out) {
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        return VKC_DEVICE;
    }
    vkc_ctx *ctx = new vkc_ctx;
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->ev_start) != cudaSuccess ||
        cudaEventCreate(&ctx->ev_stop) != cudaSuccess) {
        cudaGetLastError();
        delete ctx;
        return VKC_DEVICE;
    }
    ctx->stream = ctx->own_stream;
    ctx->box = std::make_shared<StreamBox>();
    ctx->box->stream = ctx->own_stream;
    ctx->box->device = device;
    // Freed blocks stay in the device pool, so per-statement allocations are cheap.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    void *p = nullptr;
    if (cudaMalloc(&p, sizeof(DevStatus) + kCounterSlots * sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        delete ctx;
        return VKC_DEVICE;
    }
    ctx->status = static_cast<DevStatus *>(p);
    if (cudaMallocHost(reinterpret_cast<void **>(&ctx->status_host), sizeof(DevStatus)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(p);
        delete ctx;
        return VKC_DEVICE;
    }
    ctx->counters = reinterpret_cast<unsigned *>(static_cast<char *>(p) + sizeof(DevStatus));
    DevStatus clean{~0ull, 0, 0};
    cudaMemcpy(ctx->status, &clean, sizeof clean, cudaMemcpyHostToDevice);
    cudaMemset(ctx->counters, 0, kCounterSlots * sizeof(unsigned));
    *out = ctx;
    return VKC_OK;
}

void vkc_close(vkc_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    for (cudaStream_t cs : {ctx->h2d, ctx->d2h})
        if (cs) {
            cudaStreamSynchronize(cs);
            cudaStreamDestroy(cs);
        }
    cudaStreamSynchronize(ctx->stream);
    if (ctx->scratch.ptr) cudaFreeAsync(ctx->scratch.ptr, ctx->stream);
    if (ctx->flags.ptr) cudaFreeAsync(ctx->flags.ptr, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->status) cudaFree(ctx->status);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->status_host) cudaFreeHost(ctx->status_host);
    if (ctx->io_buf) cudaFreeHost(ctx->io_buf);
    for (cudaEvent_t e : ctx->io_ev)
        if (e) cudaEventDestroy(e);
    cudaEventDestroy(ctx->ev_start);
    cudaEventDestroy(ctx->ev_stop);
    // The stream goes with the last allocation that still refers to it.
    ctx->box.reset();
    delete ctx;
}

const char *vkc_last_error(const vkc_ctx *ctx) { return ctx ? ctx->err.c_str() : ""; }

vkc_status vkc_set_cache_limit(vkc_ctx *ctx, size_t bytes) {
    if (!ctx || !ctx->box) return VKC_USAGE;
    bool drop;
    {
        std::lock_guard<std::mutex> lock(ctx->box->mu);
        ctx->box->limit = bytes;
        drop = ctx->box->cached > bytes;
    }
    if (drop) ctx->box->release_all();
    return VKC_OK;
}

vkc_status vkc_tune_set(vkc_ctx *ctx, const char *knob, int size_class, int value) {
    if (!ctx || !knob || size_class < 0 || size_class >= TUNE_CLASSES) return VKC_USAGE;
    // Test hooks, the same for every size class.
    const bool never = std::string(knob) == "lookback_never_ready";
    if (std::string(knob) == "spin_limit" || never) {
        if (value < 0 || (never && value > 1))
            return fail(ctx, VKC_USAGE, "value " + std::to_string(value) + " not allowed for " + knob);
        const unsigned flag = 1u << 31;
        if (never) ctx->spin_limit = (ctx->spin_limit & ~flag) | (value ? flag : 0u);
        else ctx->spin_limit = (ctx->spin_limit & flag) | static_cast<unsigned>(value);
        // The status word carries it to the kernels; a context stream is idle between calls.
        VKC_CUDA(ctx, cudaMemcpyAsync(&ctx->status->spin_limit, &ctx->spin_limit, sizeof(unsigned),
                                      cudaMemcpyHostToDevice, ctx->stream));
        VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return VKC_OK;
    }
    if (std::string(knob) == "fail_alloc_after") {
        if (value < -1)
            return fail(ctx, VKC_USAGE, "value " + std::to_string(value) + " not allowed for fail_alloc_after");
        ctx->fail_alloc_after = value;
        return VKC_OK;
    }
    for (int k = 0; k < TK_COUNT; ++k) {
        if (std::string(knob) != tune_knob_name(k)) continue;
        if (!tune_allowed(k, value))
            return fail(ctx, VKC_USAGE, std::string("value ") + std::to_string(value) + " not allowed for " + knob);
        ctx->tuning.v[k][size_class] = value;
        return VKC_OK;
    }
    return fail(ctx, VKC_USAGE, std::string("no tuning knob ") + knob);
}

vkc_status vkc_tune_get(const vkc_ctx *ctx, const char *knob, int size_class, int *value) {
    if (!ctx || !knob || !value || size_class < 0 || size_class >= TUNE_CLASSES) return VKC_USAGE;
    if (std::string(knob) == "spin_limit") {
        *value = static_cast<int>(ctx->spin_limit & ~(1u << 31));
        return VKC_OK;
    }
    if (std::string(knob) == "lookback_never_ready") {
        *value = static_cast<int>(ctx->spin_limit >> 31);
        return VKC_OK;
    }
    if (std::string(knob) == "fail_alloc_after") {
        *value = static_cast<int>(ctx->fail_alloc_after);
        return VKC_OK;
    }
    for (int k = 0; k < TK_COUNT; ++k)
        if (std::string(knob) == tune_knob_name(k)) {
            *value = ctx->tuning.v[k][size_class];
            return VKC_OK;
        }
    return VKC_USAGE;
}

vkc_status vkc_synchronize(vkc_ctx *ctx) {
    VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->h2d) VKC_CUDA(ctx, cudaStreamSynchronize(ctx->h2d));
    if (ctx->d2h) VKC_CUDA(ctx, cudaStreamSynchronize(ctx->d2h));
    if (stream_capturing(ctx->stream)) return VKC_OK;
    DevStatus ds;
    return read_status(ctx, &ds);
}

vkc_status vkc_set_stream(vkc_ctx *ctx, void *stream) {
    ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    return VKC_OK;
}

void *vkc_get_stream(const vkc_ctx *ctx) { return ctx->stream; }

uint64_t vkc_launch_count(const vkc_ctx *ctx) { return ctx->launches; }

vkc_status vkc_timer_start(vkc_ctx *ctx) {
    VKC_CUDA(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
    return VKC_OK;
}

vkc_status vkc_timer_stop(vkc_ctx *ctx, float *ms) {
    VKC_CUDA(ctx, cudaEventRecord(ctx->ev_stop, ctx->stream));
    VKC_CUDA(ctx, cudaEventSynchronize(ctx->ev_stop));
    VKC_CUDA(ctx, cudaEventElapsedTime(ms, ctx->ev_start, ctx->ev_stop));
    return VKC_OK;
}

vkc_status vkc_array_new(vkc_ctx *ctx, vkc_type type, int64_t len, vkc_array **out) {
    return new_array(ctx, type, len, true, out);
}

vkc_status vkc_array_upload(vkc_ctx *ctx, vkc_type type, const void *host, int64_t len,
                            vkc_array **out) {
    vkc_status st = new_array(ctx, type, len, false, out);
    if (st) return st;
    const size_t bytes = static_cast<size_t>(len) * type_width(type);
    if (bytes >= (size_t(1) << 20) && !stream_capturing(ctx->stream) && !copy_streams(ctx)) {
        // On the upload stream, after the buffer's allocation (ordered on the context stream);
        // the first kernel that reads the array waits for the copy's event.
        cudaEvent_t ready;
        if ((st = mark(ctx, ctx->stream, &ready))) return st;
        cudaStreamWaitEvent(ctx->h2d, ready, 0);
        cudaEventDestroy(ready);
        VKC_CUDA(ctx, cudaMemcpyAsync((*out)->data(), host, bytes, cudaMemcpyHostToDevice, ctx->h2d));
        return mark(ctx, ctx->h2d, &(*out)->buf->pending);
    }
    if (len) VKC_CUDA(ctx, cudaMemcpyAsync((*out)->data(), host, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return VKC_OK;
}

vkc_status vkc_array_download(vkc_ctx *ctx, const vkc_array *a, void *host, int64_t capacity) {
    if (!a) return fail(ctx, VKC_USAGE, "null array handle");
    int64_t n = a->len < capacity ? a->len : capacity;
    await_read(ctx, a);
    if (n > 0)
        VKC_CUDA(ctx, cudaMemcpyAsync(host, a->data(), static_cast<size_t>(n) * type_width(a->type),
                                      cudaMemcpyDeviceToHost, ctx->stream));
    VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // A wait of earlier enqueued work that ran out (its call did not wait for the device).
    DevStatus ds;
    return read_status(ctx, &ds);
}

vkc_status vkc_array_download_start(vkc_ctx *ctx, const vkc_array *a, void *host, int64_t capacity, vkc_copy **out) {
    if (!out) return VKC_USAGE;
    *out = nullptr;
    if (!a) return fail(ctx, VKC_USAGE, "null array handle");
    if (stream_capturing(ctx->stream)) return fail(ctx, VKC_USAGE, "vkc_array_download_start during a stream capture");
    vkc_status st;
    if ((st = copy_streams(ctx))) return st;
    // After the kernels queued so far (which made the array) and any upload into it.
    cudaEvent_t ready;
    if ((st = mark(ctx, ctx->stream, &ready))) return st;
    cudaStreamWaitEvent(ctx->d2h, ready, 0);
    cudaEventDestroy(ready);
    if (a->buf && a->buf->pending) cudaStreamWaitEvent(ctx->d2h, a->buf->pending, 0);
    const int64_t n = a->len < capacity ? a->len : capacity;
    if (n > 0)
        VKC_CUDA(ctx, cudaMemcpyAsync(host, a->data(), static_cast<size_t>(n) * type_width(a->type),
                                      cudaMemcpyDeviceToHost, ctx->d2h));
    auto *c = new vkc_copy{const_cast<vkc_array *>(a), nullptr};
    if ((st = mark(ctx, ctx->d2h, &c->done))) {
        delete c;
        return st;
    }
    if (a->buf) {
        // A later write to the array waits for this read (the copy stream runs in order, so
        // the newest event covers the earlier downloads).
        if (a->buf->reading) cudaEventDestroy(a->buf->reading);
        if ((st = mark(ctx, ctx->d2h, &a->buf->reading))) {
            cudaEventDestroy(c->done);
            delete c;
            return st;
        }
    }
    vkc_array_retain(c->array);
    *out = c;
    return VKC_OK;
}

vkc_status vkc_copy_wait(vkc_ctx *ctx, vkc_copy *c) {
    if (!c) return VKC_USAGE;
    const cudaError_t e = cudaEventSynchronize(c->done);
    cudaEventDestroy(c->done);
    vkc_array_release(c->array);
    delete c;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "vkc_copy_wait");
    return VKC_OK;
}

vkc_status vkc_array_slice(vkc_ctx *ctx, const vkc_array *a, int64_t start, int64_t len,
                           vkc_array **out) {
    *out = nullptr;
    if (!a) return fail(ctx, VKC_USAGE, "null array handle");
    // index.rs:76-93 (run_slice): bounds as start..end within the length.
    if (start < 0 || len < 0 || start > a->len || len > a->len - start)
        return fail(ctx, VKC_RUNTIME, "slice " + std::to_string(start) + ".." +
                                          std::to_string(start + len) + " out of range for length " +
                                          std::to_string(a->len));
    vkc_array *v = new vkc_array;
    v->buf = a->buf;
    v->offset = a->offset + start;
    v->len = len;
    v->type = a->type;
    *out = v;
    return VKC_OK;
}

int64_t vkc_array_len(const vkc_array *a) { return a ? a->len : 0; }
vkc_type vkc_array_type(const vkc_array *a) { return a ? a->type : VKC_F64; }
void *vkc_array_device_ptr(const vkc_array *a) {
    // The address may be used on any stream: an upload in flight finishes first.
    if (a && a->buf && a->buf->pending) host_wait(a->buf->pending);
    return a ? a->data() : nullptr;
}
void vkc_array_retain(vkc_array *a) {
    if (a) a->refs.fetch_add(1);
}
void vkc_array_release(vkc_array *a) {
    if (a && a->refs.fetch_sub(1) == 1) delete a;
}

int vkc_kernel_count(void) { return static_cast<int>(table().size()); }
const char *vkc_kernel_name(int id) {
    const KernelDef *d = def_of(id);
    return d ? d->name.c_str() : nullptr;
}
int vkc_kernel_lookup(const char *name) {
    const auto &t = table();
    for (size_t i = 0; i < t.size(); ++i)
        if (t[i].name == name) return static_cast<int>(i);
    return -1;
}
vkc_class vkc_kernel_class(int id) {
    const KernelDef *d = def_of(id);
    return d ? d->cls : VKC_WHOLE;
}
int vkc_kernel_arity(int id) {
    const KernelDef *d = def_of(id);
    return d ? static_cast<int>(d->inputs.size()) : -1;
}
uint64_t vkc_kernel_cost(int id) {
    const KernelDef *d = def_of(id);
    return d ? d->cost : 0;
}

vkc_status vkc_call(vkc_ctx *ctx, int id, const vkc_value *args, int nargs, vkc_value *out) {
    const KernelDef *d = def_of(id);
    if (!d) return fail(ctx, VKC_USAGE, "unknown kernel id " + std::to_string(id));
    memset(out, 0, sizeof *out);
    await_values(ctx, args, nargs);
    if (d->cls == VKC_WHOLE) {
        // Whole kernels check their arguments themselves (dispatch.rs:69-73).
        if (static_cast<int>(d->inputs.size()) != nargs)
            return fail(ctx, VKC_USAGE, arity_error(static_cast<int>(d->inputs.size()), nargs));
        for (int i = 0; i < nargs; ++i) {
            if (args[i].kind == VKC_VALUE_ARRAY && !args[i].array)
                return fail(ctx, VKC_USAGE, "null array handle");
            if (!spec_accepts(d->inputs[static_cast<size_t>(i)], args[i]))
                return fail(ctx, VKC_USAGE, kind_error(d->inputs[static_cast<size_t>(i)],
                                                       value_type_name(args[i])));
        }
        return d->whole(ctx, args, nargs, out);
    }
    std::vector<Arg> call;
    int64_t rows = -1;
    vkc_status st = prepare(ctx, *d, args, nargs, &call, &rows);
    if (st) return st;
    if (needs_array(*d) && rows < 0)
        return fail(ctx, VKC_USAGE, "an array kernel needs an array operand");
    switch (d->cls) {
    case VKC_ELEMENTWISE: {
        vkc_array *o;
        st = new_array(ctx, d->out_type, rows, false, &o);
        if (st) return st;
        if (rows > 0) st = d->elem(ctx, call.data(), nargs, rows, o);
        if (st) {
            vkc_array_release(o);
            return st;
        }
        out->kind = VKC_VALUE_ARRAY;
        out->array = o;
        return VKC_OK;
    }
    case VKC_REDUCTION: {
        if (rows < 0) return fail(ctx, VKC_USAGE, "a reduction needs an array operand");
        ReducerImpl *r = d->red(ctx);
        if (!r) return ctx->err.empty() ? fail(ctx, VKC_ALLOC, "cannot allocate a reducer") : VKC_ALLOC;
        if (rows > 0) st = r->update(ctx, call.data(), nargs);
        vkc_scalar s{};
        if (!st) st = r->finish(ctx, &s);
        delete r;
        if (st) return st;
        out->kind = VKC_VALUE_SCALAR;
        out->scalar = s;
        return VKC_OK;
    }
    case VKC_SCAN: {
        if (rows < 0) return fail(ctx, VKC_USAGE, "a scan needs an array operand");
        vkc_array *o;
        st = new_array(ctx, d->out_type, rows, false, &o);
        if (st) return st;
        if (rows > 0) {
            ScannerImpl *s = d->scan(ctx);
            st = s ? s->update(ctx, call.data(), nargs, o) : VKC_ALLOC;
            delete s;
        }
        if (st) {
            vkc_array_release(o);
            return st;
        }
        out->kind = VKC_VALUE_ARRAY;
        out->array = o;
        return VKC_OK;
    }
    case VKC_SELECTION: {
        Builder b{ctx, d->out_type, nullptr, 0, 0};
        st = d->sel(ctx, call.data(), nargs, 0, &b);
        if (st) return st;
        vkc_array *o = nullptr;
        st = finish_builder(b, &o);
        if (st) return st;
        out->kind = VKC_VALUE_ARRAY;
        out->array = o;
        return VKC_OK;
    }
    default: return fail(ctx, VKC_USAGE, "unknown kernel class");
    }
}

vkc_status vkc_reducer_new(vkc_ctx *ctx, int id, vkc_reducer **out) {
    *out = nullptr;
    const KernelDef *d = def_of(id);
    if (!d) return fail(ctx, VKC_USAGE, "unknown kernel id " + std::to_string(id));
    if (d->cls != VKC_REDUCTION) return fail(ctx, VKC_USAGE, d->name + " is not a reduction");
    ReducerImpl *r = d->red(ctx);
    if (!r) return VKC_ALLOC;
    *out = new vkc_reducer{ctx, r};
    return VKC_OK;
}

// Tile arguments arrive unchecked (src/kernels.rs:38-45); the entries check kinds and rows.
static void to_args(const vkc_value *args, int nargs, std::vector<Arg> *call) {
    call->clear();
    for (int i = 0; i < nargs; ++i) {
        Arg a;
        a.rows = args[i].kind == VKC_VALUE_ARRAY && args[i].array;
        a.a = args[i].array;
        a.s = args[i].scalar;
        call->push_back(a);
    }
}

vkc_status vkc_reducer_update(vkc_reducer *r, const vkc_value *args, int nargs) {
    await_values(r->ctx, args, nargs);
    std::vector<Arg> call;
    to_args(args, nargs, &call);
    return r->impl->update(r->ctx, call.data(), nargs);
}

vkc_status ReducerImpl::finish_into(vkc_ctx *ctx, void *) {
    return fail(ctx, VKC_USAGE, "this reduction cannot run enqueue-only");
}

vkc_status vkc_reducer_finish(vkc_reducer *r, vkc_scalar *out) {
    vkc_status st = r->impl->finish(r->ctx, out);
    delete r->impl;
    delete r;
    return st;
}

vkc_status vkc_call_into(vkc_ctx *ctx, int id, const vkc_value *args, int nargs, vkc_array *out,
                         int64_t row) {
    const KernelDef *d = def_of(id);
    if (!d) return fail(ctx, VKC_USAGE, "unknown kernel id " + std::to_string(id));
    if (d->cls != VKC_REDUCTION) return fail(ctx, VKC_USAGE, d->name + " is not a reduction");
    if (!out) return fail(ctx, VKC_USAGE, "null array handle");
    if (out->type != d->out_type)
        return fail(ctx, VKC_USAGE, d->name + " produces " + type_name(d->out_type) + ", got a " +
                                        type_name(out->type) + " destination");
    if (row < 0 || row >= out->len)
        return fail(ctx, VKC_USAGE, "destination row " + std::to_string(row) + " out of range for length " +
                                        std::to_string(out->len));
    std::vector<Arg> call;
    int64_t rows = -1;
    vkc_status st = prepare(ctx, *d, args, nargs, &call, &rows);
    if (st) return st;
    if (rows < 0) return fail(ctx, VKC_USAGE, "a reduction needs an array operand");
    await_values(ctx, args, nargs);
    await_write(ctx, out);
    ReducerImpl *r = d->red(ctx);
    if (!r) return ctx->err.empty() ? fail(ctx, VKC_ALLOC, "cannot allocate a reducer") : VKC_ALLOC;
    // As vkc_call: one update with all rows, none on empty input.
    if (rows > 0) st = r->update(ctx, call.data(), nargs);
    if (!st) st = r->finish_into(ctx, static_cast<char *>(out->data()) + row * type_width(out->type));
    delete r;
    return st;
}

void vkc_reducer_free(vkc_reducer *r) {
    if (!r) return;
    delete r->impl;
    delete r;
}

vkc_status vkc_scanner_new(vkc_ctx *ctx, int id, vkc_scanner **out) {
    *out = nullptr;
    const KernelDef *d = def_of(id);
    if (!d) return fail(ctx, VKC_USAGE, "unknown kernel id " + std::to_string(id));
    if (d->cls != VKC_SCAN) return fail(ctx, VKC_USAGE, d->name + " is not a scan");
    ScannerImpl *s = d->scan(ctx);
    if (!s) return VKC_ALLOC;
    *out = new vkc_scanner{ctx, s};
    return VKC_OK;
}

vkc_status vkc_scanner_update(vkc_scanner *s, const vkc_value *args, int nargs, vkc_array *out) {
    std::vector<Arg> call;
    to_args(args, nargs, &call);
    if (!out) return fail(s->ctx, VKC_USAGE, "null array handle");
    await_values(s->ctx, args, nargs);
    await_write(s->ctx, out);
    return s->impl->update(s->ctx, call.data(), nargs, out);
}

void vkc_scanner_free(vkc_scanner *s) {
    if (!s) return;
    delete s->impl;
    delete s;
}

vkc_status vkc_builder_new(vkc_ctx *ctx, vkc_type type, vkc_builder **out) {
    *out = new vkc_builder{Builder{ctx, type, nullptr, 0, 0}};
    return VKC_OK;
}

vkc_status vkc_builder_finish(vkc_builder *b, vkc_array **out) {
    vkc_status st = finish_builder(b->b, out);
    delete b;
    return st;
}

void vkc_builder_free(vkc_builder *b) { delete b; }

vkc_status vkc_select_tile(vkc_ctx *ctx, int id, const vkc_value *args, int nargs, int64_t base,
                           vkc_builder *out) {
    const KernelDef *d = def_of(id);
    if (!d) return fail(ctx, VKC_USAGE, "unknown kernel id " + std::to_string(id));
    if (d->cls != VKC_SELECTION) return fail(ctx, VKC_USAGE, d->name + " is not a selection");
    if (out->b.type != d->out_type)
        return fail(ctx, VKC_USAGE, d->name + " produces " + type_name(d->out_type) +
                                        " rows, got a " + type_name(out->b.type) + " builder");
    std::vector<Arg> call;
    int64_t rows;
    vkc_status st = prepare(ctx, *d, args, nargs, &call, &rows);
    if (st) return st;
    await_values(ctx, args, nargs);
    return d->sel(ctx, call.data(), nargs, base, &out->b);
}

vkc_status vkc_elementwise_tile(vkc_ctx *ctx, int id, const vkc_value *args, int nargs,
                                vkc_array *out) {
    const KernelDef *d = def_of(id);
    if (!d) return fail(ctx, VKC_USAGE, "unknown kernel id " + std::to_string(id));
    if (d->cls != VKC_ELEMENTWISE)
        return fail(ctx, VKC_USAGE, d->name + " is not an elementwise kernel");
    if (!out || out->type != d->out_type)
        return fail(ctx, VKC_USAGE, "destination is not aligned for " +
                                        std::string(type_name(d->out_type)));
    std::vector<Arg> call;
    int64_t rows;
    vkc_status st = prepare(ctx, *d, args, nargs, &call, &rows);
    if (st) return st;
    if (rows < 0) return fail(ctx, VKC_USAGE, "an array kernel needs an array operand");
    if (rows != out->len)
        return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(rows) +
                                          " rows for a destination of " + std::to_string(out->len) +
                                          " rows");
    if (rows == 0) return VKC_OK;
    await_values(ctx, args, nargs);
    await_write(ctx, out);
    return d->elem(ctx, call.data(), nargs, rows, out);
}

}  // extern "C"

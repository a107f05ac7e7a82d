// Ingestion into HBM: load_T (src/kernels/scalar/construct.rs:78-97, registered :252-257) and
// the column files of the acceptance data (src/columns.rs load_words, load_single_bytes).
//
// A file is read in 32 MiB chunks into two pinned host buffers that alternate: while the
// stream copies one chunk to the device, the host reads the next into the other buffer (its
// previous copy has finished, an event says). The device work that the formats need runs on
// the uploaded words: the sign flip of signed columns (x ^ 2^63) and the check that a
// one-byte-per-row column's ends are 1, 2, 3, ... (the first offending row by atomicMin).
// Error messages are the reference's texts; an OS error reads as Rust's io::Error does
// ("<description> (os error N)").
#include <cerrno>
#include <cstring>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include "reduce_common.h"

namespace vkc {

constexpr size_t IO_CHUNK = size_t(32) << 20;

static std::string os_error(int e) { return std::string(strerror(e)) + " (os error " + std::to_string(e) + ")"; }

// The pinned chunk buffers and their events, made on first use and kept by the context.
static vkc_status io_buffers(vkc_ctx *ctx, unsigned char **buf) {
    if (!ctx->io_buf) {
        VKC_CUDA(ctx, cudaMallocHost(&ctx->io_buf, 2 * IO_CHUNK));
        for (int k = 0; k < 2; ++k)
            if (cudaEventCreateWithFlags(&ctx->io_ev[k], cudaEventDisableTiming) != cudaSuccess)
                return cuda_fail(ctx, cudaGetLastError(), "cudaEventCreate");
    }
    *buf = static_cast<unsigned char *>(ctx->io_buf);
    return VKC_OK;
}

// Reads `bytes` bytes of the open file `fd` to device address `dst`. On a read error, *err
// gets errno and the call returns VKC_RUNTIME without a message (the caller words it).
static vkc_status stream_file(vkc_ctx *ctx, int fd, size_t bytes, void *dst, int *err) {
    unsigned char *buf = nullptr;
    vkc_status st;
    if ((st = io_buffers(ctx, &buf))) return st;
    size_t done = 0;
    for (int k = 0; done < bytes; k ^= 1) {
        // The buffer's last copy (of this call or an earlier one) has finished before it is
        // refilled; an event not yet recorded counts as finished.
        VKC_CUDA(ctx, cudaEventSynchronize(ctx->io_ev[k]));
        unsigned char *h = buf + k * IO_CHUNK;
        const size_t want = bytes - done < IO_CHUNK ? bytes - done : IO_CHUNK;
        size_t got = 0;
        while (got < want) {
            const ssize_t r = pread(fd, h + got, want - got, static_cast<off_t>(done + got));
            if (r < 0 && errno == EINTR) continue;
            if (r <= 0) {
                *err = r < 0 ? errno : EIO;  // a file that shrank while being read
                cudaStreamSynchronize(ctx->stream);
                return VKC_RUNTIME;
            }
            got += static_cast<size_t>(r);
        }
        VKC_CUDA(ctx, cudaMemcpyAsync(static_cast<unsigned char *>(dst) + done, h, want, cudaMemcpyHostToDevice,
                                      ctx->stream));
        VKC_CUDA(ctx, cudaEventRecord(ctx->io_ev[k], ctx->stream));
        done += want;
    }
    return VKC_OK;
}

// Opens `path`, returning its size; *err gets errno on failure.
static int open_sized(const char *path, size_t *size, int *err) {
    const int fd = open(path, O_RDONLY);
    if (fd < 0) {
        *err = errno;
        return -1;
    }
    struct stat sb;
    if (fstat(fd, &sb) != 0) {
        *err = errno;
        close(fd);
        return -1;
    }
    if (S_ISDIR(sb.st_mode)) {  // reading a directory fails as EISDIR, as std::fs::read does
        *err = EISDIR;
        close(fd);
        return -1;
    }
    *size = static_cast<size_t>(sb.st_size);
    return fd;
}

// The whole file at `path` as an array of `type` rows. `bad_size` words the error for a size
// that is not a whole number of rows; `io_msg` the one for a read error.
template <class BadSize, class IoMsg>
static vkc_status load_file(vkc_ctx *ctx, const char *path, vkc_type type, BadSize bad_size, IoMsg io_msg,
                            vkc_array **out) {
    *out = nullptr;
    int err = 0;
    size_t size = 0;
    const int fd = open_sized(path, &size, &err);
    if (fd < 0) return fail(ctx, VKC_RUNTIME, io_msg(err));
    const size_t w = static_cast<size_t>(type_width(type));
    if (size % w != 0) {
        close(fd);
        return fail(ctx, VKC_RUNTIME, bad_size(size));
    }
    vkc_array *a;
    vkc_status st = new_array(ctx, type, static_cast<int64_t>(size / w), false, &a);
    if (st) {
        close(fd);
        return st;
    }
    if (size) st = stream_file(ctx, fd, size, a->data(), &err);
    close(fd);
    if (st) {
        vkc_array_release(a);
        return st == VKC_RUNTIME ? fail(ctx, VKC_RUNTIME, io_msg(err)) : st;
    }
    *out = a;
    return VKC_OK;
}

// construct.rs:80-97 (run_load).
template <vkc_type T> static vkc_status load(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    if (nargs != 1) return fail(ctx, VKC_RUNTIME, arity_error(1, nargs));
    if (args[0].kind != VKC_VALUE_STR || !args[0].str)
        return fail(ctx, VKC_RUNTIME, "expected str, got " + value_type_name(args[0]));
    const std::string path = args[0].str;
    const size_t w = static_cast<size_t>(type_width(T));
    vkc_array *a;
    vkc_status st = load_file(
        ctx, path.c_str(), T,
        [&](size_t size) {
            return path + " has " + std::to_string(size) + " bytes, which is not a multiple of " + std::to_string(w);
        },
        [&](int e) { return "cannot read " + path + ": " + os_error(e); }, &a);
    if (st) return st;
    out->kind = VKC_VALUE_ARRAY;
    out->array = a;
    return VKC_OK;
}

__global__ void flip_sign_kernel(unsigned long long *p, int64_t n) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        p[i] ^= 0x8000000000000000ull;
}

// First row i whose end is not i + 1.
__global__ void ends_check_kernel(const unsigned long long *__restrict__ ends, int64_t n, DevStatus *st) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        if (ends[i] != static_cast<unsigned long long>(i + 1)) atomicMin(&st->first_bad, static_cast<unsigned long long>(i));
}

void register_io(std::vector<KernelDef> &t) {
    struct L { const char *name; vkc_type ty; WholeFn f; };
    const L ls[] = {{"load_f64", VKC_F64, load<VKC_F64>}, {"load_f32", VKC_F32, load<VKC_F32>},
                    {"load_i64", VKC_I64, load<VKC_I64>}, {"load_u64", VKC_U64, load<VKC_U64>},
                    {"load_i32", VKC_I32, load<VKC_I32>}, {"load_u8", VKC_U8, load<VKC_U8>}};
    for (const L &l : ls) {
        // construct.rs:168-185: one Str input, cost = the element width.
        KernelDef d{l.name, VKC_WHOLE, {InSpec{IN_STR, l.ty}}, true, l.ty, static_cast<uint64_t>(type_width(l.ty))};
        d.whole = l.f;
        t.push_back(d);
    }
}

}  // namespace vkc

using namespace vkc;

extern "C" {

// columns.rs load_words: 8-byte little-endian words as i64 or u64 rows, sign-flipped when asked.
vkc_status vkc_load_column_words(vkc_ctx *ctx, const char *path, vkc_type type, int flip_sign, vkc_array **out) {
    if (!ctx || !path || !out || (type != VKC_I64 && type != VKC_U64)) return VKC_USAGE;
    const std::string p = path;
    vkc_array *a;
    vkc_status st = load_file(
        ctx, path, type,
        [&](size_t size) { return p + ": " + std::to_string(size) + " bytes is not a whole number of 8-byte words"; },
        [&](int e) { return p + ": " + os_error(e); }, &a);
    if (st) return st;
    if (flip_sign && a->len > 0) {
        flip_sign_kernel<<<stream_grid(ctx, a->len, 256, 8, 4096), 256, 0, ctx->stream>>>(
            static_cast<unsigned long long *>(a->data()), a->len);
        if ((st = launched(ctx, "flip_sign"))) {
            vkc_array_release(a);
            return st;
        }
    }
    *out = a;
    return VKC_OK;
}

// columns.rs load_single_bytes: a string column of one byte per row, from its .ends and .bytes
// files, as u8 rows.
vkc_status vkc_load_column_bytes(vkc_ctx *ctx, const char *ends_path, const char *bytes_path, const char *column,
                                 vkc_array **out) {
    if (!ctx || !ends_path || !bytes_path || !column || !out) return VKC_USAGE;
    const std::string ep = ends_path, bp = bytes_path, col = column;
    // Both files are read before their sizes are checked, so a read error comes first.
    for (const std::string *path : {&ep, &bp}) {
        int err = 0;
        size_t size = 0;
        const int fd = open_sized(path->c_str(), &size, &err);
        if (fd < 0) return fail(ctx, VKC_RUNTIME, *path + ": " + os_error(err));
        close(fd);
    }
    vkc_array *ends, *bytes;
    vkc_status st = load_file(
        ctx, ends_path, VKC_U64,
        [&](size_t size) { return ep + ": " + std::to_string(size) + " bytes is not a whole number of 8-byte words"; },
        [&](int e) { return ep + ": " + os_error(e); }, &ends);
    if (st) return st;
    st = load_file(
        ctx, bytes_path, VKC_U8, [&](size_t) { return std::string(); }, [&](int e) { return bp + ": " + os_error(e); },
        &bytes);
    if (st) {
        vkc_array_release(ends);
        return st;
    }
    const int64_t rows = ends->len;
    if (bytes->len != rows) {
        vkc_array_release(ends);
        vkc_array_release(bytes);
        return fail(ctx, VKC_RUNTIME, "column '" + col + "' has " + std::to_string(rows) + " rows but " +
                                          std::to_string(bytes->len) + " bytes, so it is not one byte per row");
    }
    if (rows > 0) {
        ends_check_kernel<<<stream_grid(ctx, rows, 256, 8, 4096), 256, 0, ctx->stream>>>(
            static_cast<const unsigned long long *>(ends->data()), rows, ctx->status);
        if ((st = launched(ctx, "ends_check"))) {
            vkc_array_release(ends);
            vkc_array_release(bytes);
            return st;
        }
    }
    DevStatus ds;
    if ((st = read_status(ctx, &ds))) {
        vkc_array_release(ends);
        vkc_array_release(bytes);
        return st;
    }
    if (ds.first_bad != ~0ull) {
        void *h;
        if ((st = pinned(ctx, 8, &h))) {
            vkc_array_release(ends);
            vkc_array_release(bytes);
            return st;
        }
        VKC_CUDA(ctx, cudaMemcpyAsync(h, static_cast<const unsigned long long *>(ends->data()) + ds.first_bad, 8,
                                      cudaMemcpyDeviceToHost, ctx->stream));
        VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const unsigned long long end = *static_cast<unsigned long long *>(h);
        vkc_array_release(ends);
        vkc_array_release(bytes);
        return fail(ctx, VKC_RUNTIME, "column '" + col + "' row " + std::to_string(ds.first_bad) + " ends at byte " +
                                          std::to_string(end) + ", so it is not one byte per row");
    }
    vkc_array_release(ends);
    *out = bytes;
    return VKC_OK;
}

}  // extern "C"

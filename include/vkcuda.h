/*
 * vkcuda: the GB300 (sm_103a) kernel backend of the verkehrt array language, behind a C ABI.
 *
 * The reference interpreter (antiguru/verkehrt, Rust) resolves one entry per kernel from its
 * kernel table (src/kernels.rs:302, KernelTable; src/kernels.rs:632-644, Registry::resolve)
 * and calls it through Dispatch (src/kernels/dispatch.rs:25-268). This library is the entry
 * set of a new `cuda` ISA slot in that table. Each function below names the reference
 * interface it replaces. Arrays are device-resident handles, so bindings stay in HBM between
 * statements and host<->device copies happen only at vkc_array_upload / vkc_array_download.
 *
 * Conventions
 *  - Every function that can fail returns a vkc_status. On VKC_RUNTIME the message of
 *    vkc_last_error() is byte-identical to the reference kernel's `Err(String)`.
 *  - Input handles are borrowed and never mutated (arrays are immutable, src/value.rs:215).
 *    Output handles are new references owned by the caller (release with vkc_array_release).
 *  - Calls are synchronous from the caller's view: a returned scalar is final and a returned
 *    array may be read or passed to the next call at once (same context stream).
 *  - A context is used by one host thread at a time.
 *  - Calls whose kernels wait on one another's blocks (scans, selections, group ids) bound every
 *    wait. A wait that runs out inside a call that does not itself wait for the device (a scan)
 *    is reported as VKC_TIMEOUT by the next call that does: vkc_synchronize or
 *    vkc_array_download.
 */
#ifndef VKCUDA_H
#define VKCUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define VKC_API __attribute__((visibility("default")))
#else
#define VKC_API
#endif

/* Status codes. src/error.rs:1-40 has one runtime kind; the split below tells the caller
 * whether the message is a kernel error (RUNTIME, formatted like the reference) or a failure
 * of the backend itself. */
typedef enum {
    VKC_OK = 0,
    VKC_RUNTIME = 1, /* kernel error, reference message text in vkc_last_error */
    VKC_ALLOC = 2,   /* device allocation failed ("cannot allocate ..." message) */
    VKC_TIMEOUT = 3, /* a bounded device-side wait gave up; the context stays usable */
    VKC_DEVICE = 4,  /* CUDA runtime error */
    VKC_USAGE = 5    /* bad kernel id, arity, kind or handle */
} vkc_status;

/* Element types, src/value.rs:7-19 (ScalarType) restricted to ARRAY_TYPES (:23-31). Bool is
 * stored as one byte holding 0 or 1. */
typedef enum {
    VKC_F64 = 0,
    VKC_F32 = 1,
    VKC_I64 = 2,
    VKC_U64 = 3,
    VKC_I32 = 4,
    VKC_U8 = 5,
    VKC_BOOL = 6
} vkc_type;

/* Kernel classes, src/kernels.rs:336-343 (KernelClass). */
typedef enum {
    VKC_ELEMENTWISE = 0,
    VKC_REDUCTION = 1,
    VKC_SELECTION = 2,
    VKC_SCAN = 3,
    VKC_WHOLE = 4
} vkc_class;

typedef struct vkc_ctx vkc_ctx;
typedef struct vkc_array vkc_array;
typedef struct vkc_reducer vkc_reducer;
typedef struct vkc_scanner vkc_scanner;
typedef struct vkc_builder vkc_builder;

/* A scalar, src/value.rs (Scalar): the type and the value's bits in the low bytes of `bits`
 * (little-endian, f64 as its IEEE bits, bool as 0/1). */
typedef struct {
    vkc_type type;
    uint64_t bits;
} vkc_scalar;

/* A value, src/value.rs:640 (Value) and :464 (Arg): an array handle, a scalar, or a string
 * (Value::Str, the path argument of load_T). Arg::Rows is kind VKC_VALUE_ARRAY, Arg::Splat is
 * VKC_VALUE_SCALAR; `str` is only read for VKC_VALUE_STR (a NUL-terminated UTF-8 path). */
typedef enum { VKC_VALUE_ARRAY = 0, VKC_VALUE_SCALAR = 1, VKC_VALUE_STR = 2 } vkc_value_kind;
typedef struct {
    vkc_value_kind kind;
    vkc_array *array;
    vkc_scalar scalar;
    const char *str;
} vkc_value;

/* ------------------------------------------------------------------ context */

/* Opens a context on CUDA device `device`: one stream, one scratch arena. Replaces the
 * per-interpreter Registry::resolve (src/kernels.rs:632-644) for the `cuda` ISA; the level
 * check of features::runnable (src/kernels/features.rs:198-212) becomes "a device is
 * present", which this call reports as VKC_DEVICE when it is not. */
VKC_API vkc_status vkc_open(int device, vkc_ctx **out);
VKC_API void vkc_close(vkc_ctx *ctx);
/* The message of the last failed call on this context (empty string when none). */
VKC_API const char *vkc_last_error(const vkc_ctx *ctx);
/* Waits for all work of the context. */
VKC_API vkc_status vkc_synchronize(vkc_ctx *ctx);
/* Freed array blocks are kept for reuse by the context, up to `bytes` (48 GiB by default);
 * lowering it releases the cache at once. Several contexts on one GPU (one per stream of a
 * server) share the device, so each keeps a smaller cache. */
VKC_API vkc_status vkc_set_cache_limit(vkc_ctx *ctx, size_t bytes);
/* Launch shapes chosen per size class (0: n < 2^20, 1: n < 2^24, 2: larger) by the committed
 * autotuner table (the reference fixes its tile sizes per ISA; these are this backend's):
 * "radix_items" (rows per thread of the argsort passes: 8, 12, 16), "stream_blocks_per_sm"
 * (count/min/max/argmin/argmax/integer sums: 2, 4, 5, 6, 8, 12, 16), "gather_rows_per_thread" (1, 2, 4)
 * and "group_first_table_log2" (group_id's first hash table, 18 .. 22). vkc_tune_set
 * overrides one entry for this context (the autotuner measures candidates that way); results
 * never depend on it.
 * Three more names are test hooks of the failure paths, the same for every size class (they have
 * no counterpart in the reference): "spin_limit" sets how many polls a kernel's wait on another
 * block may take before it gives up and the call returns VKC_TIMEOUT (0 restores the built-in
 * limit of 2^22 polls, about a second; waits for a block's own copies keep the built-in limit),
 * "lookback_never_ready" 1 makes every decoupled lookback poll for records that no block writes
 * (a flag that nothing sets: with a small spin_limit, every wait on an earlier tile runs out; 0
 * turns it off), and "fail_alloc_after" k makes the array allocation after the next k ones fail as if the
 * device were out of memory (VKC_ALLOC with the reference's "cannot allocate ..." text; -1, the
 * default, injects nothing). */
VKC_API vkc_status vkc_tune_set(vkc_ctx *ctx, const char *knob, int size_class, int value);
VKC_API vkc_status vkc_tune_get(const vkc_ctx *ctx, const char *knob, int size_class, int *value);
/* Runs the context's work on `stream` (a cudaStream_t) instead of its own stream. */
VKC_API vkc_status vkc_set_stream(vkc_ctx *ctx, void *stream);
VKC_API void *vkc_get_stream(const vkc_ctx *ctx);
/* Number of kernels this library launched on the context since it was opened. */
VKC_API uint64_t vkc_launch_count(const vkc_ctx *ctx);
/* CUDA-event timing on the context stream: start, then stop returns milliseconds. */
VKC_API vkc_status vkc_timer_start(vkc_ctx *ctx);
VKC_API vkc_status vkc_timer_stop(vkc_ctx *ctx, float *ms);

/* ------------------------------------------------------------------ arrays */

/* A new zeroed array of `len` rows of `type`, src/value.rs:326-336 (Array::try_build). Fails
 * with "array of N elements is too large" (value.rs:285-289) or "cannot allocate an array of
 * N elements" (value.rs:297-307). */
VKC_API vkc_status vkc_array_new(vkc_ctx *ctx, vkc_type type, int64_t len, vkc_array **out);
/* Copies `len` rows from host memory into a new device array (program inputs). Copies of at
 * least 1 MiB run on the context's upload stream, overlapping kernels and downloads: the first
 * call that reads the array waits for the copy, on the device. Pinned host memory must stay
 * unchanged until then (or until vkc_synchronize). */
VKC_API vkc_status vkc_array_upload(vkc_ctx *ctx, vkc_type type, const void *host, int64_t len,
                            vkc_array **out);
/* Copies the array's rows into host memory, `capacity` rows at most (print and exports), and
 * waits for the copy. */
VKC_API vkc_status vkc_array_download(vkc_ctx *ctx, const vkc_array *a, void *host, int64_t capacity);
/* The same copy on the context's download stream, after the work queued so far: returns at
 * once with a handle that vkc_copy_wait waits on (and frees). The handle holds a reference to
 * the array; a later call that writes the array waits for the copy. */
typedef struct vkc_copy vkc_copy;
VKC_API vkc_status vkc_array_download_start(vkc_ctx *ctx, const vkc_array *a, void *host, int64_t capacity,
                                            vkc_copy **out);
VKC_API vkc_status vkc_copy_wait(vkc_ctx *ctx, vkc_copy *c);
/* A zero-copy view of rows start..start+len, src/value.rs:245-259 (Array::slice) and
 * src/kernels/scalar/index.rs:76-93 (slice_T). */
VKC_API vkc_status vkc_array_slice(vkc_ctx *ctx, const vkc_array *a, int64_t start, int64_t len,
                           vkc_array **out);
VKC_API int64_t vkc_array_len(const vkc_array *a);
VKC_API vkc_type vkc_array_type(const vkc_array *a);
/* Device address of row 0 of the view. */
VKC_API void *vkc_array_device_ptr(const vkc_array *a);
VKC_API void vkc_array_retain(vkc_array *a);
VKC_API void vkc_array_release(vkc_array *a);

/* ------------------------------------------------------------------ kernel table */

/* The kernels with a `cuda` entry, named as in the reference registry (src/kernels.rs:471-482,
 * Registry::new; names from the register functions of src/kernels/scalar/). Ids are dense,
 * 0..count-1. */
VKC_API int vkc_kernel_count(void);
VKC_API const char *vkc_kernel_name(int id);
/* Registry::by_name, src/kernels.rs:620-622: the id, or -1. */
VKC_API int vkc_kernel_lookup(const char *name);
VKC_API vkc_class vkc_kernel_class(int id);
VKC_API int vkc_kernel_arity(int id);
/* KernelDef::cost, src/kernels.rs:417-418: bytes moved per element. */
VKC_API uint64_t vkc_kernel_cost(int id);

/* ------------------------------------------------------------------ entries */

/* Dispatch::call, src/kernels/dispatch.rs:56-142: runs kernel `id` over whole arguments. It
 * unifies array lengths first ("length mismatch: a vs b"), then an elementwise kernel gets
 * its output allocated, a reduction is updated once with all rows (never on empty input), a
 * scan is updated once, a selection runs with base 0, and a whole kernel checks its own
 * arguments. On success `*out` holds the result value. */
VKC_API vkc_status vkc_call(vkc_ctx *ctx, int id, const vkc_value *args, int nargs, vkc_value *out);

/* vkc_call of a reduction without a host read, so it can be captured in a graph (below): the
 * result's bits go to row `row` of the device array `out` (of the kernel's result type) in the
 * order of ctx's stream, and the call only enqueues work. Argument errors are reported as by
 * vkc_call; so is an empty input where the reduction's empty result is an error (reduce_min,
 * reduce_max, argmin, argmax: src/kernels/scalar/reduce.rs:401-411, :454-467), decided from the
 * arguments' lengths. A device-side timeout is reported by the next call that waits for the
 * device. The scratch arena does not grow during a capture: a call whose scratch is larger
 * than any earlier call's fails there with VKC_USAGE, so run the sequence once before
 * capturing it. */
VKC_API vkc_status vkc_call_into(vkc_ctx *ctx, int id, const vkc_value *args, int nargs, vkc_array *out,
                                 int64_t row);

/* Reducer (src/kernels.rs:48-63) for tile-fed callers, handed out by Dispatch::reducer
 * (src/kernels/dispatch.rs:156-163). Every update but the last has a multiple of 16 rows;
 * the canonical float state carries across updates, so any such split gives the bits of one
 * update (Split::Free, src/kernels.rs:158-170). finish consumes the reducer. */
VKC_API vkc_status vkc_reducer_new(vkc_ctx *ctx, int id, vkc_reducer **out);
VKC_API vkc_status vkc_reducer_update(vkc_reducer *r, const vkc_value *args, int nargs);
VKC_API vkc_status vkc_reducer_finish(vkc_reducer *r, vkc_scalar *out);
VKC_API void vkc_reducer_free(vkc_reducer *r);

/* Scanner (src/kernels.rs:65-88) for tile-fed callers, Dispatch::scanner
 * (src/kernels/dispatch.rs:177-185). update writes exactly the tile's output rows into `out`
 * (a caller-owned array of the tile's length); the state carries to the next update. */
VKC_API vkc_status vkc_scanner_new(vkc_ctx *ctx, int id, vkc_scanner **out);
VKC_API vkc_status vkc_scanner_update(vkc_scanner *s, const vkc_value *args, int nargs, vkc_array *out);
VKC_API void vkc_scanner_free(vkc_scanner *s);

/* ArrayBuilder (src/value.rs:471-600): an appendable device array for selections. */
VKC_API vkc_status vkc_builder_new(vkc_ctx *ctx, vkc_type type, vkc_builder **out);
VKC_API vkc_status vkc_builder_finish(vkc_builder *b, vkc_array **out);
VKC_API void vkc_builder_free(vkc_builder *b);

/* Dispatch::select_tile, src/kernels/dispatch.rs:236-265: appends the selected rows of one
 * tile whose first row is row `base` of the whole array. */
VKC_API vkc_status vkc_select_tile(vkc_ctx *ctx, int id, const vkc_value *args, int nargs, int64_t base,
                           vkc_builder *out);

/* Dispatch::elementwise_tile, src/kernels/dispatch.rs:192-229: writes the tile's rows into
 * `out`, whose length must equal every array argument's. */
VKC_API vkc_status vkc_elementwise_tile(vkc_ctx *ctx, int id, const vkc_value *args, int nargs,
                                vkc_array *out);

/* ------------------------------------------------------------------ allocation-free entry */

/* scan_add_i64 (the inclusive wrapping prefix sum of `n` rows of `in` into `out`, both device
 * pointers) for callers that cannot allocate device memory: an embedding host that gives this
 * library only its own buffers (an interpreter's arena, a pool with a fixed budget), or a
 * serving loop that must not take the allocator's lock or latency per request. It has no
 * counterpart in the reference, whose kernels run on the host. It needs no vkc_ctx and calls
 * no allocator: its lookback scratch is a 4 MiB array in the library's device image, so n
 * may be at most 2^28 rows (larger n is rejected with VKC_USAGE and a message), and `in` and
 * `out` must be device (or managed) memory of `device` (NULL or host pointers are rejected with
 * VKC_USAGE). The first call on a device looks up the array's device address (once per device)
 * and keeps it for the life of the process. Every call synchronizes `stream`, so the entry
 * cannot run inside a stream capture.
 * A device reset (cudaDeviceReset) reloads the library's device image and leaves that address
 * stale, so this entry must not be called after a reset of its device. Every call shares the
 * array: calls that overlap on the GPU race,
 * so run them on one stream or one after another. Work runs on `stream` (a cudaStream_t, NULL
 * for the legacy default stream) and the call returns when the scan is complete. On failure a
 * message is written to `err` (`err_len` bytes, may be NULL). */
VKC_API vkc_status vkc_scan_add_i64_noalloc(int device, const int64_t *in, int64_t *out, int64_t n,
                                            void *stream, char *err, size_t err_len);

/* ------------------------------------------------------------------ regions */

/* A region of the reference's executor (src/exec/region.rs:22-50): elementwise kernels with
 * array outputs in post-order, each reading region inputs or the outputs of earlier kernels.
 * A source is an input position i >= 0, or -1 - k for the output of kernel k. */
typedef struct vkc_region_kernel {
    int32_t kernel; /* kernel id */
    int32_t nargs;
    int32_t args[3];
} vkc_region_kernel;

/* The value of the region's last kernel, with the values and errors of evaluating every kernel
 * whole (Tiling::Off). It runs as one pass over the rows with every intermediate value on chip;
 * a region whose whole evaluation could fail (an operand of the wrong type or kind, arrays of
 * different lengths, a zero divisor), or that holds more than 12 kernels, 8 inputs or 16 of
 * both, runs kernel by kernel instead, as the reference falls back to whole evaluation when a
 * tiled run fails (src/exec/region.rs:137-159). Replaces the tiled run of eval_region. */
VKC_API vkc_status vkc_region_eval(vkc_ctx *ctx, const vkc_region_kernel *kernels, int nkernels,
                                   const vkc_value *inputs, int ninputs, vkc_value *out);

/* A fused region (src/exec/region/fused.rs): reduction `root` over arguments `root_args`
 * (sources as above) whose region arguments are the kernels' outputs. `count`, the extremes on
 * f64 and i64 (reduce_min/max, argmin/argmax) and reduce_add_i64 over one region argument fold
 * the region's value in its own pass (count(<cmp>_T(x, c)) is count_<cmp>_T); when the region
 * matches another fused kernel's pattern of the registry (src/kernels/scalar/fused.rs:286-379:
 * dot_T, sumsq_T, condsum_<cmp>_T) that kernel runs over the pattern's operands; otherwise each
 * region argument is evaluated by vkc_region_eval and the root is called once. Values and
 * errors are those of whole evaluation. Replaces eval_fused. */
VKC_API vkc_status vkc_region_reduce(vkc_ctx *ctx, int root, const int32_t *root_args, int nroot,
                                     const vkc_region_kernel *kernels, int nkernels,
                                     const vkc_value *inputs, int ninputs, vkc_value *out);

/* ------------------------------------------------------------------ batches and graphs */

/* A batch: many arrays of one element type that run the same planned statement. The
 * reference's executor (src/exec.rs:162-231, Strategy :77-91) runs a statement once per array;
 * a batch runs it once for all of them, as one persistent launch, with no host synchronisation
 * inside the batch entries, so a sequence of them can be captured in a graph (below) and
 * replayed. These entries have no counterpart in the reference's kernel table. The batch
 * retains its arrays. vkc_batch_new copies the array table to the device (and waits for it). */
typedef struct vkc_batch vkc_batch;
VKC_API vkc_status vkc_batch_new(vkc_ctx *ctx, int n, vkc_array *const *arrays, vkc_batch **out);
VKC_API void vkc_batch_free(vkc_batch *b);
VKC_API int vkc_batch_len(const vkc_batch *b);

/* For every f64 array i of the batch, sums[i] = reduce_add_f64(filter_<cmp>_f64(array i, c)),
 * bit for bit (the reference's canonical order over the compacted rows). cmp: 0 eq, 1 ne, 2 lt,
 * 3 le, 4 gt, 5 ge (the reference's Cmp, src/kernels/scalar/fused.rs:45-54). `sums` is an f64
 * array of the batch's length. */
VKC_API vkc_status vkc_batch_filter_sum_f64(vkc_ctx *ctx, vkc_batch *b, int cmp, double c, vkc_array *sums);

/* For every f64 array i of the batch, counts[i] = length(filter_<cmp>_f64(array i, c)), i.e. the
 * rows with x <cmp> c (count_<cmp>_f64, src/kernels/scalar/fused.rs:150-179). `counts` is an i64
 * array of the batch's length. */
VKC_API vkc_status vkc_batch_count_f64(vkc_ctx *ctx, vkc_batch *b, int cmp, double c, vkc_array *counts);

/* sums[i] = dot_f64(xs[i], ys[i]) for every pair (equal lengths), bit for bit: fl(x*y) in the
 * canonical order (src/kernels/scalar/fused.rs:73-106). One block per pair: meant for short
 * arrays (a lane adds n/16 rows in sequence). `sums` is an f64 array of the batch's length. */
VKC_API vkc_status vkc_batch_dot_f64(vkc_ctx *ctx, vkc_batch *xs, vkc_batch *ys, vkc_array *sums);

/* For every i64 array i of `keys`, the stable ascending positions (argsort_i64) into the i64
 * array i of `outs` (same lengths). key_digits: bit d set when byte d of the keys' sign-flipped
 * image varies (0: all eight); a caller that knows its key range saves the passes of constant
 * bytes. The first call on a (keys, outs) pair allocates scratch: make it before capturing, and
 * give key_digits when capturing. */
VKC_API vkc_status vkc_batch_argsort_i64(vkc_ctx *ctx, vkc_batch *keys, const vkc_batch *outs,
                                         unsigned key_digits);

/* Many rand_f64 (type VKC_F64) or rand_i64 (VKC_I64) statements in one launch: outs[i] gets
 * rand(lens[i], seeds[i]), equal to that call's array (src/kernels/scalar/construct.rs:64-76).
 * The arrays are views of one allocation. A negative length fails as rand does. */
VKC_API vkc_status vkc_batch_rand(vkc_ctx *ctx, vkc_type type, int count, const int64_t *lens,
                                  const int64_t *seeds, vkc_array **outs);

/* The batch's arrays concatenated in the caller's order into a new array `rows` (the batch's
 * element type), and, when `index` is not NULL, a new i64 array naming the array of every row
 * (0 for the rows of the first array, and so on). A statement with no batched entry
 * (group_id2, reduce_into, scan_by, ...) then runs once for the whole batch, keyed or
 * segmented by that column. The call allocates its outputs, so it is not for use inside a
 * capture. */
VKC_API vkc_status vkc_batch_concat(vkc_ctx *ctx, vkc_batch *b, vkc_array **rows, vkc_array **index);

/* Ingestion of the acceptance column files (src/columns.rs load_words, load_single_bytes): the
 * file is streamed through pinned buffers into a new device array. Words are 8-byte
 * little-endian rows read as `type` (VKC_I64 or VKC_U64), with bit 63 flipped when
 * `flip_sign` (the columns the loader lists as signed); the bytes form reads `column`.ends and
 * .bytes paths and checks that row i ends at byte i + 1. Errors are the reference's texts.
 * load_T itself is the whole kernel load_<type> (construct.rs:78-97) through vkc_call. */
VKC_API vkc_status vkc_load_column_words(vkc_ctx *ctx, const char *path, vkc_type type, int flip_sign,
                                         vkc_array **out);
VKC_API vkc_status vkc_load_column_bytes(vkc_ctx *ctx, const char *ends_path, const char *bytes_path,
                                         const char *column, vkc_array **out);

/* A CUDA graph of the work the library enqueues on ctx's stream between vkc_graph_begin and
 * vkc_graph_end (stream capture), replayed by vkc_graph_launch. Only enqueue-only entries may
 * run in between: vkc_call_into (reductions into a device array), vkc_elementwise_tile (into an
 * existing array) and the batch entries above. A statement sequence of the reference's
 * executor (src/exec.rs:162-231) whose results stay on the device is captured once and then
 * replayed as one launch; the arrays it reads and writes are the ones it was captured with. */
typedef struct vkc_graph vkc_graph;
VKC_API vkc_status vkc_graph_begin(vkc_ctx *ctx);
VKC_API vkc_status vkc_graph_end(vkc_ctx *ctx, vkc_graph **out);
VKC_API vkc_status vkc_graph_launch(vkc_ctx *ctx, vkc_graph *g);
VKC_API void vkc_graph_free(vkc_graph *g);

#ifdef __cplusplus
}
#endif
#endif

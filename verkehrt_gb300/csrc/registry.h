// The kernel table of the `cuda` ISA: definitions mirror KernelDef (src/kernels.rs:411-426)
// and the entry classes mirror KernelImpl (src/kernels.rs:171-177).
#pragma once

#include <string>
#include <vector>

#include "vkc_internal.h"

namespace vkc {

// An entry argument, src/value.rs:464-467 (Arg): rows of an array, or a scalar splat.
struct Arg {
    bool rows;
    const vkc_array *a;
    vkc_scalar s;
    int64_t len() const { return rows ? a->len : 0; }
    template <class T> const T *ptr() const { return static_cast<const T *>(a->data()); }
    double f64() const { double d; __builtin_memcpy(&d, &s.bits, 8); return d; }
    int64_t i64() const { return static_cast<int64_t>(s.bits); }
};

// InputSpec, src/kernels.rs:304-329.
enum InKind { IN_ARRAY, IN_SCALAR, IN_EITHER, IN_STR };
struct InSpec {
    InKind kind;
    vkc_type type;
};

// ArrayBuilder (src/value.rs:471-600) on the device: rows [0, len) are committed.
struct Builder {
    vkc_ctx *ctx;
    vkc_type type;
    std::shared_ptr<Buffer> buf;
    int64_t len = 0, cap = 0;
    // Makes room for `more` rows past len; returns the device address of row len.
    vkc_status reserve(int64_t more, void **at);
};

// Reducer (src/kernels.rs:48-63): state on the device, one sync at finish.
struct ReducerImpl {
    virtual ~ReducerImpl() {}
    virtual vkc_status update(vkc_ctx *ctx, const Arg *args, int nargs) = 0;
    virtual vkc_status finish(vkc_ctx *ctx, vkc_scalar *out) = 0;
    // finish without a host read: the result's bits (the output type's width) go to the
    // device address dst, in the order of the context's stream. The one error a finish can
    // report, an empty input where that is an error, is decided by the rows the reducer was
    // given, which the host knows.
    virtual vkc_status finish_into(vkc_ctx *ctx, void *dst);
};

// Scanner (src/kernels.rs:65-88): carried state on the device.
struct ScannerImpl {
    virtual ~ScannerImpl() {}
    virtual vkc_status update(vkc_ctx *ctx, const Arg *args, int nargs, vkc_array *out) = 0;
};

using ElemFn = vkc_status (*)(vkc_ctx *, const Arg *, int, int64_t n, vkc_array *out);
using ReducerMake = ReducerImpl *(*)(vkc_ctx *);
using SelectFn = vkc_status (*)(vkc_ctx *, const Arg *, int, int64_t base, Builder *out);
using ScanMake = ScannerImpl *(*)(vkc_ctx *);
using WholeFn = vkc_status (*)(vkc_ctx *, const vkc_value *, int, vkc_value *out);

struct KernelDef {
    std::string name;
    vkc_class cls;
    std::vector<InSpec> inputs;
    bool out_array;
    vkc_type out_type;
    uint64_t cost;
    ElemFn elem = nullptr;
    ReducerMake red = nullptr;
    SelectFn sel = nullptr;
    ScanMake scan = nullptr;
    WholeFn whole = nullptr;
    // Elementwise kernels: the row operation, its operand type and its result type as codes
    // of the region evaluator (k_elementwise.cu); ew_fn < 0 elsewhere.
    int ew_fn = -1, ew_ty = 0, ew_dst = 0;
};

// The table's entry of that name (for entries built from other entries), or nullptr.
const KernelDef *kernel_def(const char *name);

// Registration by family (called once, in this order, to build the table).
void register_construct(std::vector<KernelDef> &t);
void register_reduce(std::vector<KernelDef> &t);
void register_select(std::vector<KernelDef> &t);
void register_scan(std::vector<KernelDef> &t);
void register_index(std::vector<KernelDef> &t);
void register_sort(std::vector<KernelDef> &t);
void register_group(std::vector<KernelDef> &t);
void register_io(std::vector<KernelDef> &t);
void register_reduce_into_f64(std::vector<KernelDef> &t);
void register_elementwise(std::vector<KernelDef> &t);
void register_families(std::vector<KernelDef> &t);

// Argument helpers with the reference's messages (src/kernels/scalar/elementwise.rs:172-199).
std::string arity_error(int want, int got);
std::string value_type_name(const Arg &a);  // "f64[]" or "f64"
std::string value_type_name(const vkc_value &v);
// rows_arg: the array operand of type t, else "expected f64[], got ...".
bool rows_arg(vkc_ctx *ctx, const Arg &a, vkc_type t, vkc_status *st);
// splat_arg: the scalar operand of type t, else "expected f64, got ...".
bool splat_arg(vkc_ctx *ctx, const Arg &a, vkc_type t, vkc_status *st);
// array_arg for whole kernels (src/kernels/scalar/reduce.rs:599-604).
bool array_arg(vkc_ctx *ctx, const vkc_value &v, vkc_type t, vkc_status *st);
bool i64_arg(vkc_ctx *ctx, const vkc_value &v, int64_t *out, vkc_status *st);

// Scalar constructors.
inline vkc_scalar scalar_f64(double d) { vkc_scalar s; s.type = VKC_F64; __builtin_memcpy(&s.bits, &d, 8); return s; }
inline vkc_scalar scalar_i64(int64_t v) { vkc_scalar s; s.type = VKC_I64; s.bits = static_cast<uint64_t>(v); return s; }

}  // namespace vkc

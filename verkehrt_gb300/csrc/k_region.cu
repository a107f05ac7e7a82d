// Regions on the device: the reference's executor runs a region (a subtree of at least two
// elementwise kernels with array outputs, src/exec/region.rs:22-50) tile by tile, and a fused
// region (a reduction over such kernels, src/exec/region/fused.rs:1-3) feeds the tiles to the
// root's accumulator. Here a region is one pass over the rows (region_kernel, every
// intermediate value on chip), with the values and errors of whole evaluation (Tiling::Off):
//  * a region that could fail, or could fail differently when fused (an operand of the wrong
//    type or kind, arrays of different lengths, a kernel without an array operand, a zero
//    divisor, more kernels or inputs than the evaluator holds), runs whole instead, kernel by
//    kernel in post-order, which raises the error whole evaluation raises, as the reference
//    does when its tiled run fails (region.rs:137-159);
//  * `count` over a region counts the region's true rows as it evaluates them, and the extremes
//    (reduce_min/max, argmin/argmax on f64 and i64) and the i64 sum fold them in the same pass;
//  * a fused root whose region matches one of the registry's fused patterns
//    (src/kernels/scalar/fused.rs:286-379: dot_T, sumsq_T and condsum_<cmp>_T are declared
//    there as those compositions) runs as that fused reduction over the pattern's
//    operands; any other root is called once over its arguments, each region argument
//    evaluated by one pass.
#include <cstring>
#include <string>
#include <vector>

#include "kcommon.cuh"
#include "region.h"
#include "registry.h"

namespace vkc {

namespace {

struct Src {
    bool kernel;  // the output of region kernel i, else region input i
    int i;
};
Src src_of(int32_t a) { return a >= 0 ? Src{false, a} : Src{true, -1 - a}; }

// Sources in range and in post-order, arities that the struct can hold.
vkc_status check_shape(vkc_ctx *ctx, const vkc_region_kernel *ks, int nk, int nin) {
    if (nk < 1) return fail(ctx, VKC_USAGE, "a region has at least one kernel");
    if (nin < 0) return fail(ctx, VKC_USAGE, "negative input count");
    for (int k = 0; k < nk; ++k) {
        if (ks[k].nargs < 0 || ks[k].nargs > 3)
            return fail(ctx, VKC_USAGE, "region kernel " + std::to_string(k) + ": 0 to 3 arguments");
        for (int j = 0; j < ks[k].nargs; ++j) {
            const Src s = src_of(ks[k].args[j]);
            if (s.kernel ? s.i >= k : s.i >= nin)
                return fail(ctx, VKC_USAGE, "region kernel " + std::to_string(k) + ": argument " + std::to_string(j) +
                                                " names no earlier kernel or input");
        }
    }
    return VKC_OK;
}

// The one-pass program of a region whose whole evaluation cannot fail, or false.
bool plan_region(const vkc_region_kernel *ks, int nk, const vkc_value *in, int nin, RegionProg *p, int64_t *n,
                 vkc_type *out_type) {
    if (nk > RG_MAX_K || nin > RG_MAX_IN || nk + nin > RG_MAX_SLOTS) return false;
    int64_t len = -1;
    memset(p, 0, sizeof *p);
    p->nk = nk;
    for (int j = 0; j < nin; ++j) {
        const vkc_value &v = in[j];
        if (v.kind == VKC_VALUE_ARRAY) {
            if (!v.array) return false;
            if (len >= 0 && v.array->len != len) return false;  // a length mismatch somewhere
            len = v.array->len;
        } else if (v.kind != VKC_VALUE_SCALAR) {
            return false;
        }
    }
    if (len < 0) return false;
    // The array inputs in input order, at most RG_MAX_ARR.
    std::vector<int> arr_no(static_cast<size_t>(nin), -1);
    int narr = 0;
    for (int j = 0; j < nin; ++j)
        if (in[j].kind == VKC_VALUE_ARRAY) {
            if (narr == RG_MAX_ARR) return false;
            arr_no[static_cast<size_t>(j)] = narr;
            p->in[narr++] = RgIn{in[j].array->data(), type_width(in[j].array->type)};
        }
    p->narr = narr;
    std::vector<vkc_type> ty(static_cast<size_t>(nk));
    std::vector<char> keep(static_cast<size_t>(nk), 0);
    for (int k = 0; k < nk; ++k) {
        const char *name = vkc_kernel_name(ks[k].kernel);
        const KernelDef *d = name ? kernel_def(name) : nullptr;
        if (!d || d->cls != VKC_ELEMENTWISE || d->ew_fn < 0) return false;
        if (static_cast<int>(d->inputs.size()) != ks[k].nargs) return false;
        bool any_array = false;
        RgOp &o = p->op[k];
        o.fn = static_cast<unsigned char>(d->ew_fn);
        o.ty = static_cast<unsigned char>(d->ew_ty);
        o.dst = static_cast<unsigned char>(d->ew_dst);
        for (int j = 0; j < 3; ++j) o.kind[j] = RK_CONST;  // unused operands read 0
        for (int j = 0; j < ks[k].nargs; ++j) {
            const Src s = src_of(ks[k].args[j]);
            const bool arr = s.kernel || in[s.i].kind == VKC_VALUE_ARRAY;
            const vkc_type t = s.kernel ? ty[s.i] : (arr ? in[s.i].array->type : in[s.i].scalar.type);
            const InSpec &spec = d->inputs[static_cast<size_t>(j)];
            if (t != spec.type || (spec.kind == IN_SCALAR && arr) || (spec.kind == IN_ARRAY && !arr)) return false;
            any_array |= arr;
            if (!s.kernel) {
                o.kind[j] = arr ? RK_IN : RK_CONST;
                o.idx[j] = static_cast<unsigned char>(arr ? arr_no[static_cast<size_t>(s.i)] : 0);
                o.c[j] = arr ? 0 : in[s.i].scalar.bits;
            } else if (s.i == k - 1) {
                o.kind[j] = RK_PREV;
            } else {
                o.kind[j] = RK_SLOT;
                o.idx[j] = static_cast<unsigned char>(s.i);  // a kernel; its slot below
                keep[static_cast<size_t>(s.i)] = 1;
            }
        }
        if (!any_array) return false;  // "an array kernel needs an array operand"
        if (d->ew_fn == EF_DIVC && !make_ew_divider(d->ew_ty, in[src_of(ks[k].args[1]).i].scalar.bits, &o.dv))
            return false;  // division by zero
        ty[static_cast<size_t>(k)] = d->out_type;
    }
    // Slots of the kept values, in kernel order.
    std::vector<int> slot(static_cast<size_t>(nk), -1);
    for (int k = 0; k < nk; ++k)
        if (keep[static_cast<size_t>(k)]) {
            slot[static_cast<size_t>(k)] = p->nslots++;
            p->op[k].keep = 1;
            p->op[k].slot = static_cast<unsigned char>(slot[static_cast<size_t>(k)]);
        }
    for (int k = 0; k < nk; ++k)
        for (int j = 0; j < 3; ++j)
            if (p->op[k].kind[j] == RK_SLOT) p->op[k].idx[j] = static_cast<unsigned char>(slot[p->op[k].idx[j]]);
    *out_type = ty.back();
    p->out_width = type_width(*out_type);
    *n = len;
    // f64 arithmetic and comparisons only, over f64 inputs: the f64 evaluator. A comparison's
    // result may feed only select_f64's mask or be the region's value.
    bool f64 = true;
    for (int j = 0; j < nin && f64; ++j)
        f64 = (in[j].kind == VKC_VALUE_ARRAY ? in[j].array->type : in[j].scalar.type) == VKC_F64;
    for (int k = 0; k < nk && f64; ++k) {
        const RgOp &o = p->op[k];
        const bool cmp = o.fn == EF_LT || o.fn == EF_LE || o.fn == EF_GT || o.fn == EF_GE || o.fn == EF_EQ || o.fn == EF_NE;
        const bool arith = o.fn == EF_ADD || o.fn == EF_SUB || o.fn == EF_MUL || o.fn == EF_DIV || o.fn == EF_MIN ||
                           o.fn == EF_MAX || o.fn == EF_NEG || o.fn == EF_ABS || o.fn == EF_SQRT || o.fn == EF_SELECT;
        f64 = o.ty == ET_F64 && (cmp || arith);
        for (int k2 = k + 1; k2 < nk && f64 && cmp; ++k2)  // who reads a comparison's value
            for (int j = 0; j < ks[k2].nargs; ++j) {
                const Src s = src_of(ks[k2].args[j]);
                if (s.kernel && s.i == k && !(p->op[k2].fn == EF_SELECT && j == 0)) f64 = false;
            }
    }
    p->f64only = f64;
    return true;
}

void release_values(std::vector<vkc_value> &vals) {
    for (vkc_value &v : vals)
        if (v.kind == VKC_VALUE_ARRAY && v.array) vkc_array_release(v.array);
    vals.clear();
}

// Whole evaluation: every kernel by vkc_call in post-order.
vkc_status eval_whole(vkc_ctx *ctx, const vkc_region_kernel *ks, int nk, const vkc_value *in, vkc_value *out) {
    std::vector<vkc_value> vals;
    for (int k = 0; k < nk; ++k) {
        vkc_value args[3];
        for (int j = 0; j < ks[k].nargs; ++j) {
            const Src s = src_of(ks[k].args[j]);
            args[j] = s.kernel ? vals[static_cast<size_t>(s.i)] : in[s.i];
        }
        vkc_value v;
        const vkc_status st = vkc_call(ctx, ks[k].kernel, args, ks[k].nargs, &v);
        if (st) {
            release_values(vals);
            return st;
        }
        vals.push_back(v);
    }
    *out = vals.back();
    vals.pop_back();
    release_values(vals);
    return VKC_OK;
}

vkc_status eval_region(vkc_ctx *ctx, const vkc_region_kernel *ks, int nk, const vkc_value *in, int nin,
                       vkc_value *out) {
    memset(out, 0, sizeof *out);
    vkc_status st = check_shape(ctx, ks, nk, nin);
    if (st) return st;
    RegionProg p;
    int64_t n;
    vkc_type t;
    if (!plan_region(ks, nk, in, nin, &p, &n, &t)) return eval_whole(ctx, ks, nk, in, out);
    await_values(ctx, in, nin);
    vkc_array *o;
    if ((st = new_array(ctx, t, n, false, &o))) return st;
    if ((st = launch_region(ctx, p, n, o->data()))) {
        vkc_array_release(o);
        return st;
    }
    out->kind = VKC_VALUE_ARRAY;
    out->array = o;
    return VKC_OK;
}

// The subtree of kernel k, renumbered in post-order, with the region's inputs.
std::vector<vkc_region_kernel> subtree(const vkc_region_kernel *ks, int k) {
    std::vector<char> seen(static_cast<size_t>(k) + 1, 0);
    // Kernels are in post-order, so the subtree is the marked kernels in index order.
    seen[static_cast<size_t>(k)] = 1;
    for (int i = k; i >= 0; --i) {
        if (!seen[static_cast<size_t>(i)]) continue;
        for (int j = 0; j < ks[i].nargs; ++j) {
            const Src s = src_of(ks[i].args[j]);
            if (s.kernel) seen[static_cast<size_t>(s.i)] = 1;
        }
    }
    std::vector<int> at(static_cast<size_t>(k) + 1, -1);
    std::vector<vkc_region_kernel> out;
    for (int i = 0; i <= k; ++i) {
        if (!seen[static_cast<size_t>(i)]) continue;
        vkc_region_kernel r = ks[i];
        for (int j = 0; j < r.nargs; ++j) {
            const Src s = src_of(r.args[j]);
            if (s.kernel) r.args[j] = -1 - at[static_cast<size_t>(s.i)];
        }
        at[static_cast<size_t>(i)] = static_cast<int>(out.size());
        out.push_back(r);
    }
    return out;
}

std::string name_of(int id) {
    const char *s = vkc_kernel_name(id);
    return s ? s : "";
}

// The fused.rs patterns over a region that runs fused (so none of its kernels can fail):
// reduce_add_T(mul_T(x, y)) is dot_T(x, y), or sumsq_T(x) when x and y are one array;
// reduce_add_T(select_T(<cmp>_T(x, c), x, e)) is condsum_<cmp>_T(x, c, e). (count(<cmp>_T(x, c)),
// count_<cmp>_T, is counted in the region's own pass.) Operands are region sources; true when one
// matched.
bool fused_pattern(const vkc_region_kernel *ks, const vkc_value *in, int root, const std::vector<Src> &args,
                   int *root2, std::vector<Src> *args2) {
    if (args.size() != 1 || !args[0].kernel) return false;
    const std::string rn = name_of(root);
    const vkc_region_kernel &k = ks[args[0].i];
    const std::string kn = name_of(k.kernel);
    auto is_array = [&](Src s) { return s.kernel || in[s.i].kind == VKC_VALUE_ARRAY; };
    auto same_array = [&](Src a, Src b) {
        if (a.kernel || b.kernel) return false;
        const vkc_value &x = in[a.i], &y = in[b.i];
        return x.kind == VKC_VALUE_ARRAY && y.kind == VKC_VALUE_ARRAY && x.array->data() == y.array->data() &&
               x.array->len == y.array->len && x.array->type == y.array->type;
    };
    auto scalar_input = [&](Src s) { return !s.kernel && in[s.i].kind == VKC_VALUE_SCALAR; };
    static const char *const types[] = {"f64", "f32", "i64", "u64", "i32"};
    static const char *const cmps[] = {"eq", "ne", "lt", "le", "gt", "ge"};
    for (const char *t : types) {
        if (rn == std::string("reduce_add_") + t && kn == std::string("mul_") + t) {
            const Src x = src_of(k.args[0]), y = src_of(k.args[1]);
            if (!is_array(x) || !is_array(y)) return false;
            const std::string f = same_array(x, y) ? std::string("sumsq_") + t : std::string("dot_") + t;
            if ((*root2 = vkc_kernel_lookup(f.c_str())) < 0) return false;
            *args2 = same_array(x, y) ? std::vector<Src>{x} : std::vector<Src>{x, y};
            return true;
        }
        for (const char *c : cmps) {
            const std::string cmp = std::string(c) + "_" + t;
            if (rn == std::string("reduce_add_") + t && kn == std::string("select_") + t) {
                const Src m = src_of(k.args[0]), a = src_of(k.args[1]), e = src_of(k.args[2]);
                if (!m.kernel || name_of(ks[m.i].kernel) != cmp || !scalar_input(e)) continue;
                const Src x = src_of(ks[m.i].args[0]), v = src_of(ks[m.i].args[1]);
                if (!same_array(x, a) || !scalar_input(v)) continue;
                if ((*root2 = vkc_kernel_lookup(("condsum_" + cmp).c_str())) < 0) return false;
                *args2 = {x, v, e};
                return true;
            }
        }
    }
    return false;
}

}  // namespace

}  // namespace vkc

using namespace vkc;

extern "C" {

vkc_status vkc_region_eval(vkc_ctx *ctx, const vkc_region_kernel *kernels, int nkernels, const vkc_value *inputs,
                           int ninputs, vkc_value *out) {
    if (!ctx || !out || (nkernels > 0 && !kernels) || (ninputs > 0 && !inputs)) return VKC_USAGE;
    return eval_region(ctx, kernels, nkernels, inputs, ninputs, out);
}

vkc_status vkc_region_reduce(vkc_ctx *ctx, int root, const int32_t *root_args, int nroot,
                             const vkc_region_kernel *kernels, int nkernels, const vkc_value *inputs, int ninputs,
                             vkc_value *out) {
    if (!ctx || !out || (nroot > 0 && !root_args) || (nkernels > 0 && !kernels) || (ninputs > 0 && !inputs))
        return VKC_USAGE;
    memset(out, 0, sizeof *out);
    if (vkc_kernel_class(root) != VKC_REDUCTION || !vkc_kernel_name(root))
        return fail(ctx, VKC_USAGE, "the root of a fused region is a reduction");
    vkc_status st = check_shape(ctx, kernels, nkernels, ninputs);
    if (st) return st;
    std::vector<Src> args;
    for (int j = 0; j < nroot; ++j) {
        const Src s = src_of(root_args[j]);
        if (s.kernel ? s.i >= nkernels : s.i >= ninputs)
            return fail(ctx, VKC_USAGE, "root argument " + std::to_string(j) + " names no kernel or input");
        args.push_back(s);
    }
    RegionProg p;
    int64_t n;
    vkc_type t;
    if (name_of(root) == "count" && args.size() == 1 && args[0].kernel) {
        // count over a region: the rows counted as the region is evaluated, nothing stored.
        const std::vector<vkc_region_kernel> sub = subtree(kernels, args[0].i);
        if (plan_region(sub.data(), static_cast<int>(sub.size()), inputs, ninputs, &p, &n, &t) && t == VKC_BOOL) {
            await_values(ctx, inputs, ninputs);
            vkc_array *c;
            if ((st = new_array(ctx, VKC_I64, 1, true, &c))) return st;
            int64_t v = 0;
            st = launch_region(ctx, p, n, c->data(), true);
            if (!st) st = vkc_array_download(ctx, c, &v, 1);
            vkc_array_release(c);
            if (st) return st;
            out->kind = VKC_VALUE_SCALAR;
            out->scalar = scalar_i64(v);
            return VKC_OK;
        }
    }
    // Extremes and the i64 sum over a region: folded in the same pass.
    static const struct {
        const char *name;
        int kind;
        bool f64;
    } folds[] = {{"reduce_min_f64", RF_MIN, true},     {"reduce_max_f64", RF_MAX, true},
                 {"argmin_f64", RF_ARGMIN, true},      {"argmax_f64", RF_ARGMAX, true},
                 {"reduce_min_i64", RF_MIN, false},    {"reduce_max_i64", RF_MAX, false},
                 {"argmin_i64", RF_ARGMIN, false},     {"argmax_i64", RF_ARGMAX, false},
                 {"reduce_add_i64", RF_SUM, false}};
    for (const auto &f : folds) {
        if (name_of(root) != f.name || args.size() != 1 || !args[0].kernel) continue;
        const std::vector<vkc_region_kernel> sub = subtree(kernels, args[0].i);
        if (!plan_region(sub.data(), static_cast<int>(sub.size()), inputs, ninputs, &p, &n, &t) ||
            t != (f.f64 ? VKC_F64 : VKC_I64) || n == 0)
            break;  // the root over the materialised value gives the value and the errors
        await_values(ctx, inputs, ninputs);
        vkc_array *w;
        const int64_t words = 4 * (RG_FOLD_MAX_GRID + 1) + 1;
        if ((st = new_array(ctx, VKC_U64, words, true, &w))) return st;
        auto *work = static_cast<RgFold *>(w->data());
        RgFold r{};
        st = launch_region_fold(ctx, p, n, f.kind, f.f64, work,
                                reinterpret_cast<unsigned *>(static_cast<unsigned long long *>(w->data()) + words - 1));
        if (!st) st = vkc_array_download(ctx, w, &r, 4);
        vkc_array_release(w);
        if (st) return st;
        out->kind = VKC_VALUE_SCALAR;
        const bool arg = f.kind == RF_ARGMIN || f.kind == RF_ARGMAX;
        if (f.kind == RF_SUM) {
            out->scalar = scalar_i64(static_cast<int64_t>(r.sum));
        } else if (arg) {  // reduce.rs:454-467: a NaN row decides
            out->scalar = scalar_i64(static_cast<int64_t>(f.f64 && r.nan_idx != ~0ull ? r.nan_idx : r.idx));
        } else if (f.f64) {  // reduce.rs:401-411: any NaN makes the result NaN
            out->scalar.type = VKC_F64;
            out->scalar.bits = r.nan_idx != ~0ull ? 0x7ff8000000000000ull : bits_of_key(r.key);
        } else {
            out->scalar = scalar_i64(r.key);
        }
        return VKC_OK;
    }
    int root2 = root;
    std::vector<Src> args2 = args;
    if (!plan_region(kernels, nkernels, inputs, ninputs, &p, &n, &t) ||
        !fused_pattern(kernels, inputs, root, args, &root2, &args2)) {
        root2 = root;
        args2 = args;
    }
    // The root's arguments left to right, each region argument by one pass over its subtree.
    std::vector<vkc_value> temps, call;
    for (const Src &s : args2) {
        if (!s.kernel) {
            call.push_back(inputs[s.i]);
            continue;
        }
        const std::vector<vkc_region_kernel> sub = subtree(kernels, s.i);
        vkc_value v;
        if ((st = eval_region(ctx, sub.data(), static_cast<int>(sub.size()), inputs, ninputs, &v))) {
            release_values(temps);
            return st;
        }
        temps.push_back(v);
        call.push_back(v);
    }
    st = vkc_call(ctx, root2, call.data(), static_cast<int>(call.size()), out);
    release_values(temps);
    return st;
}

}  // extern "C"

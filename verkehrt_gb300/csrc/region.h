// The region evaluator: a chain of elementwise kernels (a region of the reference's executor,
// src/exec/region.rs:22-50) run as one pass over the rows, every intermediate value kept on
// chip. Shared by k_elementwise.cu (the row operations and the kernel) and k_region.cu (the
// entries that check a region and fall back to whole evaluation).
#pragma once

#include "vkc_internal.h"

namespace vkc {

// Row operations of the elementwise kernels.
enum EwFn {
    EF_ADD, EF_SUB, EF_MUL, EF_MIN, EF_MAX, EF_LT, EF_LE, EF_GT, EF_GE, EF_EQ, EF_NE,
    EF_AND, EF_OR, EF_XOR, EF_DIV, EF_NEG, EF_ABS, EF_SQRT, EF_NOT, EF_BNOT, EF_SELECT,
    EF_DIVC, EF_CAST
};
// Storage types (bool is stored as u8 0/1).
enum EwTy { ET_F64, ET_F32, ET_I64, ET_U64, ET_I32, ET_U8 };

// The truncating division of div_const_T by a scalar (round-up multiply-high constants).
struct Divider {
    unsigned long long m;
    int sh1, sh2;
    unsigned long long dneg;  // signed types: all ones when the divisor is negative
};
// The divider of divisor bits `d` of storage type `ty`; false for a zero divisor.
bool make_ew_divider(int ty, unsigned long long d, Divider *out);

constexpr int RG_MAX_IN = 8;      // region inputs
constexpr int RG_MAX_ARR = 4;     // of which arrays (held in registers, one step's rows each)
constexpr int RG_MAX_K = 12;      // region kernels
constexpr int RG_MAX_SLOTS = 16;  // inputs + kernels

struct RgIn {
    const void *p;  // array rows
    int width;      // bytes per row
};
// Where an operand comes from: an array input (idx, its number among the arrays), a constant (a scalar input, or an unused
// operand), the previous kernel's value (held in registers), or the shared-memory slot of an
// earlier kernel whose value a later kernel reads (idx).
enum RgKind { RK_IN, RK_CONST, RK_PREV, RK_SLOT };
// Kernel k of the region: operation, operand type, result type, the three operands, and the
// slot its value is kept in when a kernel after the next one reads it.
struct RgOp {
    unsigned char fn, ty, dst;
    unsigned char kind[3], idx[3];
    unsigned char keep, slot;
    unsigned long long c[3];
    Divider dv;
};
struct RegionProg {
    int nk, nslots, out_width, narr;
    int f64only;  // every kernel f64 arithmetic or an f64 comparison, every input f64 (region_f64_kernel)
    RgIn in[RG_MAX_ARR];  // the array inputs, numbered in input order
    RgOp op[RG_MAX_K];
};

// Region folds: the root reduction over the region's value in the same pass.
enum RgFoldKind { RF_MIN, RF_MAX, RF_ARGMIN, RF_ARGMAX, RF_SUM };
struct RgFold {
    long long key;                // the best order key (f64) or value (i64)
    unsigned long long idx;       // its first row (~0: no row yet)
    unsigned long long nan_idx;   // the first NaN row (~0: none)
    unsigned long long sum;       // RF_SUM: the wrapping sum
};
constexpr int RG_FOLD_MAX_GRID = 4096;
// Folds `p`'s value over n > 0 rows: work[0] gets the result, work[1 ..] holds one partial per
// block (RG_FOLD_MAX_GRID at most); *done is a zeroed counter.
vkc_status launch_region_fold(vkc_ctx *ctx, const RegionProg &p, int64_t n, int kind, bool f64, RgFold *work,
                              unsigned *done);

// Runs `p` over n rows into `out` (the last kernel's rows) on the context's stream; with
// `count`, adds the number of nonzero result rows to the u64 at `out` instead.
vkc_status launch_region(vkc_ctx *ctx, const RegionProg &p, int64_t n, void *out, bool count = false);

}  // namespace vkc

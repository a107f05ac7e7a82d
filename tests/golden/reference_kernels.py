"""The reference's kernel table by name, restated from its registration functions (test
infrastructure: the cuda table must hold every kernel that can receive a device array).

Each block below follows one registration function of antiguru/verkehrt; the names are built
the same way (type names of src/value.rs ScalarType::name). Kernels whose operands are all
scalars of types that have no arrays (i8, i16, u16, u32 are scalar-only: src/value.rs:23-31
ARRAY_TYPES) run on the host whatever the ISA and are listed apart.
"""

ARRAY_TYPES = ["f64", "f32", "i64", "u64", "i32", "u8", "bool"]
SCALAR_ONLY = ["i8", "i16", "u16", "u32"]
CMPS = ["eq", "ne", "lt", "le", "gt", "ge"]


def elementwise():
    """src/kernels/scalar/elementwise.rs:757-915 (register). An operation gets an array kernel
    only when its operand and result types are all array types (add_entry_with,
    elementwise.rs:270-296); every operation also gets a host-only `<name>_s` scalar kernel,
    which runs on the host under any ISA and is not listed."""
    ops = []  # (name, types of the operands and the result)
    num = ["i8", "i16", "i32", "i64", "u8", "u16", "u32", "u64", "f32", "f64"]
    for t in num:  # register_num
        ops += [("%s_%s" % (op, t), (t, t, t)) for op in ("add", "sub", "mul", "min", "max")]
        ops += [("%s_%s" % (op, t), (t, t, "bool")) for op in ("lt", "le", "gt", "ge")]
    for t in ("i8", "i16", "i32", "i64", "f32", "f64"):  # register_signed
        ops += [("neg_" + t, (t, t)), ("abs_" + t, (t, t))]
    for t in ("f32", "f64"):  # register_float
        ops += [("div_" + t, (t, t, t)), ("sqrt_" + t, (t, t))]
    for t in ("i64", "u64", "i32", "u8"):  # register_div_const
        ops.append(("div_const_" + t, (t, t, t)))
    for t in num + ["bool"]:  # register_any (+ register_bool's)
        ops += [("eq_" + t, (t, t, "bool")), ("ne_" + t, (t, t, "bool")), ("select_" + t, ("bool", t, t, t))]
    for t in ("i32", "i64", "u8", "u64", "bool"):  # register_bits, register_bool
        ops += [("%s_%s" % (op, t), (t, t, t)) for op in ("and", "or", "xor")] + [("not_" + t, (t, t))]
    for f in num + ["bool"]:  # register_casts
        for t in num:
            ops.append(("cast_%s_%s" % (f, t), (f, t)))
    return [name for name, types in ops if all(t in ARRAY_TYPES for t in types)]


def reductions():
    """src/kernels/scalar/reduce.rs:664-726 (register_numeric, register_bits, register_bool)."""
    out = []
    for t in ("f64", "f32", "i64", "i32", "u8", "u64"):
        out += ["reduce_add_" + t, "reduce_mul_" + t, "reduce_min_" + t, "reduce_max_" + t,
                "argmin_" + t, "argmax_" + t]
    for t in ("i64", "i32", "u8", "u64"):
        out += ["reduce_and_" + t, "reduce_or_" + t, "reduce_xor_" + t]
    out += ["reduce_and_bool", "reduce_or_bool", "reduce_xor_bool", "count", "any", "all"]
    return out


def fused():
    """src/kernels/scalar/fused.rs:290-379 (register_cmp, register_type)."""
    out = []
    for t in ("f64", "f32", "i64", "u64", "i32"):
        out += ["dot_" + t, "sumsq_" + t]
        for c in CMPS:
            out += ["count_%s_%s" % (c, t), "filter_%s_%s" % (c, t), "condsum_%s_%s" % (c, t)]
    return out


def scans():
    """src/kernels/scalar/scan.rs:330-439 (register_scan for each fold, register_prev)."""
    out = []

    def fold(op, t):
        out.extend(["scan_%s_%s" % (op, t), "scan_by_%s_%s" % (op, t), "reduce_into_%s_%s" % (op, t)])

    for t in ("i64", "u64", "i32", "u8"):
        for op in ("add", "mul", "min", "max", "and", "or", "xor"):
            fold(op, t)
    for t in ("f64", "f32"):
        fold("min", t)
        fold("max", t)
    for op in ("and", "or", "xor"):
        fold(op, "bool")
    for t in ARRAY_TYPES:
        out.append("prev_" + t)
    return out


def index():
    """src/kernels/scalar/index.rs:290-325 (argsort, histogram, gather, slice)."""
    out = ["argsort_" + t for t in ("i64", "u64", "i32", "u8")] + ["histogram"]
    out += ["gather_" + t for t in ARRAY_TYPES] + ["slice_" + t for t in ARRAY_TYPES]
    return out


def group():
    """src/kernels/scalar/group.rs:352-363 (group_id, group_id2 on every pair of key types)."""
    keys = ("i64", "u64", "i32", "u8")
    return ["group_id_" + t for t in keys] + ["group_id2_%s_%s" % (a, b) for a in keys for b in keys]


def construct():
    """src/kernels/scalar/construct.rs:214-270 (iota, fill, rand, load, length, same_len)."""
    out = ["iota", "rand_i64", "rand_f64"]
    out += ["fill_" + t for t in ARRAY_TYPES]
    out += ["load_" + t for t in ("f64", "f32", "i64", "u64", "i32", "u8")]
    out += ["length_" + t for t in ARRAY_TYPES] + ["same_len_" + t for t in ARRAY_TYPES]
    return out


def select():
    """src/kernels/scalar/select.rs:236-260 (compress, where)."""
    return ["compress_" + t for t in ARRAY_TYPES] + ["where"]


def all_names():
    return elementwise() + reductions() + fused() + scans() + index() + group() + construct() + select()


def device_names():
    """Every kernel above: each can receive a device array."""
    return all_names()

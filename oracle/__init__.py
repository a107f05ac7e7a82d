"""The CPU oracle: TEST INFRASTRUCTURE ONLY.

numpy-facing ctypes wrapper over liboracle.so, the plain-C restatement of the reference's
scalar kernel entries (oracle.c cites the reference file:line of each). Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use it; the CUDA library never does.
Functions that fail raise OracleError with the reference's message text.
"""

import ctypes
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None
ERR_LEN = 256
CMPS = {"eq": 0, "ne": 1, "lt": 2, "le": 3, "gt": 4, "ge": 5}


class OracleError(Exception):
    pass


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = ctypes.CDLL(path)
        L = _lib
        P, I64, D, U64 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_uint64
        L.orc_splitmix64.restype = U64
        L.orc_splitmix64.argtypes = [U64]
        L.orc_rand_f64.argtypes = [I64, I64, P]
        L.orc_rand_i64.argtypes = [I64, I64, P]
        for name in ("orc_reduce_add_f64", "orc_reduce_mul_f64", "orc_sumsq_f64", "orc_neumaier_sum"):
            getattr(L, name).restype = D
            getattr(L, name).argtypes = [P, I64]
        L.orc_dot_f64.restype = D
        L.orc_dot_f64.argtypes = [P, P, I64]
        L.orc_count_cmp_f64.restype = I64
        L.orc_count_cmp_f64.argtypes = [P, I64, ctypes.c_int, D]
        L.orc_condsum_cmp_f64.restype = D
        L.orc_condsum_cmp_f64.argtypes = [P, I64, ctypes.c_int, D, D]
        L.orc_filter_cmp_f64.restype = I64
        L.orc_filter_cmp_f64.argtypes = [P, I64, ctypes.c_int, D, P]
        L.orc_reduce_minmax_f64.argtypes = [P, I64, ctypes.c_int, P, ctypes.c_char_p]
        L.orc_argext_f64.argtypes = [P, I64, ctypes.c_int, P, ctypes.c_char_p]
        L.orc_reduce_minmax_i64.argtypes = [P, I64, ctypes.c_int, P, ctypes.c_char_p]
        L.orc_argext_i64.argtypes = [P, I64, ctypes.c_int, P, ctypes.c_char_p]
        L.orc_reduce_add_i64.restype = I64
        L.orc_reduce_add_i64.argtypes = [P, I64]
        L.orc_compress.restype = I64
        L.orc_compress.argtypes = [P, ctypes.c_int, P, I64, P]
        L.orc_where.restype = I64
        L.orc_where.argtypes = [P, I64, I64, P]
        L.orc_scan_add_i64.argtypes = [P, I64, P]
        L.orc_scan_by_add_i64.argtypes = [P, P, I64, P]
        L.orc_scan_add_f64.argtypes = [P, I64, P]
        L.orc_scan_by_add_f64.argtypes = [P, P, I64, P]
        L.orc_prev_i64.argtypes = [P, I64, I64, P]
        L.orc_gather.argtypes = [P, ctypes.c_int, I64, P, I64, P, ctypes.c_char_p]
        L.orc_histogram.argtypes = [P, I64, I64, P, ctypes.c_char_p]
        L.orc_reduce_into_add_i64.argtypes = [P, P, I64, I64, P, ctypes.c_char_p]
        L.orc_reduce_into_add_f64.argtypes = [P, P, I64, I64, P, ctypes.c_char_p]
        L.orc_argsort_i64.argtypes = [P, I64, P, ctypes.c_char_p]
        L.orc_argsort_reference_i64.argtypes = [P, I64, P]
        L.orc_group_id_i64.argtypes = [P, I64, P, ctypes.c_char_p]
        L.orc_group_id2_i64_i64.argtypes = [P, P, I64, P, ctypes.c_char_p]
        L.orc_mul_f64.argtypes = [P, P, I64, P]
        L.orc_cmp_f64.argtypes = [P, P, I64, ctypes.c_int, P]
        L.orc_select_f64.argtypes = [P, P, P, I64, P]
        L.orc_dd_sum.argtypes = [P, I64, P, P]
        C, INT = ctypes.c_char_p, ctypes.c_int
        L.orc_ew_binary.argtypes = [C, INT, P, INT, P, INT, I64, P]
        L.orc_ew_unary.argtypes = [C, INT, P, I64, P]
        L.orc_ew_select.argtypes = [INT, P, INT, P, INT, P, INT, I64, P]
        L.orc_ew_cast.argtypes = [INT, INT, P, I64, P]
        L.orc_ew_div_const.argtypes = [INT, P, P, I64, P, C]
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _f64(x):
    return np.ascontiguousarray(x, dtype=np.float64)


def _i64(x):
    return np.ascontiguousarray(x, dtype=np.int64)


def _u8(x):
    return np.ascontiguousarray(np.asarray(x).astype(np.uint8))


def _err(rc, buf):
    if rc:
        raise OracleError(buf.value.decode())


def splitmix64(x):
    return int(lib().orc_splitmix64(x & 0xFFFFFFFFFFFFFFFF))


def rand_f64(n, seed):
    out = np.empty(n, dtype=np.float64)
    lib().orc_rand_f64(n, seed, _p(out))
    return out


def rand_i64(n, seed):
    out = np.empty(n, dtype=np.int64)
    lib().orc_rand_i64(n, seed, _p(out))
    return out


def reduce_add_f64(x):
    x = _f64(x)
    return lib().orc_reduce_add_f64(_p(x), len(x))


def reduce_mul_f64(x):
    x = _f64(x)
    return lib().orc_reduce_mul_f64(_p(x), len(x))


def dot_f64(x, y):
    x, y = _f64(x), _f64(y)
    return lib().orc_dot_f64(_p(x), _p(y), len(x))


def sumsq_f64(x):
    x = _f64(x)
    return lib().orc_sumsq_f64(_p(x), len(x))


def count_cmp_f64(x, cmp, c):
    x = _f64(x)
    return int(lib().orc_count_cmp_f64(_p(x), len(x), CMPS[cmp], c))


def condsum_cmp_f64(x, cmp, c, e):
    x = _f64(x)
    return lib().orc_condsum_cmp_f64(_p(x), len(x), CMPS[cmp], c, e)


def filter_cmp_f64(x, cmp, c):
    x = _f64(x)
    out = np.empty(len(x), dtype=np.float64)
    k = lib().orc_filter_cmp_f64(_p(x), len(x), CMPS[cmp], c, _p(out))
    return out[:k].copy()


def _ext(fn, x, is_max, dtype):
    out = np.zeros(1, dtype=dtype)
    buf = ctypes.create_string_buffer(ERR_LEN)
    _err(fn(_p(x), len(x), int(is_max), _p(out), buf), buf)
    return out[0]


def reduce_min_f64(x):
    return float(_ext(lib().orc_reduce_minmax_f64, _f64(x), False, np.float64))


def reduce_max_f64(x):
    return float(_ext(lib().orc_reduce_minmax_f64, _f64(x), True, np.float64))


def argmin_f64(x):
    return int(_ext(lib().orc_argext_f64, _f64(x), False, np.int64))


def argmax_f64(x):
    return int(_ext(lib().orc_argext_f64, _f64(x), True, np.int64))


def reduce_min_i64(x):
    return int(_ext(lib().orc_reduce_minmax_i64, _i64(x), False, np.int64))


def reduce_max_i64(x):
    return int(_ext(lib().orc_reduce_minmax_i64, _i64(x), True, np.int64))


def argmin_i64(x):
    return int(_ext(lib().orc_argext_i64, _i64(x), False, np.int64))


def argmax_i64(x):
    return int(_ext(lib().orc_argext_i64, _i64(x), True, np.int64))


def reduce_add_i64(x):
    x = _i64(x)
    return int(lib().orc_reduce_add_i64(_p(x), len(x)))


def compress(x, mask):
    x = np.ascontiguousarray(x)
    m = _u8(mask)
    out = np.empty_like(x)
    k = lib().orc_compress(_p(x), x.dtype.itemsize, _p(m), len(x), _p(out))
    return out[:k].copy()


def where(mask, base=0):
    m = _u8(mask)
    out = np.empty(len(m), dtype=np.int64)
    k = lib().orc_where(_p(m), len(m), base, _p(out))
    return out[:k].copy()


def scan_add_i64(x):
    x = _i64(x)
    out = np.empty(len(x), dtype=np.int64)
    lib().orc_scan_add_i64(_p(x), len(x), _p(out))
    return out


def scan_by_add_i64(x, starts):
    x, s = _i64(x), _u8(starts)
    out = np.empty(len(x), dtype=np.int64)
    lib().orc_scan_by_add_i64(_p(x), _p(s), len(x), _p(out))
    return out


def prev_i64(x, fill):
    x = _i64(x)
    out = np.empty(len(x), dtype=np.int64)
    lib().orc_prev_i64(_p(x), len(x), fill, _p(out))
    return out


def gather(src, idx):
    src = np.ascontiguousarray(src)
    idx = _i64(idx)
    out = np.empty(len(idx), dtype=src.dtype)
    buf = ctypes.create_string_buffer(ERR_LEN)
    _err(lib().orc_gather(_p(src), src.dtype.itemsize, len(src), _p(idx), len(idx), _p(out), buf), buf)
    return out


def _huge_buckets(keys, buckets):
    """The errors of a bucket count too large to allocate here (index.rs:116-130, then
    value.rs:285-307): a negative count, the first key out of range, the size cap, then the
    allocation failure."""
    if buckets < 0:
        raise OracleError("negative bucket count %d" % buckets)
    bad = np.nonzero(keys.view(np.uint64) >= np.uint64(buckets))[0]
    if len(bad):
        raise OracleError("bucket key %d out of range for %d buckets" % (keys[bad[0]], buckets))
    if buckets > (1 << 63) // 8 - 1:
        raise OracleError("array of %d elements is too large" % buckets)
    raise OracleError("cannot allocate an array of %d elements" % buckets)


def histogram(keys, buckets):
    keys = _i64(keys)
    if buckets > 1 << 28:
        _huge_buckets(keys, buckets)
    out = np.empty(max(0, min(buckets, 1 << 28)), dtype=np.int64)
    buf = ctypes.create_string_buffer(ERR_LEN)
    _err(lib().orc_histogram(_p(keys), len(keys), buckets, _p(out), buf), buf)
    return out


def reduce_into_add_i64(keys, vals, buckets):
    keys, vals = _i64(keys), _i64(vals)
    if len(keys) != len(vals):
        # index.rs:203-210: the key check comes first, then the length mismatch.
        buf = ctypes.create_string_buffer(ERR_LEN)
        tmp = np.empty(max(0, min(buckets, 1 << 20)), dtype=np.int64)
        if buckets >= 0 and buckets <= (1 << 20):
            _err(lib().orc_histogram(_p(keys), len(keys), buckets, _p(tmp), buf), buf)
        raise OracleError("length mismatch: %d keys for %d values" % (len(keys), len(vals)))
    if buckets > 1 << 28:
        _huge_buckets(keys, buckets)
    out = np.empty(max(0, min(buckets, 1 << 28)), dtype=np.int64)
    buf = ctypes.create_string_buffer(ERR_LEN)
    _err(lib().orc_reduce_into_add_i64(_p(keys), _p(vals), len(keys), buckets, _p(out), buf), buf)
    return out


def scan_add_f64(x):
    """Prefix canonical sums: out[i] = reduce_add_f64(x[:i + 1]) (the candidate float scan order
    of the reference's tier-2 notes; oracle.c orc_scan_add_f64)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty(len(x), dtype=np.float64)
    lib().orc_scan_add_f64(_p(x), len(x), _p(out))
    return out


def scan_by_add_f64(x, starts):
    """scan_add_f64 restarted at every set start flag (row 0 always starts)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    s = np.ascontiguousarray(starts, dtype=np.uint8)
    assert len(s) == len(x)
    out = np.empty(len(x), dtype=np.float64)
    lib().orc_scan_by_add_f64(_p(x), _p(s), len(x), _p(out))
    return out


def reduce_into_add_f64(keys, vals, buckets):
    """Per-bucket float sums in the candidate stripe order of the reference's tier-2 notes,
    with the canonical tail rule (oracle.c orc_reduce_into_add_f64)."""
    keys, vals = _i64(keys), np.ascontiguousarray(vals, dtype=np.float64)
    if len(keys) != len(vals):
        buf = ctypes.create_string_buffer(ERR_LEN)
        tmp = np.empty(max(0, min(buckets, 1 << 20)), dtype=np.int64)
        if buckets >= 0 and buckets <= (1 << 20):
            _err(lib().orc_histogram(_p(keys), len(keys), buckets, _p(tmp), buf), buf)
        raise OracleError("length mismatch: %d keys for %d values" % (len(keys), len(vals)))
    if buckets > 1 << 28:
        _huge_buckets(keys, buckets)
    out = np.empty(max(0, min(buckets, 1 << 28)), dtype=np.float64)
    buf = ctypes.create_string_buffer(ERR_LEN)
    _err(lib().orc_reduce_into_add_f64(_p(keys), _p(vals), len(keys), buckets, _p(out), buf), buf)
    return out


def argsort_i64(x):
    x = _i64(x)
    out = np.empty(len(x), dtype=np.int64)
    buf = ctypes.create_string_buffer(ERR_LEN)
    _err(lib().orc_argsort_i64(_p(x), len(x), _p(out), buf), buf)
    return out


def argsort_reference_i64(x):
    x = _i64(x)
    out = np.empty(len(x), dtype=np.int64)
    lib().orc_argsort_reference_i64(_p(x), len(x), _p(out))
    return out


def group_id_i64(x):
    x = _i64(x)
    out = np.empty(len(x), dtype=np.int64)
    buf = ctypes.create_string_buffer(ERR_LEN)
    _err(lib().orc_group_id_i64(_p(x), len(x), _p(out), buf), buf)
    return out


def group_id2_i64_i64(x, y):
    x, y = _i64(x), _i64(y)
    if len(x) != len(y):
        raise OracleError("length mismatch: %d vs %d" % (len(x), len(y)))
    out = np.empty(len(x), dtype=np.int64)
    buf = ctypes.create_string_buffer(ERR_LEN)
    _err(lib().orc_group_id2_i64_i64(_p(x), _p(y), len(x), _p(out), buf), buf)
    return out


def mul_f64(x, y):
    x, y = _f64(x), _f64(y)
    out = np.empty(len(x), dtype=np.float64)
    lib().orc_mul_f64(_p(x), _p(y), len(x), _p(out))
    return out


def cmp_f64(x, y, cmp):
    x, y = _f64(x), _f64(y)
    out = np.empty(len(x), dtype=np.uint8)
    lib().orc_cmp_f64(_p(x), _p(y), len(x), CMPS[cmp], _p(out))
    return out


def select_f64(m, a, b):
    m, a, b = _u8(m), _f64(a), _f64(b)
    out = np.empty(len(m), dtype=np.float64)
    lib().orc_select_f64(_p(m), _p(a), _p(b), len(m), _p(out))
    return out


def neumaier_sum(x):
    x = _f64(x)
    return lib().orc_neumaier_sum(_p(x), len(x))


def dd_sum(x):
    x = _f64(x)
    hi, lo = ctypes.c_double(), ctypes.c_double()
    lib().orc_dd_sum(_p(x), len(x), ctypes.byref(hi), ctypes.byref(lo))
    return hi.value, lo.value


# ---------------------------------------------------------------- elementwise, every array type

EW_TYPES = {"f64": 0, "f32": 1, "i64": 2, "u64": 3, "i32": 4, "u8": 5, "bool": 6}
EW_DTYPES = {"f64": np.float64, "f32": np.float32, "i64": np.int64, "u64": np.uint64, "i32": np.int32,
             "u8": np.uint8, "bool": np.uint8}
EW_BOOL_OUT = ("lt", "le", "gt", "ge", "eq", "ne")


def _ew_operand(x, t):
    """(contiguous array, is_splat) of operand x of element type t."""
    a = np.ascontiguousarray(np.atleast_1d(np.asarray(x)).astype(EW_DTYPES[t], copy=False))
    return a, np.ndim(x) == 0


def ew_binary(op, t, a, b):
    """elementwise.rs binary `op` on type t; a or b may be a scalar (a splat row)."""
    (xa, sa), (xb, sb) = _ew_operand(a, t), _ew_operand(b, t)
    n = max(1 if sa else len(xa), 1 if sb else len(xb)) if (sa and sb) else (len(xb) if sa else len(xa))
    out = np.empty(n, dtype=np.uint8 if (op in EW_BOOL_OUT or t == "bool") else EW_DTYPES[t])
    if lib().orc_ew_binary(op.encode(), EW_TYPES[t], _p(xa), int(sa), _p(xb), int(sb), n, _p(out)) != 0:
        raise OracleError("no %s on %s" % (op, t))
    return out


def ew_unary(op, t, a):
    x, _ = _ew_operand(a, t)
    out = np.empty(len(x), dtype=EW_DTYPES[t])
    if lib().orc_ew_unary(op.encode(), EW_TYPES[t], _p(x), len(x), _p(out)) != 0:
        raise OracleError("no %s on %s" % (op, t))
    return out


def ew_select(t, m, a, b):
    (xm, sm), (xa, sa), (xb, sb) = _ew_operand(m, "bool"), _ew_operand(a, t), _ew_operand(b, t)
    n = max(len(v) for v, s in ((xm, sm), (xa, sa), (xb, sb)) if not s) if not (sm and sa and sb) else 1
    out = np.empty(n, dtype=EW_DTYPES[t])
    lib().orc_ew_select(out.itemsize, _p(xm), int(sm), _p(xa), int(sa), _p(xb), int(sb), n, _p(out))
    return out


def ew_cast(src, dst, a):
    x, _ = _ew_operand(a, src)
    out = np.empty(len(x), dtype=EW_DTYPES[dst])
    if lib().orc_ew_cast(EW_TYPES[src], EW_TYPES[dst], _p(x), len(x), _p(out)) != 0:
        raise OracleError("no cast %s -> %s" % (src, dst))
    return out


def ew_div_const(t, a, d):
    x, _ = _ew_operand(a, t)
    dv, _ = _ew_operand(d, t)
    out = np.empty(len(x), dtype=EW_DTYPES[t])
    err = ctypes.create_string_buffer(256)
    if lib().orc_ew_div_const(EW_TYPES[t], _p(x), _p(dv), len(x), _p(out), err) != 0:
        raise OracleError(err.value.decode())
    return out


# ---------------------------------------------------------------- the families on every type (families.c)

FAMILY_TYPES = {"f64": 0, "f32": 1, "i64": 2, "u64": 3, "i32": 4, "u8": 5, "bool": 6}
FOLDS = {"add": 0, "mul": 1, "min": 2, "max": 3, "and": 4, "or": 5, "xor": 6}
NP_TYPES = {"f64": np.float64, "f32": np.float32, "i64": np.int64, "u64": np.uint64, "i32": np.int32,
            "u8": np.uint8, "bool": np.uint8}
WIDTH = {"f64": 8, "f32": 4, "i64": 8, "u64": 8, "i32": 4, "u8": 1, "bool": 1}


def _fam_lib():
    L = lib()
    if not getattr(L, "_families", False):
        P, I64, INT, U64 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_uint64
        C = ctypes.c_char_p
        L.orc_fold.argtypes = [INT, INT, P, I64, ctypes.POINTER(U64), C]
        L.orc_argext.argtypes = [INT, INT, P, I64, ctypes.POINTER(I64), C]
        L.orc_fused_sum.restype = U64
        L.orc_fused_sum.argtypes = [INT, INT, INT, P, P, I64, U64, U64]
        L.orc_count_cmp.restype = I64
        L.orc_count_cmp.argtypes = [INT, INT, P, I64, U64]
        L.orc_filter_cmp.restype = I64
        L.orc_filter_cmp.argtypes = [INT, INT, P, I64, U64, P]
        L.orc_scan.argtypes = [INT, INT, INT, P, P, I64, P]
        L.orc_reduce_into.argtypes = [INT, INT, P, I64, P, I64, I64, P, C]
        L._families = True
    return L


def sum_type(t):
    """The result type of add (reduce.rs:559-586): i32 widens to i64, u8 to u64."""
    return {"i32": "i64", "u8": "u64"}.get(t, t)


def as_type(x, t):
    return np.ascontiguousarray(np.asarray(x).astype(NP_TYPES[t]))


def word(t, v):
    """A scalar of type t as families.c's 64-bit word."""
    if t == "f64":
        return int(np.float64(v).view(np.uint64))
    if t == "f32":
        return int(np.float32(v).view(np.uint32))
    if t in ("i64", "i32"):
        return int(v) & 0xFFFFFFFFFFFFFFFF
    return int(v) & 0xFFFFFFFFFFFFFFFF


def word_bits(t, w):
    """The bits of a result word in the type's width (what the device returns in its low bytes)."""
    return int(w) & ((1 << (8 * WIDTH[t])) - 1)


def fold(t, f, x):
    """reduce_<f>_<t>: the result word (sum type for add), in the result type's width."""
    x = as_type(x, t)
    out = ctypes.c_uint64()
    buf = ctypes.create_string_buffer(ERR_LEN)
    _err(_fam_lib().orc_fold(FAMILY_TYPES[t], FOLDS[f], _p(x), len(x), ctypes.byref(out), buf), buf)
    return word_bits(sum_type(t) if f == "add" else t, out.value)


def argext(t, is_max, x):
    x = as_type(x, t)
    out = ctypes.c_int64()
    buf = ctypes.create_string_buffer(ERR_LEN)
    _err(_fam_lib().orc_argext(FAMILY_TYPES[t], int(is_max), _p(x), len(x), ctypes.byref(out), buf), buf)
    return out.value


def fused_sum(t, what, x, y=None, cmp="eq", c=0, e=0):
    """dot / sumsq / condsum_<cmp> on t: the result word in the sum type's width."""
    x = as_type(x, t)
    y = as_type(y, t) if y is not None else x
    w = _fam_lib().orc_fused_sum(FAMILY_TYPES[t], {"dot": 0, "sumsq": 1, "condsum": 2}[what], CMPS[cmp],
                                 _p(x), _p(y), len(x), word(t, c), word(t, e))
    return word_bits(sum_type(t), w)


def count_cmp(t, cmp, x, c):
    x = as_type(x, t)
    return int(_fam_lib().orc_count_cmp(FAMILY_TYPES[t], CMPS[cmp], _p(x), len(x), word(t, c)))


def filter_cmp(t, cmp, x, c):
    x = as_type(x, t)
    out = np.empty(len(x), dtype=NP_TYPES[t])
    k = _fam_lib().orc_filter_cmp(FAMILY_TYPES[t], CMPS[cmp], _p(x), len(x), word(t, c), _p(out))
    return out[:k]


def scan(t, f, x, starts=None):
    """scan_<f>_<t> (starts None) or scan_by_<f>_<t>: the output rows (sum type for add)."""
    x = as_type(x, t)
    ot = sum_type(t) if f == "add" else t
    out = np.empty(len(x), dtype=NP_TYPES[ot])
    s = _u8(starts) if starts is not None else np.zeros(1, np.uint8)
    _fam_lib().orc_scan(FAMILY_TYPES[t], FOLDS[f], int(starts is not None), _p(x), _p(s), len(x), _p(out))
    return out


def reduce_into(t, f, keys, vals, buckets):
    """reduce_into_<f>_<t>: the bucket rows (sum type for add), errors as the reference's."""
    keys, vals = _i64(keys), as_type(vals, t)
    ot = sum_type(t) if f == "add" else t
    if buckets > 1 << 28 and len(keys) == len(vals):
        _huge_buckets(keys, buckets)
    out = np.empty(max(0, min(buckets, 1 << 28)), dtype=NP_TYPES[ot])
    buf = ctypes.create_string_buffer(ERR_LEN)
    _err(_fam_lib().orc_reduce_into(FAMILY_TYPES[t], FOLDS[f], _p(keys), len(keys), _p(vals), len(vals),
                                    buckets, _p(out), buf), buf)
    return out

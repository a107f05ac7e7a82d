"""The elementwise kernels of every array type (src/kernels/scalar/elementwise.rs:757-873) equal
the oracle bit for bit (a NaN only has to be NaN): Num ops, neg/abs, div/sqrt, eq/ne/select,
bits, bool ops, Rust `as` casts and div_const, with array and scalar operands and the edge
values of each type. The CPU test checks that the table holds every array kernel the
reference registers, with its cost."""

import numpy as np
import pytest

import oracle
from verkehrt_gb300 import Scalar

TYPES = ["f64", "f32", "i64", "u64", "i32", "u8"]
SIGNED = ["f64", "f32", "i64", "i32"]
BITS = ["i64", "u64", "i32", "u8"]
DIV_CONST = ["i64", "u64", "i32", "u8"]
WIDTH = {"f64": 8, "f32": 4, "i64": 8, "u64": 8, "i32": 4, "u8": 1, "bool": 1}
NUM_OPS = ["add", "sub", "mul", "min", "max", "lt", "le", "gt", "ge"]
BOOL_OUT = ("lt", "le", "gt", "ge", "eq", "ne")


def expected_table():
    """Every array elementwise kernel of the reference's registration (name -> cost)."""
    t = {}
    for ty in TYPES:
        w = WIDTH[ty]
        for op in NUM_OPS:
            t["%s_%s" % (op, ty)] = 2 * w + (1 if op in BOOL_OUT else w)
    for ty in SIGNED:
        t["neg_" + ty] = t["abs_" + ty] = 2 * WIDTH[ty]
    for ty in ("f64", "f32"):
        t["div_" + ty] = 3 * WIDTH[ty]
        t["sqrt_" + ty] = 2 * WIDTH[ty]
    for ty in DIV_CONST:
        t["div_const_" + ty] = 3 * WIDTH[ty]
    for ty in TYPES + ["bool"]:
        w = WIDTH[ty]
        t["eq_" + ty] = t["ne_" + ty] = 2 * w + 1
        t["select_" + ty] = 1 + 3 * w
    for ty in BITS:
        w = WIDTH[ty]
        for op in ("and", "or", "xor"):
            t["%s_%s" % (op, ty)] = 3 * w
        t["not_" + ty] = 2 * w
    for op in ("and", "or", "xor"):
        t[op + "_bool"] = 3
    t["not_bool"] = 2
    for src in TYPES + ["bool"]:
        for dst in TYPES:
            t["cast_%s_%s" % (src, dst)] = WIDTH[src] + WIDTH[dst]
    return t


def test_table_holds_every_array_elementwise_kernel():
    import verkehrt_gb300 as vk

    got = {name: (cls, cost) for name, cls, _, cost in vk.kernels()}
    want = expected_table()
    assert len(want) == 153
    for name, cost in want.items():
        assert name in got, name
        assert got[name] == ("elementwise", cost), name


def edge_values(ty):
    if ty in ("f64", "f32"):
        v = [0.0, -0.0, 1.0, -1.0, 0.5, -2.5, 3.5, np.inf, -np.inf, np.nan, 1e-310, -1e-310, 1e38, -1e38,
             3.4e38, 1e300, -1e300, 2.0 ** 31, -(2.0 ** 31), 2.0 ** 31 - 0.5, 2.0 ** 63, -(2.0 ** 63),
             2.0 ** 64, 255.5, 256.0, -0.5, 4294967295.0, 9007199254740993.0]
        with np.errstate(over="ignore"):
            return np.array(v, dtype=np.float64 if ty == "f64" else np.float32)
    info = np.iinfo({"i64": np.int64, "u64": np.uint64, "i32": np.int32, "u8": np.uint8}[ty])
    v = [0, 1, 2, 3, 7, info.max, info.max - 1, info.min, info.min + 1 if info.min else 5, 100]
    if info.min < 0:
        v += [-1, -2, -3, -7, -100]
    return np.array(v, dtype=info.dtype)


def values(ty, n, seed):
    """n values of type ty: the edge values, then seeded random bits (floats: varied magnitudes)."""
    e = edge_values(ty)
    r = oracle.rand_i64(n, seed).view(np.uint64)
    if ty == "f64":
        rnd = (oracle.rand_f64(n, seed) - 0.5) * np.exp2((r % np.uint64(80)).astype(np.float64) - 40)
    elif ty == "f32":
        rnd = ((oracle.rand_f64(n, seed) - 0.5) * np.exp2((r % np.uint64(60)).astype(np.float64) - 30)).astype(np.float32)
    else:
        rnd = r.astype(e.dtype) if ty != "i32" else (r & np.uint64(0xFFFFFFFF)).astype(np.uint32).view(np.int32)
        if ty == "u8":
            rnd = (r % np.uint64(256)).astype(np.uint8)
        if ty == "i64":
            rnd = r.view(np.int64)
    out = np.concatenate([e, rnd.astype(e.dtype)])[:n]
    return out


def same(got, want):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape
    if got.dtype.kind == "f":
        nan = np.isnan(want)
        assert np.array_equal(np.isnan(got), nan)
        ui = np.uint64 if got.dtype == np.float64 else np.uint32
        return bool(np.array_equal(got[~nan].view(ui), want[~nan].view(ui)))
    return bool(np.array_equal(got.astype(want.dtype), want))


N = 5003


@pytest.mark.gpu
@pytest.mark.parametrize("ty", TYPES)
def test_num_ops(ctx, ty):
    a, b = values(ty, N, 1), values(ty, N, 2)
    b[: len(edge_values(ty))] = edge_values(ty)[::-1]
    da, db = ctx.upload(a, ty), ctx.upload(b, ty)
    ops = NUM_OPS + ["eq", "ne"] + (["and", "or", "xor"] if ty in BITS else []) + (["div"] if ty in ("f64", "f32") else [])
    for op in ops:
        name = "%s_%s" % (op, ty)
        assert same(ctx.call(name, da, db).numpy(), oracle.ew_binary(op, ty, a, b)), name
        s = b[3].item()
        assert same(ctx.call(name, da, Scalar(ty, s)).numpy(), oracle.ew_binary(op, ty, a, np.array(s, dtype=a.dtype))), name
        assert same(ctx.call(name, Scalar(ty, s), db).numpy(), oracle.ew_binary(op, ty, np.array(s, dtype=a.dtype), b)), name


@pytest.mark.gpu
@pytest.mark.parametrize("ty", TYPES + ["bool"])
def test_unary_select_and_bool(ctx, ty):
    if ty == "bool":
        p = (oracle.rand_i64(N, 5) % 2).astype(np.uint8)
        q = (oracle.rand_i64(N, 6) % 2).astype(np.uint8)
        dp, dq = ctx.upload(p, "bool"), ctx.upload(q, "bool")
        for op in ("and", "or", "xor", "eq", "ne"):
            assert same(ctx.call(op + "_bool", dp, dq).numpy(), oracle.ew_binary(op, "bool", p, q).astype(bool)), op
        assert same(ctx.call("not_bool", dp).numpy(), oracle.ew_unary("not", "bool", p).astype(bool))
        got = ctx.call("select_bool", dp, dq, Scalar("bool", True)).numpy()
        assert same(got, oracle.ew_select("bool", p, q, np.array(1, dtype=np.uint8)).astype(bool))
        return
    a = values(ty, N, 3)
    da = ctx.upload(a, ty)
    unary = (["neg", "abs"] if ty in SIGNED else []) + (["sqrt"] if ty in ("f64", "f32") else []) + \
            (["not"] if ty in BITS else [])
    for op in unary:
        assert same(ctx.call("%s_%s" % (op, ty), da).numpy(), oracle.ew_unary(op, ty, a)), op
    m = (oracle.rand_i64(N, 4) % 2).astype(np.uint8)
    b = values(ty, N, 9)
    got = ctx.call("select_" + ty, ctx.upload(m, "bool"), da, ctx.upload(b, ty)).numpy()
    want = oracle.ew_select(ty, m, a, b)
    # select moves bits, NaN payloads included.
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    s = a[5].item()
    got = ctx.call("select_" + ty, ctx.upload(m, "bool"), Scalar(ty, s), da).numpy()
    assert np.array_equal(got.view(np.uint8), oracle.ew_select(ty, m, np.array(s, dtype=a.dtype), a).view(np.uint8))


@pytest.mark.gpu
@pytest.mark.parametrize("src", TYPES + ["bool"])
def test_casts(ctx, src):
    a = (oracle.rand_i64(N, 7) % 2).astype(np.uint8) if src == "bool" else values(src, N, 7)
    da = ctx.upload(a, src)
    for dst in TYPES:
        name = "cast_%s_%s" % (src, dst)
        assert same(ctx.call(name, da).numpy(), oracle.ew_cast(src, dst, a)), name


@pytest.mark.gpu
@pytest.mark.parametrize("ty", DIV_CONST)
def test_div_const(ctx, ty):
    a = values(ty, N, 11)
    da = ctx.upload(a, ty)
    e = edge_values(ty)
    r = oracle.rand_i64(64, 12).view(np.uint64)
    divisors = list(e[e != 0]) + [x for x in r.astype(a.dtype) if x != 0][:40] + [3, 5, 7, 10, 255, 641]
    if ty in ("i64", "i32"):
        divisors += [-3, -10, -641]
    for d in divisors:
        d = np.array(d).astype(a.dtype)
        if d == 0:
            continue
        got = ctx.call("div_const_" + ty, da, Scalar(ty, d.item())).numpy()
        assert same(got, oracle.ew_div_const(ty, a, d)), (ty, d)
    with pytest.raises(Exception, match="^div_const: division by zero$"):
        ctx.call("div_const_" + ty, da, Scalar(ty, 0))

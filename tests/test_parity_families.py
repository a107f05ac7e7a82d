"""The kernel families on every element type against the oracle (oracle/families.c): the
reductions, argmin/argmax, fused kernels, scans, segmented scans, bucket folds and prev of the
reference's registry on f64/f32/i64/u64/i32/u8/bool, plus argsort, group ids, fill, slice and
same_len on the other key types. Integers and indices bit for bit; floats bit for bit, except
that a NaN only has to be NaN (tests/isa_variants.rs:300-309)."""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TYPES = ["f64", "f32", "i64", "u64", "i32", "u8", "bool"]
INT_TYPES = ["i64", "u64", "i32", "u8"]
SIZES = [0, 1, 15, 16, 17, 1000, 4097, 70_001]


def data(t, n, seed):
    """Seeded rows of type t with the type's edge values mixed in."""
    r = oracle.rand_i64(n, seed)
    if t in ("f64", "f32"):
        x = (oracle.rand_f64(n, seed) - 0.5) * 8.0
        sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e300 if t == "f64" else 3e38, -2.5])
        pick = (r.view(np.uint64) % np.uint64(41)).astype(np.int64)
        for i, v in enumerate(sp):
            x = np.where(pick == i, v, x)
        return x.astype(np.float64 if t == "f64" else np.float32)
    if t == "bool":
        return (r & 1).astype(np.uint8)
    if t == "u8":
        return (r & 0xFF).astype(np.uint8)
    if t == "i32":
        x = (r & 0xFFFFFFFF).astype(np.uint32).view(np.int32).copy()
        if n > 3:
            x[1], x[2] = np.iinfo(np.int32).min, np.iinfo(np.int32).max
        return x
    if t == "u64":
        return r.view(np.uint64).copy()
    x = r.copy()
    if n > 3:
        x[1], x[2] = np.iinfo(np.int64).min, np.iinfo(np.int64).max
    return x


def small(t, n, seed):
    """Rows of few distinct values (products that do not vanish at once, ties for extremes)."""
    r = (oracle.rand_i64(n, seed).view(np.uint64) % np.uint64(7)).astype(np.int64) - 3
    if t in ("f64", "f32"):
        return (1.0 + r / 64.0).astype(oracle.NP_TYPES[t])
    if t in ("u64", "u8", "bool"):
        return np.abs(r).astype(oracle.NP_TYPES[t]) & (1 if t == "bool" else 0xFF)
    return r.astype(oracle.NP_TYPES[t])


def scalar(t, v):
    import verkehrt_gb300 as vk

    return vk.Scalar(t, v)


def same_word(t, got_bits, want_bits):
    w = oracle.WIDTH[t] * 8
    g, e = got_bits & ((1 << w) - 1), want_bits & ((1 << w) - 1)
    if t == "f64":
        gf, ef = np.uint64(g).view(np.float64), np.uint64(e).view(np.float64)
        return g == e or (np.isnan(gf) and np.isnan(ef))
    if t == "f32":
        gf, ef = np.uint32(g).view(np.float32), np.uint32(e).view(np.float32)
        return g == e or (np.isnan(gf) and np.isnan(ef))
    return g == e


def same_rows(t, got, want):
    got, want = np.asarray(got), np.asarray(want)
    if got.shape != want.shape:
        return False
    if t in ("f64", "f32"):
        ui = np.uint64 if t == "f64" else np.uint32
        gb, wb = got.astype(oracle.NP_TYPES[t]).view(ui), want.astype(oracle.NP_TYPES[t]).view(ui)
        nan = np.isnan(got.astype(np.float64)) & np.isnan(want.astype(np.float64))
        return bool(np.all((gb == wb) | nan))
    return bool(np.array_equal(got.astype(oracle.NP_TYPES[t]).view(np.uint8),
                               want.astype(oracle.NP_TYPES[t]).view(np.uint8)))


def err_of(fn):
    import verkehrt_gb300 as vk

    try:
        fn()
    except (vk.KernelError, oracle.OracleError) as e:
        return str(e)
    return None


REDUCE_FOLDS = {t: ["add", "mul", "min", "max"] + (["and", "or", "xor"] if t in INT_TYPES else [])
                for t in ["f64", "f32", "i64", "i32", "u8", "u64"]}
REDUCE_FOLDS["bool"] = ["and", "or", "xor"]


@pytest.mark.parametrize("t", TYPES)
def test_reductions(ctx, t):
    for f in REDUCE_FOLDS[t]:
        for n in SIZES:
            for gen in (data, small):
                x = gen(t, n, n + 3)
                dx = ctx.upload(x, t)
                name = "reduce_%s_%s" % (f, t)
                want_err = err_of(lambda: oracle.fold(t, f, x))
                if want_err:
                    assert err_of(lambda: ctx.call(name, dx)) == want_err, (name, n)
                    continue
                rt = oracle.sum_type(t) if f == "add" else t
                got = ctx.call(name, dx, raw=True)[2]
                assert same_word(rt, got, oracle.fold(t, f, x)), (name, n, gen.__name__)


def test_bool_folds(ctx):
    for n in SIZES:
        x = data("bool", n, n)
        dx = ctx.upload(x, "bool")
        assert ctx.call("any", dx) == bool(np.any(x))
        assert ctx.call("all", dx) == bool(np.all(x))
        assert ctx.call("count", dx) == int(np.count_nonzero(x))
    assert ctx.call("all", ctx.upload(np.ones(5000, np.uint8), "bool")) is True


@pytest.mark.parametrize("t", ["f64", "f32", "i64", "u64", "i32", "u8"])
def test_argmin_argmax(ctx, t):
    for n in SIZES:
        for gen in (data, small):
            x = gen(t, n, n + 5)
            dx = ctx.upload(x, t)
            for is_max, name in ((False, "argmin_" + t), (True, "argmax_" + t)):
                want = err_of(lambda: oracle.argext(t, is_max, x)) or oracle.argext(t, is_max, x)
                got = err_of(lambda: ctx.call(name, dx)) or ctx.call(name, dx)
                assert got == want, (name, n, gen.__name__)


def test_tile_fed_reducers(ctx):
    # Split::Free: tiles of multiples of 16 rows give the one-shot result, including the
    # canonical float chains (lanes and tail carried) and argmin's row offsets.
    for t, name in (("f32", "reduce_add_f32"), ("f64", "reduce_mul_f64"), ("i32", "argmin_i32"),
                    ("u8", "reduce_add_u8"), ("f32", "argmax_f32")):
        x = small(t, 5000, 9) if "mul" in name else data(t, 5000, 9)
        r = ctx.reducer(name)
        for a, b in ((0, 992), (992, 2016), (2016, 5000)):
            r.update(ctx.upload(x[a:b], t))
        one = ctx.call(name, ctx.upload(x, t), raw=True)
        got = r.finish(raw=True)
        assert got[2] == one[2] or (np.isnan(got[1]) and np.isnan(one[1])), name


@pytest.mark.parametrize("t", ["f32", "i64", "u64", "i32"])
def test_fused(ctx, t):
    for n in SIZES + [1 << 18]:
        x, y = data(t, n, n + 1), data(t, n, n + 2)
        dx, dy = ctx.upload(x, t), ctx.upload(y, t)
        st = oracle.sum_type(t)
        assert same_word(st, ctx.call("dot_" + t, dx, dy, raw=True)[2], oracle.fused_sum(t, "dot", x, y)), n
        assert same_word(st, ctx.call("sumsq_" + t, dx, raw=True)[2], oracle.fused_sum(t, "sumsq", x)), n
        for c in ([0.0, 1.5, np.nan] if t == "f32" else [0, 5, -7 if t in ("i64", "i32") else 200]):
            for cmp in oracle.CMPS:
                cs = scalar(t, c)
                assert ctx.call("count_%s_%s" % (cmp, t), dx, cs) == oracle.count_cmp(t, cmp, x, c), (cmp, c, n)
                got = ctx.call("filter_%s_%s" % (cmp, t), dx, cs).numpy()
                assert same_rows(t, got, oracle.filter_cmp(t, cmp, x, c)), (cmp, c, n)
                e = 2.5 if t == "f32" else 3
                got = ctx.call("condsum_%s_%s" % (cmp, t), dx, cs, scalar(t, e), raw=True)[2]
                assert same_word(st, got, oracle.fused_sum(t, "condsum", x, cmp=cmp, c=c, e=e)), (cmp, c, n)


SCAN_FOLDS = {t: ["add", "mul", "min", "max", "and", "or", "xor"] for t in INT_TYPES}
SCAN_FOLDS.update({"f64": ["min", "max"], "f32": ["min", "max"], "bool": ["and", "or", "xor"]})


@pytest.mark.parametrize("t", ["f64", "f32", "i64", "u64", "i32", "u8", "bool"])
def test_scans(ctx, t):
    for f in SCAN_FOLDS[t]:
        for n in SIZES + [(1 << 20) + 3]:
            x = small(t, n, n) if f == "mul" else data(t, n, n)
            s = (oracle.rand_i64(n, n + 7) % 5 == 0).astype(np.uint8)
            dx, ds = ctx.upload(x, t), ctx.upload(s, "bool")
            rt = oracle.sum_type(t) if f == "add" else t
            got = ctx.call("scan_%s_%s" % (f, t), dx).numpy()
            assert same_rows(rt, got, oracle.scan(t, f, x)), (f, n)
            got = ctx.call("scan_by_%s_%s" % (f, t), dx, ds).numpy()
            assert same_rows(rt, got, oracle.scan(t, f, x, s)), (f, n)


def test_scanner_tiles_carry(ctx):
    # The carried state continues a segment into the next tile (scan.rs:248-282).
    for t, f in (("i32", "add"), ("f32", "min"), ("u8", "xor"), ("bool", "or")):
        n = 9000
        x = data(t, n, 4)
        s = (oracle.rand_i64(n, 5) % 11 == 0).astype(np.uint8)
        rt = oracle.sum_type(t) if f == "add" else t
        for by in (False, True):
            name = ("scan_by_%s_%s" if by else "scan_%s_%s") % (f, t)
            sc = ctx.scanner(name)
            parts = []
            for a, b in ((0, 37), (37, 4100), (4100, n)):
                out = ctx.new_array(rt, b - a)
                args = [ctx.upload(x[a:b], t)] + ([ctx.upload(s[a:b], "bool")] if by else [])
                sc.update(args, out)
                parts.append(out.numpy())
            assert same_rows(rt, np.concatenate(parts), oracle.scan(t, f, x, s if by else None)), name


@pytest.mark.parametrize("t", ["f64", "f32", "i64", "u64", "i32", "u8", "bool"])
def test_reduce_into(ctx, t):
    for f in SCAN_FOLDS[t]:
        if t == "i64" and f == "add":
            continue  # the specialised entry, covered in test_parity_index
        for n, nb in ((0, 0), (0, 3), (5, 4), (1000, 7), (70_001, 100), (70_001, 5000)):
            keys = (oracle.rand_i64(n, n + nb).view(np.uint64) % np.uint64(max(nb, 1))).astype(np.int64)
            vals = small(t, n, n + 11) if f == "mul" else data(t, n, n + 11)
            rt = oracle.sum_type(t) if f == "add" else t
            got = ctx.call("reduce_into_%s_%s" % (f, t), ctx.upload(keys), ctx.upload(vals, t), nb).numpy()
            assert same_rows(rt, got, oracle.reduce_into(t, f, keys, vals, nb)), (f, n, nb)
    # Errors in the reference's order: the key check, then the lengths, negative counts.
    name = "reduce_into_%s_%s" % (SCAN_FOLDS[t][0], t)
    for keys, vals, nb in (([0, 3], [1, 1], 3), ([0, -1], [1, 1], 3), ([0, 1], [1], 3), ([0], [1], -2)):
        k, v = np.array(keys, np.int64), np.array(vals).astype(oracle.NP_TYPES[t])
        want = err_of(lambda: oracle.reduce_into(t, SCAN_FOLDS[t][0], k, v, nb))
        assert err_of(lambda: ctx.call(name, ctx.upload(k), ctx.upload(v, t), nb)) == want, (keys, nb)


def test_grouping_golden_buckets(ctx):
    # tests/programs/grouping.dd:46-56: reduce_into with min on f64 and with and on bool.
    keys = ctx.upload(np.array([1, 0, 1, 3, 1]))
    got = ctx.call("reduce_into_min_f64", keys, ctx.upload(np.array([1.5, 2.5, 0.5, 9.0, 4.0])), 4).numpy()
    assert got.tolist() == [2.5, 0.5, np.inf, 9.0]
    got = ctx.call("reduce_into_and_bool", keys, ctx.upload(np.array([1, 0, 1, 1, 1], np.uint8), "bool"), 4).numpy()
    assert got.tolist() == [False, True, True, True]


@pytest.mark.parametrize("t", ["f64", "f32", "u64", "i32", "u8", "bool"])
def test_prev(ctx, t):
    for n in SIZES:
        x = data(t, n, n)
        fill = 1 if t != "f32" else 1.5
        got = ctx.call("prev_" + t, ctx.upload(x, t), scalar(t, fill)).numpy()
        want = np.concatenate([np.array([fill]).astype(oracle.NP_TYPES[t]), x[:-1]]) if n else x
        assert same_rows(t, got, want), n


def first_occurrence_ids(cols):
    """group_id_reference (src/kernels/scalar/group/tests.rs:24-35): ids by first occurrence."""
    n = len(cols[0])
    seen, out = {}, np.empty(n, np.int64)
    rows = list(zip(*[c.tolist() for c in cols]))
    for i, k in enumerate(rows):
        out[i] = seen.setdefault(k, len(seen))
    return out


@pytest.mark.parametrize("t", ["u64", "i32", "u8"])
def test_argsort_and_group_id_other_keys(ctx, t):
    for n in (0, 1, 1000, 9000, 300_001):
        x = data(t, n, n + 1) if n < 5000 else (small(t, n, n) if t == "u8" else data(t, n, n + 1))
        dx = ctx.upload(x, t)
        assert np.array_equal(ctx.call("argsort_" + t, dx).numpy(), np.argsort(x, kind="stable")), n
        if n <= 9000:
            assert np.array_equal(ctx.call("group_id_" + t, dx).numpy(), first_occurrence_ids([x])), n
    # Sign order of i32 and the full range of u64.
    x = np.array([3, -1, 2**31 - 1, -2**31, 0, -1], dtype=np.int32) if t == "i32" else np.array([5, 200, 0, 255, 5], np.uint8) if t == "u8" else np.array([2**63, 1, 2**64 - 1, 0, 2**63], np.uint64)
    assert np.array_equal(ctx.call("argsort_" + t, ctx.upload(x, t)).numpy(), np.argsort(x, kind="stable"))


def test_group_id2_every_pair(ctx):
    # grouping.dd:36: group_id([5u8, 5u8, 9u8], [-1i32, -1i32, -1i32]) = [0, 0, 1].
    assert ctx.call("group_id2_u8_i32", ctx.upload(np.array([5, 5, 9], np.uint8), "u8"),
                    ctx.upload(np.array([-1, -1, -1], np.int32), "i32")).numpy().tolist() == [0, 0, 1]
    for a in INT_TYPES:
        for b in INT_TYPES:
            n = 3000
            xa, xb = small(a, n, 1) & 3, small(b, n, 2) & 3
            got = ctx.call("group_id2_%s_%s" % (a, b), ctx.upload(xa, a), ctx.upload(xb, b)).numpy()
            assert np.array_equal(got, first_occurrence_ids([xa, xb])), (a, b)
    assert err_of(lambda: ctx.call("group_id2_u8_i32", ctx.upload(np.array([1], np.uint8), "u8"),
                                   ctx.upload(np.array([1, 2], np.int32), "i32"))) == "length mismatch: 1 vs 2"


@pytest.mark.parametrize("t", TYPES)
def test_fill_slice_same_len(ctx, t):
    v = {"f64": 2.5, "f32": -1.25, "i64": -7, "u64": 2**63 + 5, "i32": -3, "u8": 200, "bool": True}[t]
    for n in (0, 1, 5000):
        got = ctx.call("fill_" + t, n, scalar(t, v)).numpy()
        assert same_rows(t, got, np.array([v] * n, dtype=oracle.NP_TYPES[t])), n
    assert err_of(lambda: ctx.call("fill_" + t, -2, scalar(t, v))) == "negative length -2"
    x = data(t, 100, 3)
    dx = ctx.upload(x, t)
    assert same_rows(t, ctx.call("slice_" + t, dx, 10, 40).numpy(), x[10:40])
    assert len(ctx.call("slice_" + t, dx, 7, 7).numpy()) == 0
    for s, e in ((5, 101), (-1, 3), (9, 8)):
        assert err_of(lambda: ctx.call("slice_" + t, dx, s, e)) == "slice %d..%d out of range for length 100" % (s, e)
    assert same_rows(t, ctx.call("same_len_" + t, dx, 100).numpy(), x)
    assert err_of(lambda: ctx.call("same_len_" + t, dx, 99)) == "length mismatch: 100 vs 99"

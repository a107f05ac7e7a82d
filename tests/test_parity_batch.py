"""Batched statements (vkc_batch_*) equal the per-array kernels and the oracle, alone and replayed
from a captured CUDA graph."""

import numpy as np
import pytest

import oracle
from helpers import with_specials

pytestmark = pytest.mark.gpu

LENGTHS = [0, 1, 15, 16, 17, 31, 1000, 2047, 2048, 2049, 4097, 100_003]


def f64bits(a):
    return np.asarray(a, dtype=np.float64).view(np.uint64)


def test_batch_filter_sum_equals_filter_then_sum(ctx):
    xs = [with_specials(n, 40 + i) for i, n in enumerate(LENGTHS)]
    xs.append(oracle.rand_f64(300_001, 9) - 0.25)
    arrays = [ctx.upload(x) for x in xs]
    b = ctx.batch(arrays)
    for cmp, c in (("gt", 0.9), ("gt", 0.0), ("ge", -0.0), ("lt", 0.5), ("ne", 0.5), ("eq", np.inf),
                   ("gt", np.nan), ("ne", np.nan), ("le", -1e300)):
        sums = ctx.new_array("f64", len(xs))
        ctx.batch_filter_sum(b, cmp, c, sums)
        got = f64bits(sums.numpy())
        want = f64bits([oracle.reduce_add_f64(oracle.filter_cmp_f64(x, cmp, c)) for x in xs])
        same = (got == want) | (np.isnan(sums.numpy()) & np.isnan(want.view(np.float64)))
        assert same.all(), (cmp, c, np.flatnonzero(~same))
        one = np.array([ctx.call("reduce_add_f64", ctx.call("filter_%s_f64" % cmp, a, c)) for a in arrays])
        assert ((got == f64bits(one)) | (np.isnan(sums.numpy()) & np.isnan(one))).all(), (cmp, c)


def test_batch_argsort_equals_argsort(ctx):
    keys = [oracle.rand_i64(n, 60 + i) for i, n in enumerate(LENGTHS)]
    keys[3] = np.full(16, -1)
    keys[4] = np.array([2**63 - 1, 0, -2**63, -1, 2**63 - 1, -2**63, 0, -1] * 2 + [5])
    keys.append((oracle.rand_i64(300_001, 70) % 100).astype(np.int64))
    arrays = [ctx.upload(k) for k in keys]
    kb = ctx.batch(arrays)
    outs = [ctx.new_array("i64", len(k)) for k in keys]
    ob = ctx.batch(outs)
    ctx.batch_argsort(kb, ob)
    for k, o in zip(keys, outs):
        assert np.array_equal(o.numpy(), oracle.argsort_i64(k)), len(k)


def test_batch_argsort_narrow_keys_and_many_arrays(ctx):
    rng = np.random.default_rng(5)
    lens = [int(2 ** u) for u in rng.uniform(0, 12, 700)]
    keys = [(oracle.rand_i64(n, 1000 + i).view(np.uint64) % np.uint64(1 << 16)).astype(np.int64)
            for i, n in enumerate(lens)]
    kb = ctx.batch([ctx.upload(k) for k in keys])
    outs = [ctx.new_array("i64", n) for n in lens]
    ctx.batch_argsort(kb, ctx.batch(outs), key_digits=0b11)  # keys below 2^16: bytes 0 and 1 vary
    for k, o in zip(keys, outs):
        assert np.array_equal(o.numpy(), oracle.argsort_i64(k))


def test_batch_graph_replay(ctx):
    xs = [oracle.rand_f64(n, 80 + i) for i, n in enumerate(LENGTHS)]
    keys = [(oracle.rand_i64(n, 90 + i).view(np.uint64) % np.uint64(1 << 16)).astype(np.int64)
            for i, n in enumerate(LENGTHS)]
    xb = ctx.batch([ctx.upload(x) for x in xs])
    kb = ctx.batch([ctx.upload(k) for k in keys])
    outs = [ctx.new_array("i64", len(k)) for k in keys]
    ob = ctx.batch(outs)
    sums = ctx.new_array("f64", len(xs))
    ctx.batch_argsort(kb, ob, key_digits=0b11)  # the first call makes the scratch
    ctx.synchronize()
    ctx.graph_begin()
    ctx.batch_filter_sum(xb, "gt", 0.9, sums)
    ctx.batch_argsort(kb, ob, key_digits=0b11)
    g = ctx.graph_end()
    for _ in range(3):
        g.launch()
        ctx.synchronize()
        want = f64bits([oracle.reduce_add_f64(oracle.filter_cmp_f64(x, "gt", 0.9)) for x in xs])
        assert np.array_equal(f64bits(sums.numpy()), want)
        for k, o in zip(keys, outs):
            assert np.array_equal(o.numpy(), oracle.argsort_i64(k))


def test_batch_count_and_dot(ctx):
    xs = [with_specials(n, 200 + i) for i, n in enumerate(LENGTHS)]
    ys = [oracle.rand_f64(n, 300 + i) - 0.5 for i, n in enumerate(LENGTHS)]
    xb, yb = ctx.batch([ctx.upload(x) for x in xs]), ctx.batch([ctx.upload(y) for y in ys])
    counts = ctx.new_array("i64", len(xs))
    ctx.batch_count(xb, "gt", 0.99, counts)
    assert list(counts.numpy()) == [oracle.count_cmp_f64(x, "gt", 0.99) for x in xs]
    ctx.batch_count(xb, "le", 0.0, counts)
    assert list(counts.numpy()) == [oracle.count_cmp_f64(x, "le", 0.0) for x in xs]
    sums = ctx.new_array("f64", len(xs))
    ctx.batch_dot(xb, yb, sums)
    got = sums.numpy()
    want = np.array([oracle.dot_f64(x, y) for x, y in zip(xs, ys)])
    assert ((f64bits(got) == f64bits(want)) | (np.isnan(got) & np.isnan(want))).all()

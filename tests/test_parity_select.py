"""Selections on the GPU equal the oracle: filter_<cmp>_f64, compress_T and where, one-shot
and as tiles appended to one builder (select_tile with the tile's base row)."""

import numpy as np
import pytest

import oracle
from helpers import GPU_LENGTHS, LENGTHS, TILE_CUTS, uniform, with_specials

pytestmark = pytest.mark.gpu

CMPS = ["eq", "ne", "lt", "le", "gt", "ge"]


def same_rows(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.dtype == b.dtype and a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_filter_every_comparison(ctx):
    for n in LENGTHS + GPU_LENGTHS:
        x = with_specials(n, n)
        dx = ctx.upload(x)
        for c in (0.5, 0.0, -0.0, np.nan, np.inf):
            for cmp in CMPS:
                got = ctx.call("filter_%s_f64" % cmp, dx, c).numpy()
                assert same_rows(got, oracle.filter_cmp_f64(x, cmp, c)), (n, c, cmp)


@pytest.mark.parametrize("sel", [0.99, 0.5, 0.01])
def test_filter_selectivity_large(ctx, sel):
    n = (1 << 22) + 5
    dx = ctx.call("rand_f64", n, 4)
    x = oracle.rand_f64(n, 4)
    got = ctx.call("filter_gt_f64", dx, sel).numpy()
    assert same_rows(got, oracle.filter_cmp_f64(x, "gt", sel))


def test_filter_large_many_tiles(ctx):
    # Far more tiles than resident blocks, so every block takes tickets after its first ring.
    n = (1 << 26) + 3
    dx = ctx.call("rand_f64", n, 6)
    x = oracle.rand_f64(n, 6)
    got = ctx.call("filter_gt_f64", dx, 0.5).numpy()
    assert len(got) == ctx.call("count_gt_f64", dx, 0.5)
    assert same_rows(got, x[x > 0.5])
    m = x < 0.25
    assert same_rows(ctx.call("where", ctx.upload(m)).numpy(), np.flatnonzero(m).astype(np.int64))


@pytest.mark.parametrize("t", ["f64", "i64", "u64", "i32", "f32", "u8", "bool"])
def test_compress_types(ctx, t):
    for n in LENGTHS + GPU_LENGTHS:
        raw = oracle.rand_i64(n, n)
        x = {"f64": raw.view(np.float64), "i64": raw, "u64": raw.view(np.uint64),
             "i32": raw.astype(np.int32), "f32": (raw % 1000).astype(np.float32),
             "u8": (raw % 256).astype(np.uint8), "bool": (raw % 2 == 0)}[t]
        m = oracle.rand_i64(n, n + 1) % 3 == 0
        got = ctx.call("compress_" + t, ctx.upload(x, t), ctx.upload(m)).numpy()
        assert same_rows(got, oracle.compress(x, m)), (t, n)


def test_compress_length_mismatch(ctx):
    with pytest.raises(Exception, match="^length mismatch: 2 vs 1$"):
        ctx.call("compress_f64", ctx.upload(np.array([1.0, 2.0])), ctx.upload(np.array([True])))


def test_where(ctx):
    for n in LENGTHS + GPU_LENGTHS:
        m = oracle.rand_i64(n, n + 2) % 2 == 0
        assert same_rows(ctx.call("where", ctx.upload(m)).numpy(), oracle.where(m)), n
    # tests/programs/arrays.dd: where(x > 0.0)
    assert list(ctx.call("where", ctx.upload(np.array([True, False, True, False, True]))).numpy()) == [0, 2, 4]


def test_select_tiles_append_with_base(ctx):
    # tests/isa_variants.rs:440-447 (select_tiled): tiles 0..37, 37..100, 100..n.
    for n in (150, 4500, 10_000):
        x = uniform(n, n)
        m = oracle.rand_i64(n, 5) % 2 == 0
        dx, dm = ctx.upload(x), ctx.upload(m)
        for name, args_of, want, t in (
                ("filter_gt_f64", lambda s, e: [dx.slice(s, e), 0.5], oracle.filter_cmp_f64(x, "gt", 0.5), "f64"),
                ("compress_f64", lambda s, e: [dx.slice(s, e), dm.slice(s, e)], oracle.compress(x, m), "f64"),
                ("where", lambda s, e: [dm.slice(s, e)], oracle.where(m), "i64")):
            b = ctx.builder(t)
            start = 0
            for c in TILE_CUTS + [n]:
                ctx.select_tile(name, args_of(start, c), start, b)
                start = c
            assert same_rows(b.finish().numpy(), want), (name, n)


def test_misaligned_selection(ctx):
    x = uniform(10_000, 9)
    dx = ctx.upload(x)
    for off in (1, 5):
        got = ctx.call("filter_gt_f64", dx.slice(off, 9_000), 0.3).numpy()
        assert same_rows(got, oracle.filter_cmp_f64(x[off:9_000], "gt", 0.3))

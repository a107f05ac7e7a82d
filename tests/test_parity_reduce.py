"""Reductions on the GPU equal the oracle bit for bit: the canonical f64 sums (every length,
data that takes the integer transfer path and data that takes the sequential path), counts,
extremes and integer sums, one-shot and fed in tiles."""

import numpy as np
import pytest

import oracle
from helpers import (GPU_LENGTHS, LENGTHS, REDUCE_CUTS, bits, same_f64, uniform, varied,
                     with_specials)

pytestmark = pytest.mark.gpu

DATASETS = {
    "uniform": uniform,
    "varied": varied,
    "specials": with_specials,
    # Lanes start at 2^20, then rows of 1 + 2^-33 (and neighbours) fall exactly halfway
    # between two sums: round-half-even on every step, the two-parity transfer path.
    "ties": lambda n, s=0: np.where(np.arange(n) < 16, 2.0 ** 20, np.choose(
        oracle.rand_i64(n, s + 5) % 3, [1.0 + 2.0 ** -33, 1.0 + 3 * 2.0 ** -33, 1.0])),
    "small_then_big": lambda n, s=0: np.where(np.arange(n) < n // 2, 1e-300, 1e300) * uniform(n, s + 3),
    "negative": lambda n, s=0: -uniform(n, s + 4),
    # Quarters below 16: rows with few mantissa bits, so the quick no-tie test fails on most
    # segments and the exact test decides (no row is halfway: the lane sums stay far below
    # 2^51). On lanes that start at 2^53 (spacing 2) a quarter k/4 is halfway when k = 4 mod 8.
    "quarters": lambda n, s=0: (oracle.rand_i64(n, s + 8).view(np.uint64) % np.uint64(64)).astype(np.float64) / 4,
    "quarters_on_2^53": lambda n, s=0: np.where(np.arange(n) < 16, 2.0 ** 53, (
        oracle.rand_i64(n, s + 9).view(np.uint64) % np.uint64(64)).astype(np.float64) / 4),
    "zeros": lambda n, s=0: np.where(oracle.rand_i64(n, s + 6) % 3 == 0, 0.0, uniform(n, s + 6)),
}


@pytest.mark.parametrize("data", sorted(DATASETS))
def test_reduce_add_f64_every_length(ctx, data):
    for n in LENGTHS + GPU_LENGTHS:
        x = DATASETS[data](n, n)
        got = ctx.call("reduce_add_f64", ctx.upload(x), raw=True)[2]
        assert got == bits(oracle.reduce_add_f64(x)) or (
            np.isnan(oracle.reduce_add_f64(x)) and np.isnan(np.uint64(got).view(np.float64))), (data, n)


def test_reduce_add_f64_large_uniform(ctx):
    # Many binade crossings and tiles: every lane runs from 0 up through 2^16.
    for n in (1 << 20, (1 << 22) + 13, 3_000_017):
        x = uniform(n, 11)
        assert ctx.call("reduce_add_f64", ctx.upload(x), raw=True)[2] == bits(oracle.reduce_add_f64(x)), n


def test_signed_inputs_large(ctx):
    # Signed rows take signed transfer functions (and negative lane states their mirror image):
    # all negative, mostly positive, mixed, magnitudes over 80 binades, and dot products of
    # signed vectors; then a tiled reducer whose lanes turn negative before positive rows.
    n = (1 << 22) + 13
    u = uniform(n, 21)
    cases = {"negative": -u, "mostly_positive": u - 0.25, "mixed": u - 0.5, "varied": varied(n, 22)}
    for name, x in cases.items():
        got = ctx.call("reduce_add_f64", ctx.upload(x), raw=True)[2]
        assert got == bits(oracle.reduce_add_f64(x)), name
    y = uniform(n, 23) - 0.75
    dx, dy = ctx.upload(u - 0.25), ctx.upload(y)
    assert ctx.call("dot_f64", dx, dy, raw=True)[2] == bits(oracle.dot_f64(u - 0.25, y))
    first = -uniform(1 << 20, 24) * 8.0
    second = uniform(1 << 21, 25)
    r = ctx.reducer("reduce_add_f64")
    r.update(ctx.upload(first))
    r.update(ctx.upload(second))
    assert r.finish(raw=True)[2] == bits(oracle.reduce_add_f64(np.concatenate([first, second])))


def test_sums_that_wander_at_2p26(ctx):
    # Inputs whose lane sums keep leaving their binade: mean-centred rows (the sum wanders
    # around zero), magnitudes as large as the sum, all negative. The walk stops after a budget
    # of tiles and the lane chain finishes each lane; the bits are the reference order's.
    n = 1 << 26
    u = uniform(n, 41)
    for name, x in (("centred", u - 0.5), ("wide", varied(n, 42)), ("negative", -u)):
        dx = ctx.upload(x)
        assert ctx.call("reduce_add_f64", dx, raw=True)[2] == bits(oracle.reduce_add_f64(x)), name
        del dx
    y = uniform(n, 43) - 0.5
    x = u - 0.5
    assert ctx.call("dot_f64", ctx.upload(x), ctx.upload(y), raw=True)[2] == bits(oracle.dot_f64(x, y))
    assert ctx.call("sumsq_f64", ctx.upload(x), raw=True)[2] == bits(oracle.sumsq_f64(x))
    assert ctx.call("condsum_gt_f64", ctx.upload(x), -0.25, 0.125, raw=True)[2] == bits(
        oracle.condsum_cmp_f64(x, "gt", -0.25, 0.125))
    # Tile-fed: the chain's lane states carry into the next update.
    r = ctx.reducer("reduce_add_f64")
    r.update(ctx.upload(x[: 1 << 25]))
    r.update(ctx.upload(x[1 << 25:]))
    assert r.finish(raw=True)[2] == bits(oracle.reduce_add_f64(x))


def test_reduce_add_f64_device_generated_large(ctx):
    n = 1 << 24
    got = ctx.call("reduce_add_f64", ctx.call("rand_f64", n, 7), raw=True)[2]
    assert got == bits(oracle.reduce_add_f64(oracle.rand_f64(n, 7)))


def test_misaligned_views(ctx):
    x = uniform(20_000, 3)
    dx = ctx.upload(x)
    for off in (1, 3, 7):
        for n in (17, 1000, 8193, 19_000):
            v = dx.slice(off, off + n)
            assert ctx.call("reduce_add_f64", v, raw=True)[2] == bits(oracle.reduce_add_f64(x[off:off + n]))
            y = x[::-1].copy()
            dy = ctx.upload(y).slice(0, n)
            assert ctx.call("dot_f64", v, dy, raw=True)[2] == bits(oracle.dot_f64(x[off:off + n], y[:n]))


@pytest.mark.parametrize("data", ["uniform", "varied"])
def test_tiled_reducer_matches_one_shot(ctx, data):
    # Split::Free (src/kernels.rs:158-170): any split into 16-row multiples gives the same bits.
    for n in (1000, 50_000, 200_000):
        x = DATASETS[data](n, 1)
        dx = ctx.upload(x)
        cuts = [c for c in REDUCE_CUTS + [8192 * 2 + 48, 65_536 + 16, 120_000] if c < n]
        r = ctx.reducer("reduce_add_f64")
        start = 0
        for c in cuts + [n]:
            r.update(dx.slice(start, c))
            start = c
        assert r.finish(raw=True)[2] == bits(oracle.reduce_add_f64(x)), (data, n)


def test_partial_block_then_update_is_an_error(ctx):
    r = ctx.reducer("reduce_add_f64")
    r.update(ctx.upload(np.ones(17)))
    with pytest.raises(Exception, match="canonical update after a partial block"):
        r.update(ctx.upload(np.ones(16)))


@pytest.mark.parametrize("data", sorted(DATASETS))
def test_dot_sumsq_condsum(ctx, data):
    for n in [0, 1, 17, 300, 4500, 8193, 100_003]:
        x = DATASETS[data](n, n + 1)
        y = DATASETS["uniform"](n, n + 2)
        dx, dy = ctx.upload(x), ctx.upload(y)
        assert same_f64(np.uint64(ctx.call("dot_f64", dx, dy, raw=True)[2]).view(np.float64),
                        oracle.dot_f64(x, y)), (data, n)
        assert same_f64(np.uint64(ctx.call("sumsq_f64", dx, raw=True)[2]).view(np.float64),
                        oracle.sumsq_f64(x)), (data, n)
        for cmp in ("gt", "le", "ne"):
            got = np.uint64(ctx.call("condsum_%s_f64" % cmp, dx, 0.25, -1.5, raw=True)[2]).view(np.float64)
            assert same_f64(got, oracle.condsum_cmp_f64(x, cmp, 0.25, -1.5)), (data, n, cmp)


def test_fused_equals_unfused_on_device(ctx):
    # tests/fused_oracle.rs: dot == reduce_add(mul), condsum == reduce_add(select(cmp)).
    for n in (17, 1000, 8192 * 5 + 3, 1 << 20):
        x, y = varied(n, 2), uniform(n, 3)
        dx, dy = ctx.upload(x), ctx.upload(y)
        fused = ctx.call("dot_f64", dx, dy, raw=True)[2]
        unfused = ctx.call("reduce_add_f64", ctx.call("mul_f64", dx, dy), raw=True)[2]
        assert fused == unfused == bits(oracle.dot_f64(x, y))
        m = ctx.call("gt_f64", dx, 0.5)
        sel = ctx.call("select_f64", m, dx, -1.0)
        assert ctx.call("condsum_gt_f64", dx, 0.5, -1.0, raw=True)[2] == \
            ctx.call("reduce_add_f64", sel, raw=True)[2]


def test_readme_program(ctx):
    # README.md:40-69, config 1: bit-exact against the scalar entries.
    x = ctx.call("rand_f64", 1_000_000, 1)
    y = ctx.call("rand_f64", 1_000_000, 2)
    assert repr(ctx.call("dot_f64", x, y)) == "249724.39002046228"
    assert ctx.call("count_gt_f64", x, 0.5) == 499521
    assert ctx.call("length_f64", ctx.call("filter_gt_f64", x, 0.99)) == 9851


CMPS = ["eq", "ne", "lt", "le", "gt", "ge"]


def test_count_every_comparison(ctx):
    for n in LENGTHS + [8193, 100_003]:
        x = with_specials(n, n)
        dx = ctx.upload(x)
        for c in [0.5, 0.0, -0.0, np.inf, -np.inf, np.nan, 2.0]:
            for cmp in CMPS:
                assert ctx.call("count_%s_f64" % cmp, dx, c) == oracle.count_cmp_f64(x, cmp, c), (n, c, cmp)


def test_count_bool(ctx):
    for n in LENGTHS + [4097, 100_003]:
        m = (oracle.rand_i64(n, n) % 3 == 0)
        assert ctx.call("count", ctx.upload(m)) == int(m.sum())
        if n > 8:
            assert ctx.call("count", ctx.upload(m).slice(3, n)) == int(m[3:].sum())


@pytest.mark.parametrize("name", ["reduce_min_f64", "reduce_max_f64", "argmin_f64", "argmax_f64"])
def test_extremes_f64(ctx, name):
    fn = getattr(oracle, name)
    for n in LENGTHS[1:] + GPU_LENGTHS:
        for x in (with_specials(n, n), uniform(n, n), np.where(uniform(n, n) < 0.5, 0.0, -0.0)):
            got = ctx.call(name, ctx.upload(x))
            want = fn(x)
            if name.startswith("arg"):
                assert got == want, (name, n)
            else:
                assert same_f64(got, want), (name, n)
    with pytest.raises(Exception, match="^%s of an empty array$" % name.replace("_f64", "")):
        ctx.call(name, ctx.upload(np.array([], dtype=np.float64)))


def test_extremes_tiled_and_vectors(ctx):
    nan = float("nan")
    assert ctx.call("argmin_f64", ctx.upload(np.array([3.0, nan, nan]))) == 1
    assert ctx.call("argmax_f64", ctx.upload(np.array([-0.0, 0.0]))) == 1
    assert bits(ctx.call("reduce_min_f64", ctx.upload(np.array([0.0, -0.0])))) == bits(-0.0)
    x = with_specials(50_000, 5)
    dx = ctx.upload(x)
    for name in ("argmin_f64", "argmax_f64", "reduce_min_f64"):
        r = ctx.reducer(name)
        start = 0
        for c in [64, 384, 992, 30_000, 50_000]:
            r.update(dx.slice(start, c))
            start = c
        got, want = r.finish(), getattr(oracle, name)(x)
        assert same_f64(got, want) if name.startswith("reduce") else got == want


@pytest.mark.parametrize("name", ["reduce_min_i64", "reduce_max_i64", "argmin_i64", "argmax_i64",
                                  "reduce_add_i64"])
def test_i64_reductions(ctx, name):
    fn = getattr(oracle, name)
    for n in LENGTHS[1:] + GPU_LENGTHS:
        x = oracle.rand_i64(n, n) % 1000 if n % 2 else oracle.rand_i64(n, n)
        assert ctx.call(name, ctx.upload(x)) == fn(x), (name, n)

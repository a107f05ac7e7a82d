"""Elementwise kernels on the GPU equal the oracle (unfused plans), with array and scalar
operands, and rand_* equal the reference generator."""

import numpy as np
import pytest

import oracle
from helpers import GPU_LENGTHS, LENGTHS, bits, with_specials

pytestmark = pytest.mark.gpu


def test_rand(ctx):
    for n in LENGTHS + [8193, 1 << 20]:
        for seed in (0, 1, 2, -5, 2**62):
            assert np.array_equal(ctx.call("rand_f64", n, seed).numpy().view(np.uint64),
                                  oracle.rand_f64(n, seed).view(np.uint64)), (n, seed)
            assert np.array_equal(ctx.call("rand_i64", n, seed).numpy(), oracle.rand_i64(n, seed))
    assert list(ctx.call("rand_i64", 2, 0).numpy()) == [-2152535657050944081, -7995527694508729151]
    with pytest.raises(Exception, match="^negative length -1$"):
        ctx.call("rand_f64", -1, 0)


def test_mul_cmp_select(ctx):
    for n in LENGTHS + GPU_LENGTHS:
        x, y = with_specials(n, n), with_specials(n, n + 1)
        dx, dy = ctx.upload(x), ctx.upload(y)
        got, want = ctx.call("mul_f64", dx, dy).numpy(), oracle.mul_f64(x, y)
        # Equal bits, except that a NaN only has to be NaN (tests/isa_variants.rs:300-309).
        nan = np.isnan(want)
        assert np.array_equal(np.isnan(got), nan)
        assert np.array_equal(got[~nan].view(np.uint64), want[~nan].view(np.uint64)), n
        for cmp in ("eq", "ne", "lt", "le", "gt", "ge"):
            got = ctx.call("%s_f64" % cmp, dx, dy).numpy()
            assert np.array_equal(got.astype(np.uint8), oracle.cmp_f64(x, y, cmp)), (n, cmp)
            gs = ctx.call("%s_f64" % cmp, dx, 0.0).numpy()
            assert np.array_equal(gs.astype(np.uint8), oracle.cmp_f64(x, np.zeros(n), cmp)), (n, cmp)
        m = oracle.cmp_f64(x, y, "gt")
        got = ctx.call("select_f64", ctx.upload(m.astype(bool)), dx, -1.0).numpy()
        # select moves bits, NaN payloads included.
        assert np.array_equal(got.view(np.uint64), oracle.select_f64(m, x, np.full(n, -1.0)).view(np.uint64))


def test_integer_and_bool_ops(ctx):
    a = oracle.rand_i64(5000, 1)
    b = oracle.rand_i64(5000, 2)
    da, db = ctx.upload(a), ctx.upload(b)
    with np.errstate(over="ignore"):
        assert np.array_equal(ctx.call("add_i64", da, db).numpy(), a + b)
        assert np.array_equal(ctx.call("sub_i64", da, db).numpy(), a - b)
        assert np.array_equal(ctx.call("mul_i64", da, db).numpy(), a * b)
    assert np.array_equal(ctx.call("min_i64", da, 7).numpy(), np.minimum(a, 7))
    assert np.array_equal(ctx.call("ne_i64", da, db).numpy(), a != b)
    p, q = a % 2 == 0, b % 3 == 0
    assert np.array_equal(ctx.call("or_bool", ctx.upload(p), ctx.upload(q)).numpy(), p | q)
    assert np.array_equal(ctx.call("and_bool", ctx.upload(p), True).numpy(), p)
    assert np.array_equal(ctx.call("not_bool", ctx.upload(p)).numpy(), ~p)
    assert np.array_equal(ctx.call("iota", 10).numpy(), np.arange(10))


def test_elementwise_tile_and_errors(ctx):
    x = np.arange(100, dtype=np.float64)
    out = ctx.new_array("f64", 40)
    ctx.elementwise_tile("mul_f64", [ctx.upload(x).slice(10, 50), 2.0], out)
    assert np.array_equal(out.numpy(), x[10:50] * 2)
    with pytest.raises(Exception, match="^length mismatch: 3 vs 2$"):
        ctx.call("mul_f64", ctx.upload(np.ones(3)), ctx.upload(np.ones(2)))
    with pytest.raises(Exception, match="^expected f64 or f64\\[\\], got i64\\[\\]$"):
        ctx.call("mul_f64", ctx.upload(np.ones(3)), ctx.upload(np.ones(3, dtype=np.int64)))
    with pytest.raises(Exception, match="^expected 2 arguments, got 1$"):
        ctx.call("mul_f64", ctx.upload(np.ones(3)))

"""reduce_into_add_f64, the float per-bucket sum the reference's tier-2 design notes describe
(docs/superpowers/specs/2026-10-31-verkehrt-tier2-design.md:171-172; the reference itself has
no float reduce_into). Parity is pinned by the notes' own property, checked on the oracle and on
the GPU: with every key equal, the bucket holds exactly the bits of reduce_add_f64 (for every
length, so the canonical tail rule is exercised). The GPU equals the oracle bit for bit (a NaN
only has to be NaN) on both of its paths (at most 16 buckets: masked canonical sums; more: the
sorted stripe chains), and the errors are reduce_into_add_i64's."""

import numpy as np
import pytest

import oracle
from helpers import LENGTHS, uniform, varied, with_specials

DATA = {"uniform": uniform, "varied": varied, "specials": with_specials}


def bits(v):
    return np.asarray(v, dtype=np.float64).view(np.uint64)


def same(got, want):
    got, want = np.asarray(got, dtype=np.float64), np.asarray(want, dtype=np.float64)
    nan = np.isnan(want)
    return got.shape == want.shape and np.array_equal(np.isnan(got), nan) and np.array_equal(bits(got[~nan]), bits(want[~nan]))


def test_oracle_equal_keys_give_the_canonical_sum():
    for n in LENGTHS + [4095, 4096, 4097, 100_003]:
        for name, f in DATA.items():
            x = f(n, n + 3)
            for nb, k in ((1, 0), (7, 5)):
                got = oracle.reduce_into_add_f64(np.full(n, k, dtype=np.int64), x, nb)
                assert same(got[k], oracle.reduce_add_f64(x)), (name, n, nb)
                assert np.array_equal(bits(np.delete(got, k)), np.zeros(nb - 1, dtype=np.uint64))


def test_oracle_buckets_are_masked_canonical_sums():
    n = 10_007
    x = varied(n, 4)
    keys = (oracle.rand_i64(n, 5).view(np.uint64) % np.uint64(9)).astype(np.int64)
    got = oracle.reduce_into_add_f64(keys, x, 11)
    for k in range(11):
        assert same(got[k], oracle.reduce_add_f64(np.where(keys == k, x, 0.0))), k


def test_oracle_errors_are_the_i64_entrys():
    x = np.array([1.0, 2.0, 3.0])
    for keys, nb in (([0, 3, 1], 3), ([0, -1, 1], 2), ([0, 1, 2], -1)):
        with pytest.raises(oracle.OracleError) as want:
            oracle.reduce_into_add_i64(keys, [1, 2, 3], nb)
        with pytest.raises(oracle.OracleError, match="^%s$" % str(want.value)):
            oracle.reduce_into_add_f64(keys, x, nb)
    with pytest.raises(oracle.OracleError, match="^length mismatch: 2 keys for 3 values$"):
        oracle.reduce_into_add_f64([0, 1], x, 2)


def keysets(n, seed):
    u = oracle.rand_i64(n, seed).view(np.uint64)
    r = oracle.rand_f64(n, seed + 1)
    return {
        "one_bucket": (np.zeros(n, dtype=np.int64), 1),
        "three": ((u % np.uint64(3)).astype(np.int64), 4),
        "five": ((u % np.uint64(5)).astype(np.int64), 5),
        "nine": ((u % np.uint64(9)).astype(np.int64), 9),
        "seventeen": ((u % np.uint64(17)).astype(np.int64), 17),
        "many": ((u % np.uint64(1000)).astype(np.int64), 1000),
        "skewed": (np.minimum((1.0 / (r + 1e-9)).astype(np.int64), 5000) - 1, 5000),
        "sparse": ((u % np.uint64(50)).astype(np.int64) * 1000, 60_000),
    }


@pytest.mark.gpu
@pytest.mark.parametrize("data", sorted(DATA))
def test_gpu_equals_oracle(ctx, data):
    for n in LENGTHS + [4096, 4111, 100_003, (1 << 20) + 5]:
        x = DATA[data](n, n + 1)
        dx = ctx.upload(x)
        for name, (keys, nb) in keysets(n, n + 2).items():
            got = ctx.call("reduce_into_add_f64", ctx.upload(keys), dx, nb).numpy()
            assert same(got, oracle.reduce_into_add_f64(keys, x, nb)), (data, n, name)


@pytest.mark.gpu
def test_gpu_equal_keys_give_reduce_add_bits(ctx):
    for n in (17, 4097, 100_003, 1 << 22):
        x = varied(n, 8)
        dx = ctx.upload(x)
        want = ctx.call("reduce_add_f64", dx, raw=True)[2]
        for nb, k in ((1, 0), (17, 4)):  # the masked path and the sorted path
            got = ctx.call("reduce_into_add_f64", ctx.upload(np.full(n, k, dtype=np.int64)), dx, nb).numpy()
            assert int(bits(got[k])) == want, (n, nb)
            assert not bits(np.delete(got, k)).any()


@pytest.mark.gpu
def test_gpu_errors(ctx):
    x = ctx.upload(np.array([1.0, 2.0, 3.0]))
    for keys, nb, msg in (([0, 3, 1], 3, "bucket key 3 out of range for 3 buckets"),
                          ([0, -1, 1], 2, "bucket key -1 out of range for 2 buckets"),
                          ([0, 1, 2], -1, "negative bucket count -1")):
        with pytest.raises(Exception, match="^%s$" % msg):
            ctx.call("reduce_into_add_f64", ctx.upload(np.array(keys)), x, nb)
    with pytest.raises(Exception, match="^length mismatch: 2 keys for 3 values$"):
        ctx.call("reduce_into_add_f64", ctx.upload(np.array([0, 1])), x, 2)
    with pytest.raises(Exception, match=r"^expected f64\[\], got i64\[\]$"):
        ctx.call("reduce_into_add_f64", ctx.upload(np.array([0, 1])), ctx.upload(np.array([1, 2])), 2)
    assert len(ctx.call("reduce_into_add_f64", ctx.upload(np.array([], dtype=np.int64)),
                        ctx.upload(np.array([], dtype=np.float64)), 0)) == 0

"""gather, histogram and reduce_into on the GPU equal the oracle, including the reference's
error messages for the first offending index or key."""

import numpy as np
import pytest

import oracle
from oracle import OracleError

pytestmark = pytest.mark.gpu


def err_of(fn):
    try:
        fn()
    except (OracleError, Exception) as e:  # noqa: B014
        return str(e)
    return None


@pytest.mark.parametrize("t", ["i64", "f64", "bool", "u8", "i32"])
def test_gather(ctx, t):
    for n in (0, 1, 5, 300, 4097, 100_003):
        raw = oracle.rand_i64(n, n)
        src = {"i64": raw, "f64": raw.view(np.float64), "bool": raw % 2 == 0,
               "u8": (raw % 256).astype(np.uint8), "i32": raw.astype(np.int32)}[t]
        idx = (oracle.rand_i64(3 * n + 1, 9).view(np.uint64) % np.uint64(max(n, 1))).astype(np.int64) if n else np.array([], dtype=np.int64)
        got = ctx.call("gather_" + t, ctx.upload(src, t), ctx.upload(idx)).numpy()
        want = oracle.gather(src, idx)
        assert np.array_equal(got.view(np.uint8), np.asarray(want).view(np.uint8)), (t, n)


def test_gather_errors(ctx):
    xs = ctx.upload(np.array([10, 20, 30]))
    for idx, first in (([0, 3], 3), ([-1, 0], -1), ([2, 5, -4, 7], 5)):
        with pytest.raises(Exception, match="^gather index %d out of range for length 3$" % first):
            ctx.call("gather_i64", xs, ctx.upload(np.array(idx)))
    with pytest.raises(Exception, match="^gather index 0 out of range for length 0$"):
        ctx.call("gather_i64", ctx.upload(np.array([], dtype=np.int64)), ctx.upload(np.array([0])))
    # The first offender in index order, far into a large index array.
    n = 1 << 20
    idx = np.zeros(n, dtype=np.int64)
    idx[700_001] = 99
    idx[900_000] = -5
    with pytest.raises(Exception, match="^gather index 99 out of range for length 3$"):
        ctx.call("gather_i64", xs, ctx.upload(idx))
    # The context stays usable.
    assert list(ctx.call("gather_i64", xs, ctx.upload(np.array([2, 0]))).numpy()) == [30, 10]


def test_gather_large_uniform(ctx):
    n = 1 << 22
    src = ctx.call("rand_i64", n, 1)
    idx_h = (oracle.rand_i64(n, 2).view(np.uint64) % np.uint64(n)).astype(np.int64)
    got = ctx.call("gather_i64", src, ctx.upload(idx_h)).numpy()
    assert np.array_equal(got, oracle.gather(oracle.rand_i64(n, 1), idx_h))


def test_gather_partitioned(ctx):
    # Sources of 2^26 rows or more (four times L2) and at least half as many index rows take
    # the partitioned path: uniform indices, indices crowded into one source region, the first
    # and last rows, a ragged last tile, and 8-byte floats whose bits (NaN payloads) must
    # survive.
    nsrc = (1 << 26) + 3
    src_h = oracle.rand_i64(nsrc, 1)
    src = ctx.upload(src_h)
    n = (1 << 25) + 5
    r = oracle.rand_i64(n, 2).view(np.uint64)
    cases = {
        "uniform": (r % np.uint64(nsrc)).astype(np.int64),
        "one_region": (r % np.uint64(1000)).astype(np.int64) + (nsrc - 5000),
        "ends": np.where(r % np.uint64(2) == 0, 0, nsrc - 1).astype(np.int64),
    }
    for name, idx in cases.items():
        got = ctx.call("gather_i64", src, ctx.upload(idx)).numpy()
        assert np.array_equal(got, oracle.gather(src_h, idx)), name
    idx = cases["uniform"]
    got = ctx.call("gather_f64", ctx.upload(src_h.view(np.float64), "f64"), ctx.upload(idx)).numpy()
    assert np.array_equal(got.view(np.int64), src_h[idx])
    # The first offender in index order, and the context stays usable.
    bad = idx.copy()
    bad[30_000_001] = nsrc
    bad[31_500_000] = -1
    with pytest.raises(Exception, match="^gather index %d out of range for length %d$" % (nsrc, nsrc)):
        ctx.call("gather_i64", src, ctx.upload(bad))
    assert np.array_equal(ctx.call("gather_i64", src, ctx.upload(idx[:5])).numpy(), src_h[idx[:5]])


def test_histogram_and_reduce_into(ctx):
    for n in (0, 5, 1000, 100_003):
        for nb in (1, 5, 1024, 4096, 4097, 100_000):
            keys = (oracle.rand_i64(n, n).view(np.uint64) % np.uint64(nb)).astype(np.int64)
            v = oracle.rand_i64(n, n + 1)
            assert np.array_equal(ctx.call("histogram", ctx.upload(keys), nb).numpy(),
                                  oracle.histogram(keys, nb)), (n, nb)
            assert np.array_equal(ctx.call("reduce_into_add_i64", ctx.upload(keys), ctx.upload(v), nb).numpy(),
                                  oracle.reduce_into_add_i64(keys, v, nb)), (n, nb)


def test_histogram_and_reduce_into_skewed(ctx):
    # Most rows on a few buckets, in runs and scattered: the warp-combined atomics.
    n = 300_001
    r = oracle.rand_i64(n, 77).view(np.uint64)
    for nb in (7, 4096, 4097, 1 << 20):
        hot = (r % np.uint64(3)).astype(np.int64)
        cold = (r % np.uint64(nb)).astype(np.int64)
        for keys in (np.where(r % np.uint64(100) == 0, cold, hot), np.sort(cold), np.zeros(n, np.int64)):
            v = oracle.rand_i64(n, 78)
            assert np.array_equal(ctx.call("histogram", ctx.upload(keys), nb).numpy(), oracle.histogram(keys, nb)), nb
            assert np.array_equal(ctx.call("reduce_into_add_i64", ctx.upload(keys), ctx.upload(v), nb).numpy(),
                                  oracle.reduce_into_add_i64(keys, v, nb)), nb


def test_buckets_over_sorted_runs(ctx):
    # Runs of 1 to 5000 equal keys (run numbers of a sorted group-by): runs are summed in the
    # warp and carried across 32-row groups; keys large and small, runs split at any row.
    lens = 1 + (oracle.rand_i64(4000, 91).view(np.uint64) % np.uint64(5000)).astype(np.int64)
    for nb, stride in ((1 << 20, 97), (4096, 1), (5000, 1)):
        keys = np.repeat((np.arange(len(lens)) * stride) % nb, lens).astype(np.int64)
        v = oracle.rand_i64(len(keys), 92)
        assert np.array_equal(ctx.call("histogram", ctx.upload(keys), nb).numpy(), oracle.histogram(keys, nb))
        assert np.array_equal(ctx.call("reduce_into_add_i64", ctx.upload(keys), ctx.upload(v), nb).numpy(),
                              oracle.reduce_into_add_i64(keys, v, nb))
    # A bad key inside a long run and another later: the first one is reported.
    keys = np.repeat(np.arange(100, dtype=np.int64), 1000)
    keys[51_234] = -5
    keys[70_000] = 10 ** 9
    want = err_of(lambda: oracle.histogram(keys, 100))
    assert want == "bucket key -5 out of range for 100 buckets"
    assert err_of(lambda: ctx.call("histogram", ctx.upload(keys), 100)) == want


def test_bucket_errors(ctx):
    # src/kernels/tests.rs:1576-1620
    for keys, nb in (([0, 3], 3), ([0, -1], 3), ([0, 0], 0), ([], -1), ([0], 1 << 62), ([0], 1 << 50),
                     ([5, 0], 1 << 50)):
        k = np.array(keys, dtype=np.int64)
        want_h = err_of(lambda: oracle.histogram(k, nb))
        assert err_of(lambda: ctx.call("histogram", ctx.upload(k), nb)) == want_h, (keys, nb)
        vals = np.ones(len(k), dtype=np.int64)
        want_r = err_of(lambda: oracle.reduce_into_add_i64(k, vals, nb))
        assert err_of(lambda: ctx.call("reduce_into_add_i64", ctx.upload(k), ctx.upload(vals), nb)) == want_r
    # The key check comes before the length check (index.rs:203-210).
    assert err_of(lambda: ctx.call("reduce_into_add_i64", ctx.upload(np.array([0, 7])),
                                   ctx.upload(np.array([1])), 3)) == "bucket key 7 out of range for 3 buckets"
    assert err_of(lambda: ctx.call("reduce_into_add_i64", ctx.upload(np.array([0, 1])),
                                   ctx.upload(np.array([1])), 3)) == "length mismatch: 2 keys for 1 values"

"""Scans on the GPU equal the oracle: scan_add_i64, scan_by_add_i64 and prev_i64, one-shot and
fed in tiles (the state carries across updates)."""

import numpy as np
import pytest

import oracle
from helpers import GPU_LENGTHS, LENGTHS, TILE_CUTS

pytestmark = pytest.mark.gpu


def vals(n, seed):
    # The sweep workload's scan values: uniform in [-2^20, 2^20).
    return (oracle.rand_i64(n, seed).view(np.uint64) % np.uint64(1 << 21)).astype(np.int64) - (1 << 20)


def test_scan_add(ctx):
    for n in LENGTHS + GPU_LENGTHS + [1 << 20]:
        x = vals(n, n)
        assert np.array_equal(ctx.call("scan_add_i64", ctx.upload(x)).numpy(), oracle.scan_add_i64(x)), n
    w = np.array([2**63 - 1, 1])
    assert list(ctx.call("scan_add_i64", ctx.upload(w)).numpy()) == [2**63 - 1, -2**63]


def test_scan_by_add(ctx):
    for n in LENGTHS + GPU_LENGTHS + [1 << 20]:
        for p in (2, 7, 5000):
            x = vals(n, n)
            s = oracle.rand_i64(n, n + 1) % p == 0
            got = ctx.call("scan_by_add_i64", ctx.upload(x), ctx.upload(s)).numpy()
            assert np.array_equal(got, oracle.scan_by_add_i64(x, s)), (n, p)
    # tests/programs/grouping.dd
    got = ctx.call("scan_by_add_i64", ctx.upload(np.arange(1, 6)),
                   ctx.upload(np.array([False, False, True, False, True]))).numpy()
    assert list(got) == [1, 3, 3, 7, 5]


@pytest.mark.parametrize("name", ["scan_add_i64", "scan_by_add_i64", "prev_i64"])
def test_scanner_tiles(ctx, name):
    # tests/isa_variants.rs (scan_tiled): any split into tiles gives the one-shot rows.
    for n in (150, 5000, 20_000):
        x = vals(n, n + 3)
        s = oracle.rand_i64(n, n + 4) % 9 == 0
        dx, ds = ctx.upload(x), ctx.upload(s)
        want = {"scan_add_i64": oracle.scan_add_i64(x), "scan_by_add_i64": oracle.scan_by_add_i64(x, s),
                "prev_i64": oracle.prev_i64(x, -7)}[name]
        sc = ctx.scanner(name)
        parts, start = [], 0
        for c in TILE_CUTS + [4099, n]:
            if c <= start or c > n:
                continue
            out = ctx.new_array("i64", c - start)
            args = {"scan_add_i64": [dx.slice(start, c)], "scan_by_add_i64": [dx.slice(start, c), ds.slice(start, c)],
                    "prev_i64": [dx.slice(start, c), -7]}[name]
            sc.update(args, out)
            parts.append(out.numpy())
            start = c
        assert np.array_equal(np.concatenate(parts), want), (name, n)


def test_scan_last_equals_sum_large(ctx):
    # Size-independent property at a large size: the last prefix is the wrapping sum.
    n = 1 << 26
    x = ctx.call("rand_i64", n, 3)
    s = ctx.call("scan_add_i64", x)
    last = s.slice(n - 1, n).numpy()[0]
    assert last == ctx.call("reduce_add_i64", x)

"""Copies that overlap kernels: uploads of at least 1 MiB run on the context's upload stream
and the first call that reads the array waits for them; downloads started with
download_start run on the download stream after the work queued so far. Results equal the
oracle whatever the copies overlap, an array in flight may be released, and a call that writes
an array waits for a download of it."""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def pinned(n, dtype):
    torch = pytest.importorskip("torch")
    t = torch.empty(n, dtype={np.float64: torch.float64, np.int64: torch.int64}[dtype], pin_memory=True)
    return t, t.data_ptr()


def test_uploads_then_kernels_in_any_order(ctx):
    n = (1 << 20) + 7  # 8 MiB per array
    hs = [oracle.rand_f64(n, s) for s in range(5)]
    bufs = []
    for h in hs:
        t, p = pinned(n, np.float64)
        t.numpy()[:] = h
        bufs.append((t, p))
    arrs = [ctx.upload_ptr(p, n, "f64") for _, p in bufs]
    # The last upload is read first: each call waits only for its own arrays.
    for i in reversed(range(5)):
        got = ctx.call("reduce_add_f64", arrs[i], raw=True)[2]
        assert got == int(np.float64(oracle.reduce_add_f64(hs[i])).view(np.uint64)), i
    assert ctx.call("dot_f64", arrs[0], arrs[4]) == oracle.dot_f64(hs[0], hs[4])


def test_download_start_overlaps_and_keeps_the_array(ctx):
    n = 1 << 21
    x = ctx.call("rand_f64", n, 3)
    outs, copies = [], []
    for c in (0.25, 0.5, 0.75):
        f = ctx.call("filter_gt_f64", x, c)
        t, p = pinned(n, np.float64)
        copies.append((ctx.download_start(f, p, n), t, len(f), c))
        del f  # the copy holds its own reference
    xs = oracle.rand_f64(n, 3)
    for cp, t, k, c in copies:
        cp.wait()
        assert np.array_equal(t.numpy()[:k], oracle.filter_cmp_f64(xs, "gt", c)), c


def test_write_waits_for_a_download_of_the_array(ctx):
    n = 1 << 21
    a = ctx.upload(oracle.rand_f64(n, 5))
    b = ctx.upload(oracle.rand_f64(n, 6))
    out = ctx.new_array("f64", n)
    ctx.elementwise_tile("mul_f64", [a, b], out)
    t, p = pinned(n, np.float64)
    cp = ctx.download_start(out, p, n)
    ctx.elementwise_tile("add_f64", [a, b], out)  # overwrites `out` after the copy has read it
    cp.wait()
    assert np.array_equal(t.numpy(), oracle.mul_f64(oracle.rand_f64(n, 5), oracle.rand_f64(n, 6)))
    assert np.array_equal(out.numpy(), oracle.rand_f64(n, 5) + oracle.rand_f64(n, 6))


def test_released_uploads_and_cache_reuse(ctx):
    n = 1 << 20
    for s in range(4):
        t, p = pinned(n, np.int64)
        t.numpy()[:] = oracle.rand_i64(n, s)
        a = ctx.upload_ptr(p, n, "i64")
        del a  # released with its copy in flight: the block returns to the cache after it
        ctx.synchronize()
    t, p = pinned(n, np.int64)
    t.numpy()[:] = oracle.rand_i64(n, 9)
    a = ctx.upload_ptr(p, n, "i64")
    assert ctx.call("reduce_add_i64", a) == oracle.reduce_add_i64(oracle.rand_i64(n, 9))


def test_copies_and_graph_capture(ctx):
    n = 1 << 20
    h = oracle.rand_f64(n, 7)
    t, p = pinned(n, np.float64)
    t.numpy()[:] = h
    y = ctx.upload_ptr(p, n, "f64")  # its copy may still be in flight when the capture starts
    out = ctx.new_array("f64", n)
    ctx.graph_begin()
    ctx.elementwise_tile("mul_f64", [y, y], out)  # the host waits for the copy: no cross-capture wait
    with pytest.raises(Exception, match="during a stream capture"):
        ctx.download_start(y, p, n)
    g = ctx.graph_end()
    g.launch()
    ctx.synchronize()
    assert np.array_equal(out.numpy(), oracle.mul_f64(h, h))

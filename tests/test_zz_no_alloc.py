"""The allocation-free scan entry, vkc_scan_add_i64_noalloc, against the allocating entry.

Some callers cannot allocate device memory while they run a kernel: a host that embeds this
library and gives it only buffers from its own arena, or a serving loop that must not wait on
the allocator per request. This entry serves them with scratch that lives in the library's
device image. This file is collected last, so a run that stops at its first failure has run
every other test before it.
"""

import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def values(n, seed):
    return (oracle.rand_i64(n, seed).view(np.uint64) % np.uint64(1 << 21)).astype(np.int64) - (1 << 20)


def noalloc(lib, ctx, x, out, n):
    err = ctypes.create_string_buffer(256)
    st = lib.vkc_scan_add_i64_noalloc(0, x.device_ptr if x is not None else None,
                                      out.device_ptr if out is not None else None, n,
                                      ctx.stream, err, len(err))
    return st, err.value.decode()


def test_noalloc_scan_matches_the_allocating_entry(ctx):
    import verkehrt_gb300 as vk

    lib = vk.load()
    # Two calls in a row share the scratch array; the second is shorter, so it starts from
    # what the first left behind.
    for n, seed in ((1_000_003, 1), (70_001, 2), (4096, 3)):
        x = ctx.upload(values(n, seed))
        want = ctx.call("scan_add_i64", x).numpy()
        out = ctx.new_array("i64", n)
        st, msg = noalloc(lib, ctx, x, out, n)
        assert st == 0, msg
        assert np.array_equal(out.numpy(), want), n
    # A view that starts off the 16-byte grid.
    x = ctx.upload(values(10_000, 4))
    v = x.slice(1, 10_000)
    out = ctx.new_array("i64", 9_999)
    st, msg = noalloc(lib, ctx, v, out, 9_999)
    assert st == 0, msg
    assert np.array_equal(out.numpy(), ctx.call("scan_add_i64", v).numpy())


def test_noalloc_scan_rejects_sizes_beyond_its_maximum(ctx):
    import verkehrt_gb300 as vk

    lib = vk.load()
    st, msg = noalloc(lib, ctx, None, None, (1 << 28) + 1)
    assert st == 5  # VKC_USAGE, nothing launched
    assert "maximum of 268435456 rows" in msg
    st, msg = noalloc(lib, ctx, None, None, 0)
    assert st == 0
    # NULL and host pointers are refused before any launch.
    st, msg = noalloc(lib, ctx, None, None, 16)
    assert st == 5 and "NULL" in msg
    host = np.zeros(16, dtype=np.int64)
    err = ctypes.create_string_buffer(256)
    st = lib.vkc_scan_add_i64_noalloc(0, host.ctypes.data, host.ctypes.data, 16, ctx.stream, err, len(err))
    assert st == 5 and b"device or managed memory" in err.value

"""Parity at the benchmark configurations' own sizes: the primitive sweep at n = 2^28 rows and
the argsort/group-by pipeline at n = 2^27 rows for uniform 32-bit keys and Zipf s=1.1 keys. Every
output of the bench's calls (the same kernels, seeds and call order as bench.py) is compared with
the oracle's restatement (tests/golden/full_size.py): bit for bit, floats by their bits.

The group-by pipeline is the reference's sorted idiom (tests/programs/grouping.dd:12-31) composed
on the device, plus the hashed group-by; besides matching the oracle call by call, its two forms
must agree with each other (the same per-key sums and counts).
"""

import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))

import full_size  # noqa: E402
from full_size import bench  # noqa: E402

pytestmark = pytest.mark.gpu

SWEEP_N = 1 << 28
SORT_N = 1 << 27


def same(got, want):
    """Bit equality of a device result (Array or Python scalar) with the oracle's value."""
    if hasattr(got, "handle"):
        g = got.numpy()
        w = np.asarray(want)
        if g.dtype == np.bool_ or w.dtype == np.bool_:
            return g.shape == w.shape and np.array_equal(g.astype(np.uint8), w.astype(np.uint8))
        return g.dtype == w.dtype and g.shape == w.shape and np.array_equal(
            g.view(np.uint64 if g.itemsize == 8 else g.dtype), w.view(np.uint64 if w.itemsize == 8 else w.dtype))
    if isinstance(want, float):
        return np.float64(got).view(np.uint64) == np.float64(want).view(np.uint64)
    return int(got) == int(want)


def device_stream(ctx):
    import torch

    return torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", ctx.device))


def test_primitive_sweep_at_2p28(ctx):
    n = SWEEP_N
    dev = bench.make_inputs(ctx, n)
    got = {}
    env = dict(dev)
    for label, kernel, names, extra, _ in bench.sweep_plan(n):
        out = ctx.call(kernel, *[env[a] for a in names], *extra)
        if kernel == "mul_f64":
            env["xy"] = out
        got[label] = out
    del env, dev
    host = full_size.sweep_inputs(n)
    checked = []
    for label, want in full_size.sweep_outputs(n, host):
        assert same(got.pop(label), want), label
        checked.append(label)
    assert len(checked) == len(bench.sweep_plan(n))


def _sortgroup(ctx, dist):
    n = SORT_N
    stream = device_stream(ctx)
    keys, vf, vi = full_size.sortgroup_inputs(n, dist)
    if dist == "uniform32":
        dk = ctx.call("and_i64", ctx.call("rand_i64", n, 23), (1 << 32) - 1)
    else:
        dk = ctx.upload(keys)
    dvf = ctx.call("rand_f64", n, 21)
    dvi = ctx.call("sub_i64", ctx.call("and_i64", ctx.call("rand_i64", n, 22), (1 << 21) - 1), 1 << 20)
    _, res = bench.sortgroup_step(ctx, dk, dvf, dvi, stream)
    del dk, dvf, dvi
    checked = 0
    for label, want in full_size.sortgroup_outputs(n, dist, (keys, vf, vi)):
        assert same(res[label], want), (dist, label)
        checked += 1
    assert checked == 18
    # The sorted idiom's two forms agree, and with the hashed group-by: per-key sums and counts.
    sums = res["compress_i64(sums)"].numpy()
    assert np.array_equal(sums, res["reduce_into_add_i64(runs)"].numpy())
    uk = res["compress_i64(keys)"].numpy()
    g = res["group_id_i64"].numpy()
    assert len(uk) == res["reduce_max_i64"] + 1 == res["count"]
    # Ids number groups by first occurrence: a row is its group's first when its id exceeds
    # every earlier id.
    cm = np.maximum.accumulate(g)
    first = np.flatnonzero(np.concatenate([[True], g[1:] > cm[:-1]]))
    assert np.array_equal(g[first], np.arange(len(uk)))
    order = np.argsort(keys[first], kind="stable")
    assert np.array_equal(keys[first][order], uk)
    assert np.array_equal(res["reduce_into_add_i64"].numpy()[order], sums)
    counts = np.diff(np.append(np.flatnonzero(res["run_starts"].numpy()), len(g)))
    assert np.array_equal(res["histogram"].numpy()[order], counts)


def test_sort_groupby_uniform32_at_2p27(ctx):
    _sortgroup(ctx, "uniform32")


def test_sort_groupby_zipf_at_2p27(ctx):
    _sortgroup(ctx, "zipf1.1")

"""The committed golden fixtures (tests/golden): the reference's known answers, reproduced by the
oracle on the CPU and by the CUDA path on the GPU, and the oracle's own outputs on seeded
inputs, which pin the oracle (CPU) and are the expected values of the GPU path."""

import json
import os
import sys

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)


def known():
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        return json.load(f)


def vectors():
    return dict(np.load(os.path.join(GOLDEN, "oracle_vectors.npz")))


def f64bits(x):
    return np.float64(x).view(np.uint64)


def test_oracle_reproduces_known_answers():
    k = known()
    assert oracle.splitmix64(0) == int(k["splitmix64(0)"]["value"], 16)
    assert list(oracle.rand_i64(2, 0)) == k["rand_i64(2, 0)"]["value"]
    readme = k["README example"]["value"]
    x, y = oracle.rand_f64(1_000_000, 1), oracle.rand_f64(1_000_000, 2)
    assert f64bits(oracle.dot_f64(x, y)) == f64bits(readme["dot"])
    assert oracle.count_cmp_f64(x, "gt", 0.5) == readme["count_gt_0.5"]
    assert len(oracle.filter_cmp_f64(x, "gt", 0.99)) == readme["filter_gt_0.99_length"]
    g = k["grouping.dd group_id"]
    assert list(oracle.group_id_i64(g["input"])) == g["value"]
    a = k["argsort i64 extremes"]
    assert list(oracle.argsort_i64(a["input"])) == a["value"]


def test_oracle_reproduces_its_vectors():
    import make_golden

    want, got = vectors(), make_golden.vectors()
    assert sorted(want) == sorted(got)
    for name in want:
        a, b = np.atleast_1d(np.asarray(want[name])), np.atleast_1d(np.asarray(got[name]))
        assert a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8)), name


@pytest.mark.gpu
def test_gpu_matches_golden_vectors(ctx):
    g = vectors()
    x, y, v = ctx.upload(g["x"]), ctx.upload(g["y"]), ctx.upload(g["v"])
    assert f64bits(ctx.call("reduce_add_f64", x)) == g["reduce_add_bits"]
    assert f64bits(ctx.call("dot_f64", x, y)) == g["dot_bits"]
    assert f64bits(ctx.call("sumsq_f64", x)) == g["sumsq_bits"]
    assert ctx.call("count_gt_f64", x, 0.5) == g["count_gt_0.5"]
    assert np.array_equal(ctx.call("filter_gt_f64", x, 0.9).numpy().view(np.uint64), g["filter_gt_0.9"].view(np.uint64))
    assert f64bits(ctx.call("reduce_min_f64", x)) == g["min_bits"]
    assert f64bits(ctx.call("reduce_max_f64", x)) == g["max_bits"]
    assert ctx.call("argmin_f64", x) == g["argmin"] and ctx.call("argmax_f64", x) == g["argmax"]
    assert np.array_equal(ctx.call("scan_add_i64", v).numpy(), g["scan_add"])
    assert np.array_equal(ctx.call("scan_by_add_i64", v, ctx.upload(g["starts"])).numpy(), g["scan_by_add"])
    assert np.array_equal(ctx.call("prev_i64", v, 7).numpy(), g["prev"])
    assert np.array_equal(ctx.call("gather_i64", ctx.upload(g["src"]), ctx.upload(g["idx"])).numpy(), g["gather"])
    assert np.array_equal(ctx.call("argsort_i64", ctx.upload(g["keys"])).numpy(), g["argsort"])
    ids = ctx.call("group_id_i64", ctx.upload(g["gkeys"]))
    assert np.array_equal(ids.numpy(), g["group_id"])
    nb = len(g["histogram"])
    assert np.array_equal(ctx.call("histogram", ids, nb).numpy(), g["histogram"])
    assert np.array_equal(ctx.call("reduce_into_add_i64", ids, v, nb).numpy(), g["reduce_into"])
    m = ctx.upload(g["mask"])
    assert np.array_equal(ctx.call("compress_f64", x, m).numpy().view(np.uint64), g["compress"].view(np.uint64))
    assert np.array_equal(ctx.call("where", m).numpy(), g["where"])


@pytest.mark.gpu
def test_gpu_readme_example(ctx):
    readme = known()["README example"]["value"]
    x, y = ctx.call("rand_f64", 1_000_000, 1), ctx.call("rand_f64", 1_000_000, 2)
    assert f64bits(ctx.call("dot_f64", x, y)) == f64bits(readme["dot"])
    assert ctx.call("count_gt_f64", x, 0.5) == readme["count_gt_0.5"]
    assert len(ctx.call("filter_gt_f64", x, 0.99)) == readme["filter_gt_0.99_length"]

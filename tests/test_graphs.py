"""Reductions enqueued into device arrays (vkc_call_into) and statement sequences captured as
CUDA graphs and replayed, checked against the oracle and against vkc_call's own results.

The README program (README.md:40-69 of antiguru/verkehrt: dot, count_gt 0.5, length of
filter_gt 0.99) is the sequence captured: its results stay on the device, so one graph launch
runs all three statements.
"""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

WIDTH_VIEW = {"f64": np.uint64, "i64": np.uint64, "u64": np.uint64, "f32": np.uint32,
              "i32": np.uint32, "u8": np.uint8, "bool": np.uint8}


def bits(a, t):
    return np.ascontiguousarray(a).view(WIDTH_VIEW[t])


def zero(ctx, arr, t):
    """arr *= 0 (arr &= false for bool) on the device, in place (elementwise_tile)."""
    import verkehrt_gb300 as vk

    if t == "bool":
        ctx.elementwise_tile("and_bool", [arr, vk.Scalar("bool", False)], arr)
    else:
        ctx.elementwise_tile("mul_" + t, [arr, vk.Scalar(t, 0)], arr)


def test_readme_program_replayed_from_a_graph(ctx):
    n = 1_000_000
    x = ctx.call("rand_f64", n, 1)
    y = ctx.call("rand_f64", n, 2)
    hx, hy = oracle.rand_f64(n, 1), oracle.rand_f64(n, 2)
    dots = ctx.new_array("f64", 1)
    counts = ctx.new_array("i64", 2)

    def program():
        ctx.call_into("dot_f64", x, y, out=dots, row=0)
        ctx.call_into("count_gt_f64", x, 0.5, out=counts, row=0)
        # length(filter_gt_f64(x, 0.99)) is the count of the same comparison.
        ctx.call_into("count_gt_f64", x, 0.99, out=counts, row=1)

    program()  # sizes the scratch arena outside the capture
    ctx.synchronize()
    ctx.graph_begin()
    program()
    g = ctx.graph_end()
    want_dot = oracle.dot_f64(hx, hy)
    assert repr(float(want_dot)) == "249724.39002046228"
    for _ in range(3):
        zero(ctx, dots, "f64")
        zero(ctx, counts, "i64")
        g.launch()
        d, c = dots.numpy(), counts.numpy()
        assert bits(d, "f64")[0] == bits(np.array([want_dot]), "f64")[0]
        assert list(c) == [499521, 9851]
        assert list(c) == [oracle.count_cmp_f64(hx, "gt", 0.5), oracle.count_cmp_f64(hx, "gt", 0.99)]


# One kernel of every reducer kind: canonical f64 sums, counts, extremes, the integer sum, the
# order-free folds of every type, the arg folds and the canonical f32 and product chains.
CASES = [
    ("reduce_add_f64", ["f64"]), ("dot_f64", ["f64", "f64"]), ("sumsq_f64", ["f64"]),
    ("condsum_gt_f64", ["f64", 0.5, -1.0]), ("count_gt_f64", ["f64", 0.5]), ("count", ["bool"]),
    ("reduce_min_f64", ["f64"]), ("reduce_max_f64", ["f64"]), ("argmin_f64", ["f64"]),
    ("argmax_f64", ["f64"]), ("reduce_add_i64", ["i64"]), ("reduce_min_i64", ["i64"]),
    ("reduce_add_i32", ["i32"]), ("reduce_mul_i64", ["i64"]), ("reduce_and_u8", ["u8"]),
    ("reduce_xor_u64", ["u64"]), ("reduce_min_f32", ["f32"]), ("argmax_i32", ["i32"]),
    ("reduce_add_f32", ["f32"]), ("dot_f32", ["f32", "f32"]), ("reduce_mul_f64", ["f64"]),
    ("dot_i64", ["i64", "i64"]), ("any", ["bool"]), ("all", ["bool"]), ("reduce_or_bool", ["bool"]),
]


def column(t, n, seed):
    r = oracle.rand_i64(n, seed).view(np.uint64)
    if t == "f64":
        return oracle.rand_f64(n, seed) - 0.25
    if t == "f32":
        return (oracle.rand_f64(n, seed) - 0.25).astype(np.float32)
    if t == "bool":
        return (r % np.uint64(7)) != 0
    if t == "u8":
        return (r % np.uint64(251)).astype(np.uint8) | np.uint8(1)
    if t == "i32":
        return (r % np.uint64(2001)).astype(np.int32) - 1000
    if t == "u64":
        return r
    return (r % np.uint64(2001)).astype(np.int64) - 1000


@pytest.mark.parametrize("n", [1, 17, 4096 + 3, 300_001])
def test_enqueued_reductions_equal_the_call(ctx, n):
    for name, spec in CASES:
        args = [ctx.upload(column(a, n, 11 + i)) if isinstance(a, str) else a for i, a in enumerate(spec)]
        t, _, want = ctx.call(name, *args, raw=True)
        out = ctx.new_array(t, 3)
        ctx.call_into(name, *args, out=out, row=2)
        got = bits(out.numpy(), t)[2]
        assert int(got) == int(want) & ((1 << (8 * bits(out.numpy(), t).itemsize)) - 1), (name, n)


def test_enqueued_reductions_in_a_graph(ctx):
    n = 123_457
    data = {name: [ctx.upload(column(a, n, 31 + i)) if isinstance(a, str) else a for i, a in enumerate(spec)]
            for name, spec in CASES}
    want = {name: ctx.call(name, *args, raw=True) for name, args in data.items()}
    outs = {t: ctx.new_array(t, len(CASES)) for t in {w[0] for w in want.values()}}

    def program():
        for i, (name, args) in enumerate(data.items()):
            ctx.call_into(name, *args, out=outs[want[name][0]], row=i)

    program()
    ctx.synchronize()
    ctx.graph_begin()
    program()
    g = ctx.graph_end()
    for _ in range(2):
        for t, o in outs.items():
            zero(ctx, o, t)
        g.launch()
        got = {t: bits(o.numpy(), t) for t, o in outs.items()}
        for i, (name, (t, _, w)) in enumerate(want.items()):
            assert int(got[t][i]) == int(w) & ((1 << (8 * got[t].itemsize)) - 1), name


def test_call_into_errors(ctx):
    import verkehrt_gb300 as vk

    x = ctx.upload(oracle.rand_f64(100, 1))
    empty = ctx.upload(np.zeros(0))
    out = ctx.new_array("f64", 2)
    with pytest.raises(vk.KernelError) as e:
        ctx.call_into("reduce_min_f64", empty, out=out)
    assert (e.value.status, e.value.message) == ("RUNTIME", "reduce_min of an empty array")
    with pytest.raises(vk.KernelError) as e:
        ctx.call_into("argmax_i32", ctx.upload(np.zeros(0, np.int32)), out=ctx.new_array("i64", 1))
    assert e.value.message == "argmax of an empty array"
    with pytest.raises(vk.KernelError) as e:
        ctx.call_into("count_gt_f64", x, 0.5, out=out)
    assert e.value.status == "USAGE"
    assert e.value.message == "count_gt_f64 produces i64, got a f64 destination"
    with pytest.raises(vk.KernelError) as e:
        ctx.call_into("reduce_add_f64", x, out=out, row=2)
    assert e.value.message == "destination row 2 out of range for length 2"
    with pytest.raises(vk.KernelError) as e:
        ctx.call_into("add_f64", x, x, out=out)
    assert e.value.message == "add_f64 is not a reduction"
    # An empty sum is the identity, written like any other result.
    ctx.call_into("reduce_add_f64", empty, out=out, row=1)
    assert bits(out.numpy(), "f64")[1] == 0


def test_a_capture_never_grows_the_arena():
    import verkehrt_gb300 as vk

    c = vk.Context(0)
    try:
        n = 1 << 22
        x = c.upload(oracle.rand_f64(n, 5) - 0.5)
        out = c.new_array("f64", 1)
        want = bits(np.array([oracle.reduce_add_f64(oracle.rand_f64(n, 5) - 0.5)]), "f64")[0]
        c.graph_begin()
        with pytest.raises(vk.KernelError) as e:
            c.call_into("reduce_add_f64", x, out=out)
        assert e.value.status == "USAGE"
        assert "would grow during a capture" in e.value.message
        c.graph_end()  # the capture itself is still whole
        c.call_into("reduce_add_f64", x, out=out)  # grows the arena outside a capture
        c.synchronize()
        c.graph_begin()
        c.call_into("reduce_add_f64", x, out=out)
        g = c.graph_end()
        for _ in range(2):
            zero(c, out, "f64")
            g.launch()
            assert bits(out.numpy(), "f64")[0] == want
        del g
    finally:
        c.close()

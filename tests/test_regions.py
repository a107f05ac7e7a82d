"""Regions (src/exec/region.rs) run as one pass on the device: the value of random elementwise
trees over every type equals the kernels run one by one and the oracle's composition of the
same kernels (src/kernels/scalar/elementwise.rs); regions that would fail, or fail differently
when fused, give whole evaluation's error; fused roots (src/exec/region/fused.rs) give the
root's value over the region, through the registry's fused patterns where one matches
(src/kernels/scalar/fused.rs:286-379)."""

import random

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

NUM = ["f64", "f32", "i64", "u64", "i32", "u8"]
SIGNED = ["f64", "f32", "i64", "i32"]
BITS = ["i64", "u64", "i32", "u8"]
NP = {"f64": np.float64, "f32": np.float32, "i64": np.int64, "u64": np.uint64, "i32": np.int32,
      "u8": np.uint8, "bool": np.uint8}
UINT = {"f64": np.uint64, "f32": np.uint32, "i64": np.uint64, "u64": np.uint64, "i32": np.uint32,
        "u8": np.uint8, "bool": np.uint8}


def column(t, n, seed):
    """Values of type t with the type's edge cases among them."""
    r = oracle.rand_i64(n, seed).view(np.uint64)
    if t in ("f64", "f32"):
        x = (oracle.rand_f64(n, seed) - 0.5) * 8.0
        edge = [0.0, -0.0, np.inf, -np.inf, np.nan, 1e300 if t == "f64" else 3e38, -1.5, 2.5]
        x[: min(n, len(edge))] = edge[: min(n, len(edge))]
        return x.astype(NP[t])
    if t == "bool":
        return (r % np.uint64(3) == 0).astype(np.uint8)
    x = r.astype(NP[t]) if t != "i64" else r.view(np.int64)
    if t in ("i64", "i32"):
        x = x.copy()
        x[1::3] = (r[1::3] % np.uint64(200)).astype(NP[t]) - 100
    return x


def scalar_value(t, rng):
    if t in ("f64", "f32"):
        return rng.choice([0.5, -2.0, 0.0, 3.25, -0.0])
    if t == "bool":
        return rng.choice([0, 1])
    if t == "u8":
        return rng.randrange(1, 256)
    if t == "u64":
        return rng.randrange(1, 1 << 40)
    return rng.choice([-7, 3, 1, -1, 100])


class Tree:
    """A random region: kernels in post-order with sources, inputs (arrays and scalars)."""

    def __init__(self, rng, n, seed, max_kernels=8):
        self.rng, self.n, self.seed = rng, n, seed
        self.kernels, self.inputs, self.types = [], [], []
        self.arrays = {}
        self.max_kernels = max_kernels

    def array(self, t):
        if t not in self.arrays:
            self.arrays[t] = len(self.inputs)
            self.inputs.append(("array", t, column(t, self.n, self.seed * 10 + len(self.inputs))))
        return self.arrays[t]

    def scalar(self, t):
        self.inputs.append(("scalar", t, scalar_value(t, self.rng)))
        return len(self.inputs) - 1

    def kernel(self, name, srcs, out_t):
        self.kernels.append((name, srcs))
        self.types.append(out_t)
        return -1 - (len(self.kernels) - 1)

    def gen(self, t, depth, may_scalar=False):
        """A source of type t (an array unless may_scalar lets it be a scalar)."""
        if depth == 0 or len(self.kernels) >= self.max_kernels or self.rng.random() < 0.25:
            return self.scalar(t) if may_scalar and self.rng.random() < 0.4 else self.array(t)
        r = self.rng
        if t == "bool":
            c = r.random()
            if c < 0.45:
                s = r.choice(NUM)
                op = r.choice(["lt", "le", "gt", "ge", "eq", "ne"])
                a, b = self.gen(s, depth - 1), self.gen(s, depth - 1, True)
                return self.kernel("%s_%s" % (op, s), [a, b], "bool")
            if c < 0.7:
                op = r.choice(["and", "or", "xor", "eq", "ne"])
                return self.kernel("%s_bool" % op, [self.gen("bool", depth - 1), self.gen("bool", depth - 1, True)], "bool")
            if c < 0.85:
                return self.kernel("not_bool", [self.gen("bool", depth - 1)], "bool")
            return self.kernel("select_bool", [self.gen("bool", depth - 1, True), self.gen("bool", depth - 1),
                                               self.gen("bool", depth - 1, True)], "bool")
        choices = ["bin", "select", "cast"]
        if t in SIGNED:
            choices.append("un")
        if t in ("f64", "f32"):
            choices += ["div", "sqrt"]
        if t in BITS:
            choices += ["bits", "div_const"]
        c = r.choice(choices)
        if c == "bin":
            op = r.choice(["add", "sub", "mul", "min", "max"])
            return self.kernel("%s_%s" % (op, t), [self.gen(t, depth - 1), self.gen(t, depth - 1, True)], t)
        if c == "un":
            return self.kernel("%s_%s" % (r.choice(["neg", "abs"]), t), [self.gen(t, depth - 1)], t)
        if c == "div":
            return self.kernel("div_" + t, [self.gen(t, depth - 1), self.gen(t, depth - 1, True)], t)
        if c == "sqrt":
            return self.kernel("sqrt_" + t, [self.gen(t, depth - 1)], t)
        if c == "bits":
            if r.random() < 0.25:
                return self.kernel("not_" + t, [self.gen(t, depth - 1)], t)
            op = r.choice(["and", "or", "xor"])
            return self.kernel("%s_%s" % (op, t), [self.gen(t, depth - 1), self.gen(t, depth - 1, True)], t)
        if c == "div_const":
            return self.kernel("div_const_" + t, [self.gen(t, depth - 1), self.scalar(t)], t)
        if c == "select":
            return self.kernel("select_" + t, [self.gen("bool", depth - 1, True), self.gen(t, depth - 1),
                                               self.gen(t, depth - 1, True)], t)
        s = r.choice(NUM + ["bool"])
        return self.kernel("cast_%s_%s" % (s, t), [self.gen(s, depth - 1)], t)


class F64Tree(Tree):
    """Random regions of f64 arithmetic and comparisons (the f64 evaluator's regions): a
    comparison feeds a select's mask or is the region's value."""

    def gen(self, t, depth, may_scalar=False):
        r = self.rng
        if t == "bool":  # always a comparison (the evaluator's inputs are f64)
            op = r.choice(["lt", "le", "gt", "ge", "eq", "ne"])
            d = max(depth - 1, 0)
            return self.kernel(op + "_f64", [self.gen("f64", d), self.gen("f64", d, True)], "bool")
        if depth == 0 or len(self.kernels) >= self.max_kernels or r.random() < 0.25:
            return self.scalar("f64") if may_scalar and r.random() < 0.4 else self.array("f64")
        c = r.random()
        if c < 0.5:
            op = r.choice(["add", "sub", "mul", "div", "min", "max"])
            return self.kernel(op + "_f64", [self.gen("f64", depth - 1), self.gen("f64", depth - 1, True)], "f64")
        if c < 0.75:
            op = r.choice(["neg", "abs", "sqrt"])
            return self.kernel(op + "_f64", [self.gen("f64", depth - 1)], "f64")
        return self.kernel("select_f64", [self.gen("bool", depth - 1), self.gen("f64", depth - 1),
                                          self.gen("f64", depth - 1, True)], "f64")


def device_inputs(ctx, tree):
    import verkehrt_gb300 as vk

    out = []
    for kind, t, v in tree.inputs:
        out.append(ctx.upload(v, t) if kind == "array" else vk.Scalar(t, v))
    return out


def whole(ctx, kernels, inputs):
    vals = []
    for name, srcs in kernels:
        vals.append(ctx.call(name, *[inputs[s] if s >= 0 else vals[-1 - s] for s in srcs]))
    return vals[-1]


def oracle_eval(tree):
    vals = []
    for (name, srcs), t in zip(tree.kernels, tree.types):
        args = []
        for s in srcs:
            if s >= 0:
                kind, ty, v = tree.inputs[s]
                args.append(v)
            else:
                args.append(vals[-1 - s])
        parts = name.split("_")
        if parts[0] == "cast":
            vals.append(oracle.ew_cast(parts[1], parts[2], args[0]))
        elif parts[0] == "select":
            vals.append(oracle.ew_select(parts[1], args[0], args[1], args[2]))
        elif name.startswith("div_const_"):
            vals.append(oracle.ew_div_const(parts[2], args[0], args[1]))
        elif len(args) == 1:
            vals.append(oracle.ew_unary(parts[0], parts[1], args[0]))
        else:
            vals.append(oracle.ew_binary(parts[0], parts[1], args[0], args[1]))
    return vals[-1]


def same(a, b, t):
    """Bit for bit; a NaN of a float type only has to be a NaN."""
    a, b = np.ascontiguousarray(a).astype(NP[t], copy=False), np.ascontiguousarray(b).astype(NP[t], copy=False)
    ua, ub = a.view(UINT[t]), b.view(UINT[t])
    if t in ("f64", "f32"):
        return bool(np.all((ua == ub) | (np.isnan(a) & np.isnan(b))))
    return bool(np.array_equal(ua, ub))


@pytest.mark.parametrize("n", [1, 777, 100_003])
def test_random_regions_equal_whole_evaluation_and_the_oracle(ctx, n):
    rng = random.Random(n)
    checked = 0
    for case in range(40):
        tree = Tree(rng, n, case)
        t = rng.choice(NUM + ["bool"])
        top = tree.gen(t, depth=rng.randint(1, 4))
        if top >= 0:  # a leaf: make it a region of one kernel
            top = tree.kernel("add_%s" % t if t != "bool" else "or_bool", [top, top], t)
        dev = device_inputs(ctx, tree)
        got = ctx.region(tree.kernels, dev)
        want = whole(ctx, tree.kernels, dev)
        assert same(got.numpy(), want.numpy(), t), (n, case, tree.kernels)
        assert same(got.numpy(), oracle_eval(tree), t), (n, case, tree.kernels)
        checked += 1
    assert checked == 40


@pytest.mark.parametrize("n", [1, 777, 100_003])
def test_random_f64_regions(ctx, n):
    rng = random.Random(7 * n)
    for case in range(40):
        tree = F64Tree(rng, n, 100 + case)
        t = rng.choice(["f64", "f64", "bool"])
        top = tree.gen(t, depth=rng.randint(1, 4))
        if top >= 0:  # a leaf (f64 only): make it a region of one kernel
            top = tree.kernel("add_f64", [top, top], "f64")
        dev = device_inputs(ctx, tree)
        got = ctx.region(tree.kernels, dev)
        assert same(got.numpy(), whole(ctx, tree.kernels, dev).numpy(), t), (n, case, tree.kernels)
        assert same(got.numpy(), oracle_eval(tree), t), (n, case, tree.kernels)
        if t == "bool":
            k = len(tree.kernels) - 1
            want = int(np.count_nonzero(oracle_eval(tree)))
            assert ctx.region_reduce("count", [-1 - k], tree.kernels, dev) == want


def test_region_errors_are_whole_evaluation_errors(ctx):
    import verkehrt_gb300 as vk

    x = ctx.upload(column("f64", 1000, 1))
    y = ctx.upload(column("f64", 999, 2))
    k = vk.region_kernel

    def both(kernels, inputs):
        with pytest.raises(vk.KernelError) as e1:
            ctx.region(kernels, inputs)
        with pytest.raises(vk.KernelError) as e2:
            whole(ctx, kernels, inputs)
        assert (e1.value.status, e1.value.message) == (e2.value.status, e2.value.message)
        return e1.value.message

    assert both([("mul_f64", [0, 1]), ("add_f64", [k(0), 0])], [x, y]) == "length mismatch: 1000 vs 999"
    i = ctx.upload(column("i64", 1000, 3))
    assert both([("add_i64", [0, 0]), ("div_const_i64", [k(0), 1])], [i, vk.Scalar("i64", 0)]) == \
        "div_const: division by zero"
    assert both([("add_f64", [0, 0]), ("mul_f64", [k(0), 1])], [x, i]).startswith("expected f64")
    assert both([("add_f64", [0, 1]), ("neg_f64", [k(0)])], [0.5, 1.0]) == "an array kernel needs an array operand"


def test_long_regions_run_whole_with_the_same_value(ctx):
    import verkehrt_gb300 as vk

    n = 5000
    xs = [column("f64", n, 40 + i) for i in range(3)]
    kernels = [("add_f64", [0, 1])]
    for j in range(15):  # more kernels than the one-pass evaluator holds
        kernels.append(("mul_f64" if j % 2 else "add_f64", [vk.region_kernel(len(kernels) - 1), 2 if j % 3 else 0]))
    dev = [ctx.upload(x) for x in xs]
    assert same(ctx.region(kernels, dev).numpy(), whole(ctx, kernels, dev).numpy(), "f64")


def test_fused_roots(ctx):
    import verkehrt_gb300 as vk

    k = vk.region_kernel
    n = 300_001
    x, y = column("f64", n, 7), column("f64", n, 8)
    x[:8] = np.arange(8) + 1.0  # no NaN or inf in the sums below
    y[:8] = 1.0
    dx, dy = ctx.upload(x), ctx.upload(y)

    def check(root, root_args, kernels, inputs, want_bits=None):
        got = ctx.region_reduce(root, root_args, kernels, inputs, raw=True)
        vals = []
        for name, srcs in kernels:
            vals.append(ctx.call(name, *[inputs[s] if s >= 0 else vals[-1 - s] for s in srcs]))
        args = [inputs[s] if s >= 0 else vals[-1 - s] for s in root_args]
        want = ctx.call(root, *args, raw=True)
        assert (got[0], got[2]) == (want[0], want[2]), (root, kernels)  # type and bits
        if want_bits is not None:
            assert got[2] == want_bits
        return got

    bits = lambda v: int(np.array([v], np.float64).view(np.uint64)[0])
    # reduce_add(mul) is dot; with one array twice it is sumsq.
    check("reduce_add_f64", [k(0)], [("mul_f64", [0, 1])], [dx, dy], bits(oracle.dot_f64(x, y)))
    check("reduce_add_f64", [k(0)], [("mul_f64", [0, 1])], [dx, dx], bits(oracle.sumsq_f64(x)))
    # count(gt(x * 2, c)): the comparison's operand is a region kernel.
    c = check("count", [k(1)], [("mul_f64", [0, 1]), ("gt_f64", [k(0), 2])], [dx, 2.0, 0.5])
    assert c[1] == oracle.count_cmp_f64(oracle.mul_f64(x, np.full(n, 2.0)), "gt", 0.5)
    # condsum: reduce_add(select(lt(x, c), x, e)).
    check("reduce_add_f64", [k(1)], [("lt_f64", [0, 1]), ("select_f64", [k(0), 2, 3])], [dx, 0.25, dx, -1.0],
          bits(oracle.condsum_cmp_f64(x, "lt", 0.25, -1.0)))
    # Roots without a pattern: the root over the region's value.
    check("reduce_min_f64", [k(0)], [("add_f64", [0, 1])], [dx, dy])
    check("argmax_f64", [k(1)], [("sub_f64", [0, 1]), ("abs_f64", [k(0)])], [dx, dy])
    check("reduce_add_f64", [k(1)], [("mul_f64", [0, 1]), ("add_f64", [k(0), 2])], [dx, dy, 0.125])
    i = ctx.upload(column("i32", n, 9))
    check("reduce_add_i32", [k(0)], [("mul_i32", [0, 0])], [i, i])  # sumsq_i32
    check("reduce_max_i32", [k(0)], [("xor_i32", [0, 1])], [i, vk.Scalar("i32", 12345)])
    # Extremes and the i64 sum folded in the region's pass: NaN rows, -0 and +0, ties.
    xn = column("f64", n, 17)  # NaN, infinities and signed zeros among the first rows
    dxn = ctx.upload(xn)
    for root in ("reduce_min_f64", "reduce_max_f64", "argmin_f64", "argmax_f64"):
        check(root, [k(0)], [("mul_f64", [0, 1])], [dxn, dy])
        check(root, [k(0)], [("mul_f64", [0, 1])], [dxn, 0.0])  # every row +-0 or NaN
        check(root, [k(1)], [("abs_f64", [0]), ("neg_f64", [k(0)])], [dx])
    ii = ctx.upload(column("i64", n, 19))
    for root in ("reduce_min_i64", "reduce_max_i64", "argmin_i64", "argmax_i64", "reduce_add_i64"):
        check(root, [k(0)], [("mul_i64", [0, 1])], [ii, ii])
        check(root, [k(0)], [("and_i64", [0, 1])], [ii, vk.Scalar("i64", 7)])  # many ties
    want = oracle.argmin_f64(oracle.ew_binary("mul", "f64", xn, y))
    assert ctx.region_reduce("argmin_f64", [k(0)], [("mul_f64", [0, 1])], [dxn, dy]) == want
    # dot over two region kernels, and its length mismatch error as whole evaluation gives it.
    check("dot_f64", [k(0), k(1)], [("neg_f64", [0]), ("abs_f64", [1])], [dx, dy])
    short = ctx.upload(column("f64", 10, 3))
    with pytest.raises(vk.KernelError) as e:
        ctx.region_reduce("dot_f64", [k(0), k(1)], [("neg_f64", [0]), ("abs_f64", [1])], [dx, short])
    assert e.value.message == "length mismatch: %d vs 10" % n
    # An empty region under an extreme: the root's own error.
    empty = ctx.upload(np.zeros(0))
    with pytest.raises(vk.KernelError) as e:
        ctx.region_reduce("reduce_min_f64", [k(0)], [("add_f64", [0, 0])], [empty])
    assert e.value.message == "reduce_min of an empty array"

"""The oracle's outputs for the bench's full-size workloads (test infrastructure only).

`sweep_outputs(n)` restates the primitive sweep of bench.py (inputs of `make_inputs`, calls of
`sweep_plan`) at n rows with the oracle; `sortgroup_outputs(n, dist)` restates `sortgroup_step`:
stable argsort, the gathers by the permutation, the sorted group-by idiom of the reference's
tests/programs/grouping.dd:12-31 (run starts and ends, scan_by add over the runs, per-group sums
and keys by compress, and the same sums through reduce_into over the run numbers) and the hashed
group-by (group_id, then reduce_into add and histogram over the ids). Both yield (label, value)
pairs in call order, with the labels the bench prints; a value is a numpy array for an array
result and a Python float or int for a scalar. `bench.digest` turns either into the digest that
`full_size_digests.json` holds (written by make_full_digests.py).
"""

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402  (digest, zipf_keys, SELECTIVITY)
import oracle  # noqa: E402


def sweep_inputs(n):
    """bench.make_inputs, on the host."""
    assert n & (n - 1) == 0
    return {
        "x": oracle.rand_f64(n, 1),
        "y": oracle.rand_f64(n, 2),
        "src": oracle.rand_i64(n, 3),
        "idx": oracle.rand_i64(n, 4) & np.int64(n - 1),
        "v": (oracle.rand_i64(n, 5) & np.int64((1 << 21) - 1)) - np.int64(1 << 20),
    }


def sweep_outputs(n, inputs=None):
    """(label, value) of every call of bench.sweep_plan(n), in order."""
    d = inputs if inputs is not None else sweep_inputs(n)
    x, y = d["x"], d["y"]
    yield "reduce_add_f64", oracle.reduce_add_f64(x)
    yield "dot_f64", oracle.dot_f64(x, y)
    yield "reduce_min_f64", oracle.reduce_min_f64(x)
    yield "reduce_max_f64", oracle.reduce_max_f64(x)
    yield "argmin_f64", int(oracle.argmin_f64(x))
    yield "argmax_f64", int(oracle.argmax_f64(x))
    for c in bench.SELECTIVITY:
        yield "count_gt_f64@%g" % c, int(oracle.count_cmp_f64(x, "gt", c))
    for c in bench.SELECTIVITY:
        yield "filter_gt_f64@%g" % c, oracle.filter_cmp_f64(x, "gt", c)
    yield "gather_i64", oracle.gather(d["src"], d["idx"])
    yield "scan_add_i64", oracle.scan_add_i64(d["v"])
    xy = oracle.mul_f64(x, y)
    yield "mul_f64", xy
    yield "reduce_add_f64(mul)", oracle.reduce_add_f64(xy)


def sortgroup_inputs(n, dist):
    """Keys and values of bench.run_sort_groupby, on the host."""
    vf = oracle.rand_f64(n, 21)
    vi = (oracle.rand_i64(n, 22) & np.int64((1 << 21) - 1)) - np.int64(1 << 20)
    if dist == "uniform32":
        keys = oracle.rand_i64(n, 23) & np.int64((1 << 32) - 1)
    elif dist == "zipf1.1":
        keys = bench.zipf_keys(n)
    else:
        raise ValueError(dist)
    return keys, vf, vi


def sortgroup_outputs(n, dist, inputs=None):
    """(label, value) of every call of bench.sortgroup_step, in order."""
    keys, vf, vi = inputs if inputs is not None else sortgroup_inputs(n, dist)
    rows = np.arange(n, dtype=np.int64)
    perm = oracle.argsort_i64(keys)
    yield "argsort_i64", perm
    sk = oracle.gather(keys, perm)
    yield "gather_i64(keys)", sk
    yield "gather_f64(vals)", oracle.gather(vf, perm)
    sv = oracle.gather(vi, perm)
    yield "gather_i64(vals)", sv
    pk = oracle.prev_i64(sk, 0)
    yield "prev_i64", pk
    s = (sk != pk) | (rows == 0)
    yield "run_starts", s
    nk = oracle.gather(sk, np.minimum(rows + 1, n - 1))
    yield "gather_i64(next)", nk
    e = (sk != nk) | (rows == n - 1)
    yield "run_ends", e
    sb = oracle.scan_by_add_i64(sv, s)
    yield "scan_by_add_i64", sb
    yield "compress_i64(sums)", oracle.compress(sb, e)
    yield "compress_i64(keys)", oracle.compress(sk, s)
    runs = int(np.count_nonzero(s))
    yield "count", runs
    seg = oracle.scan_add_i64(s.astype(np.int64)) - 1
    yield "run_numbers", seg
    yield "reduce_into_add_i64(runs)", oracle.reduce_into_add_i64(seg, sv, runs)
    del sk, pk, nk, sb, seg
    g = oracle.group_id_i64(keys)
    yield "group_id_i64", g
    nb = int(g.max()) + 1 if n else 0
    yield "reduce_max_i64", nb - 1
    yield "reduce_into_add_i64", oracle.reduce_into_add_i64(g, vi, nb)
    yield "histogram", oracle.histogram(g, nb)

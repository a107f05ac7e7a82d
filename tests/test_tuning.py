"""The autotuner's knobs change launch shapes only: every candidate of every knob gives the
oracle's results (argsort, the streaming reductions, gather, group_id), and the committed table
holds allowed values that match its measurements file."""

import json
import os
import re

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_committed_table_is_consistent():
    from verkehrt_gb300 import autotune

    with open(os.path.join(ROOT, "verkehrt_gb300", "csrc", "tuning_table.h")) as f:
        text = f.read()
    rows = re.search(r"#define VKC_TUNE_TABLE \{(.*)\}", text).group(1)
    table = [[int(v) for v in r.split(",")] for r in re.findall(r"\{([^{}]*)\}", rows)]
    assert len(table) == len(autotune.KNOBS)
    for knob, row in zip(autotune.KNOBS, table):
        assert len(row) == len(autotune.CLASS_ROWS)
        assert all(v in autotune.CANDIDATES[knob] for v in row), knob
    path = os.path.join(ROOT, "verkehrt_gb300", "tuning_table.json")
    if os.path.exists(path):
        with open(path) as f:
            meas = json.load(f)
        assert [meas["table"][k] for k in autotune.KNOBS] == table


@pytest.mark.gpu
def test_every_candidate_gives_the_same_results(ctx):
    from verkehrt_gb300 import autotune

    cases = [300_001, (1 << 21) + 7]  # size classes 0 and 1
    for n in cases:
        c = 0 if n < (1 << 20) else 1
        keys = (oracle.rand_i64(n, 3).view(np.uint64) >> np.uint64(29)).astype(np.int64)
        x = oracle.rand_f64(n, 4)
        src = oracle.rand_i64(n, 5)
        idx = (oracle.rand_i64(n, 6).view(np.uint64) % np.uint64(n)).astype(np.int64)
        g = (oracle.rand_i64(n, 7).view(np.uint64) % np.uint64(1 << 17)).astype(np.int64)
        dk, dx, ds, di, dg = (ctx.upload(v) for v in (keys, x, src, idx, g))
        want = {
            "radix_items": oracle.argsort_i64(keys),
            "stream_blocks_per_sm": (oracle.count_cmp_f64(x, "gt", 0.5), oracle.reduce_min_f64(x), oracle.argmax_f64(x)),
            "gather_rows_per_thread": oracle.gather(src, idx),
            "group_first_table_log2": oracle.group_id_i64(g),
            "canon_chain_rows": np.float64(oracle.reduce_add_f64(x - 0.5)).view(np.uint64),
        }
        dc = ctx.upload(x - 0.5)
        for knob in autotune.KNOBS:
            before = ctx.tune_get(knob, c)
            for v in autotune.CANDIDATES[knob]:
                ctx.tune_set(knob, c, v)
                if knob == "radix_items":
                    assert np.array_equal(ctx.call("argsort_i64", dk).numpy(), want[knob]), (n, v)
                elif knob == "stream_blocks_per_sm":
                    got = (ctx.call("count_gt_f64", dx, 0.5), ctx.call("reduce_min_f64", dx), ctx.call("argmax_f64", dx))
                    assert got == want[knob], (n, v)
                elif knob == "gather_rows_per_thread":
                    assert np.array_equal(ctx.call("gather_i64", ds, di).numpy(), want[knob]), (n, v)
                elif knob == "canon_chain_rows":
                    assert ctx.call("reduce_add_f64", dc, raw=True)[2] == int(want[knob]), (n, v)
                else:
                    assert np.array_equal(ctx.call("group_id_i64", dg).numpy(), want[knob]), (n, v)
            ctx.tune_set(knob, c, before)


@pytest.mark.gpu
def test_tune_set_rejects_bad_values(ctx):
    with pytest.raises(Exception, match="not allowed"):
        ctx.tune_set("radix_items", 0, 7)
    with pytest.raises(Exception, match="no tuning knob"):
        ctx.tune_set("no_such_knob", 0, 8)

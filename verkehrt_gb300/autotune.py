"""The autotuner: picks each launch-shape knob per size class by measuring every candidate on
the GPU, and writes the table the library compiles in (csrc/tuning_table.h) plus the
measurements (tuning_table.json).

Knobs (csrc/tuning.h) and the workload each is timed on, at the representative size of each
class (2^18, 2^22, 2^26 rows; inputs generated on the device by the reference's generators):

  radix_items             argsort_i64 of 32-bit keys (four passes)
  stream_blocks_per_sm    count_gt_f64, reduce_min_f64 and argmax_f64 of rand_f64
  gather_rows_per_thread  gather_i64 with indices uniform over the source
  group_first_table_log2  group_id_i64 of keys with 2^12 and with 2^18 distinct values
  canon_chain_rows        reduce_add_f64 of rand_f64 - 0.5 (a mean-centred sum: the lane chain)

Every candidate gives the same results (the tests check the committed table's and the
others'); only the time differs. Usage, on a GPU machine, from the repository root:

    python -m verkehrt_gb300.autotune [--out DIR] [--reps K] [--knobs a,b]

(--knobs measures only those knobs and keeps the committed table's other rows)

then rebuild (the library recompiles when the table changes).
"""

import argparse
import datetime
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
KNOBS = ["radix_items", "stream_blocks_per_sm", "gather_rows_per_thread", "group_first_table_log2",
         "canon_chain_rows"]
CANDIDATES = {
    "radix_items": [8, 12, 16],
    "stream_blocks_per_sm": [2, 4, 5, 6, 8, 12, 16],
    "gather_rows_per_thread": [1, 2, 4],
    "group_first_table_log2": [18, 19, 20, 21, 22],
    "canon_chain_rows": [4, 8, 16],
}
CLASS_ROWS = [1 << 18, 1 << 22, 1 << 26]


def workloads(ctx, n):
    """knob -> a function that runs the knob's workload once (enqueued and synchronised)."""
    x = ctx.call("rand_f64", n, 1)
    k32 = ctx.call("and_i64", ctx.call("rand_i64", n, 2), 0xFFFFFFFF)
    src = ctx.call("rand_i64", n, 3)
    # Indices uniform over [0, n): the high bits of splitmix64 scaled down (n is a power of two).
    idx = ctx.call("and_i64", ctx.call("rand_i64", n, 4), n - 1)
    g12 = ctx.call("and_i64", ctx.call("rand_i64", n, 5), (1 << 12) - 1)
    g18 = ctx.call("and_i64", ctx.call("rand_i64", n, 6), (1 << 18) - 1)
    centred = ctx.call("sub_f64", x, 0.5)
    ctx.synchronize()

    def run(fn):
        def f():
            fn()
            ctx.synchronize()
        return f

    return {
        "radix_items": run(lambda: ctx.call("argsort_i64", k32)),
        "stream_blocks_per_sm": run(lambda: (ctx.call("count_gt_f64", x, 0.5), ctx.call("reduce_min_f64", x),
                                             ctx.call("argmax_f64", x))),
        "gather_rows_per_thread": run(lambda: ctx.call("gather_i64", src, idx)),
        "group_first_table_log2": run(lambda: (ctx.call("group_id_i64", g12), ctx.call("group_id_i64", g18))),
        "canon_chain_rows": run(lambda: ctx.call("reduce_add_f64", centred)),
    }


def median_time(f, reps):
    f()  # warm-up (allocations, first launch)
    ts = []
    for _ in range(reps):
        t = time.perf_counter()
        f()
        ts.append(time.perf_counter() - t)
    return float(np.median(ts))


def tune(ctx, reps, knobs=KNOBS):
    table, measured = {}, {}
    for c, n in enumerate(CLASS_ROWS):
        work = workloads(ctx, n)
        r = reps if n >= (1 << 24) else reps * 4
        for knob in knobs:
            times = {}
            for v in CANDIDATES[knob]:
                ctx.tune_set(knob, c, v)
                times[v] = median_time(work[knob], r)
            best = min(times, key=times.get)
            ctx.tune_set(knob, c, best)
            table.setdefault(knob, [None] * len(CLASS_ROWS))[c] = best
            measured.setdefault(knob, {})[str(n)] = {str(v): round(t * 1e3, 4) for v, t in times.items()}
            print("class %d (n=%d) %-24s %s -> %d" % (c, n, knob, measured[knob][str(n)], best), flush=True)
        del work
    return table, measured


def device_name():
    try:
        import torch

        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown GPU"


def write(table, measured, out):
    os.makedirs(out, exist_ok=True)
    stamp = datetime.date.today().isoformat()
    rows = ", ".join("{%s}" % ", ".join(str(v) for v in table[k]) for k in KNOBS)
    header = (
        "// The autotuner's table: written by `python -m verkehrt_gb300.autotune` from measurements on\n"
        "// the GPU named below; edit by rerunning it. Rows are the knobs in TuneKnob order (radix rows\n"
        "// per thread, streaming-reduction blocks per SM, gather rows per thread, log2 of the group_id\n"
        "// first table's slots, rows per thread of the canonical sums' lane chain); columns are the\n"
        "// size classes n < 2^20, n < 2^24, and larger.\n"
        "// Measured on: %s, %s (median of the runs in tuning_table.json).\n"
        "#pragma once\n"
        "#define VKC_TUNE_TABLE { %s }\n" % (device_name(), stamp, rows))
    with open(os.path.join(out, "tuning_table.h"), "w") as f:
        f.write(header)
    with open(os.path.join(out, "tuning_table.json"), "w") as f:
        json.dump({"device": device_name(), "date": stamp, "size_classes": CLASS_ROWS,
                   "table": table, "median_ms": measured}, f, indent=1)
        f.write("\n")


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", default=None, help="directory for tuning_table.h/.json (default: the package)")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--knobs", default=",".join(KNOBS), help="the knobs to measure (comma-separated)")
    args = ap.parse_args(argv)
    import verkehrt_gb300 as vk

    knobs = [k for k in args.knobs.split(",") if k]
    unknown = set(knobs) - set(KNOBS)
    if unknown:
        ap.error("unknown knobs: %s" % ", ".join(sorted(unknown)))
    ctx = vk.Context(0)
    table, measured = tune(ctx, args.reps, knobs)
    if set(knobs) != set(KNOBS):
        # The other rows stay as committed (their measurements with them).
        with open(os.path.join(HERE, "tuning_table.json")) as f:
            old = json.load(f)
        for k in KNOBS:
            if k not in table:
                table[k] = old["table"].get(k) or [ctx.tune_get(k, c) for c in range(len(CLASS_ROWS))]
                if k in old.get("median_ms", {}):
                    measured[k] = old["median_ms"][k]
    if args.out is None:
        write(table, measured, os.path.join(HERE, "csrc"))
        os.replace(os.path.join(HERE, "csrc", "tuning_table.json"), os.path.join(HERE, "tuning_table.json"))
    else:
        write(table, measured, args.out)
    print(json.dumps(table))


if __name__ == "__main__":
    sys.exit(main())

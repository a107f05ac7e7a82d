#!/usr/bin/env python3
"""Benchmark of the verkehrt kernel-table primitives on GB300 (the `cuda` ISA).

Workload: the primitive sweep at n = 2^28 rows (the reference's headline "HBM GB/s per kernel"
sweep at its largest size): reduce_add/dot/min/max/argmin/argmax over f64 uniform [0,1),
count_gt and filter_gt at 1%/50%/99% selectivity, gather_i64 with indices uniform in [0,n),
scan_add_i64 over values uniform in [-2^20, 2^20), and the unfused dot (mul_f64 then
reduce_add_f64), which must give the fused bits. One step runs every primitive once as a plain
per-statement call through the C ABI.

value   algorithmic bytes of the step / device time of the step (GB/s, inputs resident in HBM,
        every array 2 GiB, larger than the 126 MB L2, so no flush is needed)
e2e     the same bytes / time of the step through the C ABI with host buffers: the step's inputs
        uploaded from pinned host memory and its array results downloaded, every step
roofline  the dominant kernel's algorithmic GB/s against the measured HBM copy bandwidth
cpu_baseline  the oracle port of the reference's scalar entries (single thread, like the
        reference) on a bounded sample of the same workload, on this machine's host

--impl reference times that CPU implementation as the reference arm. With N > 1 ranks (torchrun)
every rank runs an independent replica ("replicas only": the primitives have no exchange step).
"""

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "HBM GB/s per kernel vs peak; batched/served req/s and p99 vs plain GPU path"
UNIT = "GB/s"
SELECTIVITY = (0.99, 0.5, 0.01)  # thresholds of count_gt/filter_gt: 1%, 50%, 99% kept


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic():
    """Per-launch DRAM bytes of the dominant kernels from the committed ncu captures."""
    path = os.path.join(ROOT, "profiles", "dram_traffic_sweep_n2p28.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


# ---------------------------------------------------------------------------- clocks


class ClockSampler:
    """Samples nvidia-smi every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------- the sweep


def sweep_plan(n):
    """(label, kernel, argument names, extra scalars, fixed algorithmic bytes)."""
    plan = [
        ("reduce_add_f64", "reduce_add_f64", ["x"], [], 8 * n),
        ("dot_f64", "dot_f64", ["x", "y"], [], 16 * n),
        ("reduce_min_f64", "reduce_min_f64", ["x"], [], 8 * n),
        ("reduce_max_f64", "reduce_max_f64", ["x"], [], 8 * n),
        ("argmin_f64", "argmin_f64", ["x"], [], 8 * n),
        ("argmax_f64", "argmax_f64", ["x"], [], 8 * n),
    ]
    for c in SELECTIVITY:
        plan.append(("count_gt_f64@%g" % c, "count_gt_f64", ["x"], [c], 8 * n))
    for c in SELECTIVITY:
        plan.append(("filter_gt_f64@%g" % c, "filter_gt_f64", ["x"], [c], 8 * n))  # + 8k
    plan += [
        ("gather_i64", "gather_i64", ["src", "idx"], [], 24 * n),
        ("scan_add_i64", "scan_add_i64", ["v"], [], 16 * n),
        ("mul_f64", "mul_f64", ["x", "y"], [], 24 * n),
        ("reduce_add_f64(mul)", "reduce_add_f64", ["xy"], [], 8 * n),
    ]
    return plan


def make_inputs(ctx, n):
    """Seeded inputs generated on the device with the reference's rand_* kernels."""
    assert n & (n - 1) == 0, "n must be a power of two (indices are rand mod n)"
    x = ctx.call("rand_f64", n, 1)
    y = ctx.call("rand_f64", n, 2)
    src = ctx.call("rand_i64", n, 3)
    idx = ctx.call("and_i64", ctx.call("rand_i64", n, 4), n - 1)
    v = ctx.call("sub_i64", ctx.call("and_i64", ctx.call("rand_i64", n, 5), (1 << 21) - 1), 1 << 20)
    ctx.synchronize()
    return {"x": x, "y": y, "src": src, "idx": idx, "v": v}


def run_step(ctx, n, inputs, events, host_out=None):
    """One pass of the sweep. Returns {label: (ms, bytes)} measured with CUDA events on the
    library's stream, the step's device time, and the results."""
    import torch

    plan = sweep_plan(n)
    marks = []
    results = {}
    env = dict(inputs)
    stream = events["stream"]
    with torch.cuda.stream(stream):
        start = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for label, kernel, names, extra, nbytes in plan:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = ctx.call(kernel, *[env[a] for a in names], *extra)
            e1.record(stream)
            if kernel == "filter_gt_f64":
                nbytes += 8 * len(out)
            if kernel == "mul_f64":
                env["xy"] = out
            results[label] = out
            marks.append((label, e0, e1, nbytes))
        stop = torch.cuda.Event(enable_timing=True)
        stop.record(stream)
    stop.synchronize()
    per = {label: (e0.elapsed_time(e1), b) for label, e0, e1, b in marks}
    return per, start.elapsed_time(stop), results


def check_results(results):
    """The unfused dot must give the fused bits (fused-equals-unfused on device)."""
    a = results["dot_f64"]
    b = results["reduce_add_f64(mul)"]
    if np.float64(a).view(np.uint64) != np.float64(b).view(np.uint64):
        raise SystemExit("fused dot %r != unfused %r" % (a, b))


# ---------------------------------------------------------------------------- parity digests


DIGESTS = os.path.join(ROOT, "tests", "golden", "full_size_digests.json")


def digest(value):
    """SHA-256 (first 32 hex digits) of a result's little-endian bytes: an array's rows (bool as
    0/1 bytes), an f64 scalar's IEEE bits, an integer scalar as an i64."""
    import hashlib

    if hasattr(value, "handle"):
        value = value.numpy()
    if isinstance(value, np.ndarray):
        a = value.view(np.uint8) if value.dtype == np.bool_ else value
        data = np.ascontiguousarray(a).tobytes()
    elif isinstance(value, float):
        data = np.float64(value).tobytes()
    else:
        data = np.int64(value).tobytes()
    return hashlib.sha256(data).hexdigest()[:32]


def committed_digests():
    """The oracle's digests of the full-size workloads' outputs (tests/golden/make_full_digests.py)."""
    if os.path.exists(DIGESTS):
        with open(DIGESTS) as f:
            return json.load(f)
    return {}


def check_digests(results, want, n, want_n):
    """Compares every result that has a committed digest with it (outside the timed region)."""
    if not want or want_n != n:
        return {"parity_checked": None, "why": "no committed oracle digests at n=%d" % n}
    bad = [label for label, d in want.items() if label not in results or digest(results[label]) != d]
    return {"parity_checked": not bad, "outputs_checked": len(want), "mismatches": bad}


# ---------------------------------------------------------------------------- argsort and group-by


def splitmix64_np(x):
    """splitmix64 of uint64 counters (the generator behind rand_i64), vectorised."""
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def zipf_keys(n, s=1.1, distinct=1 << 20, seed=11):
    """Keys with Zipf(s) frequencies over `distinct` ranks: inverse CDF of a host table driven
    by a seeded splitmix stream; key = splitmix64(rank), so keys span the full 64 bits."""
    w = np.arange(1, distinct + 1, dtype=np.float64) ** -s
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    out = np.empty(n, dtype=np.int64)
    chunk = 1 << 24
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        u = (splitmix64_np(np.arange(seed + a, seed + b, dtype=np.uint64)) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
        rank = np.minimum(np.searchsorted(cdf, u, side="right"), distinct - 1).astype(np.uint64)
        out[a:b] = splitmix64_np(rank).view(np.int64)
    return out


def sortgroup_step(ctx, keys, vf, vi, stream):
    """One group-by pass at n rows, as a program of per-statement calls. The sorted idiom of the
    reference's tests/programs/grouping.dd:12-31: stable argsort, the keys and values gathered by
    the permutation, run starts s = (k != prev(k, 0)) | (row == 0) and ends e = (k != next(k)) |
    (row == n - 1), scan_by add over the runs, per-group sums compress(scan_by, e) and keys
    compress(k, s), and the same sums as reduce_into(scan(cast_i64(s)) - 1, v, count(s), add).
    Then the hashed group-by: group_id, reduce_into add and histogram over the ids. Returns
    ([(label, ms, algorithmic bytes)], {label: result})."""
    import torch

    n = len(keys)
    marks, res = [], {}

    def timed(label, fn, nbytes):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        k = len(out) if hasattr(out, "handle") else 0
        marks.append((label, e0, e1, nbytes(k) if callable(nbytes) else nbytes))
        res[label] = out
        return out

    c = ctx.call
    with torch.cuda.stream(stream):
        perm = timed("argsort_i64", lambda: c("argsort_i64", keys), 16 * n)
        sk = timed("gather_i64(keys)", lambda: c("gather_i64", keys, perm), 24 * n)
        timed("gather_f64(vals)", lambda: c("gather_f64", vf, perm), 24 * n)
        sv = timed("gather_i64(vals)", lambda: c("gather_i64", vi, perm), 24 * n)
        io = timed("iota", lambda: c("iota", n), 8 * n)
        pk = timed("prev_i64", lambda: c("prev_i64", sk, 0), 16 * n)
        ne = timed("ne_i64(starts)", lambda: c("ne_i64", sk, pk), 17 * n)
        first = timed("eq_i64(first)", lambda: c("eq_i64", io, 0), 9 * n)
        s = timed("run_starts", lambda: c("or_bool", ne, first), 3 * n)
        nxt = timed("add_i64(next)", lambda: c("add_i64", io, 1), 16 * n)
        nxt = timed("min_i64(next)", lambda: c("min_i64", nxt, n - 1), 16 * n)
        nk = timed("gather_i64(next)", lambda: c("gather_i64", sk, nxt), 24 * n)
        ne = timed("ne_i64(ends)", lambda: c("ne_i64", sk, nk), 17 * n)
        last = timed("eq_i64(last)", lambda: c("eq_i64", io, n - 1), 9 * n)
        e = timed("run_ends", lambda: c("or_bool", ne, last), 3 * n)
        sb = timed("scan_by_add_i64", lambda: c("scan_by_add_i64", sv, s), 17 * n)
        timed("compress_i64(sums)", lambda: c("compress_i64", sb, e), lambda k: 9 * n + 8 * k)
        timed("compress_i64(keys)", lambda: c("compress_i64", sk, s), lambda k: 9 * n + 8 * k)
        runs = timed("count", lambda: c("count", s), n)
        si = timed("cast_bool_i64", lambda: c("cast_bool_i64", s), 9 * n)
        si = timed("scan_add_i64(runs)", lambda: c("scan_add_i64", si), 16 * n)
        seg = timed("run_numbers", lambda: c("sub_i64", si, 1), 16 * n)
        timed("reduce_into_add_i64(runs)", lambda: c("reduce_into_add_i64", seg, sv, runs), 16 * n + 8 * runs)
        g = timed("group_id_i64", lambda: c("group_id_i64", keys), 16 * n)
        nb = timed("reduce_max_i64", lambda: c("reduce_max_i64", g), 8 * n) + 1
        timed("reduce_into_add_i64", lambda: c("reduce_into_add_i64", g, vi, nb), 16 * n + 8 * nb)
        timed("histogram", lambda: c("histogram", g, nb), 8 * n + 8 * nb)
    torch.cuda.current_stream().synchronize()
    stream.synchronize()
    return [(label, e0.elapsed_time(e1), b) for label, e0, e1, b in marks], res


def run_sort_groupby(ctx, n, stream, steps, warmup, digests=None):
    """Argsort and group-by at n rows for both key distributions: per-call ms, GB/s and rows/s,
    and the last step's outputs checked against the committed oracle digests."""
    out = {}
    vf = ctx.call("rand_f64", n, 21)
    vi = ctx.call("sub_i64", ctx.call("and_i64", ctx.call("rand_i64", n, 22), (1 << 21) - 1), 1 << 20)
    for dist in ("uniform32", "zipf1.1"):
        if dist == "uniform32":
            keys = ctx.call("and_i64", ctx.call("rand_i64", n, 23), (1 << 32) - 1)
        else:
            keys = ctx.upload(zipf_keys(n))
        for _ in range(warmup):
            sortgroup_step(ctx, keys, vf, vi, stream)
        acc = {}
        for _ in range(steps):
            res = None  # free the previous step's outputs first
            per, res = sortgroup_step(ctx, keys, vf, vi, stream)
            for label, ms, nbytes in per:
                a = acc.setdefault(label, [0.0, 0])
                a[0] += ms
                a[1] = nbytes
        nb = res["reduce_max_i64"] + 1
        calls = {}
        for label, (ms_sum, nbytes) in acc.items():
            ms = ms_sum / steps
            calls[label] = {"ms": round(ms, 4), "GB/s": round(nbytes / (ms / 1e3) / 1e9, 1),
                            "Grows/s": round(n / (ms / 1e3) / 1e9, 3)}
        total = sum(a[0] for a in acc.values()) / steps
        sorted_ms = sum(a[0] for k, a in acc.items() if k not in HASHED_GROUPBY) / steps
        out[dist] = {"groups": int(nb), "pipeline_ms": round(total, 3),
                     "sorted_idiom_ms": round(sorted_ms, 3), "hashed_ms": round(total - sorted_ms, 3),
                     "kernels": calls,
                     "parity": check_digests(res, (digests or {}).get(dist), n, (digests or {}).get("n"))}
        del keys, res
    return {"workload": "n=2^%d i64 keys (uniform over [0,2^32); Zipf s=1.1 over 2^20 keys, "
                        "key = splitmix64(rank)), f64 and i64 values; stable argsort, gathers by "
                        "the permutation, the sorted group-by idiom (run starts/ends, scan_by add, "
                        "compress of sums and keys, reduce_into over run numbers), and group_id + "
                        "reduce_into + histogram" % (n.bit_length() - 1),
            "steps": steps, "warmup": warmup, **out}


# Calls of the hashed group-by in sortgroup_step (the rest is the sorted idiom).
HASHED_GROUPBY = ("group_id_i64", "reduce_max_i64", "reduce_into_add_i64", "histogram")


def run_f64_scans(ctx, n, stream, steps=3, warmup=1):
    """scan_add_f64 at n rows (uniform [0,1)) and scan_by_add_f64 at n/2 rows with segments of
    about 128 rows (start flags set with probability 1/128): CUDA-event ms and GB/s of the
    algorithmic bytes (read 8 + write 8 per row, plus the start flag's byte for scan_by)."""
    import torch

    x = ctx.call("rand_f64", n, 31)
    m = n // 2
    v = ctx.call("rand_f64", m, 32)
    starts = ctx.call("lt_f64", ctx.call("rand_f64", m, 33), 1.0 / 128)
    cases = (("scan_add_f64", lambda: ctx.call("scan_add_f64", x), 16 * n, n),
             ("scan_by_add_f64", lambda: ctx.call("scan_by_add_f64", v, starts), 17 * m, m))
    out = {}
    with torch.cuda.stream(stream):
        for label, fn, nbytes, rows in cases:
            for _ in range(warmup):
                fn()
            ts = []
            for _ in range(steps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                stream.synchronize()
                ts.append(e0.elapsed_time(e1))
            ms = sorted(ts)[len(ts) // 2]
            out[label] = {"rows": rows, "ms": round(ms, 4), "GB/s": round(nbytes / (ms / 1e3) / 1e9, 1)}
    return {"workload": "scan_add_f64 at n=2^%d uniform [0,1); scan_by_add_f64 at n=2^%d, segments of "
                        "about 128 rows; the candidate float scan order (prefix canonical sums)"
                        % (n.bit_length() - 1, m.bit_length() - 1), **out}


# ---------------------------------------------------------------------------- canonical sums on hard inputs


def adversarial_inputs(ctx, n):
    """Inputs whose lane sums keep leaving their binade, generated on the device: mean-centred
    rows u - 0.5, all-negative rows -u, and signed rows over about 31 binades, (u - 0.5) * k^8
    with k uniform in 0..15."""
    u = ctx.call("rand_f64", n, 61)
    k = ctx.call("cast_i64_f64", ctx.call("and_i64", ctx.call("rand_i64", n, 62), 15))
    k2 = ctx.call("mul_f64", k, k)
    k4 = ctx.call("mul_f64", k2, k2)
    return {"centred": ctx.call("sub_f64", u, 0.5),
            "negative": ctx.call("neg_f64", u),
            "wide": ctx.call("mul_f64", ctx.call("sub_f64", u, 0.5), ctx.call("mul_f64", k4, k4))}


def run_canon_adversarial(ctx, sizes, stream, steps=3, cpu_n=1 << 24, no_cpu=False):
    """reduce_add_f64 on the hard inputs at each size (CUDA events, median of `steps`), beside the
    oracle port of the reference's scalar sum (one thread, as the reference) on the same kind of
    input at cpu_n rows, scaled to rows/s."""
    import torch

    out = {}
    for n in sizes:
        xs = adversarial_inputs(ctx, n)
        for name, x in xs.items():
            ctx.call("reduce_add_f64", x)
            ts = []
            with torch.cuda.stream(stream):
                for _ in range(steps):
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    ctx.call("reduce_add_f64", x)
                    e1.record(stream)
                    stream.synchronize()
                    ts.append(e0.elapsed_time(e1))
            ms = sorted(ts)[len(ts) // 2]
            out.setdefault(name, {})["n=2^%d" % (n.bit_length() - 1)] = {
                "ms": round(ms, 3), "GB/s": round(8 * n / (ms / 1e3) / 1e9, 1), "Grows/s": round(n / ms / 1e6, 3)}
        del xs
    cpu = None
    if not no_cpu:
        cpu = cpu_sum_rates(cpu_n)
        for name, rate in cpu.items():
            out[name]["cpu_port_1_thread_Grows/s"] = rate
    return {"workload": "reduce_add_f64 on mean-centred (u - 0.5), all-negative (-u) and (u - 0.5) * k^8 "
                        "(k uniform in 0..15, about 31 binades) rows; CPU: the oracle port on one host thread "
                        "at n=2^%d"
                        % (cpu_n.bit_length() - 1), **out}


def run_regions(ctx, n, stream, steps=3):
    """Regions as one pass (vkc_region_eval, vkc_region_reduce) against their kernels run whole
    (Tiling::Off), at n rows of rand_f64 inputs: x * y + z, sum(x * y) (the dot pattern) beside
    dot_f64 itself, count(x * y > 0.25) and min(x * y + z). Every region value is checked
    against whole evaluation's."""
    import torch
    import verkehrt_gb300 as vk

    k = vk.region_kernel
    x, y, z = (ctx.call("rand_f64", n, 71 + i) for i in range(3))

    def med(fn):
        fn()
        ts = []
        with torch.cuda.stream(stream):
            for _ in range(steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                stream.synchronize()
                ts.append(e0.elapsed_time(e1))
        return sorted(ts)[len(ts) // 2]

    fma = [("mul_f64", [0, 1]), ("add_f64", [k(0), 2])]
    out = {}

    def case(name, region, whole, nbytes):
        r = region()
        w = whole()
        if isinstance(r, vk.Array):
            ok = bool(np.array_equal(r.numpy().view(np.uint64), w.numpy().view(np.uint64)))
        else:
            ok = r == w
        del r, w
        tr, tw = med(region), med(whole)
        out[name] = {"region_ms": round(tr, 3), "whole_ms": round(tw, 3), "speedup": round(tw / tr, 2),
                     "region_GB/s": round(nbytes / (tr / 1e3) / 1e9, 1), "equal_to_whole": ok}

    case("x*y+z", lambda: ctx.region(fma, [x, y, z]),
         lambda: ctx.call("add_f64", ctx.call("mul_f64", x, y), z), 32 * n)
    case("sum(x*y)", lambda: ctx.region_reduce("reduce_add_f64", [k(0)], fma[:1], [x, y], raw=True),
         lambda: ctx.call("reduce_add_f64", ctx.call("mul_f64", x, y), raw=True), 16 * n)
    out["sum(x*y)"]["dot_f64_ms"] = round(med(lambda: ctx.call("dot_f64", x, y)), 3)
    case("count(x*y>0.25)", lambda: ctx.region_reduce("count", [k(1)], [fma[0], ("gt_f64", [k(0), 2])], [x, y, 0.25]),
         lambda: ctx.call("count", ctx.call("gt_f64", ctx.call("mul_f64", x, y), 0.25)), 16 * n)
    case("min(x*y+z)", lambda: ctx.region_reduce("reduce_min_f64", [k(1)], fma, [x, y, z], raw=True),
         lambda: ctx.call("reduce_min_f64", ctx.call("add_f64", ctx.call("mul_f64", x, y), z), raw=True), 24 * n)
    del x, y, z
    return {"workload": "n=2^%d rand_f64 columns; region_GB/s counts each input read once and the result "
                        "written once" % (n.bit_length() - 1), **out}


def cpu_sum_rates(n):
    """Rows/s (in G) of the oracle port's canonical sum on the hard inputs, one thread."""
    import oracle

    u = oracle.rand_f64(n, 61)
    k = (oracle.rand_i64(n, 62) & 15).astype(np.float64)
    rates = {}
    k4 = (k * k) * (k * k)
    for name, x in (("centred", u - 0.5), ("negative", -u), ("wide", (u - 0.5) * (k4 * k4))):
        oracle.reduce_add_f64(x)
        t0 = time.perf_counter()
        reps = 3
        for _ in range(reps):
            oracle.reduce_add_f64(x)
        rates[name] = round(reps * n / (time.perf_counter() - t0) / 1e9, 3)
    return rates


# ---------------------------------------------------------------------------- batched statements


def batch_lengths(count, lo, hi, seed=13):
    """Lengths floor(2^U), U uniform in [lo, hi], from a seeded splitmix stream."""
    u = (splitmix64_np(np.arange(seed, seed + count, dtype=np.uint64)) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    return np.floor(2.0 ** (lo + (hi - lo) * u)).astype(np.int64)


def run_batched(ctx, count=4096, lo=10, hi=18, reps=2):
    """Batched statements: `count` independent arrays, each running filter_gt(0.9) -> sum on f64 values and
    argsort of i64 keys below 2^16, three ways: the plain per-array GPU path (one synchronous
    call per statement, as the reference executor runs them), the batched entries (one
    persistent launch for the filter-sum, one batched radix sort), and a captured CUDA graph of
    the batch replayed. Each timed run includes reading the sums back to the host."""
    lens = batch_lengths(count, lo, hi)
    xs = [ctx.call("rand_f64", int(n), 100 + i) for i, n in enumerate(lens)]
    ks = [ctx.call("and_i64", ctx.call("rand_i64", int(n), 50_000 + i), 0xFFFF) for i, n in enumerate(lens)]
    ctx.synchronize()

    def plain():
        sums, perms = [], []
        for x, k in zip(xs, ks):
            sums.append(ctx.call("reduce_add_f64", ctx.call("filter_gt_f64", x, 0.9)))
            perms.append(ctx.call("argsort_i64", k))
        ctx.synchronize()
        return sums, perms

    xb, kb = ctx.batch(xs), ctx.batch(ks)
    outs = [ctx.new_array("i64", int(n)) for n in lens]
    ob = ctx.batch(outs)
    sums_arr = ctx.new_array("f64", count)
    ctx.batch_argsort(kb, ob, key_digits=0b11)  # first call: scratch
    ctx.synchronize()

    def batched():
        ctx.batch_filter_sum(xb, "gt", 0.9, sums_arr)
        ctx.batch_argsort(kb, ob, key_digits=0b11)
        return sums_arr.numpy()

    ctx.graph_begin()
    ctx.batch_filter_sum(xb, "gt", 0.9, sums_arr)
    ctx.batch_argsort(kb, ob, key_digits=0b11)
    graph = ctx.graph_end()

    def replay():
        graph.launch()
        return sums_arr.numpy()

    def timed(fn):
        fn()  # warm-up
        best = None
        for _ in range(reps):
            t0 = time.perf_counter()
            out = fn()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        return best, out

    t_plain, (psums, pperms) = timed(plain)
    t_batch, bsums = timed(batched)
    t_graph, gsums = timed(replay)
    want = np.array(psums, dtype=np.float64).view(np.uint64)
    exact = bool(np.array_equal(bsums.view(np.uint64), want) and np.array_equal(gsums.view(np.uint64), want))
    sample = range(0, count, max(1, count // 64))
    perms_ok = all(np.array_equal(outs[i].numpy(), pperms[i].numpy()) for i in sample)
    rows = int(lens.sum())

    def line(t):
        return {"s": round(t, 4), "arrays_per_s": round(count / t, 1), "rows_per_s": round(rows / t, 1)}

    return {"workload": "%d arrays, lengths floor(2^U) with U uniform in [%d, %d] (%d rows, %.2f GiB of f64 "
                        "values and i64 keys); per array filter_gt_f64(0.9) -> reduce_add_f64 and "
                        "argsort_i64 of keys below 2^16" % (count, lo, hi, rows, 16 * rows / 2 ** 30),
            "plain": line(t_plain), "batched": line(t_batch), "graph": line(t_graph),
            "speedup_batched": round(t_plain / t_batch, 2), "speedup_graph": round(t_plain / t_graph, 2),
            "sums_bit_exact": exact, "argsort_sample_equal": bool(perms_ok)}


# ---------------------------------------------------------------------------- served requests


# Two request mixes: the full range of sizes, where large argsorts and group-bys keep the device
# busy whatever the scheduling, and small requests only, where per-statement launches and
# synchronisations dominate the plain path.
SERVED_MIXES = {
    "mixed": {"n_lo": 1e3, "n_hi": 1e8, "rates": (500, 1000, 1500, 2000, 2500, 3000, 4000, 6400),
              "p99_bound_ms": 100.0},
    "small": {"n_lo": 1e3, "n_hi": 1e5, "rates": (1000, 2500, 5000, 10000, 20000, 40000, 60000, 80000, 120000),
              "p99_bound_ms": 20.0},
}


def run_served(ctx, count=3000, slots=4, budget=150e9):
    """Served requests: Poisson arrivals of programs drawn from {dot, filter_gt + length, argsort,
    group-by sum} with n = floor(10^U), U uniform over each mix's range, inputs generated on the
    device; the plain GPU path (one request at a time, one synchronous call per statement)
    against the server (continuous batching over `slots` streams, same-kind coalescing,
    admission by a 150 GB HBM budget). Latency is arrival to answer. Every rate runs `count`
    requests. gpu_busy is the time the streams spent on requests (CUDA events around every
    request or group) over the wall time: for the plain path's one stream, the share of the run
    the device was working for it."""
    import verkehrt_gb300 as vk
    from verkehrt_gb300 import serve

    ctx.set_cache_limit(16 << 30)
    workers = [vk.Context(ctx.device) for _ in range(slots)]
    for w in workers:
        w.set_cache_limit(16 << 30)
    # Warm-up of both paths on a short mix.
    serve.serve([ctx], serve.poisson_requests(16, 1e4, seed=1, n_hi=1e5), budget, batching=False)
    serve.serve(workers, serve.poisson_requests(16, 1e4, seed=1, n_hi=1e5), budget)
    result = {}
    for mix, spec in SERVED_MIXES.items():
        out = []
        for rate in spec["rates"]:
            row = {"offered_req_per_s": rate}
            runs = {}
            for mode, ws, batching in (("plain", [ctx], False), ("served", workers, True)):
                reqs = serve.poisson_requests(count, rate, seed=rate, n_lo=spec["n_lo"], n_hi=spec["n_hi"])
                dev = []
                wall = serve.serve(ws, reqs, budget, batching=batching, device_ms=dev)
                row[mode] = serve.summary(reqs, wall)
                row[mode]["gpu_busy"] = round(sum(dev) / 1e3 / wall, 3) if wall > 0 else None
                runs[mode] = reqs
            row["scalar_results_equal"] = bool(all(a.result == b.result for a, b in zip(runs["plain"], runs["served"])
                                                   if a.kind in ("dot", "filter_len")))
            out.append(row)
            del runs
        bound = spec["p99_bound_ms"]

        def knee(mode):
            ok = [r for r in out if r[mode]["p99_ms"] <= bound]
            return max(ok, key=lambda r: r[mode]["req_per_s"]) if ok else None

        kp, ks = knee("plain"), knee("served")
        at = {"p99_bound_ms": bound, "plain_req_per_s": kp["plain"]["req_per_s"] if kp else None,
              "served_req_per_s": ks["served"]["req_per_s"] if ks else None,
              "plain_gpu_busy_at_knee": kp["plain"]["gpu_busy"] if kp else None}
        if at["plain_req_per_s"] and at["served_req_per_s"]:
            at["ratio"] = round(at["served_req_per_s"] / at["plain_req_per_s"], 2)
        result[mix] = {"at_equal_p99": at,
                       "workload": "%d requests per rate and path, kinds uniform over dot_f64 / filter_gt_f64+length "
                                   "/ argsort_i64 / group-by sum, n = floor(10^U) with U uniform in [%g, %g], seeded "
                                   "inputs generated on the device; server: %d streams, requests up to 2^20 rows "
                                   "coalesced per kind, 150 GB admission budget"
                                   % (count, np.log10(spec["n_lo"]), np.log10(spec["n_hi"]), slots),
                       "rates": out}
    for w in workers:
        w.close()
    return result


# ---------------------------------------------------------------------------- e2e


# The order in which the e2e step uploads its inputs: the inputs of the calls whose results
# come back to the host first, so that downloads start while the other inputs still arrive.
E2E_UPLOADS = ["x", "v", "src", "idx", "y"]


class HostInputs:
    """The step's inputs in pinned host memory, and one pinned host buffer per array result
    (downloads of different results are in flight together)."""

    def __init__(self, ctx, inputs, n):
        import torch

        self.n = n
        self.host = {}
        for name in E2E_UPLOADS:
            arr = inputs[name]
            t = torch.empty(n, dtype=torch.float64 if arr.type == "f64" else torch.int64, pin_memory=True)
            ctx.download_ptr(arr, t.data_ptr(), n)
            self.host[name] = (t, arr.type)
        outs = sum(1 for _, kernel, _, _, _ in sweep_plan(n) if kernel in ARRAY_RESULTS)
        self.out = [torch.empty(n, dtype=torch.int64, pin_memory=True) for _ in range(outs)]

    def upload(self, ctx):
        """Starts every upload (each a copy on the library's upload stream; a call that reads an
        input waits for that input only)."""
        return {name: ctx.upload_ptr(t.data_ptr(), self.n, ty) for name, (t, ty) in self.host.items()}


# Sweep calls whose result is an array (downloaded in the e2e step); mul_f64's product only
# feeds the next call.
ARRAY_RESULTS = ("filter_gt_f64", "gather_i64", "scan_add_i64")


def e2e_order(plan):
    """The sweep's calls, each once, ordered by the arrival of their last input (stable)."""
    last = {name: i for i, name in enumerate(E2E_UPLOADS)}
    return sorted(plan, key=lambda call: max(last.get(a, len(E2E_UPLOADS)) for a in call[2]))


def run_e2e_step(ctx, n, hin):
    """Upload the inputs from pinned host memory, run the sweep, download the array results,
    through the library's public calls: uploads and downloads run on its copy streams and
    overlap each other and the kernels. Returns (seconds, h2d bytes, d2h bytes)."""
    t0 = time.perf_counter()
    inputs = hin.upload(ctx)
    h2d = sum(8 * n for _ in inputs)
    env = dict(inputs)
    d2h = 0
    copies = []
    for label, kernel, names, extra, _ in e2e_order(sweep_plan(n)):
        out = ctx.call(kernel, *[env[a] for a in names], *extra)
        if kernel == "mul_f64":
            env["xy"] = out
        if hasattr(out, "handle"):
            if kernel in ARRAY_RESULTS:
                copies.append(ctx.download_start(out, hin.out[len(copies)].data_ptr(), n))
                d2h += 8 * len(out)
        else:
            d2h += 8  # the scalar result
    for c in copies:
        c.wait()
    ctx.synchronize()
    return time.perf_counter() - t0, h2d, d2h


# ---------------------------------------------------------------------------- CPU baseline


def cpu_baseline(n_sample, budget_s=12.0, barrier=None):
    """Times the oracle port of the reference's scalar entries (one thread, as each of the
    reference's kernels runs) over the same sweep at a sample size. Returns (GB/s, passes).
    With `barrier`, the timing starts when every replica process has its inputs."""
    import oracle

    x, y = oracle.rand_f64(n_sample, 1), oracle.rand_f64(n_sample, 2)
    src = oracle.rand_i64(n_sample, 3)
    idx = (oracle.rand_i64(n_sample, 4) & (n_sample - 1)).astype(np.int64)
    v = (oracle.rand_i64(n_sample, 5) & ((1 << 21) - 1)) - (1 << 20)
    n = n_sample
    steps = [
        (lambda: oracle.reduce_add_f64(x), 8 * n),
        (lambda: oracle.dot_f64(x, y), 16 * n),
        (lambda: oracle.reduce_min_f64(x), 8 * n),
        (lambda: oracle.reduce_max_f64(x), 8 * n),
        (lambda: oracle.argmin_f64(x), 8 * n),
        (lambda: oracle.argmax_f64(x), 8 * n),
    ]
    for c in SELECTIVITY:
        steps.append((lambda c=c: oracle.count_cmp_f64(x, "gt", c), 8 * n))
    for c in SELECTIVITY:
        steps.append((lambda c=c: oracle.filter_cmp_f64(x, "gt", c), None))
    steps += [
        (lambda: oracle.gather(src, idx), 24 * n),
        (lambda: oracle.scan_add_i64(v), 16 * n),
        (lambda: oracle.reduce_add_f64(oracle.mul_f64(x, y)), 32 * n),
    ]
    total_b, total_t, passes = 0, 0.0, 0
    if barrier is not None:
        barrier.wait()
    t_start = time.perf_counter()
    while passes < 2 or (time.perf_counter() - t_start < budget_s and passes < 50):
        for fn, b in steps:
            t0 = time.perf_counter()
            r = fn()
            total_t += time.perf_counter() - t0
            total_b += b if b is not None else 8 * n + 8 * len(r)
        passes += 1
    return total_b / total_t / 1e9, passes


def _cpu_replica(n_sample, budget_s, barrier, results):
    sys.path.insert(0, ROOT)
    results.put(cpu_baseline(n_sample, budget_s, barrier))


def cpu_replicas(n_sample, budget_s, procs):
    """The oracle port on `procs` host processes at once, each over its own copy of the sample
    (the reference's programs are Send + Sync, so a host runs independent executions side by
    side). Returns (aggregate GB/s, total passes)."""
    if procs <= 1:
        return cpu_baseline(n_sample, budget_s)
    import multiprocessing

    mp = multiprocessing.get_context("spawn")
    barrier, results = mp.Barrier(procs), mp.Queue()
    ps = [mp.Process(target=_cpu_replica, args=(n_sample, budget_s, barrier, results)) for _ in range(procs)]
    for p in ps:
        p.start()
    got = [results.get(timeout=budget_s + 600) for _ in ps]
    for p in ps:
        p.join(timeout=60)
    return sum(g for g, _ in got), sum(k for _, k in got)


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------- main


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return world, rank, local


def reduce_max(value, world):
    """Max over ranks (the slowest replica sets the aggregate time)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def aggregate(bytes_per_step, steps, max_total_ms, world):
    """Whole-job GB/s: every replica moves bytes_per_step per step; the slowest sets the time."""
    return world * bytes_per_step * steps / (max_total_ms / 1e3) / 1e9


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=1 << 28)
    ap.add_argument("--e2e-steps", type=int, default=9)
    ap.add_argument("--cpu-sample", type=int, default=1 << 23)
    ap.add_argument("--cpu-procs", type=int, default=0,
                    help="host processes of the reference arm (0: every core this process may use)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--sort-n", type=int, default=1 << 27, help="0 skips the argsort/group-by section")
    ap.add_argument("--scan-n", type=int, default=1 << 28, help="0 skips the float scan section")
    ap.add_argument("--region-n", type=int, default=1 << 28, help="0 skips the region section")
    ap.add_argument("--hard-sizes", default="26,28",
                    help="log2 sizes of the canonical sums on hard inputs (empty skips the section)")
    ap.add_argument("--batch-arrays", type=int, default=4096, help="0 skips the batched section")
    ap.add_argument("--serve-requests", type=int, default=3000,
                    help="requests per rate and path in the served section (0 skips it)")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    n = args.n
    config = {"workload": "primitive sweep, n=2^%d rows per array (f64 uniform [0,1), i64 gather "
                          "indices uniform in [0,n), i64 scan values uniform in [-2^20,2^20))"
                          % (n.bit_length() - 1),
              "n": n, "kernels": [p[0] for p in sweep_plan(n)],
              "l2": "inputs larger than L2 (2 GiB arrays), no flush",
              "parallelism": "replicas" if world > 1 else "single GPU"}

    if args.impl == "reference":
        if rank != 0:
            return
        procs = args.cpu_procs or host_cores()
        gbs, passes = cpu_replicas(args.cpu_sample, max(3.0, 2.0 * args.steps), procs)
        sample = ("oracle port of the scalar entries, sweep at n=2^%d, %d processes side by side (one per "
                  "host core, each its own copy of the sample), %d passes in all" % (
                      args.cpu_sample.bit_length() - 1, procs, passes))
        # What this arm ran: the same kernels and data distributions, at the sample size, as
        # independent replicas on every host core.
        config = dict(config, n=args.cpu_sample, processes=procs,
                      workload="primitive sweep (the GPU arm's kernels and distributions) at n=2^%d rows "
                               "per array, %d independent host processes" % (
                                   args.cpu_sample.bit_length() - 1, procs),
                      gpu_arm_n=n)
        line = {"impl": "reference", "metric": METRIC, "value": round(gbs, 3), "unit": UNIT,
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64+i64",
                "data": "synthetic (seeded rand_f64/rand_i64, the reference generators)",
                "config": config,
                "cpu_baseline": {"value": round(gbs, 3), "unit": UNIT, "cores": procs, "kind": "port",
                                 "sample": sample},
                "e2e": {"value": round(gbs, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch

    import verkehrt_gb300 as vk
    from verkehrt_gb300 import build as vbuild

    vbuild.build()
    torch.cuda.set_device(local)
    ctx = vk.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    events = {"stream": stream}
    inputs = make_inputs(ctx, n)

    for _ in range(args.warmup):
        _, _, res = run_step(ctx, n, inputs, events)
        check_results(res)

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(1.0)  # nvidia-smi's start-up stalls the GPU briefly: keep it out of the timed steps
    barrier(world)
    launches0 = ctx.launch_count()
    per_label = {}
    step_ms = []
    for _ in range(args.steps):
        per, ms, res = run_step(ctx, n, inputs, events)
        step_ms.append(ms)
        for label, (t, b) in per.items():
            acc = per_label.setdefault(label, [0.0, 0, 0])
            acc[0] += t
            acc[1] += b
            acc[2] += 1
    launches = ctx.launch_count() - launches0
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    check_results(res)

    bytes_per_step = sum(v[1] for v in per_label.values()) / args.steps
    total_ms = reduce_max(sum(step_ms), world)
    value = aggregate(bytes_per_step, args.steps, total_ms, world)

    # Dominant kernel: the largest share of the step's kernel time.
    dom = max(per_label, key=lambda k: per_label[k][0])
    dom_ms = per_label[dom][0] / per_label[dom][2]
    dom_bytes = per_label[dom][1] / per_label[dom][2]
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = committed_traffic().get(dom.split("@")[0])
    kernels = {k: {"ms": round(v[0] / v[2], 4), "GB/s": round(v[1] / v[2] / (v[0] / v[2] / 1e3) / 1e9, 1),
                   "frac": round(v[1] / v[2] / (v[0] / v[2] / 1e3) / 1e9 / peak, 3)}
               for k, v in per_label.items()}

    # e2e through the C ABI with pinned host buffers, after two untimed steps (measured on
    # GB300: the first two steps of a process take 98 and 78 ms, then every step 64 ms).
    hin = HostInputs(ctx, inputs, n)
    for _ in range(2):  # the copy streams, the device blocks and the first DMA to the host pages
        run_e2e_step(ctx, n, hin)
    e2e = []
    for _ in range(max(1, args.e2e_steps)):
        e2e.append(run_e2e_step(ctx, n, hin))
    # The median step (max over ranks): the host link of a shared machine is not always quiet,
    # and one step that waited on another tenant's copies would otherwise set the figure.
    e2e_s = reduce_max(float(np.median([t for t, _, _ in e2e])), world)
    e2e_value = world * bytes_per_step / e2e_s / 1e9

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        gbs, passes = cpu_baseline(args.cpu_sample)
        cpu = {"value": round(gbs, 3), "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "oracle port of the scalar entries (one thread, as the reference), the sweep "
                         "at n=2^%d, %d passes" % (args.cpu_sample.bit_length() - 1, passes)}

    # The last timed step's outputs against the oracle's digests (after every timed leg: the check
    # downloads and hashes the outputs on the host).
    digests = committed_digests()
    sweep_parity = check_digests(res, digests.get("sweep", {}).get("outputs"), n,
                                 digests.get("sweep", {}).get("n"))

    # Argsort and group-by, batched statements and served requests, reported beside the headline sweep.
    c3 = None
    del inputs, hin, res
    if args.sort_n > 0:
        c3 = run_sort_groupby(ctx, args.sort_n, stream, steps=3, warmup=1,
                              digests=digests.get("sort_groupby"))
    c6 = run_f64_scans(ctx, args.scan_n, stream) if args.scan_n > 0 else None
    c8 = run_regions(ctx, args.region_n, stream) if args.region_n > 0 else None
    hard = [1 << int(v) for v in args.hard_sizes.split(",") if v.strip()]
    c7 = run_canon_adversarial(ctx, hard, stream, no_cpu=args.no_cpu or rank != 0) if hard else None
    c4 = run_batched(ctx, args.batch_arrays) if args.batch_arrays > 0 else None
    # The configuration's other reading: its length range [2^10, 2^24] taken literally, with fewer
    # arrays (512, about 14 GiB of values and keys) so that the inputs and the sort's scratch fit.
    c4w = run_batched(ctx, 512, lo=10, hi=24) if args.batch_arrays > 0 else None
    c5 = run_served(ctx, count=args.serve_requests) if args.serve_requests > 0 else None

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+i64",
            "data": "synthetic (seeded rand_f64/rand_i64 generated on device, the reference generators)",
            "config": config,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1),
                         "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "traffic": traffic, "peak_kind": peak_kind},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "statistic": "median of %d steps" % len(e2e),
                    "step_ms": [round(t * 1e3, 1) for t, _, _ in e2e],
                    "h2d_bytes_per_step": e2e[0][1], "d2h_bytes_per_step": e2e[0][2]},
            "clocks": clk,
            "gpu_launches": launches,
            "parity_checked": sweep_parity["parity_checked"],
            "parity": sweep_parity,
            "kernels": kernels,
            "sort_groupby": c3,
            "f64_scans": c6,
            "regions": c8,
            "canon_adversarial": c7,
            "batched": c4,
            "batched_wide": c4w,
            "served": c5,
        }
        print(json.dumps(line), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()

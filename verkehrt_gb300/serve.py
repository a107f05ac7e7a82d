"""Serving: verkehrt programs answered as they arrive, with continuous batching on one GPU.

The reference answers one program at a time (Prepared::execute, src/interp.rs:446-516): each
statement runs to completion before the next. Here requests arrive on their own clock and a
server keeps the GPU busy with them:

* every worker owns a context (its own CUDA stream and allocator cache), so the work of
  different workers overlaps on the device;
* a worker that frees up takes the oldest waiting request's kind and coalesces every waiting
  small request of that kind into one batched launch (vkc_batch_*, the requests' generator
  statements included), as long as the group fits
  the free part of the device-memory budget; a large request runs alone through the plain
  entries;
* admission: a request is only started when the bytes it holds at its peak fit the budget left
  by the requests in flight, so the server never oversubscribes HBM;
* inputs are generated on the device and results stay there (arrays) unless they are scalars.

A request's result is the same whether it ran alone or in a mix: every entry used is
deterministic and bit-exact (the canonical sums, counts, stable argsort, first-occurrence
group ids), so tests compare the two exactly.

Program kinds (the served mix): dot (x = rand_f64(n, s); y = rand_f64(n, s + 1); dot_f64),
filter_len (length(filter_gt_f64(rand_f64(n, s), 0.9))), argsort (argsort_i64(rand_i64(n, s))),
group_sum (group-by sum of i64 values over keys below 2^16: group_id_i64, reduce_into_add_i64).

group_sum has no batched entry of its own: a group of them runs as one statement over the
concatenated keys (vkc_batch_concat), keyed by (request, key) with group_id2, so each request's
groups get consecutive ids in its own first-occurrence order, offset by the groups of the
requests before it; one reduce_into sums them all and each request's result is its slice.
"""

import collections
import threading
import time

import numpy as np

KINDS = ("dot", "filter_len", "argsort", "group_sum")
BATCHED = KINDS  # kinds that coalesce (group_sum through a concatenation)
THRESHOLD = 0.9
KEY_MASK = (1 << 16) - 1


class Request:
    """One program to answer: kind, rows, seed, arrival time (seconds from the run's start)."""

    __slots__ = ("rid", "kind", "n", "seed", "arrival", "start", "done", "result", "batched")

    def __init__(self, rid, kind, n, seed, arrival=0.0):
        self.rid, self.kind, self.n, self.seed, self.arrival = rid, kind, int(n), int(seed), arrival
        self.start = self.done = None
        self.result = None
        self.batched = False

    @property
    def latency(self):
        return self.done - self.arrival


def request_bytes(kind, n):
    """Device bytes a request holds at its peak (inputs, outputs and scratch), for admission."""
    if kind == "dot":
        return 16 * n
    if kind == "filter_len":
        return 16 * n
    if kind == "argsort":
        return 48 * n
    slots = 2
    while slots < 2 * n:
        slots <<= 1
    return 40 * n + 24 * slots


def poisson_requests(count, rate, seed=1, n_lo=1e3, n_hi=1e8, kinds=KINDS):
    """`count` requests with exponential gaps of mean 1/rate, kinds uniform, n = floor(10^U) with
    U uniform in [log10 n_lo, log10 n_hi] (a seeded numpy stream)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, count)
    arrivals = np.cumsum(gaps) - gaps[0]
    ns = np.floor(10.0 ** rng.uniform(np.log10(n_lo), np.log10(n_hi), count)).astype(np.int64)
    ks = rng.integers(0, len(kinds), count)
    return [Request(i, kinds[ks[i]], ns[i], 1000 + 7 * i, arrivals[i]) for i in range(count)]


# ---------------------------------------------------------------------------- execution


def run_one(ctx, r):
    """The plain per-statement GPU path for one request (each entry returns when done)."""
    n, s = r.n, r.seed
    if r.kind == "dot":
        r.result = ctx.call("dot_f64", ctx.call("rand_f64", n, s), ctx.call("rand_f64", n, s + 1), raw=True)[2]
    elif r.kind == "filter_len":
        r.result = len(ctx.call("filter_gt_f64", ctx.call("rand_f64", n, s), THRESHOLD))
    elif r.kind == "argsort":
        r.result = ctx.call("argsort_i64", ctx.call("rand_i64", n, s))
    else:
        keys = ctx.call("and_i64", ctx.call("rand_i64", n, s), KEY_MASK)
        vals = ctx.call("and_i64", ctx.call("rand_i64", n, s + 1), KEY_MASK)
        g = ctx.call("group_id_i64", keys)
        nb = ctx.call("reduce_max_i64", g) + 1 if n else 0
        r.result = ctx.call("reduce_into_add_i64", g, vals, nb)
    ctx.synchronize()


def run_batch(ctx, reqs):
    """Same-kind requests as one batched launch; their generator statements are batched too
    (vkc_batch_rand: one launch for every request's rand call, each array that call's)."""
    kind = reqs[0].kind
    lens = [r.n for r in reqs]
    seeds = [r.seed for r in reqs]
    seeds1 = [r.seed + 1 for r in reqs]
    if kind == "dot":
        xs = ctx.batch_rand("f64", lens, seeds)
        ys = ctx.batch_rand("f64", lens, seeds1)
        sums = ctx.new_array("f64", len(reqs))
        ctx.batch_dot(ctx.batch(xs), ctx.batch(ys), sums)
        out = sums.numpy().view(np.uint64)
        for r, v in zip(reqs, out):
            r.result = int(v)
    elif kind == "filter_len":
        xs = ctx.batch_rand("f64", lens, seeds)
        counts = ctx.new_array("i64", len(reqs))
        ctx.batch_count(ctx.batch(xs), "gt", THRESHOLD, counts)
        for r, v in zip(reqs, counts.numpy()):
            r.result = int(v)
    elif kind == "argsort":
        ks = ctx.batch_rand("i64", lens, seeds)
        outs = [ctx.new_array("i64", r.n) for r in reqs]
        ctx.batch_argsort(ctx.batch(ks), ctx.batch(outs))
        for r, o in zip(reqs, outs):
            r.result = o
    else:
        # The masks apply row by row, so they run once over the concatenations.
        kraw, index = ctx.batch_concat(ctx.batch(ctx.batch_rand("i64", lens, seeds)))
        vraw = ctx.batch_concat(ctx.batch(ctx.batch_rand("i64", lens, seeds1)), index=False)
        kcat = ctx.call("and_i64", kraw, KEY_MASK)
        vcat = ctx.call("and_i64", vraw, KEY_MASK)
        g = ctx.call("group_id2_i64_i64", index, kcat)
        nb = ctx.call("reduce_max_i64", g) + 1 if len(g) else 0
        sums = ctx.call("reduce_into_add_i64", g, vcat, nb)
        # The first group id of every request with rows (ids are consecutive per request).
        starts = np.cumsum([0] + [r.n for r in reqs[:-1]])
        live = [i for i, r in enumerate(reqs) if r.n > 0]
        first = ctx.call("gather_i64", g, ctx.upload(starts[live].astype(np.int64))).numpy() if live else []
        bounds = dict(zip(live, first))
        ends = list(first[1:]) + [nb]
        for j, i in enumerate(live):
            reqs[i].result = sums.slice(int(bounds[i]), int(ends[j]))
        for r in reqs:
            if r.n == 0:
                r.result = sums.slice(0, 0)
    ctx.synchronize()
    for r in reqs:
        r.batched = True


# ---------------------------------------------------------------------------- scheduling


class Scheduler:
    """Admission and coalescing, independent of the device (unit-tested on the CPU).

    take() hands a worker the next group: the oldest waiting request's kind; if that request is
    small and its kind has a batched entry, every waiting small request of the kind, oldest
    first, up to `max_group` and within the free budget; otherwise that request alone. A request
    larger than the whole budget is admitted alone when nothing else is in flight."""

    def __init__(self, budget, small_rows=1 << 20, max_group=512, batching=True):
        self.budget, self.small_rows, self.max_group, self.batching = budget, small_rows, max_group, batching
        self.pending = collections.deque()
        self.in_flight = 0
        self.closed = False
        self.cv = threading.Condition()

    def submit(self, r):
        with self.cv:
            self.pending.append(r)
            self.cv.notify_all()

    def close(self):
        with self.cv:
            self.closed = True
            self.cv.notify_all()

    def _group(self):
        if not self.pending:
            return None
        head = self.pending[0]
        free = self.budget - self.in_flight
        need = request_bytes(head.kind, head.n)
        if need > free and not (self.in_flight == 0 and need > self.budget):
            return None
        small = head.n <= self.small_rows and head.kind in BATCHED and self.batching
        if not small:
            self.pending.popleft()
            return [head], need
        group, used = [], 0
        keep = collections.deque()
        while self.pending:
            r = self.pending.popleft()
            b = request_bytes(r.kind, r.n)
            if (r.kind == head.kind and r.n <= self.small_rows and len(group) < self.max_group
                    and used + b <= max(free, need)):
                group.append(r)
                used += b
            else:
                keep.append(r)
        self.pending = keep
        return group, used

    def take(self):
        """The next group and its bytes, or None once closed and drained (blocks meanwhile)."""
        with self.cv:
            while True:
                g = self._group()
                if g is not None:
                    self.in_flight += g[1]
                    return g
                if self.closed and not self.pending:
                    return None
                self.cv.wait()

    def release(self, nbytes):
        with self.cv:
            self.in_flight -= nbytes
            self.cv.notify_all()


def serve(contexts, requests, budget=150e9, small_rows=1 << 20, batching=True, device_ms=None):
    """Answers `requests` (sorted by arrival), released at their arrival times from now on, with
    one worker per context. Returns the wall time from the first arrival to the last answer.
    With a list `device_ms`, every group appends the time its context's stream took for it
    (CUDA events around the group): the sum over the wall time is the share of the run that the
    device spent on requests."""
    sched = Scheduler(budget, small_rows, batching=batching)
    t0 = time.perf_counter()
    errors = []

    def worker(ctx):
        try:
            while True:
                g = sched.take()
                if g is None:
                    return
                group, nbytes = g
                now = time.perf_counter() - t0
                for r in group:
                    r.start = now
                try:
                    if device_ms is not None:
                        ctx.timer_start()
                    if len(group) > 1:
                        run_batch(ctx, group)
                    else:
                        run_one(ctx, group[0])
                    if device_ms is not None:
                        device_ms.append(ctx.timer_stop())
                finally:
                    done = time.perf_counter() - t0
                    for r in group:
                        r.done = done
                    sched.release(nbytes)
        except Exception as e:  # surfaced after the run
            errors.append(e)
            sched.close()

    threads = [threading.Thread(target=worker, args=(c,), daemon=True) for c in contexts]
    for t in threads:
        t.start()
    for r in requests:
        delay = r.arrival - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        sched.submit(r)
    sched.close()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return max(r.done for r in requests) if requests else 0.0


def summary(requests, wall):
    lat = np.array([r.latency for r in requests]) * 1e3
    return {"requests": len(requests), "wall_s": round(wall, 4),
            "req_per_s": round(len(requests) / wall, 1) if wall > 0 else None,
            "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
            "batched_fraction": round(sum(r.batched for r in requests) / max(1, len(requests)), 3)}

"""The serving loop: admission and coalescing (CPU, with fake executors), and on the GPU, every
request's result is the same alone and in a concurrent, coalesced mix."""

import threading
import time

import numpy as np
import pytest

from verkehrt_gb300 import serve
from verkehrt_gb300.serve import Request, Scheduler, request_bytes


def test_scheduler_coalesces_the_head_kind():
    s = Scheduler(budget=1e12, small_rows=1000)
    for i, (k, n) in enumerate([("dot", 10), ("argsort", 10), ("dot", 20), ("group_sum", 5), ("dot", 5000), ("dot", 30)]):
        s.submit(Request(i, k, n, i))
    group, nbytes = s.take()
    assert [r.rid for r in group] == [0, 2, 5]  # the small dots, oldest first; the large one waits
    assert nbytes == sum(request_bytes("dot", n) for n in (10, 20, 30))
    group, _ = s.take()
    assert [r.rid for r in group] == [1]  # argsort, alone in the queue
    group, _ = s.take()
    assert [r.rid for r in group] == [3]  # group_sum, alone in the queue
    group, _ = s.take()
    assert [r.rid for r in group] == [4]  # large: alone


def test_scheduler_admission_budget():
    s = Scheduler(budget=request_bytes("dot", 100) * 2, small_rows=1000)
    for i in range(5):
        s.submit(Request(i, "dot", 100, i))
    group, nbytes = s.take()
    assert len(group) == 2 and nbytes == request_bytes("dot", 100) * 2  # fills the budget
    got = []
    t = threading.Thread(target=lambda: got.append(s.take()))
    t.start()
    time.sleep(0.05)
    assert not got  # nothing fits until bytes come back
    s.release(nbytes)
    t.join(timeout=5)
    assert len(got[0][0]) == 2
    # A request larger than the whole budget runs alone once nothing is in flight.
    s2 = Scheduler(budget=10, small_rows=0)
    s2.submit(Request(0, "argsort", 1000, 0))
    assert [r.rid for r in s2.take()[0]] == [0]


def test_scheduler_without_batching_is_fifo():
    s = Scheduler(budget=1e12, batching=False)
    for i, k in enumerate(["dot", "dot", "argsort"]):
        s.submit(Request(i, k, 10, i))
    assert [s.take()[0][0].rid for _ in range(3)] == [0, 1, 2]


def test_serve_completes_every_request(monkeypatch):
    calls = []

    def one(ctx, r):
        time.sleep(0.001)
        r.result = ("one", r.rid)
        calls.append((ctx, [r.rid]))

    def batch(ctx, reqs):
        time.sleep(0.001)
        for r in reqs:
            r.result = ("batch", r.rid)
            r.batched = True
        calls.append((ctx, [r.rid for r in reqs]))

    monkeypatch.setattr(serve, "run_one", one)
    monkeypatch.setattr(serve, "run_batch", batch)
    reqs = serve.poisson_requests(200, rate=5000, seed=3, n_lo=1e3, n_hi=1e7)
    wall = serve.serve(["c0", "c1", "c2"], reqs, budget=1e12, small_rows=1 << 20)
    assert wall > 0 and all(r.done is not None and r.done >= r.arrival for r in reqs)
    assert sorted(rid for _, ids in calls for rid in ids) == list(range(200))
    assert any(len(ids) > 1 for _, ids in calls)  # coalesced
    assert {c for c, _ in calls} == {"c0", "c1", "c2"}  # every worker took work
    s = serve.summary(reqs, wall)
    assert s["requests"] == 200 and s["p50_ms"] <= s["p99_ms"]


def _value(r):
    if r.kind in ("argsort", "group_sum"):
        return r.result.numpy().tobytes()
    return r.result


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix(ctx):
    import verkehrt_gb300 as vk

    mix = serve.poisson_requests(48, rate=20_000, seed=11, n_lo=1e3, n_hi=3e5)
    alone = [Request(r.rid, r.kind, r.n, r.seed) for r in mix]
    for r in alone:
        serve.run_one(ctx, r)
    workers = [vk.Context(0) for _ in range(3)]
    serve.serve(workers, mix, budget=150e9, small_rows=1 << 20)
    assert sum(r.batched for r in mix) > 0  # small requests of one kind were coalesced
    for a, m in zip(alone, mix):
        assert _value(a) == _value(m), (a.kind, a.n)


@pytest.mark.gpu
def test_batched_group_sums_equal_the_plain_ones(ctx):
    # Requests of different sizes, one empty, coalesced through the concatenation.
    reqs = [Request(i, "group_sum", n, 500 + 3 * i) for i, n in enumerate([1000, 1, 70_000, 0, 4097, 65_536 * 3])]
    alone = [Request(r.rid, r.kind, r.n, r.seed) for r in reqs]
    for r in alone:
        serve.run_one(ctx, r)
    serve.run_batch(ctx, reqs)
    for a, b in zip(alone, reqs):
        assert b.batched
        assert np.array_equal(a.result.numpy(), b.result.numpy()), a.n
    # Batched generators equal their own calls.
    lens, seeds = [0, 1, 5, 1000, 70_001], [3, 4, 5, 6, 7]
    for t in ("f64", "i64"):
        got = ctx.batch_rand(t, lens, seeds)
        for a, n, sd in zip(got, lens, seeds):
            assert np.array_equal(a.numpy(), ctx.call("rand_" + t, n, sd).numpy())
    # The concatenation and its index column.
    arrays = [ctx.upload(np.arange(k, dtype=np.int64) * 3) for k in (5, 0, 3)]
    rows, index = ctx.batch_concat(ctx.batch(arrays))
    assert list(rows.numpy()) == [0, 3, 6, 9, 12, 0, 3, 6]
    assert list(index.numpy()) == [0, 0, 0, 0, 0, 2, 2, 2]
    big = [ctx.upload(np.full(n, i, np.uint8)) for i, n in enumerate([20_000, 8192, 8193, 1])]
    rows = ctx.batch_concat(ctx.batch(big), index=False)
    assert np.array_equal(rows.numpy(), np.concatenate([np.full(n, i, np.uint8) for i, n in enumerate([20_000, 8192, 8193, 1])]))
    # Four-byte rows, views that start inside their arrays, and an empty batch.
    src = np.arange(50_000, dtype=np.int32) * 7 - 3
    whole = ctx.upload(src)
    views = [whole.slice(5, 20_005), whole.slice(1, 2), whole.slice(30_000, 49_999)]
    rows, index = ctx.batch_concat(ctx.batch(views))
    assert np.array_equal(rows.numpy(), np.concatenate([src[5:20_005], src[1:2], src[30_000:49_999]]))
    assert np.array_equal(index.numpy(), np.repeat(np.arange(3), [20_000, 1, 19_999]))
    rows, index = ctx.batch_concat(ctx.batch([]))
    assert len(rows) == 0 and len(index) == 0

"""argsort_i64 and group_id on the GPU equal the oracle (src/kernels/scalar/index/tests.rs and
src/kernels/scalar/group/tests.rs input classes)."""

import numpy as np
import pytest

import oracle
from helpers import LENGTHS

pytestmark = pytest.mark.gpu

I64_MIN, I64_MAX = -2**63, 2**63 - 1


def boundary_pool():
    """Values at and around every digit boundary, and their negatives (index/tests.rs:73-91)."""
    raw = [0, 1]
    for k in range(8):
        raw += [1 << (8 * k), (1 << (8 * k)) - 1]
    for k in range(6):
        raw += [(1 << (11 * k)) + 1, (1 << (11 * k)) - 1]
    raw += [(-v) & 0xFFFFFFFFFFFFFFFF for v in raw]
    return np.array(raw, dtype=np.uint64).view(np.int64)


def classes(n, seed):
    r = oracle.rand_i64(n, seed)
    u = r.view(np.uint64)
    pick = lambda pool: pool[(u % np.uint64(len(pool))).astype(np.int64)]
    base = np.uint64(oracle.splitmix64(seed))
    k = seed % 8
    return {
        "few": pick(oracle.rand_i64(3, seed + 1)),
        "extreme": pick(np.array([I64_MIN, I64_MAX, -1, 0, 1], dtype=np.int64)),
        "sorted": np.sort(r),
        "reversed": np.sort(r)[::-1].copy(),
        "random": r,
        "small": (u % np.uint64(300)).astype(np.int64),
        "small_signed": (u % np.uint64(600)).astype(np.int64) - 300,
        "one_byte": (base ^ ((u & np.uint64(0xFF)) << np.uint64(8 * k))).view(np.int64),
        "boundary": pick(boundary_pool()),
        "u32": (u >> np.uint64(32)).astype(np.int64),
    }


def test_argsort_classes(ctx):
    for n in LENGTHS + [1023, 1024, 1025, 2047, 2048, 2049, 4095, 4096, 4097, 5000, 8191, 8192, 8193, 70_001]:
        for name, xs in classes(n, n + 7).items():
            got = ctx.call("argsort_i64", ctx.upload(xs)).numpy()
            assert np.array_equal(got, oracle.argsort_i64(xs)), (name, n)


def test_argsort_reference_vectors(ctx):
    # index/tests.rs:246-266
    i64s = np.array([I64_MAX, 0, I64_MIN, -1, I64_MAX, I64_MIN, 0, -1])
    assert list(ctx.call("argsort_i64", ctx.upload(i64s)).numpy()) == [2, 5, 3, 7, 1, 6, 0, 4]
    near64 = np.array([0xFE, -2, I64_MIN + 1, 1, I64_MAX, -1, 0xFF, I64_MIN])
    assert list(ctx.call("argsort_i64", ctx.upload(near64)).numpy()) == [7, 2, 1, 5, 3, 0, 6, 4]
    # :268-280: all equal rows give the identity (every digit constant, no pass runs).
    n = 100_000
    assert np.array_equal(ctx.call("argsort_i64", ctx.upload(np.full(n, -1))).numpy(), np.arange(n))
    # :304-321: exactly two active digits.
    h = np.array([oracle.splitmix64(i) for i in range(2000)], dtype=np.uint64)
    xs = (np.uint64(0x0101010101010101) ^ (h % np.uint64(16)) ^
          (((h >> np.uint64(8)) % np.uint64(16)) << np.uint64(24))).view(np.int64)
    assert np.array_equal(ctx.call("argsort_i64", ctx.upload(xs)).numpy(), oracle.argsort_reference_i64(xs))


def test_argsort_large(ctx):
    n = 1 << 22
    u32 = (oracle.rand_i64(n, 3).view(np.uint64) >> np.uint64(32)).astype(np.int64)
    got = ctx.call("argsort_i64", ctx.upload(u32)).numpy()
    assert np.array_equal(got, np.argsort(u32, kind="stable"))
    r = oracle.rand_i64(n, 4)
    assert np.array_equal(ctx.call("argsort_i64", ctx.upload(r)).numpy(), np.argsort(r, kind="stable"))


def first_occurrence(keys):
    seen = {}
    return np.array([seen.setdefault(k, len(seen)) for k in keys], dtype=np.int64)


def test_group_id_classes(ctx):
    for n in LENGTHS + [4097, 5000, 70_001]:
        for name, xs in classes(n, n + 11).items():
            got = ctx.call("group_id_i64", ctx.upload(xs)).numpy()
            assert np.array_equal(got, oracle.group_id_i64(xs)), (name, n)


def test_group_id_vectors(ctx):
    # tests/programs/grouping.dd
    assert list(ctx.call("group_id_i64", ctx.upload(np.array([7, -1, 7, 3, -1, 7]))).numpy()) == [0, 1, 0, 2, 1, 0]
    got = ctx.call("group_id2_i64_i64", ctx.upload(np.array([1, 2, 1, 2])), ctx.upload(np.array([2, 1, 2, 2])))
    assert list(got.numpy()) == [0, 1, 0, 2]
    with pytest.raises(Exception, match="^length mismatch: 2 vs 1$"):
        ctx.call("group_id2_i64_i64", ctx.upload(np.array([1, 2])), ctx.upload(np.array([1])))


def test_group_id2_classes(ctx):
    for n in (0, 1, 17, 300, 5000, 70_001):
        a = (oracle.rand_i64(n, n).view(np.uint64) % np.uint64(40)).astype(np.int64)
        b = (oracle.rand_i64(n, n + 1).view(np.uint64) % np.uint64(30)).astype(np.int64) - 15
        got = ctx.call("group_id2_i64_i64", ctx.upload(a), ctx.upload(b)).numpy()
        assert np.array_equal(got, oracle.group_id2_i64_i64(a, b)), n


def test_group_id_large(ctx):
    n = 1 << 22
    for mod in (1 << 16, 1 << 40):
        xs = (oracle.rand_i64(n, 5).view(np.uint64) % np.uint64(mod)).astype(np.int64)
        got = ctx.call("group_id_i64", ctx.upload(xs)).numpy()
        assert np.array_equal(got, oracle.group_id_i64(xs)), mod


def test_group_id_region_partitioned(ctx):
    # Many distinct single keys on 2^22 rows or more take the region-partitioned tables: keys
    # repeated far apart (first occurrences in earlier tiles), the free-slot pattern as a key,
    # one key in the first and the last row, and a ragged last tile.
    n = (1 << 23) + 77
    xs = (oracle.rand_i64(n, 15).view(np.uint64) % np.uint64(1 << 22)).astype(np.int64)
    empty = np.uint64(0x8080808080808080).view(np.int64)
    xs[[5, 70_000, 4_000_000, n - 2]] = empty
    xs[0] = xs[n - 1] = 123_456_789_012
    got = ctx.call("group_id_i64", ctx.upload(xs)).numpy()
    assert np.array_equal(got, oracle.group_id_i64(xs))
    u = oracle.rand_i64(1 << 22, 16)  # every key distinct (almost)
    assert np.array_equal(ctx.call("group_id_i64", ctx.upload(u)).numpy(), oracle.group_id_i64(u))


def test_group_id_free_slot_pattern_and_table_switch(ctx):
    # The key whose bytes are all 0x80 marks a free slot of the GPU table; rows holding it take
    # their own slot. Pairs with one such half probe like any other pair.
    e = np.uint64(0x8080808080808080).view(np.int64)
    xs = np.array([5, e, 5, e, -1, e, 0], dtype=np.int64)
    assert np.array_equal(ctx.call("group_id_i64", ctx.upload(xs)).numpy(), oracle.group_id_i64(xs))
    a = np.array([e, e, 1, e, e, 1, e], dtype=np.int64)
    b = np.array([e, 1, e, e, 1, e, 2], dtype=np.int64)
    got = ctx.call("group_id2_i64_i64", ctx.upload(a), ctx.upload(b)).numpy()
    assert np.array_equal(got, oracle.group_id2_i64_i64(a, b))
    # Above 2^20 rows: few keys stay in the small table; about 2^20 distinct keys (the small
    # table's limit) and many distinct pairs move to the full table part-way.
    n = (1 << 21) + 5
    r = oracle.rand_i64(n, 21).view(np.uint64)
    for mod in (1000, (1 << 20) - 3, (1 << 20) + 3):
        xs = (r % np.uint64(mod)).astype(np.int64)
        xs[::4097] = e
        got = ctx.call("group_id_i64", ctx.upload(xs)).numpy()
        assert np.array_equal(got, oracle.group_id_i64(xs)), mod
    for mod in (50, 1 << 12):
        a = (r % np.uint64(mod)).astype(np.int64)
        b = ((r >> np.uint64(20)) % np.uint64(mod)).astype(np.int64)
        a[::999] = e
        got = ctx.call("group_id2_i64_i64", ctx.upload(a), ctx.upload(b)).numpy()
        assert np.array_equal(got, oracle.group_id2_i64_i64(a, b)), mod

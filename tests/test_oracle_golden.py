"""Pins the CPU oracle to the reference's own golden vectors and known answers, before any
GPU comparison trusts it. Sources are files of antiguru/verkehrt."""

import numpy as np
import pytest

import oracle
from oracle import OracleError


def bits(x):
    return int(np.float64(x).view(np.uint64))


def test_splitmix_and_rand():
    # src/kernels/tests.rs:1167-1181
    assert oracle.splitmix64(0) == 0xE220A8397B1DCDAF
    assert oracle.rand_i64(3, 7)[1] == np.int64(np.uint64(oracle.splitmix64(8)).view(np.int64))
    r = oracle.rand_f64(1000, 1)
    assert np.all((r >= 0.0) & (r < 1.0))
    assert bits(r[0]) == bits((oracle.splitmix64(1) >> 11) * 2.0 ** -53)
    # tests/programs/random.dd:4-9
    assert list(oracle.rand_i64(2, 0)) == [-2152535657050944081, -7995527694508729151]
    assert len(oracle.rand_f64(10, 1)) == 10


def varied(n):
    """src/kernels/tests.rs:664-673: data spanning magnitudes, so the order matters."""
    out = []
    for i in range(n):
        unit = (oracle.splitmix64(i) >> 11) * 2.0 ** -53
        out.append((unit - 0.5) * 10.0 ** ((i % 9) * 2))
    return np.array(out)


def reference_sum(xs):
    """src/kernels/tests.rs:676-696: the spec's order written bullet by bullet."""
    n = len(xs)
    b = n - n % 16
    acc = [0.0] * 16
    for j in range(16):
        i = j
        while i < b:
            acc[j] += xs[i]
            i += 16
    for step in (8, 4, 2, 1):
        for j in range(step):
            acc[j] += acc[j + step]
    for x in xs[b:]:
        acc[0] += x
    return acc[0]


def test_canonical_sum_follows_the_spec_order():
    # src/kernels/tests.rs:698-720
    xs = np.array([1e16 if i == 0 else (-1e16 if i == 16 else 1.0) for i in range(35)])
    assert bits(oracle.reduce_add_f64(xs)) == bits(reference_sum(xs))
    naive = 0.0
    for x in xs:
        naive += x
    assert bits(naive) != bits(reference_sum(xs))
    v = varied(35)
    assert bits(oracle.reduce_add_f64(v)) == bits(reference_sum(v))
    for n in (0, 1, 15, 16, 17, 63, 64, 65, 300, 1000):
        v = varied(n)
        assert bits(oracle.reduce_add_f64(v)) == bits(reference_sum(v)), n


def test_canonical_sum_golden_values():
    # src/kernels/tests.rs:761-791: the bits of the literal 50.16
    xs = np.array([
        1e16, 0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 1.1, 1.2, 1.3, 1.4, 1.5, 1.6,
        -1e16, 1.7, 1.8, 1.9, 2.1, 2.2, 2.3, 2.4, 2.5, 2.6, 2.7, 2.8, 2.9, 3.1, 3.2, 3.3,
        0.01, 0.02, 0.03])
    assert bits(oracle.reduce_add_f64(xs)) == 0x4049147AE147AE14
    naive = 0.0
    for x in xs:
        naive += x
    assert naive == 49.56


def test_canonical_empty_and_product():
    # src/kernels/tests.rs:722-727, :1000-1010
    assert bits(oracle.reduce_add_f64(np.array([]))) == bits(0.0)
    assert oracle.reduce_mul_f64(np.array([])) == 1.0
    assert oracle.reduce_mul_f64(np.array([2.0, 3.0, 4.0])) == 24.0


def test_fused_equals_unfused():
    # tests/fused_oracle.rs: dot == reduce_add(mul), bit for bit
    x, y = varied(1000), varied(1000)[::-1].copy()
    assert bits(oracle.dot_f64(x, y)) == bits(oracle.reduce_add_f64(oracle.mul_f64(x, y)))
    sel = oracle.select_f64(oracle.cmp_f64(x, np.full(1000, 0.5), "gt"), x, np.full(1000, -1.0))
    assert bits(oracle.condsum_cmp_f64(x, "gt", 0.5, -1.0)) == bits(oracle.reduce_add_f64(sel))


def test_arrays_dd_programs():
    # tests/programs/arrays.dd
    assert oracle.dot_f64(np.array([1.0, 2.0, 3.0]), np.array([4.0, 5.0, 6.0])) == 32.0
    x = np.array([1.0, -2.0, 3.0, -4.0, 5.0])
    assert list(oracle.filter_cmp_f64(x, "gt", 0.0)) == [1.0, 3.0, 5.0]
    assert oracle.count_cmp_f64(x, "gt", 0.0) == 3
    assert list(oracle.where(x > 0.0)) == [0, 2, 4]
    assert len(oracle.filter_cmp_f64(x, "gt", 100.0)) == 0
    assert oracle.reduce_add_f64(oracle.filter_cmp_f64(x, "gt", 100.0)) == 0.0
    xi = np.arange(10)
    assert list(oracle.gather(xi * 10, [9, 0, 4, 4])) == [90, 0, 40, 40]
    assert oracle.reduce_add_i64(oracle.gather(xi, xi[0:5])) == 10
    assert list(oracle.prev_i64([1, 2, 3], 0)) == [0, 1, 2]
    r = np.array([3.0, 1.0, 4.0, 1.0, 5.0])
    assert oracle.reduce_max_f64(r) == 5.0
    assert oracle.reduce_min_f64(r) == 1.0
    assert oracle.reduce_mul_f64(r) == 60.0
    assert oracle.argmin_f64(r) == 1


def test_grouping_dd_programs():
    # tests/programs/grouping.dd
    x = np.array([1, 2, 3, 4, 5])
    assert list(oracle.scan_add_i64(x)) == [1, 3, 6, 10, 15]
    assert list(oracle.scan_by_add_i64(x, [0, 0, 1, 0, 1])) == [1, 3, 3, 7, 5]
    k = np.array([1, 1, 2, 2, 2, 5])
    v = np.array([1, 2, 3, 4, 5, 6])
    n = len(k)
    s = (k != oracle.prev_i64(k, 0)) | (np.arange(n) == 0)
    e = (k != oracle.gather(k, np.minimum(np.arange(n) + 1, n - 1))) | (np.arange(n) == n - 1)
    assert list(oracle.compress(oracle.scan_by_add_i64(v, s), e)) == [3, 12, 6]
    ids = oracle.scan_add_i64(s.astype(np.int64)) - 1
    assert list(oracle.reduce_into_add_i64(ids, v, int(s.sum()))) == [3, 12, 6]
    assert list(oracle.compress(k, s)) == [1, 2, 5]
    g = oracle.group_id_i64([7, -1, 7, 3, -1, 7])
    assert list(g) == [0, 1, 0, 2, 1, 0]
    assert oracle.reduce_max_i64(g) + 1 == 3
    assert list(oracle.group_id2_i64_i64([1, 2, 1, 2], [2, 1, 2, 2])) == [0, 1, 0, 2]
    keys = np.array([1, 0, 1, 3, 1])
    assert list(oracle.histogram(keys, 5)) == [1, 3, 0, 1, 0]
    assert list(oracle.reduce_into_add_i64(keys, [5, 7, 9, 2, 1], 4)) == [7, 15, 0, 2]
    assert len(oracle.histogram(keys, 4)) == 4


def test_kernel_unit_vectors():
    # src/kernels/tests.rs:861-905 (IEEE min/max, argmin/argmax ties and NaN)
    nan = float("nan")
    assert np.isnan(oracle.reduce_min_f64([1.0, nan, 0.0]))
    assert bits(oracle.reduce_min_f64([0.0, -0.0])) == bits(-0.0)
    assert bits(oracle.reduce_max_f64([-0.0, 0.0])) == bits(0.0)
    with pytest.raises(OracleError, match="reduce_min of an empty array"):
        oracle.reduce_min_f64([])
    assert oracle.argmin_f64([3.0, 1.0, 1.0]) == 1
    assert oracle.argmin_f64([3.0, nan, nan]) == 1
    assert oracle.argmin_f64([0.0, -0.0]) == 1
    assert oracle.argmax_f64([-0.0, 0.0]) == 1
    assert oracle.argmax_f64([1.0, 5.0, 5.0]) == 1
    assert oracle.argmax_f64([1.0, nan, 5.0]) == 1
    with pytest.raises(OracleError, match="argmax of an empty array"):
        oracle.argmax_f64([])
    # :1416-1430 and :1446-1454 (scans)
    assert list(oracle.scan_add_i64([1, 2, 3, 4])) == [1, 3, 6, 10]
    assert list(oracle.scan_add_i64([2**63 - 1, 1])) == [2**63 - 1, -2**63]
    assert list(oracle.scan_by_add_i64([1, 2], [1, 0])) == [1, 3]
    # :1511-1540 (gather)
    assert list(oracle.gather(np.array([10, 20, 30]), [2, 0, 2])) == [30, 10, 30]
    assert len(oracle.gather(np.array([10, 20, 30]), [])) == 0
    with pytest.raises(OracleError, match="^gather index 3 out of range for length 3$"):
        oracle.gather(np.array([10, 20, 30]), [0, 3])
    with pytest.raises(OracleError, match="^gather index -1 out of range for length 3$"):
        oracle.gather(np.array([10, 20, 30]), [-1, 0])
    with pytest.raises(OracleError, match="^gather index 0 out of range for length 0$"):
        oracle.gather(np.array([], dtype=np.int64), [0])
    # :1576-1600 (histogram, bucket key errors)
    assert list(oracle.histogram([0, 2, 2, 3], 5)) == [1, 0, 2, 1, 0]
    assert len(oracle.histogram([], 0)) == 0
    assert list(oracle.histogram([], 3)) == [0, 0, 0]
    for key, n in [(3, 3), (-1, 3), (0, 0)]:
        first = 0 if n == 0 else key
        want = "bucket key %d out of range for %d buckets" % (first, n)
        with pytest.raises(OracleError, match="^%s$" % want):
            oracle.histogram([0, key], n)
        with pytest.raises(OracleError, match="^%s$" % want):
            oracle.reduce_into_add_i64([0, key], [1, 1], n)
    with pytest.raises(OracleError, match="^negative bucket count -1$"):
        oracle.histogram([], -1)
    with pytest.raises(OracleError, match="too large"):
        oracle.histogram([0], 1 << 62)
    with pytest.raises(OracleError, match="cannot allocate"):
        oracle.histogram([0], 1 << 50)
    assert list(oracle.reduce_into_add_i64([1, 0, 1], [5, 7, 9], 3)) == [7, 14, 0]


def test_argsort_reference_vectors():
    # src/kernels/scalar/index/tests.rs:246-266
    i64s = [2**63 - 1, 0, -2**63, -1, 2**63 - 1, -2**63, 0, -1]
    assert list(oracle.argsort_i64(i64s)) == [2, 5, 3, 7, 1, 6, 0, 4]
    near64 = [0xFE, -2, -2**63 + 1, 1, 2**63 - 1, -1, 0xFF, -2**63]
    assert list(oracle.argsort_i64(near64)) == [7, 2, 1, 5, 3, 0, 6, 4]
    # :268-280: all-equal rows give the identity, through the radix path
    n = 100_000
    assert np.array_equal(oracle.argsort_i64(np.full(n, -1)), np.arange(n))
    # radix path (> 1024 rows) equals the comparison restatement, two active passes
    # (:304-321) and random keys
    h = np.array([oracle.splitmix64(i) for i in range(2000)], dtype=np.uint64)
    base = np.uint64(0x0101010101010101)
    xs = (base ^ (h % np.uint64(16)) ^ (((h >> np.uint64(8)) % np.uint64(16)) << np.uint64(24))).view(np.int64)
    assert np.array_equal(oracle.argsort_i64(xs), oracle.argsort_reference_i64(xs))
    r = oracle.rand_i64(5000, 9)
    assert np.array_equal(oracle.argsort_i64(r), oracle.argsort_reference_i64(r))
    assert np.array_equal(oracle.argsort_i64(r), np.argsort(r, kind="stable"))


def test_group_id_first_occurrence():
    # src/kernels/scalar/group/tests.rs:24-35 (group_id_reference) over a growth-crossing column
    r = oracle.rand_i64(5000, 3) % 700
    seen = {}
    want = [seen.setdefault(int(v), len(seen)) for v in r]
    assert list(oracle.group_id_i64(r)) == want
    d = oracle.rand_i64(5000, 4)  # all distinct: several growths
    assert list(oracle.group_id_i64(d)) == list(range(5000))


def test_readme_example():
    # README.md:40-69: x = rand_f64(1e6, 1), y = rand_f64(1e6, 2)
    x, y = oracle.rand_f64(1_000_000, 1), oracle.rand_f64(1_000_000, 2)
    assert repr(oracle.dot_f64(x, y)) == "249724.39002046228"
    assert oracle.count_cmp_f64(x, "gt", 0.5) == 499521
    assert len(oracle.filter_cmp_f64(x, "gt", 0.99)) == 9851

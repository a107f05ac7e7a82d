"""scan_add_f64 and scan_by_add_f64, the float scans the reference's tier-2 design notes describe
(docs/superpowers/specs/2026-10-31-verkehrt-tier2-design.md:172; the reference itself has no
float scan, src/kernels/scalar/scan.rs:408-415). Parity is pinned by the notes' own definition,
checked on the oracle: out[i] is reduce_add_f64 of the prefix x[0..=i] (so out[n - 1] is the
array's canonical sum), and scan_by is that restarted at each set start flag. The GPU equals
the oracle bit for bit (a NaN only has to be NaN) on every path: one tile, the canonical pass in
record mode (whole chunks, tile by tile, signed rows), slices that are not 16-byte aligned, and
for scan_by short segments in registers and long ones through the tiled scan."""

import numpy as np
import pytest

import oracle
from helpers import GPU_LENGTHS, LENGTHS, uniform, varied, with_specials


def ties(n, seed=0):
    """Rows that round exactly halfway: after a first block of 2^53 every lane holds a state in
    [2^53, 2^54) (ulp 2), and the odd integer rows fall halfway between two states."""
    x = (oracle.rand_i64(n, seed).view(np.uint64) % np.uint64(500)).astype(np.float64) * 2 + 1
    x[:16] = 2.0 ** 53
    return x


DATA = {"uniform": uniform, "varied": varied, "specials": with_specials, "ties": ties}


def bits(v):
    return np.asarray(v, dtype=np.float64).view(np.uint64)


def same(got, want):
    got, want = np.asarray(got, dtype=np.float64), np.asarray(want, dtype=np.float64)
    nan = np.isnan(want)
    return got.shape == want.shape and np.array_equal(np.isnan(got), nan) and np.array_equal(bits(got[~nan]), bits(want[~nan]))


def starts_of(n, density, seed):
    s = (oracle.rand_f64(n, seed) < density).astype(np.uint8)
    if n:
        s[0] = 0  # row 0 starts whatever its flag
    return s


def test_oracle_scan_is_the_prefix_canonical_sum():
    for n in LENGTHS[:15] + [33, 47, 48, 49, 257, 300]:
        for name, f in DATA.items():
            x = f(n, n + 1)
            want = np.array([oracle.reduce_add_f64(x[: i + 1]) for i in range(n)], dtype=np.float64)
            assert same(oracle.scan_add_f64(x), want), (name, n)


def test_oracle_scan_ends_with_the_sum():
    for n in (4095, 4096, 4097, 100_003):
        for name, f in DATA.items():
            x = f(n, n + 5)
            assert same(oracle.scan_add_f64(x)[-1], oracle.reduce_add_f64(x)), (name, n)


def test_oracle_scan_by_restarts_per_segment():
    n = 5000
    x = varied(n, 3)
    for density in (0.0, 0.5, 0.02):
        s = starts_of(n, density, 7)
        s[0] = 1
        got = oracle.scan_by_add_f64(x, s)
        heads = list(np.flatnonzero(s)) + [n]
        for a, b in zip(heads[:-1], heads[1:]):
            assert same(got[a:b], oracle.scan_add_f64(x[a:b])), (density, a)
    # every row a segment: +0.0 + x[i]
    s = np.ones(n, dtype=np.uint8)
    assert same(oracle.scan_by_add_f64(x, s), 0.0 + x)


@pytest.mark.gpu
@pytest.mark.parametrize("data", sorted(DATA))
def test_gpu_scan_equals_oracle(ctx, data):
    for n in LENGTHS + GPU_LENGTHS + [(1 << 20) + 5]:
        x = DATA[data](n, n + 1)
        got = ctx.call("scan_add_f64", ctx.upload(x)).numpy()
        assert same(got, oracle.scan_add_f64(x)), (data, n)


@pytest.mark.gpu
def test_gpu_scan_large(ctx):
    # Whole chunks (uniform), negative rows (the signed walk), a sum that crosses zero.
    n = (1 << 24) + 7
    cases = {"uniform": uniform(n, 2), "negative": -uniform(n, 3), "mostly_positive": uniform(n, 4) - 0.3,
             "ties": ties(n, 5)}
    for name, x in cases.items():
        dx = ctx.upload(x)
        got = ctx.call("scan_add_f64", dx).numpy()
        assert same(got, oracle.scan_add_f64(x)), name
        assert int(bits(got[-1])) == ctx.call("reduce_add_f64", dx, raw=True)[2], name


@pytest.mark.gpu
def test_gpu_scan_unaligned_slices(ctx):
    x = uniform(300_000, 6)
    dx = ctx.upload(x)
    for off, n in ((1, 200_001), (3, 4097), (17, 65_536)):
        got = ctx.call("scan_add_f64", dx.slice(off, off + n)).numpy()
        assert same(got, oracle.scan_add_f64(x[off : off + n])), (off, n)


@pytest.mark.gpu
@pytest.mark.parametrize("data", sorted(DATA))
def test_gpu_scan_by_equals_oracle(ctx, data):
    for n in LENGTHS + GPU_LENGTHS + [(1 << 20) + 5]:
        x = DATA[data](n, n + 2)
        dx = ctx.upload(x)
        for density in (0.0, 0.5, 0.01, 1e-4):
            s = starts_of(n, density, n + 3)
            got = ctx.call("scan_by_add_f64", dx, ctx.upload(s.astype(bool))).numpy()
            assert same(got, oracle.scan_by_add_f64(x, s)), (data, n, density)


@pytest.mark.gpu
def test_gpu_scan_by_long_segments(ctx):
    # Segments beyond 2^16 rows take the tiled scan on their rows (some not 16-byte aligned).
    n = (1 << 19) + 3
    x = uniform(n, 8) - 0.1
    s = np.zeros(n, dtype=np.uint8)
    for h in (70_001, 70_002, 200_000, 200_017, 300_000, 450_000):
        s[h] = 1
    dx, ds = ctx.upload(x), ctx.upload(s.astype(bool))
    got = ctx.call("scan_by_add_f64", dx, ds).numpy()
    assert same(got, oracle.scan_by_add_f64(x, s))
    # one segment: the scan itself
    z = np.zeros(n, dtype=bool)
    assert same(ctx.call("scan_by_add_f64", dx, ctx.upload(z)).numpy(), oracle.scan_add_f64(x))


@pytest.mark.gpu
def test_gpu_scan_by_segment_edges(ctx):
    # Segment lengths at the edges of the 16-row blocks, of the 1024-row head tiles and of the
    # 1536-row shared-memory runs and windows, and start flags read from views at every offset
    # modulo 16 (the flags are read 16 bytes at a time only where aligned).
    lens = [1536, 1537, 1535, 1, 1024, 1023, 3072, 3073, 15, 16, 17, 31, 32, 33, 4608, 2, 1536 * 5 + 7]
    lens += [1] * 40 + [16] * 20 + [1500, 36, 1537]
    n = sum(lens)
    s = np.zeros(n + 16, dtype=np.uint8)
    at = 0
    for L in lens:
        s[at] = 1
        at += L
    x = varied(n + 16, 21)
    dx = ctx.upload(x)
    ds = ctx.upload(s.astype(bool))
    for off in range(16):
        m = n - 16 + off
        got = ctx.call("scan_by_add_f64", dx.slice(off, off + m), ds.slice(off, off + m)).numpy()
        assert same(got, oracle.scan_by_add_f64(x[off : off + m], s[off : off + m])), off


@pytest.mark.gpu
def test_gpu_scan_by_many_long_segments(ctx):
    # Many segments beyond 2^16 rows: one block per segment in windows (some starting at rows
    # that are not 16-byte aligned), rows of mixed sign and magnitude.
    n = (1 << 22) + 5
    rng = np.random.default_rng(11)
    heads = np.cumsum(rng.integers(65_537, 90_000, size=60))
    heads = heads[heads < n]
    s = np.zeros(n, dtype=np.uint8)
    s[heads] = 1
    for x in (uniform(n, 12) - 0.2, varied(n, 13)):
        got = ctx.call("scan_by_add_f64", ctx.upload(x), ctx.upload(s.astype(bool))).numpy()
        assert same(got, oracle.scan_by_add_f64(x, s))


@pytest.mark.gpu
def test_gpu_scan_errors_and_empty(ctx):
    x = ctx.upload(np.array([1.0, 2.0, 3.0]))
    with pytest.raises(Exception, match=r"^expected f64\[\], got i64\[\]$"):
        ctx.call("scan_add_f64", ctx.upload(np.array([1, 2])))
    with pytest.raises(Exception, match="^length mismatch: 3 vs 2$"):
        ctx.call("scan_by_add_f64", x, ctx.upload(np.array([True, False])))
    e = ctx.upload(np.array([], dtype=np.float64))
    assert len(ctx.call("scan_add_f64", e)) == 0
    assert len(ctx.call("scan_by_add_f64", e, ctx.upload(np.array([], dtype=bool)))) == 0

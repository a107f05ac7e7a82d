"""Ingestion into HBM: load_T (src/kernels/scalar/construct.rs:78-97) and the acceptance column
files (src/columns.rs load_words / load_single_bytes, and its tests' cases), streamed through
pinned buffers. The data arrives bit for bit, and the errors are the reference's texts."""

import numpy as np
import pytest

import oracle

LOADS = {"f64": np.float64, "f32": np.float32, "i64": np.int64, "u64": np.uint64, "i32": np.int32, "u8": np.uint8}


def test_load_entries_in_the_table():
    import verkehrt_gb300 as vk

    table = {name: (cls, arity, cost) for name, cls, arity, cost in vk.kernels()}
    for t, dt in LOADS.items():
        assert table["load_" + t] == ("whole", 1, np.dtype(dt).itemsize)


@pytest.mark.gpu
def test_load_every_type(ctx, tmp_path):
    raw = oracle.rand_i64(10_007, 3).view(np.uint8)
    for t, dt in LOADS.items():
        w = np.dtype(dt).itemsize
        data = raw[: (len(raw) // w) * w]
        p = tmp_path / ("x." + t)
        p.write_bytes(data.tobytes())
        got = ctx.call("load_" + t, str(p)).numpy()
        assert got.dtype == dt and np.array_equal(got.view(np.uint8), data), t
    e = tmp_path / "empty"
    e.write_bytes(b"")
    assert len(ctx.call("load_f64", str(e))) == 0


@pytest.mark.gpu
def test_load_larger_than_the_staging_buffers(ctx, tmp_path):
    # 9 chunks of 32 MiB and a ragged end: both pinned buffers are reused several times.
    n = (9 * (32 << 20) + 4096 + 8) // 8
    x = oracle.rand_f64(n, 5)
    p = tmp_path / "big.f64"
    p.write_bytes(x.tobytes())
    a = ctx.call("load_f64", str(p))
    b = ctx.call("load_f64", str(p))  # a second load right after reuses the buffers
    assert np.array_equal(a.numpy().view(np.uint64), x.view(np.uint64))
    assert np.array_equal(b.numpy().view(np.uint64), x.view(np.uint64))
    assert ctx.call("reduce_add_f64", a, raw=True)[2] == int(np.float64(oracle.reduce_add_f64(x)).view(np.uint64))


@pytest.mark.gpu
def test_load_errors(ctx, tmp_path):
    p = tmp_path / "seven"
    p.write_bytes(b"1234567")
    with pytest.raises(Exception, match="^%s has 7 bytes, which is not a multiple of 8$" % p):
        ctx.call("load_i64", str(p))
    assert len(ctx.call("load_u8", str(p))) == 7
    missing = tmp_path / "missing.f64"
    with pytest.raises(Exception, match=r"^cannot read %s: No such file or directory \(os error 2\)$" % missing):
        ctx.call("load_f64", str(missing))
    with pytest.raises(Exception, match="^expected str, got i64$"):
        ctx.call("load_f64", 3)


def words(v):
    return np.asarray(v, dtype=np.uint64).tobytes()


@pytest.mark.gpu
def test_column_words_and_bytes(ctx, tmp_path):
    # columns.rs tests: load_inputs_reads_u64_and_bytes.
    (tmp_path / "a.u64").write_bytes(words([1, 2, 2**64 - 1]))
    (tmp_path / "b.u64").write_bytes(words([2**64 - 1, 7, 0]))
    (tmp_path / "s.ends").write_bytes(words([1, 2, 3]))
    (tmp_path / "s.bytes").write_bytes(b"xyz")
    assert list(ctx.load_column_words(tmp_path / "a.u64", "u64").numpy()) == [1, 2, 2**64 - 1]
    assert list(ctx.load_column_words(tmp_path / "b.u64", "i64").numpy()) == [-1, 7, 0]
    assert bytes(ctx.load_column_bytes(tmp_path / "s.ends", tmp_path / "s.bytes", "s").numpy()) == b"xyz"
    # Signed columns are stored with the sign bit flipped (CLICKBENCH_SIGNED).
    v = oracle.rand_i64(100_003, 9)
    (tmp_path / "w.u64").write_bytes((v.view(np.uint64) ^ np.uint64(1 << 63)).tobytes())
    assert np.array_equal(ctx.load_column_words(tmp_path / "w.u64", "i64", flip_sign=True).numpy(), v)


@pytest.mark.gpu
def test_column_errors(ctx, tmp_path):
    (tmp_path / "odd.u64").write_bytes(b"123456789")
    with pytest.raises(Exception, match="^%s: 9 bytes is not a whole number of 8-byte words$" % (tmp_path / "odd.u64")):
        ctx.load_column_words(tmp_path / "odd.u64", "u64")
    (tmp_path / "c.ends").write_bytes(words([1, 2, 4, 4]))
    (tmp_path / "c.bytes").write_bytes(b"abcd")
    with pytest.raises(Exception, match="^column 'c' row 2 ends at byte 4, so it is not one byte per row$"):
        ctx.load_column_bytes(tmp_path / "c.ends", tmp_path / "c.bytes", "c")
    (tmp_path / "d.ends").write_bytes(words([1, 2]))
    (tmp_path / "d.bytes").write_bytes(b"abc")
    with pytest.raises(Exception, match="^column 'd' has 2 rows but 3 bytes, so it is not one byte per row$"):
        ctx.load_column_bytes(tmp_path / "d.ends", tmp_path / "d.bytes", "d")
    with pytest.raises(Exception, match=r"^%s: No such file or directory \(os error 2\)$" % (tmp_path / "e.bytes")):
        (tmp_path / "e.ends").write_bytes(b"123")  # a bad size, but the missing bytes file comes first
        ctx.load_column_bytes(tmp_path / "e.ends", tmp_path / "e.bytes", "e")

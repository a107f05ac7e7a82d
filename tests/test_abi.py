"""The C-ABI library loads, exports every entry point include/vkcuda.h declares, and carries
the kernel-table entries of the hot path. No compute call is made (no GPU needed)."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    text = open(os.path.join(ROOT, "include", "vkcuda.h")).read()
    return sorted(set(re.findall(r"VKC_API[^;(]*?\b(vkc_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from verkehrt_gb300 import build as vbuild

    vbuild.build()
    import verkehrt_gb300 as vk

    return vk.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 35
    for n in names:
        assert hasattr(lib, n), n
    import verkehrt_gb300 as vk

    assert sorted(vk.exported_symbols()) == names


def test_only_the_abi_is_exported(lib):
    # The library exports the C ABI and hides its internals (built -fvisibility=hidden).
    with pytest.raises(AttributeError):
        getattr(lib, "_ZN3vkc10new_arrayEP7vkc_ctx8vkc_typelbPP9vkc_array")


HOT_PATH = [
    # README program and primitive sweep
    "rand_f64", "rand_i64", "length_f64", "dot_f64", "count_gt_f64", "filter_gt_f64",
    "reduce_add_f64", "reduce_min_f64", "reduce_max_f64", "argmin_f64", "argmax_f64",
    "compress_f64", "compress_i64", "compress_bool", "where", "gather_i64", "gather_f64",
    "scan_add_i64", "scan_by_add_i64",
    # group-by
    "histogram", "reduce_into_add_i64",
    # unfused plans
    "mul_f64", "gt_f64", "select_f64",
    # sort and group-by
    "argsort_i64", "group_id_i64", "group_id2_i64_i64", "prev_i64", "iota",
]


def test_kernel_table(lib):
    import verkehrt_gb300 as vk

    table = {name: (cls, arity, cost) for name, cls, arity, cost in vk.kernels()}
    for name in HOT_PATH:
        assert name in table, name
    # KernelDef::cost of the reference (bytes per element).
    assert table["dot_f64"][2] == 16
    assert table["reduce_add_f64"] == ("reduction", 1, 8)
    assert table["filter_gt_f64"][:2] == ("selection", 2)
    assert table["gather_i64"][2] == 24
    assert table["where"][2] == 9
    assert lib.vkc_kernel_lookup(b"no_such_kernel") == -1


def test_open_without_a_device_fails_cleanly(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a device is present")
    h = ctypes.c_void_p()
    assert lib.vkc_open(0, ctypes.byref(h)) == 4  # VKC_DEVICE


def test_missing_library_raises_instead_of_falling_back(tmp_path, monkeypatch):
    # The CUDA library is the only compute path: without it every entry raises.
    import verkehrt_gb300 as vk

    monkeypatch.setattr(vk, "_lib", None)
    monkeypatch.setattr(vk, "LIB_PATH", str(tmp_path / "libvkcuda.so"))
    with pytest.raises(RuntimeError, match="not built"):
        vk.load()
    with pytest.raises(RuntimeError, match="not built"):
        vk.Context(0)


def test_table_covers_the_reference_registry(lib):
    # Every kernel of the reference's registry that can receive a device array has a cuda entry
    # (tests/golden/reference_kernels.py restates the registration functions), so `select`
    # (src/kernels.rs:342-368) never falls back to a host entry for device-resident values.
    import sys

    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import reference_kernels
    import verkehrt_gb300 as vk

    ours = {name for name, _, _, _ in vk.kernels()}
    missing = sorted(set(reference_kernels.device_names()) - ours)
    assert not missing, missing
    # Beyond the reference: the float extensions of its tier-2 design notes only.
    assert sorted(ours - set(reference_kernels.all_names())) == [
        "reduce_into_add_f64", "scan_add_f64", "scan_by_add_f64"]

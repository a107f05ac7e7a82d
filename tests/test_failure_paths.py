"""The failure paths, made to happen on the host or by a wait that runs out, never by a GPU fault.

* A wait on another block that runs out: the "lookback_never_ready" test hook makes every
  decoupled lookback of scan_add_i64 poll for records that no block writes (a flag that
  nothing sets), and the "spin_limit" hook bounds each wait to a few dozen polls. Each waiting
  block records the timeout in the status word and goes on (its outputs stay in bounds: a
  lookback that gives up uses the scan's identity as its prefix). A scan's call only enqueues
  its kernels, so the next call that waits for the device (a download, vkc_synchronize)
  reports VKC_TIMEOUT; a selection waits for its count and reports it itself. The same
  context then gives the oracle's results again.
* An allocation that fails: the "fail_alloc_after" hook makes one array allocation of the
  context report failure, as a device out of memory would. The call returns VKC_ALLOC with
  the reference's text (src/kernels/scalar/index/radix.rs:151-157 for argsort scratch,
  src/kernels/scalar/group.rs:128-137 for the group_id table, src/value.rs:297-307 for an
  array), as in src/kernels/scalar/index/tests.rs:324-330, and the context stays usable.
"""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture()
def fresh():
    """A context of its own, so the hooks touch no other test."""
    import verkehrt_gb300 as vk

    c = vk.Context(0)
    yield c
    c.close()


def scan_values(n, seed):
    return (oracle.rand_i64(n, seed).view(np.uint64) % np.uint64(1 << 21)).astype(np.int64) - (1 << 20)


def test_a_wait_that_runs_out_reports_a_timeout_and_the_context_recovers(fresh):
    import verkehrt_gb300 as vk

    n = 1 << 24
    v = scan_values(n, 3)
    dv = fresh.upload(v)
    want = oracle.scan_add_i64(v)
    assert np.array_equal(fresh.call("scan_add_i64", dv).numpy(), want)
    fresh.tune_set("spin_limit", 0, 64)
    fresh.tune_set("lookback_never_ready", 0, 1)
    assert fresh.tune_get("spin_limit", 0) == 64
    assert fresh.tune_get("lookback_never_ready", 0) == 1
    # A scan only enqueues its kernels: the next call that waits for the device reports it.
    out = fresh.call("scan_add_i64", dv)
    with pytest.raises(vk.KernelError) as e:
        out.numpy()
    assert (e.value.status, e.value.message) == ("TIMEOUT", "a device-side wait gave up")
    fresh.call("scan_add_i64", dv)
    with pytest.raises(vk.KernelError) as e:
        fresh.synchronize()
    assert (e.value.status, e.value.message) == ("TIMEOUT", "a device-side wait gave up")
    # A selection waits for its count, so the call itself reports it.
    with pytest.raises(vk.KernelError) as e:
        fresh.call("filter_gt_f64", fresh.call("rand_f64", 1 << 24, 1), 0.5)
    assert (e.value.status, e.value.message) == ("TIMEOUT", "a device-side wait gave up")
    fresh.tune_set("lookback_never_ready", 0, 0)
    fresh.tune_set("spin_limit", 0, 0)
    assert (fresh.tune_get("spin_limit", 0), fresh.tune_get("lookback_never_ready", 0)) == (0, 0)
    for _ in range(3):
        assert np.array_equal(fresh.call("scan_add_i64", dv).numpy(), want)
    assert fresh.call("reduce_add_i64", dv) == int(v.sum())


def test_an_allocation_failure_is_an_error_and_the_context_recovers(fresh):
    import verkehrt_gb300 as vk

    n = 100_000
    keys = oracle.rand_i64(n, 5)
    dk = fresh.upload(keys)
    want = oracle.argsort_i64(keys)
    # The first allocation is argsort's output, the second its key-image scratch.
    fresh.tune_set("fail_alloc_after", 0, 1)
    with pytest.raises(vk.KernelError) as e:
        fresh.call("argsort_i64", dk)
    assert e.value.status == "ALLOC"
    assert e.value.message == "cannot allocate argsort scratch for %d rows" % n
    assert fresh.tune_get("fail_alloc_after", 0) == -1  # one failure, then none
    assert np.array_equal(fresh.call("argsort_i64", dk).numpy(), want)
    # group_id: the output, then the table.
    fresh.tune_set("fail_alloc_after", 0, 1)
    with pytest.raises(vk.KernelError) as e:
        fresh.call("group_id_i64", dk)
    assert e.value.status == "ALLOC"
    assert e.value.message == "cannot allocate a group_id table of 262144 slots"
    assert np.array_equal(fresh.call("group_id_i64", dk).numpy(), oracle.group_id_i64(keys))
    # A plain array.
    fresh.tune_set("fail_alloc_after", 0, 0)
    with pytest.raises(vk.KernelError) as e:
        fresh.call("rand_f64", 1000, 1)
    assert (e.value.status, e.value.message) == ("ALLOC", "cannot allocate an array of 1000 elements")
    assert np.array_equal(fresh.call("rand_f64", 1000, 1).numpy(), oracle.rand_f64(1000, 1))


def test_hook_values_are_checked(fresh):
    import verkehrt_gb300 as vk

    with pytest.raises(vk.KernelError):
        fresh.tune_set("spin_limit", 0, -1)
    with pytest.raises(vk.KernelError):
        fresh.tune_set("fail_alloc_after", 0, -2)
    with pytest.raises(vk.KernelError):
        fresh.tune_set("lookback_never_ready", 0, 2)

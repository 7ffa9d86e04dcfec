"""Failure paths without a GPU fault.

A bounded device wait that never ends is made on purpose: one onesweep pass
whose only tile waits for a predecessor that nothing publishes.  The wait must
give up after its poll limit, raise status bit 1, return, and leave the
context usable.  The wait-limit setting itself is host state and is checked
without a GPU."""
import time

import numpy as np
import pytest


def test_wait_limit_setting_roundtrip():
    from del_msh_gb300 import _native
    _native.load(build_if_missing=True)
    before = _native.get_wait_limit()
    assert before == 1 << 22
    try:
        _native.set_wait_limit(5000)
        assert _native.get_wait_limit() == 5000
        _native.set_wait_limit(0)  # 0 restores the default
        assert _native.get_wait_limit() == 1 << 22
    finally:
        _native.set_wait_limit(before)


def test_selftest_rejects_bad_arguments():
    from del_msh_gb300 import _native
    L = _native.load(build_if_missing=True)
    need = L.dm_selftest_bounded_wait_scratch_bytes()
    assert need > 0
    with pytest.raises(_native.DelMshError):
        _native.call("dm_selftest_bounded_wait", 0, 0, None, need)  # polls 0
    with pytest.raises(_native.DelMshError):
        _native.call("dm_selftest_bounded_wait", 0, 100, None, need)  # no scratch


@pytest.mark.gpu
def test_bounded_wait_gives_up_and_reports(cuda):
    torch = cuda
    from del_msh_gb300 import _native
    L = _native.load()
    assert _native.device_status(clear=True) == 0
    need = L.dm_selftest_bounded_wait_scratch_bytes()
    scratch = torch.empty((need,), dtype=torch.uint8, device="cuda:0")
    sp = torch.cuda.current_stream().cuda_stream
    t0 = time.perf_counter()
    _native.call("dm_selftest_bounded_wait", sp, 2000, scratch.data_ptr(), need)
    elapsed = time.perf_counter() - t0
    assert elapsed < 10.0
    bits = _native.device_status(clear=False)
    assert bits & 1, bits  # the wait gave up and said so
    assert _native.device_status(clear=True) & 1
    assert _native.device_status(clear=False) == 0  # cleared
    # the context is still usable: a real sort right after is correct and clean
    rng = np.random.default_rng(1)
    keys = rng.integers(0, 1 << 30, 100_000, dtype=np.uint32)
    d_keys = torch.from_numpy(keys.view(np.int32)).to("cuda:0")
    idx = torch.empty_like(d_keys)
    n = keys.size
    sb = L.dm_array1d_argsort_scratch_bytes(n)
    s2 = torch.empty((sb,), dtype=torch.uint8, device="cuda:0")
    _native.call("dm_array1d_argsort", sp, n, d_keys.data_ptr(), idx.data_ptr(), s2.data_ptr(), sb)
    torch.cuda.synchronize()
    assert np.array_equal(idx.cpu().numpy().view(np.uint32), np.argsort(keys, kind="stable"))
    assert _native.device_status(clear=True) == 0

"""The allocation-free scan (sr_exclusive_scan_i32_noalloc), through the C ABI.

It is for callers that cannot allocate device memory: hosts that give all
device memory to their own allocator or run under a hard memory budget, and
frame loops that cannot risk an allocation call that may wait on the device.
Its scratch is a fixed array inside the library, shared by every call, so the
test makes two calls in a row: the second must not see the first's state.
The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scan_both(sr, a):
    """Returns (allocation-free result, allocating result) for host array a."""
    import torch
    n = a.size
    d_in = torch.from_numpy(a).cuda()
    out_free = torch.full((n + 1,), -1, dtype=torch.int32, device="cuda")
    out_ref = torch.full((n + 1,), -2, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    L = sr.lib()
    assert L.sr_exclusive_scan_i32_noalloc(d_in.data_ptr(), out_free.data_ptr(), n, stream) == 0, \
        L.sr_last_error()
    assert L.sr_exclusive_scan_i32(d_in.data_ptr(), out_ref.data_ptr(), n, stream) == 0, L.sr_last_error()
    torch.cuda.synchronize()
    sr.scan_status(stream)
    return out_free.cpu().numpy(), out_ref.cpu().numpy()


def test_two_calls_in_a_row_match_the_allocating_scan(gpu):
    rng = np.random.default_rng(2024)
    # first call at the largest size the fixed scratch holds, then a smaller one
    first = rng.integers(-1000, 1000, size=gpu.NOALLOC_SCAN_MAX_N, dtype=np.int32)
    second = rng.integers(-7, 8, size=1_000_003, dtype=np.int32)
    for a in (first, second):
        got, want = _scan_both(gpu, a)
        assert np.array_equal(got, want)
        assert got[0] == 0 and got[-1] == np.int32(a.astype(np.int64).sum())


def test_calls_leave_free_device_memory_unchanged_and_scan_in_place(gpu):
    """Once the library's device code is loaded (the first call on a device
    may load it), further calls take no device memory: the free bytes the
    driver reports are the same before and after.  In place (d_in == d_out)
    at a size that is not a whole number of 4,096-element tiles."""
    import torch
    n = 1_000_003
    rng = np.random.default_rng(7)
    a = rng.integers(-50, 50, size=n, dtype=np.int32)
    buf = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    L = gpu.lib()
    assert L.sr_exclusive_scan_i32_noalloc(buf.data_ptr(), buf.data_ptr(), n, None) == 0, L.sr_last_error()
    torch.cuda.synchronize()
    buf[:n] = torch.from_numpy(a).cuda()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert L.sr_exclusive_scan_i32_noalloc(buf.data_ptr(), buf.data_ptr(), n, None) == 0, L.sr_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    gpu.scan_status()
    assert free1 == free0
    want = np.zeros(n + 1, np.int64)
    np.cumsum(a.astype(np.int64), out=want[1:])
    assert np.array_equal(buf.cpu().numpy(), want.astype(np.int32))


def test_sizes_beyond_the_fixed_scratch_are_rejected(gpu):
    L = gpu.lib()
    rc = L.sr_exclusive_scan_i32_noalloc(None, None, gpu.NOALLOC_SCAN_MAX_N + 1, None)
    assert rc == 1
    assert b"outside" in L.sr_last_error()

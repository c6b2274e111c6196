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


def test_sizes_beyond_the_fixed_scratch_are_rejected(gpu):
    L = gpu.lib()
    rc = L.sr_exclusive_scan_i32_noalloc(None, None, gpu.NOALLOC_SCAN_MAX_N + 1, None)
    assert rc == 1
    assert b"outside" in L.sr_last_error()

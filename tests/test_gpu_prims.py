"""GPU tests of the standalone device primitives exposed by the C ABI."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _excl_scan_ref(a):
    out = np.zeros(a.size + 1, np.int64)
    np.cumsum(a.astype(np.int64), out=out[1:])
    return out.astype(np.int32)   # wraps like the device scan


@pytest.mark.parametrize("n", [0, 1, 31, 4095, 4096, 4097, 100003, 1 << 21])
def test_exclusive_scan_matches_numpy(gpu, n):
    import torch
    rng = np.random.default_rng(n)
    a = rng.integers(-5, 6, size=n, dtype=np.int32)
    d_in = torch.from_numpy(a).cuda() if n else torch.zeros(1, dtype=torch.int32, device="cuda")
    d_out = torch.full((n + 1,), -7, dtype=torch.int32, device="cuda")
    gpu.exclusive_scan_i32(d_in.data_ptr(), d_out.data_ptr(), n)
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy(), _excl_scan_ref(a))


def test_exclusive_scan_in_place_and_wrapping(gpu):
    import torch
    n = 300000
    a = np.full(n, 1 << 20, np.int32)   # total overflows int32
    buf = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    buf[:n] = torch.from_numpy(a).cuda()
    gpu.exclusive_scan_i32(buf.data_ptr(), buf.data_ptr(), n)
    torch.cuda.synchronize()
    assert np.array_equal(buf.cpu().numpy(), _excl_scan_ref(a))


def test_exclusive_scan_rejects_bad_sizes(gpu):
    import torch
    d = torch.zeros(4, dtype=torch.int32, device="cuda")
    with pytest.raises(gpu.SRError):
        gpu.exclusive_scan_i32(d.data_ptr(), d.data_ptr(), -1)
    with pytest.raises(gpu.SRError):
        gpu.exclusive_scan_i32(d.data_ptr(), None, 3)


def test_scan_status_is_ok_after_good_scans(gpu):
    import torch
    a = np.arange(50000, dtype=np.int32)
    d_in = torch.from_numpy(a).cuda()
    d_out = torch.zeros(a.size + 1, dtype=torch.int32, device="cuda")
    gpu.exclusive_scan_i32(d_in.data_ptr(), d_out.data_ptr(), a.size)
    gpu.exclusive_scan_i32_noalloc(d_in.data_ptr(), d_out.data_ptr(), a.size)
    gpu.scan_status()
    assert np.array_equal(d_out.cpu().numpy(), _excl_scan_ref(a))


def test_bounded_wait_gives_up_and_the_context_stays_usable(gpu):
    """A look-back whose predecessor never publishes (tile 0 is skipped)
    gives up after the spin limit; the scan reports SR_ERR_TIMEOUT through
    sr_scan_status, and the next scan on the same device is correct."""
    import torch
    n = 64 * 4096 + 5
    a = np.ones(n, np.int32)
    d_in = torch.from_numpy(a).cuda()
    d_out = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    L = gpu.lib()
    gpu.set_spin_limit(2000)
    try:
        assert L.sr_debug_scan_without_first_tile(d_in.data_ptr(), d_out.data_ptr(), n, None) == 0, \
            L.sr_last_error()
        with pytest.raises(gpu.SRError) as e:
            gpu.scan_status()
        assert e.value.code == 4 and "timed out" in str(e.value)
        gpu.scan_status()   # the report was cleared
    finally:
        gpu.set_spin_limit(0)
    gpu.exclusive_scan_i32(d_in.data_ptr(), d_out.data_ptr(), n)
    gpu.scan_status()
    assert np.array_equal(d_out.cpu().numpy(), _excl_scan_ref(a))

"""The render server's host logic without a GPU: the admission rule and
argument checks."""
import ctypes

import vkscanlinepr_gb300 as sr


def test_admission_takes_the_longest_fitting_prefix():
    assert sr.admission_take([10, 20, 30], 0, 100) == (3, False)
    assert sr.admission_take([10, 20, 30], 50, 100) == (2, False)
    assert sr.admission_take([10, 20, 30], 95, 100) == (0, False)
    # order is kept: a small request behind a large one waits
    assert sr.admission_take([60, 5], 50, 100) == (0, False)
    assert sr.admission_take([10, 20, 30], 0, 100, max_take=2) == (2, False)


def test_admission_rejects_a_request_larger_than_the_budget():
    assert sr.admission_take([150, 10], 0, 100) == (0, True)
    assert sr.admission_take([], 0, 100) == (0, False)


def test_admission_does_not_overflow():
    big = (1 << 64) - 10
    assert sr.admission_take([5, 5], big - 20, big) == (2, False)
    assert sr.admission_take([5, big], 0, big) == (1, False)


def test_server_arguments_are_checked_without_a_gpu():
    L = sr.lib()
    assert L.sr_server_create(None, None, None) == 1
    o = sr.ServerOpts(ctypes.sizeof(sr.ServerOpts), 1, 0, 0, 64, 0, 1 << 30)
    h = ctypes.c_void_p()
    assert L.sr_server_create(ctypes.byref(o), None, ctypes.byref(h)) == 1   # zero slots
    assert b"slots" in L.sr_last_error()
    assert L.sr_server_submit(None, 1, 1, None, None, None) == 1

"""The C ABI library: builds for sm_103a, loads without a GPU, and exports
every function include/sr.h declares.  No device work is done here."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    txt = open(os.path.join(REPO, "include", "sr.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = set(re.findall(r"\b(sr_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ("sr_create", "sr_load_scene", "sr_set_mvp", "sr_render", "sr_destroy"):
        assert n in names


def test_library_exports_every_declared_symbol(srlib):
    L = ctypes.CDLL(srlib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    assert set(srlib.EXPORTS) <= set(declared_functions())


def test_errors_cross_the_abi_as_status_codes(srlib):
    L = srlib.lib()
    # no context and no GPU needed for argument checks
    assert L.sr_create(0, 0, None, ctypes.byref(ctypes.c_void_p())) == 1
    assert b"canvas" in L.sr_last_error()
    assert L.sr_set_mvp(None, None) == 1
    assert L.sr_render(None, None, 0, None) == 1
    assert L.sr_exclusive_scan_i32(None, None, -1, None) == 1


def test_host_scene_sources_work_without_gpu(srlib):
    sc = srlib.synth_scene(0, 0, width=128, height=96, n_paths=20)
    assert sc.width == 128 and sc.height == 96 and sc.n_paths == 20
    assert set(sc.arrays()["curve_type"].tolist()) == {4}


def test_cuda_sources_compile_for_sm103a_only():
    from vkscanlinepr_gb300 import builder
    assert builder.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert "--fmad=false" in builder.NVCC_FLAGS


def test_tuning_values_are_checked(srlib):
    L = srlib.lib()
    t = srlib.Tuning(ctypes.sizeof(srlib.Tuning), 10, 16, 8)
    assert L.sr_set_tuning(None, ctypes.byref(t)) == 1
    assert L.sr_batch_set_tuning(None, ctypes.byref(t)) == 1

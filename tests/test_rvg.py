"""The .rvg reader behind sr_rvg_load (host code, no GPU)."""
import os

import numpy as np
import pytest

import oracle

REF_RVG = "/root/reference/workdir/input/rvg"

SMALL = """viewport 0,0 40,30
window 0,0 40,30
scene dyn_identity
  1 element nzfill dyn_concrete 0,0 0,0 0,0: M 2,2 L 20,2 L 20,12 L 2,12 Z dyn_identity dyn_paint 1 solid rgba(1,0,0,1)
  1 element ofill dyn_concrete 0,0 0,0 0,0: M 5,5 C 10,0 20,0 25,5 L 25,20 dyn_identity dyn_paint 0.5 solid rgba(0,0,1,1)
  1 element stroke 3 dyn_identity
"""


def test_small_rvg(tmp_path, srlib):
    p = tmp_path / "small.rvg"
    p.write_text(SMALL)
    sc, vp = srlib.load_rvg(str(p))
    assert list(vp) == [0, 0, 40, 30]
    a = sc.arrays()
    # path 0: four lines, explicitly closed by Z (no extra line);
    # path 1: cubic + line, open -> closed with a line (rvg.cpp:211-223)
    assert a["curve_type"].tolist() == [2, 2, 2, 4, 2, 2]
    assert a["curve_path_idx"].tolist() == [0, 0, 0, 1, 1, 1]
    assert a["fill_rule"].tolist()[:2] == [0, 1]
    # colour packing of loadVG: u8(c*255), alpha *= opacity (scanline_rasterizer.cpp:107-118)
    assert a["fill_info"][0] == 0xFF0000FF
    assert a["fill_info"][1] == (0x7F << 24) | (0xFF << 16)
    last = a["position"].reshape(-1, 2)[a["curve_pos_map"][5]:][:2]
    assert np.array_equal(last, [[25, 20], [5, 5]])


@pytest.mark.skipif(not os.path.isdir(REF_RVG), reason="reference scenes not present")
@pytest.mark.parametrize("name", ["test.rvg", "drops.rvg"])
def test_reference_scenes_render_in_reference_mode(srlib, name):
    sc, vp = srlib.load_rvg(os.path.join(REF_RVG, name))
    a = sc.arrays()
    assert a["curve_type"].size > 0 and set(np.unique(a["curve_type"]).tolist()) <= {2, 4}
    w, h = int(vp[2]), int(vp[3])
    s = oracle.Scene(w, h, a["position"], a["pos_path_idx"], a["curve_pos_map"], a["curve_type"],
                     a["curve_path_idx"], a["fill_rule"], a["fill_info"])
    f = oracle.Frame(s, mode=oracle.MODE_REFERENCE)
    assert f.n_intersections > 0 and f.n_draw > 0

"""The .rvg reader behind sr_rvg_load (host code, no GPU), on a hand-written
scene and on the reference's eight shipped scenes (tests/golden/rvg)."""
import numpy as np
import pytest

import oracle
import rvg_scenes
import scenes

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


# curves and paths each shipped scene parses to, as the reference's reader
# sees them (the arc scenes stop at their first 'A': rvg.cpp has no case for it)
EXPECTED = {"car": (6881, 237), "chord": (0, 1), "chord-black": (0, 1), "drops": (859, 81),
            "embrace": (3687, 184), "reschart": (8705, 747), "test": (264, 17), "tiger": (28042, 302)}


@pytest.mark.parametrize("name", rvg_scenes.NAMES)
def test_reference_scenes_parse(srlib, tmp_path, name):
    d, vp = rvg_scenes.load(srlib, name, tmp_path)
    assert (d["curve_type"].size, d["fill_rule"].size) == EXPECTED[name]
    assert set(np.unique(d["curve_type"]).tolist()) <= {2, 4}
    assert vp[0] == 0 and vp[1] == 0 and vp[2] > 0 and vp[3] > 0


@pytest.mark.parametrize("name", ["test", "drops", "tiger"])
def test_reference_scenes_render_on_the_oracle(srlib, tmp_path, name):
    d, _ = rvg_scenes.load(srlib, name, tmp_path)
    for mode in (oracle.MODE_REFERENCE, oracle.MODE_PIXEL):
        f = oracle.Frame(scenes.to_oracle(d), mode=mode)
        assert f.n_intersections > 0 and f.n_draw > 0
        assert f.get("image").shape == (d["height"], d["width"], 4)


def test_full_reader_reads_arcs_and_quadratics(srlib, tmp_path):
    """The full reader keeps what RVG::load drops: 'A' segments as arcs
    (4 slots: P0, homogeneous control point, P2, (w, w)) and 'Q' segments."""
    p = tmp_path / "arc.rvg"
    p.write_text("""viewport 0,0 40,30
window 0,0 40,30
scene dyn_identity
  1 element nzfill dyn_concrete 0,0 0,0 0,0: M 2,20 A 0,-10,0 30,20 Q 16,28 2,20 Z dyn_identity dyn_paint 1 solid rgba(1,0,0,1)
""")
    ref, _ = srlib.load_rvg(str(p))
    assert ref.arrays()["curve_type"].size == 0          # the reference reader stops at the 'A'
    sc, vp = srlib.load_rvg(str(p), full=True)
    a = sc.arrays()
    assert a["curve_type"].tolist() == [0x13, 3]
    pos = a["position"].reshape(-1, 2)
    assert pos[:4].tolist() == [[2, 20], [0, -10], [30, 20], [0, 0]]
    assert pos[4:7].tolist() == [[30, 20], [16, 28], [2, 20]]


@pytest.mark.parametrize("name,arcs", [("car", 124), ("chord", 9312), ("chord-black", 9312), ("drops", 0)])
def test_full_reader_on_reference_scenes(srlib, tmp_path, name, arcs):
    d, _ = rvg_scenes.load(srlib, name, tmp_path, full=True)
    assert int((d["curve_type"] == 0x13).sum()) == arcs
    w = d["position"].reshape(-1, 2)[d["curve_pos_map"][d["curve_type"] == 0x13] + 3]
    assert np.all(w[:, 0] == w[:, 1]) and np.all(w[:, 0] > -1)

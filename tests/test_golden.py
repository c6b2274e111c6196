"""Golden fixtures (tests/golden/): the oracle must reproduce them on the CPU,
and the CUDA renderer must reproduce them on the GPU."""
import ctypes
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))
MOCK = os.path.join(HERE, "golden", "ref_mock_drawlists.npz")
STAGES = ["curve_count", "curve_offset", "intersection", "frag_key", "frag_winding", "sorted_key",
          "sorted_index", "winding_scan", "frag_flag", "span_flag", "draw_list", "image"]
SYN = {"star1024_seed0": (0, 0, 0, 0, 0), "mixed1000x750_seed7": (1, 7, 1000, 750, 1500)}


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _scene(name):
    if name in SYN:
        preset, seed, w, h, p = SYN[name]
        return oracle.synth(preset, seed, width=w, height=h, n_paths=p)
    return scenes.to_oracle(scenes.ALL[name]())


CASES = [(grp, n, m) for grp in ("synthetic", "handmade") for n in sorted(GOLD[grp]) for m in (0, 1)]


@pytest.mark.parametrize("grp,name,mode", CASES)
def test_oracle_matches_golden(grp, name, mode):
    want = GOLD[grp][name]["mode%d" % mode]
    f = oracle.Frame(_scene(name), mode=mode)
    assert f.n_intersections == want["n_intersections"] and f.n_draw == want["n_draw"]
    for s in STAGES:
        assert sha(f.get(s)) == want[s], s


def test_reference_mock_draw_lists_format():
    z = np.load(MOCK)
    for nm in ("test_data", "test_data3"):
        a = z[nm]
        frag = a[:, 3] != 0
        assert np.all(a[frag, 1] == 2)                               # FRAG_SIZE 2
        assert np.array_equal(a[frag, 3], np.arange(1, frag.sum() + 1))
        assert np.all((a[:, 0] >> 16) < 1024) and np.all((a[:, 0] & 0xFFFF) <= 1202)
        img = oracle.resolve(a, 1200, 1024, oracle.MODE_REFERENCE)
        assert np.array_equal(img, z[nm + "_image"])


@pytest.mark.gpu
@pytest.mark.parametrize("grp,name,mode", CASES)
def test_gpu_matches_golden(gpu, grp, name, mode):
    want = GOLD[grp][name]["mode%d" % mode]
    sc = _scene(name)
    r = gpu.ScanlineVGRasterizer(mode=mode, keep_stages=True)
    r.initialize(None, sc.width, sc.height)
    c = gpu.VGContainer.from_arrays(sc.width, sc.height, sc.position, sc.pos_path_idx, sc.curve_pos_map,
                                    sc.curve_type, sc.curve_path_idx, sc.fill_rule, sc.fill_info)
    if sc.paints:
        c.paints = (gpu.Paint * len(sc.paints))()
        ctypes.memmove(c.paints, sc.paints, ctypes.sizeof(gpu.Paint) * len(sc.paints))
    r.loadVG(c)
    img = r.render()
    for s in STAGES:
        got = img if s == "image" else r.dump(s)
        assert sha(got) == want[s], s
    r.close()


@pytest.mark.gpu
@pytest.mark.parametrize("nm", ["test_data", "test_data3"])
def test_gpu_paints_reference_mock_draw_lists(gpu, nm):
    z = np.load(MOCK)
    r = gpu.ScanlineVGRasterizer(mode=gpu.MODE_REFERENCE)
    r.initialize(None, 1200, 1024)
    img = r.render_draw_list(z[nm])
    assert np.array_equal(img, z[nm + "_image"])
    r.close()

"""Antialiased frames (sr_render_aa, the reference's comb-like multisampling
TODO) through the C ABI, bit-exact against the oracle's restatement: each
sample is the pixel-mode frame with the sample moved to the pixel centre, and
a pixel the rounded average of its samples."""
import numpy as np
import pytest

import rvg_scenes
import scenes

pytestmark = pytest.mark.gpu


def _render_aa(gpu, d, k, mvp=None):
    r = gpu.ScanlineVGRasterizer(mode=gpu.MODE_PIXEL)
    r.initialize(None, d["width"], d["height"])
    r.loadVG(scenes.to_container(d))
    if mvp is not None:
        r.setMVP(mvp)
    img = r.render_aa(k).copy()
    plain = r.render().copy()   # the context renders 1 spp again afterwards
    r.close()
    return img, plain


@pytest.mark.parametrize("k", [4, 16])
def test_star_scene(gpu, oracle_lib, k):
    s = oracle_lib.synth(0, 3, width=300, height=200, n_paths=60)
    d = dict(width=s.width, height=s.height, **{f: getattr(s, f) for f in oracle_lib.Scene.FIELDS})
    img, plain = _render_aa(gpu, d, k)
    assert np.array_equal(img, oracle_lib.render_aa(s, k))
    assert np.array_equal(plain, oracle_lib.Frame(s, mode=1).get("image"))


@pytest.mark.parametrize("name", ["arcs", "gradients", "translucent_layers"])
def test_handmade_scenes(gpu, oracle_lib, name):
    d = scenes.ALL[name]()
    img, _ = _render_aa(gpu, d, 8)
    assert np.array_equal(img, oracle_lib.render_aa(scenes.to_oracle(d), 8))


def test_reference_scene_with_a_matrix(gpu, oracle_lib, tmp_path):
    d, _ = rvg_scenes.load(gpu, "tiger", tmp_path, full=True)
    m = np.array([1.25, 0, 0, -20, 0, 1.25, 0, -15, 0, 0, 1, 0, 0, 0, 0, 1], np.float32)
    img, _ = _render_aa(gpu, d, 16, mvp=m)
    assert np.array_equal(img, oracle_lib.render_aa(scenes.to_oracle(d), 16, mvp=m))


def test_reference_mode_is_rejected(gpu):
    r = gpu.ScanlineVGRasterizer(mode=gpu.MODE_REFERENCE)
    r.initialize(None, 16, 16)
    r.loadVG(scenes.to_container(scenes.square()))
    with pytest.raises(gpu.SRError):
        r.render_aa(4)
    r.close()

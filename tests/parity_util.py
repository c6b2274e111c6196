"""Stage-by-stage comparison of the CUDA renderer (through the C ABI) with
the CPU oracle, shared by the GPU parity tests."""
import numpy as np

import scenes

STAGES_COMMON = ["transformed_pos", "path_visible", "cutpoints", "curve_count", "curve_offset",
                 "intersection", "frag_key", "frag_winding", "sorted_key", "sorted_index",
                 "winding_scan", "frag_flag", "span_flag", "draw_list", "image"]

# the leftover matrix of the reference (scanline_rasterizer.cpp:1157-1165), scaled down
MVP_ZOOM = np.array([1.75, 0, 0, -40.5, 0, 1.75, 0, -22.25, 0, 0, 1, 0, 0, 0, 0, 1], np.float32)


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a


def render_both(sr, oracle, d, mode, mvp=None, w=None, h=None):
    w = d["width"] if w is None else w
    h = d["height"] if h is None else h
    of = oracle.Frame(scenes.to_oracle(d), width=w, height=h, mvp=mvp, mode=mode, threads=0)
    r = sr.ScanlineVGRasterizer(mode=mode, keep_stages=True)
    r.initialize(None, w, h)
    r.loadVG(scenes.to_container(d))
    if mvp is not None:
        r.setMVP(mvp)
    img = r.render()
    return of, r, img


def compare_all(of, r, img, mode, stages=STAGES_COMMON):
    st = r.stats()
    assert st["n_intersections"] == of.n_intersections
    assert st["n_draw_records"] == of.n_draw
    assert st["n_merged_fragments"] == of.n_frag
    assert st["n_spans"] == of.n_span
    names = list(stages) + (["frag_left"] if mode == 1 else [])
    for name in names:
        a = _bits(r.dump(name))
        b = _bits(of.get(name))
        assert a.shape == b.shape, (name, a.shape, b.shape)
        if not np.array_equal(a, b):
            bad = np.argwhere(a != b)
            raise AssertionError("stage %s differs at %d places, first %s: gpu %s oracle %s" % (
                name, len(bad), bad[:3].tolist(), a[tuple(bad[0])], b[tuple(bad[0])]))
    assert np.array_equal(img, of.get("image"))

"""Stage-by-stage parity of the CUDA renderer (through the C ABI) with the
CPU oracle.  Every comparison is bit-exact: the path is integer, index and
IEEE float work with a fixed operation order on both sides."""
import numpy as np
import pytest

import scenes
from parity_util import MVP_ZOOM, _bits, compare_all, render_both

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("name", sorted(scenes.ALL))
def test_handmade_stages(gpu, oracle_lib, name, mode):
    d = scenes.ALL[name]()
    of, r, img = render_both(gpu, oracle_lib, d, mode)
    compare_all(of, r, img, mode)
    r.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_config0_stages(gpu, oracle_lib, mode):
    import oracle
    s = oracle.synth(0, 0)
    d = dict(width=s.width, height=s.height, **{f: getattr(s, f) for f in oracle.Scene.FIELDS})
    of, r, img = render_both(gpu, oracle_lib, d, mode)
    compare_all(of, r, img, mode)
    r.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_config0_zoomed_mvp(gpu, oracle_lib, mode):
    import oracle
    s = oracle.synth(0, 0)
    d = dict(width=s.width, height=s.height, **{f: getattr(s, f) for f in oracle.Scene.FIELDS})
    of, r, img = render_both(gpu, oracle_lib, d, mode, mvp=MVP_ZOOM)
    compare_all(of, r, img, mode)
    r.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_mixed_preset_small(gpu, oracle_lib, mode):
    import oracle
    s = oracle.synth(1, 7, width=1000, height=750, n_paths=1500)
    d = dict(width=s.width, height=s.height, **{f: getattr(s, f) for f in oracle.Scene.FIELDS})
    of, r, img = render_both(gpu, oracle_lib, d, mode)
    compare_all(of, r, img, mode)
    r.close()


def test_library_generator_matches_oracle_generator(gpu, oracle_lib):
    import oracle
    a = oracle.synth(1, 3, width=512, height=512, n_paths=300)
    b = gpu.synth_scene(1, 3, width=512, height=512, n_paths=300).arrays()
    for f in oracle.Scene.FIELDS:
        assert np.array_equal(_bits(getattr(a, f)), _bits(b[f])), f


def test_render_twice_identical(gpu, oracle_lib):
    """Buffers are reused across frames; a second frame must not see state of
    the first (path_visible is cleared every frame)."""
    import oracle
    s = oracle.synth(0, 5)
    d = dict(width=s.width, height=s.height, **{f: getattr(s, f) for f in oracle.Scene.FIELDS})
    r = gpu.ScanlineVGRasterizer(mode=1)
    r.initialize(None, d["width"], d["height"])
    r.loadVG(scenes.to_container(d))
    a = r.render().copy()
    r.setMVP(MVP_ZOOM)
    r.render()
    r.setMVP(np.eye(4, dtype=np.float32).reshape(16))
    b = r.render()
    assert np.array_equal(a, b)
    r.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_config1_full_size(gpu, oracle_lib, mode):
    """4096x4096, 20000 mixed paths, in pixel mode and in reference mode:
    intersections, sort order, winding scan, flags, draw list and image
    bit-exact against the oracle at full size."""
    import oracle
    s = oracle.synth(1, 1)
    d = dict(width=s.width, height=s.height, **{f: getattr(s, f) for f in oracle.Scene.FIELDS})
    of, r, img = render_both(gpu, oracle_lib, d, mode)
    compare_all(of, r, img, mode, stages=["curve_offset", "intersection", "sorted_key", "sorted_index",
                                           "winding_scan", "frag_flag", "span_flag", "draw_list", "image"])
    r.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_production_frame_equals_kept_stages_frame(gpu, oracle_lib, mode):
    """Without SR_FLAG_KEEP_STAGES the winding bits ride above the sort key
    (keys-only sort, no record-index gather); with it the sort carries record
    indices.  Both must give the same draw list and image."""
    import oracle
    s = oracle.synth(1, 3, width=1536, height=1024, n_paths=2000)
    d = dict(width=s.width, height=s.height, **{f: getattr(s, f) for f in oracle.Scene.FIELDS})
    out = []
    for keep in (True, False):
        r = gpu.ScanlineVGRasterizer(mode=mode, keep_stages=keep)
        r.initialize(None, d["width"], d["height"])
        r.loadVG(scenes.to_container(d))
        img = r.render().copy()
        out.append((img, r.dump("draw_list").copy()))
        r.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    want = oracle_lib.Frame(s, mode=mode).get("image")
    assert np.array_equal(out[1][0], want)


def test_segmented_sort_equals_radix_sort_at_full_size(gpu, oracle_lib):
    """The per-path segmented sort and the radix sort give the same draw
    list and image on the 4096x4096 20k-path frame (paths of up to ~58k
    records, several merge rounds)."""
    import oracle
    s = oracle.synth(1, 1)
    d = dict(width=s.width, height=s.height, **{f: getattr(s, f) for f in oracle.Scene.FIELDS})
    out = []
    for kind in (0, 1):
        r = gpu.ScanlineVGRasterizer(mode=1)
        r.initialize(None, d["width"], d["height"])
        r.set_tuning(sort_kind=kind)
        r.loadVG(scenes.to_container(d))
        img = r.render().copy()
        out.append((img, r.dump("draw_list").copy()))
        r.close()
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][0], out[1][0])


def test_presized_frames_and_the_overflow_rerun(gpu, oracle_lib):
    """sr_render pre-sizes a frame from the previous frame of a scene with the
    same curve and path counts and waits only at its end.  Going from a
    half-scale matrix (200k records) to the identity (367k) needs more than
    that: the frame overflows and is rerun with exact sizing.  Every image
    equals the oracle's."""
    import oracle
    s = oracle.synth(0, 0)
    d = dict(width=s.width, height=s.height, **{f: getattr(s, f) for f in oracle.Scene.FIELDS})
    half = np.array([0.5, 0, 0, 256, 0, 0.5, 0, 256, 0, 0, 1, 0, 0, 0, 0, 1], np.float32)
    ident = np.eye(4, dtype=np.float32).reshape(16)
    want_half = oracle_lib.Frame(s, mode=1, mvp=half).get("image")
    want_id = oracle_lib.Frame(s, mode=1).get("image")
    r = gpu.ScanlineVGRasterizer(mode=1)
    r.initialize(None, d["width"], d["height"])
    r.loadVG(scenes.to_container(d))
    r.setMVP(half)
    assert np.array_equal(r.render(), want_half)    # exact: first frame of the scene
    assert np.array_equal(r.render(), want_half)    # pre-sized from the first
    assert r.stats()["reruns"] == 0
    r.setMVP(ident)
    assert np.array_equal(r.render(), want_id)      # overflows, rerun exact
    assert r.stats()["reruns"] == 1
    assert np.array_equal(r.render(), want_id)      # pre-sized from the rerun
    r.loadVG(scenes.to_container(d))                # same scene again: still pre-sized
    r.setMVP(half)
    assert np.array_equal(r.render(), want_half)
    assert r.stats()["reruns"] == 1
    r.close()

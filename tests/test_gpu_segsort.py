"""The per-path segmented sort at its limits: a path too large for the merge
rounds of a pre-sized frame (the frame overflows and is redone with exact
sizing, which takes the radix sort), paths of every size class around the
tile and group bounds, and a scene of many one-record paths."""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


def _zigzag(w, h, teeth, width_px=3.0):
    # one even-odd path whose edges each cross every row: ~2*teeth*h records
    b = scenes.Builder(w, h)
    b.path(rule=1, rgba=(200, 40, 30, 180))
    pts = []
    for i in range(teeth):
        x = 4.0 + i * (w - 8.0) / teeth
        pts += [(x, 1.5), (x + width_px, h - 1.5)]
    b.polygon(pts)
    b.path(rule=0, rgba=(10, 90, 200, 120))   # a small second path after it
    b.polygon([(10.5, 10.5), (60.25, 14.0), (40.0, 70.75)])
    return b.arrays()


def _render(gpu, d, **tune):
    r = gpu.ScanlineVGRasterizer(mode=1)
    r.initialize(None, d["width"], d["height"])
    if tune:
        r.set_tuning(**tune)
    r.loadVG(scenes.to_container(d))
    img = r.render().copy()
    n = r.stats()["n_intersections"]
    r.close()
    return img, n


def test_path_beyond_merge_rounds_uses_radix_sort(gpu, oracle_lib):
    d = _zigzag(1024, 1024, 96)
    want = oracle_lib.Frame(scenes.to_oracle(d), mode=1).get("image")
    img, n = _render(gpu, d)
    assert n > 4096 * 32                       # more than five merge rounds of 4096-record chunks
    assert np.array_equal(img, want)
    img1, _ = _render(gpu, d, sort_kind=1)
    assert np.array_equal(img1, want)
    # pre-sized: the tables flag the path, the frame is redone with exact sizing
    b = gpu.SceneBatch(mode=1)
    b.add_scene(scenes.to_container(d))
    b.render(capacity=n, graph=False, refit=True)
    st = b.stats()
    assert st["overflows"] >= 1 and st["refits"] >= 1
    assert np.array_equal(b.image(0), want)
    b.close()


@pytest.mark.parametrize("teeth", [1, 2, 3, 4, 7, 9, 15])
def test_paths_around_tile_bounds(gpu, oracle_lib, teeth):
    # path sizes around 2048 (group bound) and 4096 (tile) records, several merge rounds
    d = _zigzag(512, 512, teeth, width_px=1.5)
    want = oracle_lib.Frame(scenes.to_oracle(d), mode=1).get("image")
    img, _ = _render(gpu, d)
    assert np.array_equal(img, want)


def test_many_tiny_paths(gpu, oracle_lib):
    rng = np.random.default_rng(3)
    b = scenes.Builder(300, 200)
    for i in range(3000):
        x, y = rng.uniform(0, 300), rng.uniform(0, 200)
        b.path(rule=int(i % 2), rgba=(int(i % 251), 90, 30, 100 + i % 150))
        b.polygon([(x, y), (x + 0.7, y + 0.2), (x + 0.3, y + 0.8)])
    d = b.arrays()
    want = oracle_lib.Frame(scenes.to_oracle(d), mode=1).get("image")
    img, _ = _render(gpu, d)
    assert np.array_equal(img, want)


def _scattered(w, h, n, seed):
    # many small paths spread over a wide canvas (some reaching past its
    # edges): a tile holds paths far apart, so its packed key fields need
    # more than the 32-bit items' bits and it is sorted with 64-bit items
    rng = np.random.default_rng(seed)
    b = scenes.Builder(w, h)
    for i in range(n):
        x, y = rng.uniform(-8, w + 8), rng.uniform(-8, h + 8)
        s = rng.uniform(2.0, 9.0)
        b.path(rule=int(i % 2), rgba=(int(i % 251), 90, 30, 100 + i % 150))
        b.polygon([(x, y), (x + s, y + 0.3 * s), (x + 0.4 * s, y + s)])
    return b.arrays()


@pytest.mark.parametrize("w,h,n,seed", [(16384, 1024, 2500, 5), (4096, 4096, 3000, 6)])
def test_tiles_sorted_with_64bit_items(gpu, oracle_lib, w, h, n, seed):
    d = _scattered(w, h, n, seed)
    of = oracle_lib.Frame(scenes.to_oracle(d), mode=1)
    r = gpu.ScanlineVGRasterizer(mode=1)
    r.initialize(None, w, h)
    r.loadVG(scenes.to_container(d))
    img = r.render()
    tiles, wide = r.sort_tiles()
    assert tiles > 0 and wide > 0
    # the draw list follows the sorted order record by record
    assert np.array_equal(r.dump("draw_list"), of.get("draw_list"))
    assert np.array_equal(img, of.get("image"))
    r.close()

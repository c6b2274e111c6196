"""Batches of uneven scenes (sr_batch_*): every scene's image must be the one
the oracle paints for that scene alone, whatever the sizing mode."""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


def _oracle_images(oracle, scs, mode):
    return [oracle.Frame(s, mode=mode).get("image") for s in scs]


def _container(sr, s):
    return sr.VGContainer.from_arrays(s.width, s.height, s.position, s.pos_path_idx, s.curve_pos_map,
                                      s.curve_type, s.curve_path_idx, s.fill_rule, s.fill_info)


def _mixed_scenes(oracle):
    out = [oracle.synth(2, 2, scene_index=i) for i in range(6)]
    out += [scenes.to_oracle(scenes.ALL[n]()) for n in ("square", "star_evenodd", "offcanvas", "degenerate")]
    out.append(oracle.synth(0, 3, width=300, height=200, n_paths=40))   # odd canvas
    return out


@pytest.mark.parametrize("mode", [0, 1])
def test_batch_images_equal_oracle_and_single_renders(gpu, oracle_lib, mode):
    scs = _mixed_scenes(oracle_lib)
    want = _oracle_images(oracle_lib, scs, mode)
    b = gpu.SceneBatch(mode=mode)
    for s in scs:
        b.add_scene(_container(gpu, s))
    b.render()
    for i, w in enumerate(want):
        assert np.array_equal(b.image(i), w), "scene %d" % i
    st = b.stats()
    assert st["n_scenes"] == len(scs)
    # the batch's records are the sum of the scenes' records
    n_single = 0
    for s in scs:
        r = gpu.ScanlineVGRasterizer(mode=mode)
        r.initialize(None, s.width, s.height)
        r.loadVG(_container(gpu, s))
        r.render()
        n_single += r.stats()["n_intersections"]
        r.close()
    assert st["n_intersections"] == n_single
    b.close()


def test_capacity_overflow_refit_and_graph_replay(gpu, oracle_lib):
    scs = _mixed_scenes(oracle_lib)
    want = _oracle_images(oracle_lib, scs, 1)
    b = gpu.SceneBatch(mode=1)
    for s in scs:
        b.add_scene(_container(gpu, s))
    b.render()
    n = b.stats()["n_intersections"]
    # exact capacity, no mid-frame wait
    b.render(capacity=n)
    assert all(np.array_equal(b.image(i), w) for i, w in enumerate(want))
    # too small: detected on the device, rerun with exact sizing
    b.render(capacity=n // 2, refit=True)
    st = b.stats()
    assert st["overflows"] == 1 and st["refits"] == 1
    assert all(np.array_equal(b.image(i), w) for i, w in enumerate(want))
    # too small without refit: an overflow status, not wrong pixels
    with pytest.raises(gpu.SRError) as ei:
        b.render(capacity=n // 2, refit=False)
    assert ei.value.code == 3
    # captured graph, replayed three times
    for _ in range(3):
        b.render(capacity=n + 1000, graph=True)
        assert b.stats()["graph_captured"] == 1
        assert all(np.array_equal(b.image(i), w) for i, w in enumerate(want))
    b.close()


def test_batch_synth_matches_oracle_synth(gpu, oracle_lib):
    b = gpu.SceneBatch(mode=1)
    first = b.add_synth(2, 9, 5)
    b.render()
    for i in range(5):
        s = oracle_lib.synth(2, 9, scene_index=i)
        assert b.size(first + i) == (s.width, s.height)
        assert np.array_equal(b.image(first + i), oracle_lib.Frame(s, mode=1).get("image"))
    b.close()


@pytest.mark.parametrize("tuning", [(8, 8, 4, 1), (16, 16, 8, 1), (12, 8, 8, 0), (8, 16, 4, 0)])
def test_every_tuning_gives_the_same_images(gpu, oracle_lib, tuning):
    scs = _mixed_scenes(oracle_lib)
    want = _oracle_images(oracle_lib, scs, 1)
    b = gpu.SceneBatch(mode=1)
    for s in scs:
        b.add_scene(_container(gpu, s))
    b.set_tuning(*tuning)
    b.render()
    for i, w in enumerate(want):
        assert np.array_equal(b.image(i), w), (tuning, i)
    b.render(capacity=b.stats()["n_intersections"], graph=True)
    for i, w in enumerate(want):
        assert np.array_equal(b.image(i), w), (tuning, i)
    b.close()


def test_autotune_caches_its_choice(gpu, tmp_path):
    import json
    path = str(tmp_path / "tuning.json")
    b = gpu.SceneBatch(mode=1)
    b.add_synth(2, 9, 16)
    t1 = b.autotune(path)
    cls = b.tuning_class()
    with open(path) as f:
        cache = json.load(f)
    assert cache[cls]["sort_items"] == t1["sort_items"] and cache[cls]["frame_ms"] > 0
    # a second batch of the same class takes the cached choice without timing
    b2 = gpu.SceneBatch(mode=1)
    b2.add_synth(2, 9, 16)
    b2.set_tuning(16 if t1["sort_items"] != 16 else 8, 8 if t1["resolve_warps"] != 8 else 16, 4)
    assert b2.autotune(path) == t1
    b.close()
    b2.close()


def test_reserve_like_grows_buffers_and_keeps_images(gpu, oracle_lib):
    # a small batch grown like a large one renders the same images; its
    # scenes are uploaded again after its buffers moved
    big = gpu.SceneBatch(mode=1)
    big.add_synth(2, 7, 24)
    big.render()
    scs = [oracle_lib.synth(2, 8, scene_index=i) for i in range(2)]
    want = _oracle_images(oracle_lib, scs, 1)
    small = gpu.SceneBatch(mode=1)
    for s in scs:
        small.add_scene(_container(gpu, s))
    small.render()
    assert all(np.array_equal(small.image(i), w) for i, w in enumerate(want))
    before = small.held_bytes()
    small.reserve_like(big)
    assert small.held_bytes() >= big.held_bytes() > before
    small.reserve_like(big)   # nothing moves the second time
    small.render()
    assert all(np.array_equal(small.image(i), w) for i, w in enumerate(want))
    n = small.stats()["n_intersections"]
    small.render(capacity=n, graph=True)   # a captured frame on the grown buffers
    assert all(np.array_equal(small.image(i), w) for i, w in enumerate(want))
    big.close()
    small.close()

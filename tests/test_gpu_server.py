"""The continuous-batching render server on the GPU: every request's image
equals the same scene rendered alone (and the oracle's), whether it is
served alone or in a mix of concurrent requests, with learned or exact
sizing, under a tight memory budget, and when the sizes are forced low."""
import threading

import numpy as np
import pytest

import sizing_util

pytestmark = pytest.mark.gpu


def _container(sr, s):
    return sr.VGContainer.from_arrays(s.width, s.height, s.position, s.pos_path_idx, s.curve_pos_map,
                                      s.curve_type, s.curve_path_idx, s.fill_rule, s.fill_info)


@pytest.fixture(scope="module")
def sizer(gpu):
    sz, _, _, _ = sizing_util.train_sizer(gpu, [301, 302], epochs=16)
    yield sz
    sz.close()


def _alone(sr, sc):
    r = sr.ScanlineVGRasterizer(mode=sr.MODE_PIXEL)
    r.initialize(None, sc.width, sc.height)
    r.loadVG(sc)
    img = r.render()
    r.close()
    return img


def test_alone_and_in_the_mix_give_the_same_image(gpu, oracle_lib, sizer):
    target = oracle_lib.synth(1, 77, width=384, height=320, n_paths=150)
    want = oracle_lib.Frame(target, mode=1).get("image")
    tc = _container(gpu, target)
    srv = gpu.RenderServer(sizer=sizer, slots=3, max_batch_scenes=16)
    t = srv.submit(tc)
    alone, info = srv.wait(t)
    assert np.array_equal(alone, want)
    assert info["batch_scenes"] == 1
    # the same scene among concurrent requests from two client threads
    others = [gpu.synth_scene(2, 5, scene_index=i) for i in range(40)]
    tickets = {}

    def client(lo, hi):
        for i in range(lo, hi):
            tickets[i] = srv.submit(others[i])
            if i == 25:
                tickets["target"] = srv.submit(tc)
    th = [threading.Thread(target=client, args=(0, 20)), threading.Thread(target=client, args=(20, 40))]
    for x in th:
        x.start()
    for x in th:
        x.join()
    mixed, info = srv.wait(tickets.pop("target"))
    assert np.array_equal(mixed, want)
    for i, tk in sorted(tickets.items()):
        img, inf = srv.wait(tk)
        assert inf["status"] == 0
        if i % 8 == 0:
            assert np.array_equal(img, _alone(gpu, others[i])), i
    st = srv.stats()
    assert st["completed"] == st["submitted"] == 42
    assert st["batches"] >= 3
    srv.close()


def test_exact_sizing_server_gives_the_same_images(gpu):
    scs = [gpu.synth_scene(2, 6, scene_index=i) for i in range(12)]
    srv = gpu.RenderServer(sizer=None, slots=2, max_batch_scenes=5)
    tk = [srv.submit(s) for s in scs]
    for s, t in zip(scs, tk):
        img, info = srv.wait(t)
        assert np.array_equal(img, _alone(gpu, s))
        assert info["batch_scenes"] <= 5
    srv.close()


def test_memory_budget_limits_what_is_in_flight(gpu, sizer):
    scs = [gpu.synth_scene(2, 7, scene_index=i) for i in range(24)]
    # learn the largest single-request share with a generous budget
    srv = gpu.RenderServer(sizer=sizer, slots=2, max_batch_scenes=1)
    shares = []
    for s in scs:
        img, info = srv.wait(srv.submit(s), fetch=False)
        shares.append(info["predicted_bytes"])
    srv.close()
    budget = int(max(shares) * 1.5)
    srv = gpu.RenderServer(sizer=sizer, slots=4, max_batch_scenes=8, memory_budget=budget)
    tk = [srv.submit(s) for s in scs]
    for s, t in zip(scs, tk):
        img, info = srv.wait(t)
        assert np.array_equal(img, _alone(gpu, s))
    st = srv.stats()
    assert st["peak_bytes"] <= budget
    assert st["budget_waits"] > 0
    srv.close()
    # a request larger than the whole budget is refused, the others still run
    srv = gpu.RenderServer(sizer=sizer, slots=2, max_batch_scenes=4, memory_budget=min(shares) // 2)
    t = srv.submit(scs[0])
    with pytest.raises(gpu.SRError):
        srv.wait(t)
    assert srv.stats()["rejected"] == 1
    srv.close()


def test_forced_low_sizes_fall_back_to_exact_count(gpu, sizer):
    scs = [gpu.synth_scene(2, 8, scene_index=i) for i in range(10)]
    srv = gpu.RenderServer(sizer=sizer, slots=2, max_batch_scenes=5, margins=(-3.0, -3.0, -3.0, -3.0))
    tk = [srv.submit(s) for s in scs]
    refit = 0
    for s, t in zip(scs, tk):
        img, info = srv.wait(t)
        refit += info["refit"]
        assert np.array_equal(img, _alone(gpu, s))
    st = srv.stats()
    assert st["overflows"] >= 1 and st["refits"] >= 1 and refit >= 1
    srv.close()

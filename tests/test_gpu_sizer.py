"""Learned sizing on the GPU (sr_sizer_*, sr_batch_plan/judge): features,
labels, gradients, Adam and predictions against the CPU restatements, and
sizing that changes no pixel.

Tolerances: the GPU network computes in FP32 with BF16 weights, the CPU
restatement in float64 with the same BF16 weights.  Predictions and loss
agree to 1e-4 relative; gradients to 2e-3 of the largest gradient entry;
features (FP32 sums, sqrtf/atan2f/log1pf) to 1e-4 relative.  Labels are
integers and must be exact."""
import numpy as np
import pytest

from oracle import mlp_ref as M

import sizing_util

pytestmark = pytest.mark.gpu


def _scenes(oracle, n=5):
    # preset-1 paths on small canvases so the oracle finishes quickly
    return [oracle.synth(1, 40 + i, width=256 + 64 * i, height=256, n_paths=120) for i in range(n)]


def _container(sr, s):
    return sr.VGContainer.from_arrays(s.width, s.height, s.position, s.pos_path_idx, s.curve_pos_map,
                                      s.curve_type, s.curve_path_idx, s.fill_rule, s.fill_info)


def _batch(sr, scs, mode=1):
    b = sr.SceneBatch(mode=mode)
    for s in scs:
        b.add_scene(_container(sr, s))
    b.commit()
    return b


@pytest.mark.parametrize("mode", [1, 0])
def test_features_and_labels_match_oracle(gpu, oracle_lib, mode):
    scs = _scenes(oracle_lib)
    b = _batch(gpu, scs, mode)
    feats = b.features().numpy()
    labels = b.labels().numpy()
    F = 1 if mode == 1 else 2
    off = 0
    for s in scs:
        fr = oracle_lib.Frame(s, mode=mode)
        tpos = fr.get("transformed_pos").view(np.float32).reshape(-1, 2)
        P = len(s.fill_rule)
        want_f = M.path_features(tpos, s.curve_pos_map, s.curve_type, s.curve_path_idx, P, s.width, s.height, F)
        got_f = feats[off:off + P]
        assert np.allclose(got_f, want_f, rtol=1e-4, atol=1e-5)
        want_l = M.path_labels(fr.get("curve_count"), s.curve_path_idx, fr.get("path_draws"), P)
        got_l = np.rint(np.expm1(labels[off:off + P].astype(np.float64))).astype(np.int64)
        assert np.array_equal(got_l, want_l)
        off += P
    assert off == feats.shape[0]
    b.close()


def _data(gpu, oracle_lib):
    b = _batch(gpu, _scenes(oracle_lib, 3))
    x = b.features()
    t = b.labels()
    return b, x, t


def test_loss_gradient_and_prediction_match_restatement(gpu, oracle_lib):
    b, x, t = _data(gpu, oracle_lib)
    xh, th = x.numpy(), t.numpy()
    sz = gpu.Sizer(seed=7)
    norm = gpu.sizer_norm(xh, th)
    sz.set_norm(norm)
    params = sz.state()["params"]
    loss, g = sz.loss_grad(x, t)
    want_loss, want_g = M.loss_grad(params, norm, xh, th)
    assert loss == pytest.approx(want_loss, rel=1e-4)
    scale = np.abs(want_g).max()
    assert np.abs(g - want_g).max() <= 2e-3 * scale, np.abs(g - want_g).max() / scale
    y = sz.predict(x).numpy()
    assert np.allclose(y, M.forward(params, norm, xh), rtol=1e-4, atol=1e-4)
    sz.close()
    b.close()


def test_adam_step_matches_restatement(gpu, oracle_lib):
    b, x, t = _data(gpu, oracle_lib)
    xh, th = x.numpy(), t.numpy()
    sz = gpu.Sizer(seed=3)
    norm = gpu.sizer_norm(xh, th)
    sz.set_norm(norm)
    p0 = sz.state()["params"]
    _, g = M.loss_grad(p0, norm, xh, th)
    # one full-batch step in row order
    sz.train(x, t, epochs=1, batch=x.shape[0], shuffle=False, lr=1e-3)
    st = sz.state()
    p1, m1, v1 = M.adam_step(p0, np.zeros_like(p0), np.zeros_like(p0), g, 1, lr=1e-3)
    assert st["step"] == 1
    strong = np.abs(g) > 1e-2 * np.abs(g).max()   # the sign of tiny gradients is rounding
    assert np.allclose(st["params"][strong], p1[strong], atol=2e-6)
    assert np.allclose(st["adam_m"], m1, atol=2e-3 * 0.1 * np.abs(g).max())
    sz.close()
    b.close()


def test_state_round_trip(gpu, oracle_lib, tmp_path):
    b, x, t = _data(gpu, oracle_lib)
    sz = gpu.Sizer(seed=5)
    sz.set_norm(gpu.sizer_norm(x.numpy(), t.numpy()))
    sz.train(x, t, epochs=3, batch=256, seed=1)
    path = str(tmp_path / "sizer.npz")
    sz.save(path)
    sz2 = gpu.Sizer(seed=99)
    sz2.load(path)
    assert sz2.state()["step"] == sz.state()["step"]
    assert np.array_equal(sz.predict(x).numpy(), sz2.predict(x).numpy())
    sz.close()
    sz2.close()
    b.close()


def _train_on_batches(gpu, seeds, epochs=40):
    return sizing_util.train_sizer(gpu, seeds, epochs=epochs)


def _overalloc(pred, exact, frac=0.01):
    """Margin that leaves `frac` of the paths over their allotment, and the
    resulting sum(allotment) / sum(exact)."""
    r = np.log1p(exact) - pred
    m = float(np.quantile(r, 1.0 - frac))
    allot = np.ceil(np.expm1(np.minimum(pred + m, 21.0)))
    return m, allot.sum() / max(exact.sum(), 1), float((exact > allot).mean())


def test_trained_sizer_beats_sizing_without_it(gpu):
    sz, x, t, losses = _train_on_batches(gpu, [101, 102, 103])
    assert losses[-1] < losses[0]
    # held-out scenes
    b = gpu.SceneBatch(mode=1)
    b.add_synth(2, 104, 24)
    b.commit()
    xv = b.features()
    tv = b.labels().numpy().astype(np.float64)
    exact = np.rint(np.expm1(tv[:, 0]))
    pred = sz.predict(xv).numpy()[:, 0].astype(np.float64)
    _, over_mlp, _ = _overalloc(pred, exact)
    # without the network: a per-segment rule fitted on the training rows
    xt, tt = x.numpy().astype(np.float64), t.numpy().astype(np.float64)
    segs_t = np.expm1(xt[:, 0])
    rate = np.expm1(tt[:, 0]).sum() / segs_t.sum()
    rule = np.log1p(rate * np.expm1(xv.numpy()[:, 0].astype(np.float64)))
    _, over_rule, _ = _overalloc(rule, exact)
    # an untrained network with the same normaliser
    raw = gpu.Sizer(seed=11)
    raw.set_norm(sz.state()["norm"])
    _, over_raw, _ = _overalloc(raw.predict(xv).numpy()[:, 0].astype(np.float64), exact)
    assert over_mlp < over_rule and over_mlp < over_raw, (over_mlp, over_rule, over_raw)
    raw.close()
    sz.close()
    b.close()


def test_planned_frames_change_no_pixel(gpu):
    sz, x, t, _ = _train_on_batches(gpu, [201, 202], epochs=16)
    ref = gpu.SceneBatch(mode=1)
    ref.add_synth(2, 205, 12)
    ref.render()
    want = [ref.image(i) for i in range(12)]
    n_exact = ref.stats()["n_intersections"]
    b = gpu.SceneBatch(mode=1)
    b.add_synth(2, 205, 12)
    b.commit()
    plan = b.plan(sz, (0.7, 0.7, 0.3, 0.3), per_scene=True)
    assert plan["scenes"][:, 0].sum() == plan["records"]
    assert plan["path_records"] >= plan["records"] and plan["draws"] <= 2 * plan["records"]
    assert plan["device_bytes"] == b.frame_bytes(plan["records"], plan["draws"])
    b.render(capacity=plan["records"], draw_capacity=plan["draws"], graph=True, refit=True)
    for i in range(12):
        assert np.array_equal(b.image(i), want[i]), i
    j = b.judge()
    assert j["records"] == n_exact and j["paths"] == b.n_paths()
    assert 0 <= j["paths_over_records"] <= j["paths"]
    # a forced under-prediction overflows on the device and falls back to the exact count pass
    low = b.plan(sz, (-3.0, -3.0, -3.0, -3.0))
    assert low["records"] < n_exact
    b.render(capacity=low["records"], draw_capacity=low["draws"], graph=False, refit=True)
    st = b.stats()
    assert st["overflows"] >= 1 and st["refits"] >= 1
    for i in range(12):
        assert np.array_equal(b.image(i), want[i]), i
    sz.close()
    b.close()
    ref.close()

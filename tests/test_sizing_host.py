"""Host-side sizing logic (no GPU): margin calibration from held-out rows."""
import numpy as np

import vkscanlinepr_gb300 as sr


def test_calibrated_margins_cover_each_scene_and_quantile_of_paths():
    rng = np.random.default_rng(0)
    P = 4000
    exact = rng.integers(0, 5000, (P, 2)).astype(np.float64)
    lab = np.log1p(exact)
    pred = lab + rng.normal(0, 0.3, (P, 2))
    ranges = np.array([0, 700, 1500, 2600, 4000])
    m = sr.calibrate_margins(pred, lab, ranges, path_quantile=0.99, frame_slack=0.0)
    for o in range(2):
        allot = np.ceil(np.expm1(pred[:, o] + m[o]))
        frac = (exact[:, o] > allot).mean()
        assert frac <= 0.0101
        cap = np.ceil(np.expm1(pred[:, o] + m[2 + o])).clip(0)
        for s in range(4):
            a, b = ranges[s], ranges[s + 1]
            assert cap[a:b].sum() >= exact[a:b, o].sum()
        # errors of many paths average out: the frame margin is the smaller one
        assert m[2 + o] < m[o]


def test_empty_scenes_are_skipped():
    pred = np.zeros((3, 2))
    lab = np.zeros((3, 2))
    m = sr.calibrate_margins(pred, lab, np.array([0, 0, 3]), frame_slack=0.01)
    assert m[2] == 0.01 and m[3] == 0.01

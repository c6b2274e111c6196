"""Seeded synthetic scenes: deterministic, identical across the library and
the oracle build, and shaped like the configurations they stand for."""
import numpy as np

import oracle


def _bits(a):
    return a.view(np.uint32) if a.dtype == np.float32 else a


def test_deterministic_and_seed_sensitive():
    a = oracle.synth(1, 3, width=512, height=512, n_paths=200)
    b = oracle.synth(1, 3, width=512, height=512, n_paths=200)
    c = oracle.synth(1, 4, width=512, height=512, n_paths=200)
    assert np.array_equal(_bits(a.position), _bits(b.position))
    assert not np.array_equal(a.position[:50], c.position[:50])


def test_library_and_oracle_generators_agree(srlib):
    a = oracle.synth(1, 11, width=700, height=500, n_paths=400)
    b = srlib.synth_scene(1, 11, width=700, height=500, n_paths=400).arrays()
    for f in oracle.Scene.FIELDS:
        assert np.array_equal(_bits(getattr(a, f)), _bits(b[f])), f


def test_star_preset_shape():
    s = oracle.synth(0, 0)
    assert (s.width, s.height, s.n_paths) == (1024, 1024, 500)
    per_path = np.bincount(s.curve_path_idx, minlength=500)
    assert per_path.min() >= 4 and per_path.max() <= 16
    assert np.all(s.curve_type == 4) and np.all(s.fill_rule == 0)
    alpha = s.fill_info >> 24
    assert alpha.min() >= 102 and alpha.max() <= 255


def test_mixed_preset_shape():
    s = oracle.synth(1, 1)
    assert (s.width, s.height, s.n_paths) == (4096, 4096, 20000)
    t = s.curve_type
    frac = [np.mean(t == k) for k in (4, 3, 2)]
    assert 0.5 < frac[0] < 0.65 and 0.25 < frac[1] < 0.33 and 0.09 < frac[2] < 0.16
    assert 0.27 < np.mean(s.fill_rule == 1) < 0.33
    # every point belongs to its curve's path
    assert np.array_equal(s.pos_path_idx[s.curve_pos_map], s.curve_path_idx)

"""Structural invariants of the oracle's stages on seeded synthetic scenes."""
import numpy as np
import pytest

import oracle


@pytest.fixture(scope="module", params=[(0, 0, 0, 0, 0), (1, 7, 640, 480, 600)])
def frames(request):
    preset, seed, w, h, p = request.param
    sc = oracle.synth(preset, seed, width=w, height=h, n_paths=p)
    return sc, {m: oracle.Frame(sc, mode=m) for m in (0, 1)}


def test_offsets_are_scan_of_counts(frames):
    sc, fr = frames
    for f in fr.values():
        cnt = f.get("curve_count").astype(np.int64)
        off = f.get("curve_offset").astype(np.int64)
        assert off[0] == 0 and np.array_equal(np.diff(off), cnt) and off[-1] == f.n_intersections


def test_records_grouped_by_curve_in_order(frames):
    sc, fr = frames
    for f in fr.values():
        rec = f.get("intersection")
        assert np.all(np.diff(rec[:, 0]) >= 0)


def test_sorted_keys_sorted_within_paths_and_permutation(frames):
    sc, fr = frames
    for f in fr.values():
        key = f.get("sorted_key")
        idx = f.get("sorted_index")
        fk = f.get("frag_key")
        assert np.array_equal(np.sort(idx), np.arange(idx.size))
        assert np.array_equal(fk[idx], key)
        path = sc.curve_path_idx[f.get("intersection")[:, 0]]
        same = path[1:] == path[:-1]
        k = key.astype(np.int64)
        assert np.all((k[1:] > k[:-1]) | ((k[1:] == k[:-1]) & (idx[1:] > idx[:-1])) | ~same)


def test_winding_scan_is_exclusive_scan_of_sorted_changes(frames):
    sc, fr = frames
    for f in fr.values():
        wn = f.get("frag_winding")[f.get("sorted_index")]
        ws = f.get("winding_scan").astype(np.int64)
        assert ws[0] == 0 and np.array_equal(np.diff(ws), wn)


def test_draw_list_format(frames):
    sc, fr = frames
    for mode, f in fr.items():
        d = f.get("draw_list")
        frag = d[:, 3] != 0
        F = 1 if mode == 1 else 2
        assert np.all(d[frag, 1] == F)
        assert np.array_equal(d[frag, 3], np.arange(1, frag.sum() + 1))
        assert np.all(d[~frag, 1] >= 1)
        assert frag.sum() == f.n_frag and (~frag).sum() == f.n_span


def test_pixel_mode_alpha_stays_opaque(frames):
    sc, fr = frames
    assert np.all(fr[1].get("image")[:, :, 3] == 255)


def test_thread_count_does_not_change_results(frames):
    sc, fr = frames
    one = oracle.Frame(sc, mode=1, threads=1)
    for s in ("sorted_index", "winding_scan", "draw_list", "image"):
        assert np.array_equal(one.get(s), fr[1].get(s))

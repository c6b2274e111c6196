"""Writes the golden fixtures under tests/golden/.

  ref_mock_drawlists.npz   the reference's own mock draw lists
                           (workdir/test_data.csv, workdir/test_data3.csv,
                           loaded by scanline_rasterizer.cpp:261-281 in its
                           MOCK_DATA mode), as int32 (n, 4) arrays, plus the
                           RGBA8 image the oracle paints from each on the
                           reference's 1200x1024 viewport (scanlinepr.vert:39)
  golden.json              per scene and mode: record counts and the
                           SHA-256 of every stage the oracle produces for the
                           seeded synthetic scenes and the hand-made scenes

Run from the repository root; the mock draw lists are read from the
reference's workdir given as the argument (only this script reads it; the
fixtures it writes travel with the repository):

  python tests/golden/make_golden.py [<reference>/workdir]
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
import scenes  # noqa: E402

STAGES = ["curve_count", "curve_offset", "intersection", "frag_key", "frag_winding", "sorted_key",
          "sorted_index", "winding_scan", "frag_flag", "span_flag", "draw_list", "image"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def frame_record(scene, mode, **kw):
    f = oracle.Frame(scene, mode=mode, **kw)
    rec = {"n_intersections": f.n_intersections, "n_draw": f.n_draw, "n_frag": f.n_frag, "n_span": f.n_span}
    for s in STAGES:
        rec[s] = sha(f.get(s))
    return rec


def main(ref=None):
    out = {"synthetic": {}, "handmade": {}}
    for name, (preset, seed, w, h, p) in {"star1024_seed0": (0, 0, 0, 0, 0),
                                           "mixed1000x750_seed7": (1, 7, 1000, 750, 1500)}.items():
        sc = oracle.synth(preset, seed, width=w, height=h, n_paths=p)
        out["synthetic"][name] = {"preset": preset, "seed": seed, "width": sc.width, "height": sc.height,
                                  "paths": int(sc.n_paths), "scene_sha": sha(sc.position)}
        for mode in (0, 1):
            out["synthetic"][name]["mode%d" % mode] = frame_record(sc, mode)
    for name, fn in sorted(scenes.ALL.items()):
        d = fn()
        out["handmade"][name] = {}
        for mode in (0, 1):
            out["handmade"][name]["mode%d" % mode] = frame_record(scenes.to_oracle(d), mode)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)

    if ref and os.path.isdir(ref):
        arrays = {}
        for nm in ("test_data", "test_data3"):
            a = np.loadtxt(os.path.join(ref, nm + ".csv"), delimiter=",", dtype=np.int64).astype(np.int32)
            arrays[nm] = a
            arrays[nm + "_image"] = oracle.resolve(a, 1200, 1024, oracle.MODE_REFERENCE, threads=4)
        np.savez_compressed(os.path.join(HERE, "ref_mock_drawlists.npz"), **arrays)
    print("golden fixtures written")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)

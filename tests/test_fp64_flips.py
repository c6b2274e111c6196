"""Samples that flip against the FP64 oracle, per scene.

The renderer computes intersections in FP32 with the oracle's operation order
(bit-exact to the oracle's FP32 instance).  The oracle's FP64 instance (double
arithmetic, 52 bisection steps) shows how many of the 1-sample-per-pixel
samples that FP32 decides differently.  The counts are deterministic; these
are the values for the seeded synthetic scenes and the reference's shipped
scenes, in reference mode (0) and pixel mode (1)."""
import pytest

import oracle
import rvg_scenes
import scenes

SYNTH = {
    # name: (preset, seed, width, height, paths) -> flips in mode 0, mode 1
    "star1024_seed0": ((0, 0, 0, 0, 0), (0, 1)),
    "mixed1000x750_seed7": ((1, 7, 1000, 750, 1500), (0, 1)),
    "mixed2048_seed1": ((1, 1, 2048, 2048, 5000), (46076, 2)),
}
RVG = {"car": (0, 0), "chord": (0, 0), "chord-black": (0, 0), "drops": (0, 0), "embrace": (0, 1),
       "reschart": (0, 0), "test": (0, 0), "tiger": (4, 1)}


@pytest.mark.parametrize("name", sorted(SYNTH))
def test_synthetic_scene_flips(name):
    (preset, seed, w, h, p), want = SYNTH[name]
    s = oracle.synth(preset, seed, width=w, height=h, n_paths=p)
    assert tuple(oracle.fp64_flips(s, mode) for mode in (0, 1)) == want


@pytest.mark.parametrize("name", sorted(RVG))
def test_reference_scene_flips(srlib, tmp_path, name):
    d, _ = rvg_scenes.load(srlib, name, tmp_path)
    s = scenes.to_oracle(d)
    assert tuple(oracle.fp64_flips(s, mode) for mode in (0, 1)) == RVG[name]


def test_a_planted_difference_is_counted():
    s = oracle.synth(0, 0, width=256, height=256, n_paths=40)
    img = oracle.Frame(s, mode=1).get("image").copy()
    base = oracle.fp64_flips(s, 1, image=img)
    img[3, 5, 0] ^= 0xFF
    img[7, 9, 2] ^= 0x01
    assert oracle.fp64_flips(s, 1, image=img) == base + 2

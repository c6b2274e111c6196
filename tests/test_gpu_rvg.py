"""The reference's eight shipped RVG scenes (tests/golden/rvg), rendered by
the CUDA renderer through the C ABI and compared stage by stage with the
oracle, in reference mode (the reference's own semantics: 2x2 cells, whole
boundary cells, the last path wins) and in pixel mode.  The scenes are read
by the library's RVG reader, which follows the reference's RVG::load; the arc
scenes (chord, chord-black) stop at their first arc as the reference's reader
does, and render as empty canvases."""
import pytest

import rvg_scenes
from parity_util import STAGES_COMMON, compare_all, render_both

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("name", rvg_scenes.NAMES)
def test_reference_scene_stages(gpu, oracle_lib, tmp_path, name, mode):
    d, _ = rvg_scenes.load(gpu, name, tmp_path)
    of, r, img = render_both(gpu, oracle_lib, d, mode)
    compare_all(of, r, img, mode, stages=STAGES_COMMON)
    r.close()


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("name", ["car", "chord", "chord-black", "drops", "embrace"])
def test_full_reader_scene_stages(gpu, oracle_lib, tmp_path, name, mode):
    """The same scenes read in full (arcs as rational quadratics, linear and
    radial gradient paints): every stage bit-exact against the oracle,
    including the arcs' transformed slots, monotonic cuts and bisected
    crossings, and every gradient pixel of the image."""
    d, _ = rvg_scenes.load(gpu, name, tmp_path, full=True)
    of, r, img = render_both(gpu, oracle_lib, d, mode)
    compare_all(of, r, img, mode, stages=STAGES_COMMON)
    r.close()


def test_rendered_scene_written_as_png(gpu, oracle_lib, tmp_path):
    """The headless stand-in for the reference's swapchain: the frame read
    back to host memory and written as a PNG file holds the same pixels."""
    from test_image_writer import _read_png
    d, _ = rvg_scenes.load(gpu, "tiger", tmp_path)
    of, r, img = render_both(gpu, oracle_lib, d, 0)
    r.close()
    gpu.write_image(tmp_path / "tiger.png", img)
    assert img.shape == (d["height"], d["width"], 4)
    assert (_read_png(tmp_path / "tiger.png") == of.get("image")).all()

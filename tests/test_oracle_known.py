"""Known-answer scenes for the CPU oracle, each answer derived by hand."""
import math

import numpy as np

import oracle
import scenes


def covered(img):
    return np.any(img != 255, axis=2)


def render(d, mode, **kw):
    return oracle.Frame(scenes.to_oracle(d), mode=mode, **kw)


def test_square_pixel_mode_is_exact():
    # pixel centres inside [2,6)x[2,6); edges on integer lines
    img = render(scenes.square(), oracle.MODE_PIXEL).get("image")
    want = np.zeros((8, 8), bool)
    want[2:6, 2:6] = True
    assert np.array_equal(covered(img), want)
    assert np.all(img[2:6, 2:6] == [255, 0, 0, 255])


def test_square_reference_mode_paints_whole_boundary_cells():
    # 2-px cells: the right edge x=6 lies in cell 6 (pixels 6,7), the top
    # edge y=6 in cell row 6 (rows 6,7) with cells x=2,4 only; no coverage
    # mask, so boundary cells are painted whole (gen_fragment.comp:202 TODO)
    img = render(scenes.square(), oracle.MODE_REFERENCE).get("image")
    want = np.zeros((8, 8), bool)
    want[2:6, 2:8] = True
    want[6:8, 2:6] = True
    assert np.array_equal(covered(img), want)


def test_star_nonzero_fills_centre_evenodd_does_not():
    c = 32
    nz = render(scenes.star(rule=0), oracle.MODE_PIXEL).get("image")
    eo = render(scenes.star(rule=1), oracle.MODE_PIXEL).get("image")
    assert covered(nz)[c, c] and not covered(eo)[c, c]
    # a point of the star (winding 1) is filled under both rules
    a = math.pi / 2
    px, py = int(32 + 20 * math.cos(a)), int(32 + 20 * math.sin(a))
    assert covered(nz)[py, px] and covered(eo)[py, px]
    # the rules differ exactly on the inner pentagon
    assert covered(nz).sum() > covered(eo).sum()


def test_figure_eight_lobes_filled_under_both_rules():
    for rule in (0, 1):
        img = render(scenes.figure_eight(rule=rule), oracle.MODE_PIXEL).get("image")
        cov = covered(img)
        assert cov[12, 14] and cov[12, 50]       # inside each lobe near the upper edge
        assert not cov[2, 32] and not cov[30, 32]


def test_offcanvas_and_clipped_paths():
    f = render(scenes.offcanvas(), oracle.MODE_PIXEL)
    img = f.get("image")
    vis = f.get("path_visible")
    # path 0 lies entirely left/below the canvas: culled, no records
    assert not (vis[0] & 0x10000001) == 0x10000001
    cov = covered(img)
    assert cov[0:12, 0:12].all()                 # clipped square covers [0,12)^2
    assert np.all(img[0:12, 0:12] == [0, 0, 255, 255])
    assert cov[20:32, 20:32].all() and not cov[12:20, 12:20].any()


def test_degenerate_paths_cover_nothing_in_pixel_mode():
    f = render(scenes.degenerate(), oracle.MODE_PIXEL)
    assert not covered(f.get("image")).any()
    assert f.n_draw == 0


def test_blend_is_source_over_in_path_order():
    # two overlapping translucent squares: red then blue over white
    b = scenes.Builder(8, 8)
    b.path(0, (255, 0, 0, 128)).polygon([(0, 0), (6, 0), (6, 6), (0, 6)])
    b.path(0, (0, 0, 255, 64)).polygon([(2, 2), (8, 2), (8, 8), (2, 8)])
    img = render(b.arrays(), oracle.MODE_PIXEL).get("image")

    def over(d, s):
        a = s[3]
        return [(s[i] * a + d[i] * (255 - a) + 127) // 255 for i in range(3)] + [255]
    white = [255, 255, 255, 255]
    red = over(white, (255, 0, 0, 128))
    both = over(red, (0, 0, 255, 64))
    assert list(img[1, 1]) == red
    assert list(img[3, 3]) == both
    assert list(img[7, 7]) == over(white, (0, 0, 255, 64))


def test_mvp_translate_moves_the_picture():
    d = scenes.square(w=16, h=16)
    mvp = np.array([1, 0, 0, 5, 0, 1, 0, 3, 0, 0, 1, 0, 0, 0, 0, 1], np.float32)
    img = render(d, oracle.MODE_PIXEL, mvp=mvp).get("image")
    want = np.zeros((16, 16), bool)
    want[5:9, 7:11] = True
    assert np.array_equal(covered(img), want)


def test_fp64_restatement_agrees_on_clean_geometry():
    for mode in (0, 1):
        a = render(scenes.mixed_curves(), mode).get("image")
        b = render(scenes.mixed_curves(), mode, fp64=True).get("image")
        assert np.any(a != b, axis=2).sum() <= 2


def test_arcs_known_answers(oracle_lib):
    """Rational quadratic arcs: a circle of four quarter arcs (w = sqrt(1/2))
    covers pi r^2 pixels up to its boundary; the half ellipse of weight 0
    reaches 25 px above its chord at its apex; both modes render."""
    import numpy as np
    d = scenes.arcs()
    img = oracle_lib.Frame(scenes.to_oracle(d), mode=oracle_lib.MODE_PIXEL).get("image")
    circle = np.all(img[:, :, :3] == [200, 30, 30], axis=2)
    assert abs(int(circle.sum()) - np.pi * 20 ** 2) < 2 * np.pi * 20 * 0.5
    assert circle[30, 28] and not circle[30, 49] and circle[30, 47]
    assert not np.all(img[16, 75] == 255) and np.all(img[14, 75] == 255)
    f0 = oracle_lib.Frame(scenes.to_oracle(d), mode=oracle_lib.MODE_REFERENCE)
    assert f0.n_intersections > 0 and f0.n_draw > 0


def test_gradient_known_answers(oracle_lib):
    """A linear gradient over the canvas: pixel x has t = (x + 0.5) / W and
    each channel trunc(t * 255); the radial disc is red at its centre; paths
    past the paint table paint nothing."""
    d = scenes.gradients()
    img = oracle_lib.Frame(scenes.to_oracle(d), mode=oracle_lib.MODE_PIXEL).get("image")
    W = d["width"]
    for x in (0, 7, 55, 119):
        v = int(np.float32(np.float32(x + 0.5) * np.float32(1.0 / W)) * np.float32(255.0))
        assert abs(int(img[2, x, 0]) - v) <= 1 and img[2, x, 1] == img[2, x, 0]
    # the radial disc's centre: red at alpha 0.9 over the linear gray
    cx = img[30, 80]
    assert cx[0] > 200 and cx[1] < 60
    # reference mode samples the cell's centre row and overwrites
    f0 = oracle_lib.Frame(scenes.to_oracle(d), mode=oracle_lib.MODE_REFERENCE)
    assert f0.n_draw > 0
    # without the paint table every gradient fill paints nothing: white
    bare = dict(d)
    bare.pop("paints")
    img2 = oracle_lib.Frame(scenes.to_oracle(bare), mode=oracle_lib.MODE_PIXEL).get("image")
    assert np.all(img2 == 255)


def test_multisampled_edge_coverage(oracle_lib):
    """A black square from x = 2.25 to 6 over white, 16 samples a pixel: the
    pixel column 2 has 12 of its 16 samples (columns 4..15 of the comb) inside,
    so its channels are (255 * 4 + 8) // 16 = 64; the columns fully inside
    are black and those outside white."""
    d = scenes.square(w=10, h=8, x0=2.25, y0=2, x1=6, y1=6, rgba=(0, 0, 0, 255))
    img = oracle_lib.render_aa(scenes.to_oracle(d), 16)
    assert img[4, 2, 0] == (255 * 4 + 8) // 16
    assert np.all(img[4, 3:6, :3] == 0) and np.all(img[4, 7, :3] == 255)
    # one sample is the plain pixel-mode frame with the sample at the centre
    one = oracle_lib.render_aa(scenes.to_oracle(d), 1)
    assert np.array_equal(one, oracle_lib.Frame(scenes.to_oracle(d), mode=1).get("image"))

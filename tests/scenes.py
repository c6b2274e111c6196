"""Hand-made scenes with known answers, shared by the oracle and GPU tests.

Each builder returns a flattened scene (numpy SoA, the reference's loadVG
layout) as a dict accepted by both oracle.Scene and
vkscanlinepr_gb300.VGContainer.from_arrays.
"""
import ctypes
import math

import numpy as np

LINE, QUADRIC, CUBIC, ARC = 2, 3, 4, 0x13


class Builder:
    def __init__(self, w, h):
        self.w, self.h = w, h
        self.pos, self.pos_path = [], []
        self.curve_pos, self.curve_type, self.curve_path = [], [], []
        self.fill_rule, self.fill_info = [], []

    def path(self, rule=0, rgba=(0, 0, 0, 255)):
        r, g, b, a = rgba
        self.fill_rule.append(rule)
        self.fill_info.append((r | (g << 8) | (b << 16) | (a << 24)) if a else 0)
        return self

    def curve(self, ctype, pts):
        p = len(self.fill_rule) - 1
        self.curve_pos.append(len(self.pos_path))
        self.curve_type.append(ctype)
        self.curve_path.append(p)
        for x, y in pts:
            self.pos.append((x, y))
            self.pos_path.append(p)
        return self

    def polygon(self, pts):
        for i in range(len(pts)):
            self.curve(LINE, [pts[i], pts[(i + 1) % len(pts)]])
        return self

    def arrays(self):
        return dict(
            width=self.w, height=self.h,
            position=np.asarray(self.pos, np.float32).reshape(-1),
            pos_path_idx=np.asarray(self.pos_path, np.uint32),
            curve_pos_map=np.asarray(self.curve_pos, np.uint32),
            curve_type=np.asarray(self.curve_type, np.uint32),
            curve_path_idx=np.asarray(self.curve_path, np.uint32),
            fill_rule=np.asarray(self.fill_rule, np.uint32),
            fill_info=np.asarray(self.fill_info, np.uint32))


def to_oracle(d):
    import oracle
    return oracle.Scene(d["width"], d["height"], d["position"], d["pos_path_idx"], d["curve_pos_map"],
                        d["curve_type"], d["curve_path_idx"], d["fill_rule"], d["fill_info"], paints=d.get("paints"))


def to_container(d):
    import vkscanlinepr_gb300 as sr
    c = sr.VGContainer.from_arrays(d["width"], d["height"], d["position"], d["pos_path_idx"],
                                   d["curve_pos_map"], d["curve_type"], d["curve_path_idx"],
                                   d["fill_rule"], d["fill_info"])
    p = d.get("paints")
    if p:
        c.paints = (sr.Paint * len(p))()
        ctypes.memmove(c.paints, p, ctypes.sizeof(sr.Paint) * len(p))
    return c


RED = (255, 0, 0, 255)
BLUE = (0, 0, 255, 255)


def square(w=8, h=8, x0=2, y0=2, x1=6, y1=6, rgba=RED, rule=0):
    return Builder(w, h).path(rule, rgba).polygon([(x0, y0), (x1, y0), (x1, y1), (x0, y1)]).arrays()


def star(w=64, h=64, rule=0, rgba=RED):
    cx, cy, r = 32.0, 32.0, 28.0
    pts = []
    for k in range(5):
        a = math.pi / 2 + k * 4 * math.pi / 5
        pts.append((cx + r * math.cos(a), cy + r * math.sin(a)))
    return Builder(w, h).path(rule, rgba).polygon(pts).arrays()


def figure_eight(w=64, h=32, rule=0, rgba=RED):
    # two diamonds joined by crossing edges: orientation flips between lobes
    pts = [(8, 8), (32, 24), (56, 8), (56, 24), (32, 8), (8, 24)]
    return Builder(w, h).path(rule, rgba).polygon(pts).arrays()


def mixed_curves(w=96, h=80):
    b = Builder(w, h)
    # cubic blob, nonzero
    b.path(0, (20, 200, 40, 255))
    b.curve(CUBIC, [(10, 40), (10, 5), (60, 5), (60, 40)])
    b.curve(CUBIC, [(60, 40), (60, 75), (10, 75), (10, 40)])
    # quadric lens, even-odd, semi-transparent
    b.path(1, (200, 30, 90, 160))
    b.curve(QUADRIC, [(30, 20), (55, 70), (85, 20)])
    b.curve(QUADRIC, [(85, 20), (55, 0), (30, 20)])
    # line triangle that hits integer grid lines exactly
    b.path(0, (0, 0, 255, 200))
    b.polygon([(40, 30), (90, 30), (40, 76)])
    return b.arrays()


def offcanvas(w=32, h=32):
    b = Builder(w, h)
    b.path(0, RED).polygon([(-40, -40), (-10, -40), (-10, -10), (-40, -10)])   # fully outside
    b.path(0, BLUE).polygon([(-8, -8), (12, -8), (12, 12), (-8, 12)])          # clipped
    b.path(0, (0, 200, 0, 255)).polygon([(20, 20), (60, 20), (60, 60), (20, 60)])
    return b.arrays()


def degenerate(w=32, h=32):
    b = Builder(w, h)
    b.path(0, RED).polygon([(4, 10), (20, 10), (28, 10)])        # zero-area, horizontal
    b.path(0, BLUE).polygon([(10, 4), (10, 20), (10, 28)])       # zero-area, vertical
    b.path(0, (0, 200, 0, 255)).polygon([(5, 5), (5, 5), (5, 5)])  # a single point
    return b.arrays()


def long_chains(w=2400, h=2400):
    """Curves crossing more than 1024 grid lines of one axis in one monotone
    piece (in both modes), which the renderer solves a warp per chain."""
    b = Builder(w, h)
    b.path(0, RED)
    b.curve(CUBIC, [(15.3, 30.7), (800.2, 700.9), (1600.5, 1500.1), (2380.6, 2210.4)])
    b.curve(CUBIC, [(2380.6, 2210.4), (2300.0, 400.0), (600.0, 100.0), (15.3, 30.7)])
    b.path(1, BLUE)
    b.curve(QUADRIC, [(5.5, 2390.2), (1200.3, 1190.7), (2395.1, 12.8)])
    b.curve(LINE, [(2395.1, 12.8), (5.5, 2390.2)])
    b.path(0, (0, 200, 0, 180))
    b.curve(CUBIC, [(10.0, 1200.0), (800.0, -900.0), (1600.0, 3300.0), (2390.0, 1210.0)])
    b.curve(LINE, [(2390.0, 1210.0), (10.0, 1200.0)])
    return b.arrays()


def opaque_layers(w=1100, h=64):
    """Wide opaque and translucent layers: spans that cover whole 256-pixel
    resolve segments (the renderer skips what an opaque span hides)."""
    b = Builder(w, h)
    b.path(0, (200, 30, 30, 255)).polygon([(0, 0), (1100, 0), (1100, 64), (0, 64)])
    b.path(0, (20, 40, 220, 120)).polygon([(100, 10), (900, 10), (900, 50), (100, 50)])
    b.path(0, (10, 190, 40, 255)).polygon([(256, 0), (780, 0), (780, 40), (256, 40)])
    b.path(1, (250, 20, 20, 90)).polygon([(0, 20), (1100, 20), (1100, 30), (0, 30)])
    b.path(1, (240, 240, 240, 255)).polygon([(600.5, 30.25), (1099.5, 31.75), (1000, 63.5), (590, 60)])
    b.path(0, (0, 0, 0, 200)).polygon([(5.5, 2.5), (1090.25, 8.5), (1080.75, 60.5), (12.5, 55.25)])
    b.path(0, (90, 90, 250, 255)).polygon([(0, 44), (1100, 44), (1100, 52), (0, 52)])
    return b.arrays()


def long_line(w=9000, h=64):
    """A line crossing more than 8192 grid columns beside cubics of a few
    hundred crossings: the line's chain must sort after the warp-solved ones."""
    b = Builder(w, h)
    b.path(0, RED)
    b.curve(LINE, [(1.5, 10.5), (8999.5, 50.5)])
    b.curve(CUBIC, [(8999.5, 50.5), (6000.0, 70.0), (3000.0, -10.0), (1.5, 10.5)])
    b.path(1, BLUE)
    b.curve(CUBIC, [(100.25, 5.5), (500.0, 60.0), (900.0, 2.0), (1300.75, 58.5)])
    b.curve(LINE, [(1300.75, 58.5), (100.25, 5.5)])
    return b.arrays()


def very_long_piece(w=16000, h=16):
    """One monotone cubic piece crossing about 16,000 grid columns (more
    than the long-piece merge keeps in shared memory) and a line back."""
    b = Builder(w, h)
    b.path(0, (30, 160, 90, 220))
    b.curve(CUBIC, [(1.5, 3.5), (5000.25, 5.5), (11000.75, 10.5), (15998.5, 12.5)])
    b.curve(LINE, [(15998.5, 12.5), (1.5, 3.5)])
    return b.arrays()


def translucent_layers(w=1300, h=48):
    """Runs of translucent layers over whole 256-pixel resolve segments between
    shapes that cover part of a segment.  A run whose composed blend sends
    every colour to one (a few layers of alpha 0.4 and more) lets the
    renderer start painting there; runs of alpha 1-3 never do; one run is
    longer than the 32 records a warp holds, and the last segment is 20
    pixels wide."""
    rng = np.random.default_rng(11)
    b = Builder(w, h)
    full = [(-1, -1), (w + 1, -1), (w + 1, h + 1), (-1, h + 1)]

    def rgb():
        return tuple(int(v) for v in rng.integers(0, 256, 3))

    def layer(lo, hi):
        b.path(0, rgb() + (int(rng.integers(lo, hi)),)).polygon(full)

    def shape():
        x, y, r = float(rng.uniform(0, w)), float(rng.uniform(0, h)), float(rng.uniform(3, 300))
        b.path(int(rng.integers(2)), rgb() + (int(rng.integers(60, 256)),)).polygon(
            [(x - r, y - 0.3 * r), (x + 0.7 * r, y - 0.4 * r), (x + 0.1 * r, y + 0.9 * r)])

    for _ in range(3):
        layer(102, 255)
    shape()
    for _ in range(40):
        layer(102, 255)
    shape()
    for _ in range(40):
        layer(1, 4)
    shape()
    shape()
    for _ in range(5):
        layer(1, 4)
    shape()
    for _ in range(6):
        for _ in range(int(rng.integers(1, 8))):
            layer(102, 255)
        shape()
    b.path(0, (10, 20, 30, 200)).polygon([(256, -1), (w + 1, -1), (w + 1, h + 1), (256, h + 1)])
    b.path(0, (200, 20, 30, 230)).polygon([(1280, -1), (w + 1, -1), (w + 1, h + 1), (1280, h + 1)])
    for _ in range(3):
        layer(1, 3)
    return b.arrays()


def deep_tail(w=2304, h=8):
    """Rows of about 1,300 records over nine resolve segments: 40 translucent
    full-canvas layers, 1,200 thin shapes in the first segment, then 10 layers
    over the other segments.  Those segments find their cut among the last
    records; the first finds none in the last 1,024, so the row is painted
    from its start in several staged chunks, and the CTA's two groups of
    segments share them."""
    rng = np.random.default_rng(23)
    b = Builder(w, h)

    def rgba(lo):
        return tuple(int(v) for v in rng.integers(0, 256, 3)) + (int(rng.integers(lo, 255)),)

    for _ in range(40):
        b.path(0, rgba(102)).polygon([(-1, -1), (w + 1, -1), (w + 1, h + 1), (-1, h + 1)])
    for k in range(1200):
        x = 0.2 * (k % 1200) + 0.25
        b.path(int(rng.integers(2)), rgba(60)).polygon([(x, -1), (x + 1.5, -1), (x + 1.5, h + 1), (x, h + 1)])
    for _ in range(10):
        b.path(0, rgba(200)).polygon([(256, -1), (w + 1, -1), (w + 1, h + 1), (256, h + 1)])
    return b.arrays()


def arcs(w=96, h=80):
    """A circle of four quarter arcs (w = sqrt(1/2)), a half ellipse closed by
    its chord (w = 0: the control point at infinity, given in homogeneous
    form), and an even-odd ring of arcs with w = 2 (hyperbolic) and w = 0.3
    (elliptic)."""
    import math
    b = Builder(w, h)
    wq = math.sqrt(0.5)
    cx, cy, r = 28.0, 30.0, 20.0
    b.path(0, (200, 30, 30, 255))
    for k in range(4):
        a0 = k * math.pi / 2
        a1 = a0 + math.pi / 2
        p0 = (cx + r * math.cos(a0), cy + r * math.sin(a0))
        p2 = (cx + r * math.cos(a1), cy + r * math.sin(a1))
        ctl = (cx + r * (math.cos(a0) + math.cos(a1)), cy + r * (math.sin(a0) + math.sin(a1)))
        b.curve(ARC, [p0, (ctl[0] * wq, ctl[1] * wq), p2, (wq, wq)])
    b.path(0, (30, 60, 200, 180))
    b.curve(ARC, [(60.0, 40.0), (0.0, -25.0), (90.0, 40.0), (0.0, 0.0)])
    b.curve(LINE, [(90.0, 40.0), (60.0, 40.0)])
    b.path(1, (20, 160, 40, 200))
    b.curve(ARC, [(50.0, 70.0), (2 * 70.0, 2 * 52.0), (90.0, 70.0), (2.0, 2.0)])
    b.curve(ARC, [(90.0, 70.0), (0.3 * 70.0, 0.3 * 78.0), (50.0, 70.0), (0.3, 0.3)])
    return b.arrays()


def gradients(w=120, h=60):
    """A full-canvas linear gradient, opaque black to opaque white from
    x = 0 to x = w (pad), under a radial gradient disc (centre (80, 30),
    radius 20, focus at the centre, red to transparent, reflect spread) and a
    linear gradient square rotated by its transform (repeat spread)."""
    import oracle
    b = Builder(w, h)
    paints = (oracle.Paint * 3)()
    lin = paints[0]
    lin.kind, lin.spread, lin.opacity, lin.n_stops = 1, 0, 1.0, 2
    lin.p0[:] = [0.0, 0.0]
    lin.p1[:] = [float(w), 0.0]
    lin.xf[:] = [1, 0, 0, 0, 1, 0]
    lin.offset[0], lin.offset[1] = 0.0, 1.0
    lin.rgba[0][:] = [0, 0, 0, 1]
    lin.rgba[1][:] = [1, 1, 1, 1]
    rad = paints[1]
    rad.kind, rad.spread, rad.opacity, rad.n_stops = 2, 2, 0.9, 3
    rad.p0[:] = [80.0, 30.0]
    rad.p1[:] = [80.0, 30.0]
    rad.radius = 20.0
    rad.xf[:] = [1, 0, 0, 0, 1, 0]
    rad.offset[0], rad.offset[1], rad.offset[2] = 0.0, 0.5, 1.0
    rad.rgba[0][:] = [1, 0, 0, 1]
    rad.rgba[1][:] = [1, 0.5, 0, 0.6]
    rad.rgba[2][:] = [1, 1, 0, 0]
    rot = paints[2]
    rot.kind, rot.spread, rot.opacity, rot.n_stops = 1, 1, 1.0, 2
    rot.p0[:] = [0.0, 0.0]
    rot.p1[:] = [8.0, 0.0]
    rot.xf[:] = [0.6, -0.8, 20.0, 0.8, 0.6, 10.0]
    rot.offset[0], rot.offset[1] = 0.0, 1.0
    rot.rgba[0][:] = [0, 0, 1, 1]
    rot.rgba[1][:] = [0, 1, 0, 1]
    b.path(0, (0, 0, 0, 255)).polygon([(0, 0), (w, 0), (w, h), (0, h)])
    b.path(0, (0, 0, 0, 255)).polygon([(60, 10), (100, 10), (100, 50), (60, 50)])
    b.path(1, (0, 0, 0, 255)).polygon([(10, 10), (40, 10), (40, 40), (10, 40)])
    d = b.arrays()
    d["fill_info"][:] = [1, 2, 3]   # SR_FILL_PAINT(0), (1), (2)
    d["paints"] = paints
    return d


ALL = {
    "arcs": arcs,
    "gradients": gradients,
    "square": square,
    "star_nonzero": lambda: star(rule=0),
    "star_evenodd": lambda: star(rule=1),
    "figure_eight": figure_eight,
    "mixed_curves": mixed_curves,
    "offcanvas": offcanvas,
    "degenerate": degenerate,
    "long_chains": long_chains,
    "opaque_layers": opaque_layers,
    "long_line": long_line,
    "very_long_piece": very_long_piece,
    "translucent_layers": translucent_layers,
    "deep_tail": deep_tail,
}

"""The resolve's collapse cut, restated on the CPU and checked against the
oracle: painting each 256-pixel segment from white at its cut gives the
oracle's image, and the warp's bit-mask walk over 32-record ballots finds the
same cut as a walk over one record at a time."""
import random

import numpy as np

import scenes

SEG = 256
TAIL = 1024   # records of a row the walk reads, from its end


def _blend(c, s, a):
    return (s * a + c * (255 - a) + 127) // 255


def _collapses(cols):
    for ch in range(3):
        lo, hi = 0, 255
        for col in cols:
            s, a = (col >> (8 * ch)) & 255, col >> 24
            lo, hi = _blend(lo, s, a), _blend(hi, s, a)
        if lo != hi:
            return False
    return True


def _test_run(run):
    """run: [(position, colour)] in draw order, at most 32; the latest start
    whose suffix collapses, or -1."""
    for t in range(len(run) - 1, -1, -1):
        if _collapses([c for _, c in run[t:]]):
            return run[t][0]
    return -1


def record_walk(recs):
    """recs: [(overlaps, covers, colour)] of a row's last records in draw
    order.  The walk one record at a time from the end: a run of covering
    records ends at a record over part of the segment; the latest 32 of a
    run are tested."""
    run, full = [], False
    for q in range(len(recs) - 1, -1, -1):
        ov, cv, col = recs[q]
        if not ov:
            continue
        if cv:
            if full:
                continue
            run.insert(0, (q, col))
            if len(run) == 32:
                c = _test_run(run)
                if c >= 0:
                    return c
                full = True
        else:
            if run and not full:
                c = _test_run(run)
                if c >= 0:
                    return c
            run, full = [], False
    if run and not full:
        return _test_run(run)
    return -1


class MaskWalk:
    """The warp's form: 32 records a step as two ballots (overlapping,
    covering); the covers above the highest partial record extend the run,
    that record ends it, and a run's records enter the buffer by rank."""

    def __init__(self):
        self.n, self.full, self.cut = 0, False, -1
        self.buf = [None] * 32

    def _collapse(self):
        run = [self.buf[k] for k in range(32 - self.n, 32)]
        return _test_run(run)

    def close(self):
        if self.n and not self.full:
            self.cut = self._collapse()
            if self.cut >= 0:
                return True
        self.n, self.full = 0, False
        return False

    def feed(self, mo, mc, lanes):
        mp = mo & ~mc
        while True:
            hp = mp.bit_length() - 1
            above = (~((2 << hp) - 1)) & 0xFFFFFFFF if mp else 0xFFFFFFFF
            run = mc & above
            if run and not self.full:
                for lane in range(32):
                    if (run >> lane) & 1:
                        rank = self.n + bin(run & (~((2 << lane) - 1) & 0xFFFFFFFF)).count("1")
                        if rank < 32:
                            self.buf[31 - rank] = lanes[lane]
                self.n += bin(run).count("1")
                if self.n >= 32:
                    self.n = 32
                    self.cut = self._collapse()
                    if self.cut >= 0:
                        return True
                    self.full = True
            if not mp:
                return False
            if self.close():
                return True
            mc &= ~above & 0xFFFFFFFF
            mp &= ~above & ((1 << hp) - 1)
            if not mc:
                return False


def mask_walk(recs):
    w = MaskWalk()
    c1 = len(recs)
    while c1 > 0:
        mo = mc = 0
        lanes = [None] * 32
        for lane in range(32):
            q = c1 - 32 + lane
            if q >= 0:
                ov, cv, col = recs[q]
                mo |= int(ov) << lane
                mc |= int(cv) << lane
                lanes[lane] = (q, col)
        if w.feed(mo, mc, lanes):
            return w.cut
        c1 -= 32
    return w.cut if w.close() else -1


def paint_from_cuts(draw, W, H):
    """Pixel-mode image of an int32x4 draw list, each segment of each row
    painted from white starting at its cut; also returns how many segments
    had one."""
    d = np.asarray(draw, np.int64).reshape(-1, 4)
    x0 = d[:, 0] & 0xFFFF
    y = d[:, 0] >> 16
    x1 = x0 + d[:, 1]
    col = d[:, 2] & 0xFFFFFFFF
    order = np.argsort(y, kind="stable")
    img = np.zeros((H, W, 4), np.uint8)
    img[..., 3] = 255
    cuts = 0
    for r in range(H):
        idx = order[y[order] == r]
        for seg in range(0, W, SEG):
            segend = min(seg + SEG, W)
            tail = idx[max(0, len(idx) - TAIL):]
            recs = [(bool(x0[i] < seg + SEG and x1[i] > seg), bool(x0[i] <= seg and x1[i] >= segend), int(col[i]))
                    for i in tail]
            cut = record_walk(recs)
            start = len(idx) - len(tail) + cut if cut >= 0 else 0
            cuts += cut >= 0
            px = np.full((3, segend - seg), 255, np.int64)
            xs = np.arange(seg, segend)
            for i in idx[start:]:
                m = (xs >= x0[i]) & (xs < x1[i])
                if not m.any():
                    continue
                a = int(col[i] >> 24)
                for ch in range(3):
                    s = int((col[i] >> (8 * ch)) & 255)
                    px[ch, m] = _blend(px[ch, m], s, a)
            img[r, seg:segend, :3] = px.T.astype(np.uint8)
    return img, cuts


def _check_scene(oracle_lib, scene):
    f = oracle_lib.Frame(scene, mode=oracle_lib.MODE_PIXEL)
    img, cuts = paint_from_cuts(f.get("draw_list"), f.width, f.height)
    assert np.array_equal(img, f.get("image"))
    return cuts


def test_painting_from_the_cut_equals_the_oracle_translucent_layers(oracle_lib):
    cuts = _check_scene(oracle_lib, scenes.to_oracle(scenes.translucent_layers()))
    assert cuts > 100


def test_painting_from_the_cut_equals_the_oracle_mixed_scene(oracle_lib):
    # many paths on a small canvas: full-canvas backgrounds between shapes
    s = oracle_lib.synth(1, 9, width=520, height=40, n_paths=2500)
    cuts = _check_scene(oracle_lib, s)
    assert cuts > 0


def test_mask_walk_finds_the_record_walk_cut():
    rng = random.Random(3)
    for _ in range(1500):
        n = rng.randint(0, 160)
        p_cover, p_over = rng.random(), rng.random()
        low_alpha = rng.random() < 0.3
        recs = []
        for _ in range(n):
            ov = rng.random() < p_over
            cv = ov and rng.random() < p_cover
            a = rng.randint(1, 4) if low_alpha and rng.random() < 0.7 else rng.randint(1, 255)
            recs.append((ov, cv, rng.randint(0, 0xFFFFFF) | (a << 24)))
        assert mask_walk(recs) == record_walk(recs)


def test_painting_from_the_cut_equals_the_oracle_deep_tail(oracle_lib):
    # segments without a cut in the row's last 1,024 records beside ones with
    cuts = _check_scene(oracle_lib, scenes.to_oracle(scenes.deep_tail()))
    assert 0 < cuts < 8 * 9

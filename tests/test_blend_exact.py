"""Exhaustive checks of the integer identities the compositing kernels use."""
import numpy as np

import oracle


def test_fma_round_trick_equals_integer_source_over():
    # u = s*a + d*(255-a); the kernel computes fma(u, fl(1/255), 1.5*2^23) - 1.5*2^23.
    # The fma rounds once: emulate exactly with integers (inv = M * 2^E).
    inv = np.float32(1.0) / np.float32(255.0)
    m, e = np.frexp(np.float64(inv))
    M, E = int(round(m * 2 ** 24)), int(e) - 24
    assert float(M) * 2.0 ** E == float(inv)
    u = np.arange(0, 65026, dtype=np.int64)
    sh = -E
    num = u * M
    rem = num & ((1 << sh) - 1)
    assert not np.any(rem == (1 << (sh - 1)))          # no rounding ties
    q_fp = (num + (1 << (sh - 1))) >> sh
    assert np.array_equal(q_fp, (u + 127) // 255)
    # every reachable u is in range and exact as a float32
    a = np.arange(256)[:, None]
    d = np.arange(256)[None, :]
    assert (d * (255 - a) + 255 * a).max() <= 65025 < 2 ** 24


def test_packed_div255_identity():
    x = np.arange(0, 65153, dtype=np.int64)
    assert np.array_equal((x + 1 + (x >> 8)) >> 8, x // 255)


def _perm_4341(x):
    # __byte_perm(x, 0, 0x4341): bytes 1 and 3 of x to bytes 0 and 2, zeros elsewhere
    return ((x >> 8) & 0xFF) | (((x >> 24) & 0xFF) << 16)


def test_packed_red_blue_blend_equals_source_over():
    # red in bits 0-7 and blue in bits 16-23 of one word:
    # u = rb * (255 - a) + ((sr*a + 128) | (sb*a + 128) << 16);
    # rb' = perm(u + perm(u)) with perm(x) = (x >> 8) & 0x00FF00FF
    u = np.arange(0, 65026, dtype=np.int64)   # every reachable c*(255-a) + s*a
    v = u + 128
    assert (v + (v >> 8)).max() < 2 ** 16      # no half carries into the other
    assert np.array_equal((v + (v >> 8)) >> 8, (u + 127) // 255)
    rng = np.random.default_rng(1)
    n = 200000
    c_r, c_b, s_r, s_b, a = (rng.integers(0, 256, n) for _ in range(5))
    a[:256] = np.arange(256)
    c_r[:256] = 255
    s_b[:256] = 255
    rb = c_r | (c_b << 16)
    uu = rb * (255 - a) + ((s_r * a + 128) | ((s_b * a + 128) << 16))
    assert uu.max() < 2 ** 32
    out = _perm_4341(uu + _perm_4341(uu))
    assert np.array_equal(out & 0xFF, (s_r * a + c_r * (255 - a) + 127) // 255)
    assert np.array_equal(out >> 16, (s_b * a + c_b * (255 - a) + 127) // 255)


def test_oracle_blend_matches_formula_and_keeps_alpha():
    rng = np.random.default_rng(0)
    for _ in range(2000):
        d = int(rng.integers(0, 2 ** 32))
        d |= 0xFF000000
        s = int(rng.integers(0, 2 ** 32))
        a = s >> 24
        got = oracle.blend(d, s)
        for ch in range(3):
            sc, dc = (s >> (8 * ch)) & 255, (d >> (8 * ch)) & 255
            assert (got >> (8 * ch)) & 255 == (sc * a + dc * (255 - a) + 127) // 255
        assert got >> 24 == 255


def _blend(c, s, a):
    return (s * a + c * (255 - a) + 127) // 255


def test_blend_is_monotone_in_the_old_value():
    # every (s, a): c -> blend(c) never decreases, so a composition of blends
    # sends every colour between what it sends 0 and 255 to
    c = np.arange(256, dtype=np.int64)
    s = np.arange(256, dtype=np.int64)[:, None, None]
    a = np.arange(256, dtype=np.int64)[None, :, None]
    v = _blend(c[None, None, :], s, a)
    assert np.all(np.diff(v, axis=2) >= 0)


def test_collapsed_runs_send_every_colour_to_one():
    # the resolve starts a segment at a run of whole-segment layers whose
    # composition sends 0 and 255 to one value: check it sends all 256 there
    rng = np.random.default_rng(5)
    hits = 0
    for _ in range(4000):
        n = int(rng.integers(1, 12))
        s = rng.integers(0, 256, n)
        a = rng.integers(1, 256, n)
        c = np.arange(256, dtype=np.int64)
        for k in range(n):
            c = _blend(c, int(s[k]), int(a[k]))
        if c[0] == c[255]:
            hits += 1
            assert np.all(c == c[0])
    assert hits > 500

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

"""The CPU restatement of the sizing network (oracle/mlp_ref.py), pinned on
its own: analytic gradients against central differences, BF16 rounding and
Adam against known answers, features of hand-made paths."""
import math

import numpy as np
import pytest

from oracle import mlp_ref as M


def _net(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(M.N_PARAMS, np.float32)
    p[M.O_W1:M.O_B1] = rng.uniform(-0.7, 0.7, M.O_B1 - M.O_W1)
    p[M.O_B1:M.O_W2] = rng.uniform(-0.1, 0.1, M.O_W2 - M.O_B1)
    p[M.O_W2:M.O_B2] = rng.uniform(-0.2, 0.2, M.O_B2 - M.O_W2)
    p[M.O_B2:M.O_W3] = rng.uniform(-0.1, 0.1, M.O_W3 - M.O_B2)
    p[M.O_W3:M.O_B3] = rng.uniform(-0.2, 0.2, M.O_B3 - M.O_W3)
    p[M.O_B3:] = rng.uniform(-0.1, 0.1, M.N_PARAMS - M.O_B3)
    norm = np.concatenate([rng.uniform(0, 2, 6), rng.uniform(0.5, 2, 6), rng.uniform(1, 3, 2),
                           rng.uniform(0.5, 2, 2)]).astype(np.float32)
    x = rng.uniform(0, 6, (24, 6))
    t = rng.uniform(0, 8, (24, 2))
    return p, norm, x, t


def test_parameter_layout():
    assert M.N_PARAMS == 4738 and M.N_NORM == 16


def test_gradient_matches_central_differences():
    p, norm, x, t = _net(1)
    _, g = M.loss_grad(p, norm, x, t, round_weights=False)
    rng = np.random.default_rng(2)
    idx = np.concatenate([rng.choice(np.arange(s, e), 6, replace=False) for s, e in
                          [(M.O_W1, M.O_B1), (M.O_B1, M.O_W2), (M.O_W2, M.O_B2), (M.O_B2, M.O_W3),
                           (M.O_W3, M.O_B3)]] + [np.arange(M.O_B3, M.N_PARAMS)])
    p64 = p.astype(np.float64)
    for i in idx:
        h = 1e-4
        a, b = p64.copy(), p64.copy()
        a[i] += h
        b[i] -= h
        # the restatement takes float32 parameters; evaluate in float64 here
        la = _loss64(a, norm, x, t)
        lb = _loss64(b, norm, x, t)
        fd = (la - lb) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def _loss64(p, norm, x, t):
    W1 = p[M.O_W1:M.O_B1].reshape(64, 6)
    W2 = p[M.O_W2:M.O_B2].reshape(64, 64)
    W3 = p[M.O_W3:M.O_B3].reshape(2, 64)
    xm, xs, ym, ys = M.split_norm(norm)
    xn = (x - xm) * xs
    h1 = M.gelu(xn @ W1.T + p[M.O_B1:M.O_W2])
    h2 = M.gelu(h1 @ W2.T + p[M.O_B2:M.O_W3])
    y = h2 @ W3.T + p[M.O_B3:]
    e = y - (t - ym) / ys
    return (e * e).sum() / e.size


def test_gelu_grad_matches_differences():
    x = np.linspace(-6, 6, 101)
    h = 1e-5
    fd = (M.gelu(x + h) - M.gelu(x - h)) / (2 * h)
    assert np.allclose(M.gelu_grad(x), fd, atol=1e-8)


def test_bf16_rounding_known_values():
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -7, -2.5, 0.0, 3.0e38], np.float32)
    got = M.bf16_round(vals)
    # bf16 keeps 7 fraction bits: 1 + 2^-8 is a tie and the even neighbour 1.0
    # wins; 1 + 3*2^-8 is a tie between 1 + 2^-7 (odd) and 1 + 2^-6 (even)
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == np.float32(1.0 + 2 ** -6)
    assert got[3] == np.float32(1.0 + 2 ** -7) and got[4] == -2.5 and got[5] == 0.0
    assert (got.view(np.uint32) & 0xFFFF).max() == 0
    assert abs(float(got[6]) - 3.0e38) / 3.0e38 < 2 ** -8


def test_adam_first_step_moves_by_lr():
    g = np.array([0.5, -2.0, 1e-3, 0.0])
    p, m, v = M.adam_step(np.zeros(4), np.zeros(4), np.zeros(4), g, 1, lr=1e-3)
    # bias-corrected first step: -lr * g / (|g| + eps)
    assert np.allclose(p[:3], -1e-3 * np.sign(g[:3]), rtol=1e-4)
    assert p[3] == 0.0
    assert np.allclose(m, 0.1 * g) and np.allclose(v, 0.001 * g * g)


def test_features_of_a_square_and_a_cubic():
    # path 0: unit-10 square of 4 lines; path 1: one cubic, partly off canvas
    tpos = np.array([[10, 10], [20, 10], [20, 10], [20, 20], [20, 20], [10, 20], [10, 20], [10, 10],
                     [-50, 5], [0, 5], [0, 15], [40, 15]], np.float32)
    curve_pos = [0, 2, 4, 6, 8]
    curve_type = [2, 2, 2, 2, 4]
    curve_path = [0, 0, 0, 0, 1]
    f = M.path_features(tpos, curve_pos, curve_type, curve_path, 2, 32, 32)
    assert np.allclose(f[0], [math.log1p(4), math.log1p(10), math.log1p(10), math.log1p(40),
                              math.log1p(0.75), 0.0])
    # cubic: bbox x clipped to [-1, 33] -> 34; polygon length 50 + 10 + 40; turns +90 and -90 degrees
    assert np.allclose(f[1], [math.log1p(1), math.log1p(34), math.log1p(10), math.log1p(100),
                              math.log1p(0.5), 1.0])


def test_forward_equals_loss_path():
    p, norm, x, t = _net(3)
    y = M.forward(p, norm, x)
    _, _, _, ys = M.split_norm(norm)
    loss, _ = M.loss_grad(p, norm, x, t)
    e = (y - t) / ys
    assert loss == pytest.approx(float((e * e).mean()), rel=1e-12)

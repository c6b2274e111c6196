"""CPU restatement of the learned-sizing network and its path features.

TEST INFRASTRUCTURE ONLY: tests, the smoke check and the bench's CPU leg use
this module to check the GPU kernels in vkscanlinepr_gb300/csrc/mlp.cu; the
product never imports it.

The reference has no sizing network: it reads the count pass back
(scanline_rasterizer.cpp:337-369) and grows buffers on demand
(vulkan_buffer.h:31-46).  What is restated here is the network the GPU
trains and runs:

  features (per path, from the transformed control points)
      log1p(segments), log1p(clipped bbox w / F), log1p(clipped bbox h / F),
      log1p(control-polygon length / F), log1p(sum |turn| / 2 pi),
      cubic fraction
  network   x -> standardise -> 64 GELU -> 64 GELU -> 2 -> de-standardise
            weights rounded to BF16 (round to nearest even), biases FP32
  loss      mean over rows and outputs of (y_std_units - t_std_units)^2
  optimiser Adam with bias correction

Everything is computed in float64; the GPU computes in FP32, so parity is a
tolerance (stated in the tests).  The analytic gradient here is pinned by
central finite differences on the unrounded network (tests/test_sizer_ref.py).
"""
import math

import numpy as np

IN, HID, OUT = 6, 64, 2
O_W1 = 0
O_B1 = O_W1 + HID * IN
O_W2 = O_B1 + HID
O_B2 = O_W2 + HID * HID
O_W3 = O_B2 + HID
O_B3 = O_W3 + OUT * HID
N_PARAMS = O_B3 + OUT
N_NORM = 2 * IN + 2 * OUT


def bf16_round(x):
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def unpack(params, round_weights=True):
    p = np.asarray(params, np.float32)
    w = bf16_round(p) if round_weights else p
    w = w.astype(np.float64)
    b = p.astype(np.float64)
    return (w[O_W1:O_B1].reshape(HID, IN), b[O_B1:O_W2], w[O_W2:O_B2].reshape(HID, HID), b[O_B2:O_W3],
            w[O_W3:O_B3].reshape(OUT, HID), b[O_B3:])


_erf = np.vectorize(math.erf, otypes=[np.float64])


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def split_norm(norm):
    n = np.asarray(norm, np.float64)
    return n[:IN], n[IN:2 * IN], n[2 * IN:2 * IN + OUT], n[2 * IN + OUT:]


def forward(params, norm, x, round_weights=True):
    """Predictions in log(1 + count) units, [n, 2]."""
    W1, b1, W2, b2, W3, b3 = unpack(params, round_weights)
    xm, xs, ym, ys = split_norm(norm)
    xn = (np.asarray(x, np.float64) - xm) * xs
    h1 = gelu(xn @ W1.T + b1)
    h2 = gelu(h1 @ W2.T + b2)
    return (h2 @ W3.T + b3) * ys + ym


def loss_grad(params, norm, x, t, round_weights=True):
    """(mean squared error in standard units, gradient [N_PARAMS])."""
    W1, b1, W2, b2, W3, b3 = unpack(params, round_weights)
    xm, xs, ym, ys = split_norm(norm)
    xn = (np.asarray(x, np.float64) - xm) * xs
    tn = (np.asarray(t, np.float64) - ym) / ys
    n = xn.shape[0]
    a1 = xn @ W1.T + b1
    h1 = gelu(a1)
    a2 = h1 @ W2.T + b2
    h2 = gelu(a2)
    y = h2 @ W3.T + b3
    e = y - tn
    loss = float((e * e).sum() / (n * OUT))
    dy = 2.0 * e / (n * OUT)
    d2 = (dy @ W3) * gelu_grad(a2)
    d1 = (d2 @ W2) * gelu_grad(a1)
    g = np.zeros(N_PARAMS)
    g[O_W1:O_B1] = (d1.T @ xn).reshape(-1)
    g[O_B1:O_W2] = d1.sum(0)
    g[O_W2:O_B2] = (d2.T @ h1).reshape(-1)
    g[O_B2:O_W3] = d2.sum(0)
    g[O_W3:O_B3] = (dy.T @ h2).reshape(-1)
    g[O_B3:] = dy.sum(0)
    return loss, g


def adam_step(params, m, v, grad, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam step (step counts from 1); returns (params, m, v)."""
    p = np.asarray(params, np.float64)
    m = b1 * np.asarray(m, np.float64) + (1.0 - b1) * grad
    v = b2 * np.asarray(v, np.float64) + (1.0 - b2) * grad * grad
    bc1 = 1.0 - b1 ** step
    bc2 = 1.0 - b2 ** step
    p = p - lr * (m / bc1) / (np.sqrt(v / bc2) + eps)
    return p, m, v


def path_features(tpos, curve_pos, curve_type, curve_path, n_paths, width, height, F=1):
    """Features [n_paths, 6] from transformed positions (float32 pairs)."""
    tp = np.asarray(tpos, np.float64).reshape(-1, 2)
    out = np.zeros((n_paths, IN))
    first = np.searchsorted(np.asarray(curve_path), np.arange(n_paths + 1), side="left")
    for p in range(n_paths):
        c0, c1 = int(first[p]), int(first[p + 1])
        segs = c1 - c0
        if segs == 0:
            out[p] = [0.0, 0.0, 0.0, 0.0, 0.0, 0.0]
            continue
        pts = []
        length = turn = 0.0
        prev = None
        cubics = 0
        for c in range(c0, c1):
            k = int(curve_type[c]) & 7
            cubics += int(curve_type[c]) == 4
            cp = tp[int(curve_pos[c]):int(curve_pos[c]) + k]
            pts.append(cp)
            for i in range(1, k):
                ex, ey = cp[i, 0] - cp[i - 1, 0], cp[i, 1] - cp[i - 1, 1]
                el = math.hypot(ex, ey)
                if el > 0.0:
                    length += el
                    if prev is not None:
                        turn += abs(math.atan2(prev[0] * ey - prev[1] * ex, prev[0] * ex + prev[1] * ey))
                    prev = (ex, ey)
        a = np.concatenate(pts)
        bw = max(min(a[:, 0].max(), width + 1.0) - max(a[:, 0].min(), -1.0), 0.0)
        bh = max(min(a[:, 1].max(), height + 1.0) - max(a[:, 1].min(), -1.0), 0.0)
        out[p] = [math.log1p(segs), math.log1p(bw / F), math.log1p(bh / F), math.log1p(length / F),
                  math.log1p(turn / (2.0 * math.pi)), cubics / segs]
    return out


def path_labels(curve_count, curve_path, path_draws, n_paths):
    """Exact per-path counts [n_paths, 2] (records, draw records) as integers."""
    rec = np.bincount(np.asarray(curve_path), weights=np.asarray(curve_count, np.float64), minlength=n_paths)
    return np.stack([rec.astype(np.int64), np.asarray(path_draws, np.int64)], 1)

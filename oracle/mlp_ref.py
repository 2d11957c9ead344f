"""CPU checker for the learned surrogate (test infrastructure only: imported
by tests/, smoke() and bench.py's CPU legs, never by the product).

The surrogate has no counterpart in the reference; this file restates the
project's own definitions so the GPU kernels can be checked:

  descriptor  4 channels x 24 Gaussian-smeared radial bins of the pairs
              (moved bead, other bead; moved pairs once) before and after a
              move: pairs up to 7.5 counted in fine bins floor(32 r + 1/2)
              (centres r_f = f / 32), then
              bin k (centre 0.125 + 0.25 k) = sum_f count_f
              round(4096 exp(-(r_f - c_k)^2 / (2 0.25^2))) / 4096
  network     x' = bf16((x - mu) isd), h1 = bf16(SiLU(W1 x' + b1)),
              h2 = SiLU(W2 h1 + b2), f = bf16(w3) . h2 + b3 with bf16 W1, W2
  surrogate   s = y_scale (f(x) - f(swap x)), swap = channels (0,1) <-> (2,3)
  loss        mean (s - t)^2, gradients by hand in float64 with the GPU's
              bf16 rounding points (x', h1, and the dz2, dz1 fed to the
              tensor cores)
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID, N_BINS = 96, 128, 24
BIN_W, CUT = 0.25, 7.5
OFF_W1 = 0
OFF_B1 = N_HID * N_IN
OFF_W2 = OFF_B1 + N_HID
OFF_B2 = OFF_W2 + N_HID * N_HID
OFF_W3 = OFF_B2 + N_HID
OFF_B3 = OFF_W3 + N_HID
N_PARAM = OFF_B3 + 1


def bf16(a):
    """Round to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF_W1:OFF_B1].reshape(N_HID, N_IN), p[OFF_B1:OFF_W2],
            p[OFF_W2:OFF_B2].reshape(N_HID, N_HID), p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3],
            p[OFF_B3])


def swap(x):
    x = np.asarray(x)
    return np.concatenate([x[:, N_IN // 2:], x[:, :N_IN // 2]], axis=1)


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def _forward(p, mu, isd, x):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    W1b = bf16(W1).astype(np.float64)
    W2b = bf16(W2).astype(np.float64)
    w3b = bf16(w3).astype(np.float64)
    xs = bf16((np.asarray(x, np.float32) - np.asarray(mu, np.float32))
              * np.asarray(isd, np.float32)).astype(np.float64)
    z1 = xs @ W1b.T + b1
    h1 = bf16(z1 * _sig(z1)).astype(np.float64)
    z2 = h1 @ W2b.T + b2
    h2 = z2 * _sig(z2)
    f = h2 @ w3b + b3
    return f, dict(xs=xs, z1=z1, h1=h1, z2=z2, h2=h2, W2b=W2b, w3b=w3b)


def predict(p, mu, isd, y_scale, x):
    """Surrogate energy change s of each descriptor row."""
    x = np.asarray(x, np.float64)
    fa, _ = _forward(p, mu, isd, x)
    fb, _ = _forward(p, mu, isd, swap(x))
    return y_scale * (fa - fb)


def grad(p, mu, isd, y_scale, x, t):
    """Gradient of mean (s - t)^2 over the parameter vector, and the loss."""
    x = np.asarray(x, np.float64)
    t = np.asarray(t, np.float64)
    n = len(x)
    fa, ca = _forward(p, mu, isd, x)
    fb, cb = _forward(p, mu, isd, swap(x))
    s = y_scale * (fa - fb)
    g = 2.0 * (s - t) * y_scale / n
    out = np.zeros(N_PARAM)
    for c, dy in ((ca, g), (cb, -g)):
        sg2 = _sig(c["z2"])
        out[OFF_W3:OFF_B3] += dy @ c["h2"]
        out[OFF_B3] += dy.sum()
        dz2 = dy[:, None] * c["w3b"][None, :] * sg2 * (1.0 + c["z2"] * (1.0 - sg2))
        out[OFF_B2:OFF_W3] += dz2.sum(axis=0)
        dz2b = bf16(dz2).astype(np.float64)
        out[OFF_W2:OFF_B2] += (dz2b.T @ c["h1"]).ravel()
        dh1 = dz2b @ c["W2b"]
        sg1 = _sig(c["z1"])
        dz1 = dh1 * sg1 * (1.0 + c["z1"] * (1.0 - sg1))
        out[OFF_B1:OFF_W2] += dz1.sum(axis=0)
        dz1b = bf16(dz1).astype(np.float64)
        out[OFF_W1:OFF_B1] += (dz1b.T @ c["xs"]).ravel()
    return out, float(np.mean((s - t) ** 2))


def loss_exact(p, mu, isd, y_scale, x, t):
    """The loss without any bf16 rounding (for finite-difference checks of
    the gradient formulas)."""
    def f(xx):
        W1, b1, W2, b2, w3, b3 = unpack(p)
        xs = (xx - mu) * isd
        z1 = xs @ W1.T + b1
        h1 = z1 * _sig(z1)
        z2 = h1 @ W2.T + b2
        return (z2 * _sig(z2)) @ w3 + b3
    x = np.asarray(x, np.float64)
    s = y_scale * (f(x) - f(swap(x)))
    return float(np.mean((s - np.asarray(t)) ** 2))


def grad_exact(p, mu, isd, y_scale, x, t):
    """grad() without bf16 rounding, for the finite-difference check."""
    x = np.asarray(x, np.float64)
    t = np.asarray(t, np.float64)
    W1, b1, W2, b2, w3, b3 = unpack(p)
    n = len(x)

    def fw(xx):
        xs = (xx - mu) * isd
        z1 = xs @ W1.T + b1
        h1 = z1 * _sig(z1)
        z2 = h1 @ W2.T + b2
        h2 = z2 * _sig(z2)
        return h2 @ w3 + b3, (xs, z1, h1, z2, h2)

    fa, ca = fw(x)
    fb, cb = fw(swap(x))
    s = y_scale * (fa - fb)
    g = 2.0 * (s - t) * y_scale / n
    out = np.zeros(N_PARAM)
    for (xs, z1, h1, z2, h2), dy in ((ca, g), (cb, -g)):
        out[OFF_W3:OFF_B3] += dy @ h2
        out[OFF_B3] += dy.sum()
        sg2 = _sig(z2)
        dz2 = dy[:, None] * w3[None, :] * sg2 * (1.0 + z2 * (1.0 - sg2))
        out[OFF_B2:OFF_W3] += dz2.sum(axis=0)
        out[OFF_W2:OFF_B2] += (dz2.T @ h1).ravel()
        sg1 = _sig(z1)
        dz1 = (dz2 @ W2) * sg1 * (1.0 + z1 * (1.0 - sg1))
        out[OFF_B1:OFF_W2] += dz1.sum(axis=0)
        out[OFF_W1:OFF_B1] += (dz1.T @ xs).ravel()
    return out


def adam(p, m, v, g, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step in float32 (the GPU's arithmetic)."""
    p, m, v, g = (np.asarray(a, np.float32).copy() for a in (p, m, v, g))
    m = np.float32(b1) * m + np.float32(1 - b1) * g
    v = np.float32(b2) * v + np.float32(1 - b2) * g * g
    c1 = np.float32(1.0 / (1.0 - b1 ** step))
    c2 = np.float32(1.0 / (1.0 - b2 ** step))
    p = p - np.float32(lr) * (m * c1) / (np.sqrt(v * c2) + np.float32(eps))
    return p, m, v


FINE = 32          # fine distance bins per sigma
N_FINE = 241       # fine bins per channel (0 - 7.5 sigma), centred on f / 32


def smear_weights():
    """Integer weights round(4096 exp(-(r_f - c_k)^2 / (2 w^2))) [fine bin][bin]."""
    rf = np.arange(N_FINE) / FINE
    ck = (np.arange(N_BINS) + 0.5) * BIN_W
    return np.rint(4096.0 * np.exp(-0.5 / BIN_W ** 2 * (rf[:, None] - ck[None, :]) ** 2))


def descriptor(before, after, lo, hi, types, box, npbc=3):
    """Descriptor of moving beads [lo, hi) from `before` to `after` (both
    [n_bead, 3]; rows outside [lo, hi) equal), types[n_bead]: pairs within
    7.5 counted per (channel, floor(32 r + 1/2)), then smeared with
    smear_weights()."""
    before = np.asarray(before, np.float64)
    after = np.asarray(after, np.float64)
    types = np.asarray(types)
    box = np.asarray(box, np.float64)
    counts = np.zeros((4, N_FINE), np.int64)
    n = len(before)
    for i in range(lo, hi):
        j = np.arange(n)
        keep = (j != i) & ~((j >= lo) & (j < hi) & (j < i))
        j = j[keep]
        cls = (types[j] != types[i]).astype(int)
        for which, pos in ((0, before), (2, after)):
            d = pos[j] - pos[i]
            for a in range(npbc):
                d[:, a] -= box[a] * np.rint(d[:, a] / box[a])
            r = np.sqrt((d * d).sum(axis=1))
            sel = r < CUT
            np.add.at(counts, (which + cls[sel], (r[sel] * FINE + 0.5).astype(int)), 1)
    return (counts @ smear_weights()).ravel() / 4096.0

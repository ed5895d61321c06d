"""numpy restatement of the correction CNN (focss_cnn_*) with the same BF16
rounding points as the GPU kernels, FP64 accumulation.

TEST INFRASTRUCTURE ONLY: the checker for the GPU forward/backward kernels.
The network has no reference counterpart.
"""
from __future__ import annotations

import numpy as np

LAYERS = ((16, 64), (64, 64), (64, 64), (64, 16))
KW, HALF = 9, 4


def bf16(x):
    a = np.ascontiguousarray(np.asarray(x, np.float32)).view(np.uint32)
    r = ((a >> 16) & 1) + np.uint32(0x7FFF)
    return ((a + r) & np.uint32(0xFFFF0000)).view(np.float32).astype(np.float64)


def unpack(flat):
    out, o = [], 0
    for cin, cout in LAYERS:
        w = np.asarray(flat[o:o + cout * KW * cin], np.float64).reshape(cout, KW, cin)
        o += cout * KW * cin
        b = np.asarray(flat[o:o + cout], np.float64)
        o += cout
        out.append((w, b))
    return out


def shift(x, d):
    """x[:, p + d, :] with zero padding (x: B, L, C)."""
    out = np.zeros_like(x)
    L = x.shape[1]
    if d >= 0:
        out[:, : L - d] = x[:, d:]
    else:
        out[:, -d:] = x[:, : L + d]
    return out


def conv(x, w, b=None):
    out = np.zeros(x.shape[:2] + (w.shape[0],))
    for kk in range(KW):
        out += shift(x, kk - HALF) @ w[:, kk, :].T
    if b is not None:
        out += b
    return out


def wgrad(g, x):
    return np.stack([np.einsum("blo,bli->oi", g, shift(x, kk - HALF)) for kk in range(KW)], axis=1)


def _at(y, d):
    """y[:, k + d] with zero outside the realization (y: B, L)."""
    out = np.zeros_like(y)
    L = y.shape[1]
    if d >= 0:
        out[:, : max(0, L - d)] = y[:, d:]
    else:
        out[:, -d:] = y[:, : L + d]
    return out


def triplet(y, m, n):
    """T(m, n)[k] = y[k+m] y[k+n] conj(y[k+m+n]) (src/focss/equalizer/sino.cpp:161-171, one mode)."""
    return _at(y, m) * _at(y, n) * np.conj(_at(y, m + n))


def triplet_features(y, pairs):
    """Feature j = T(m_j, n_j) + T(-m_j, -n_j) (T(0, 0) alone), as focss_cnn_set_triplets."""
    out = []
    for m, n in pairs:
        f = triplet(y, m, n)
        if m != 0 or n != 0:
            f = f + triplet(y, -m, -n)
        out.append(f)
    return out


def forward(flat, y, s, triplets=()):
    P = unpack(flat)
    B, L = y.shape
    x0 = np.zeros((B, L, 16))
    x0[..., 0] = y.real / s
    x0[..., 1] = y.imag / s
    # FP32 products as on the GPU, then the 1/s^3 scale
    y32 = y.astype(np.complex64)
    for j, f in enumerate(triplet_features(y32, triplets)):
        f = f.astype(np.complex64).astype(np.complex128)
        x0[..., 2 + 2 * j] = f.real / s ** 3
        x0[..., 3 + 2 * j] = f.imag / s ** 3
    acts = [bf16(x0)]
    for l in range(3):
        w, b = P[l]
        acts.append(bf16(np.maximum(conv(acts[-1], bf16(w), b), 0)))
    w, b = P[3]
    d4 = conv(acts[-1], bf16(w), b)
    z = y + s * (d4[..., 0] + 1j * d4[..., 1])
    return z, acts


def loss_grad(flat, y, tx, s, triplets=()):
    P = unpack(flat)
    z, acts = forward(flat, y, s, triplets)
    M = y.size
    d = z - tx
    loss = float(np.sum(np.abs(d) ** 2) / M)
    g = np.zeros(y.shape + (16,))
    g[..., 0] = 2 * s * d.real / M
    g[..., 1] = 2 * s * d.imag / M
    g = bf16(g)
    grads = [None] * 4
    for l in (3, 2, 1, 0):
        w, _ = P[l]
        grads[l] = (wgrad(g, acts[l]), g.sum(axis=(0, 1)))
        if l > 0:
            wt = np.flip(bf16(w), axis=1).transpose(2, 1, 0)  # W'[ci][kk'][co] = W[co][8-kk'][ci]
            g = bf16(conv(g, wt) * (acts[l] > 0))
    flat_g = []
    for gw, gb in grads:
        flat_g += [gw.ravel(), gb.ravel()]
    return loss, np.concatenate(flat_g), z

"""FP64 numpy restatement of the learned-DBP model and its gradients.

TEST INFRASTRUCTURE ONLY: the checker for the GPU forward/backward kernels
(focss_ldbp_*).  The model has no reference counterpart; it is the few-step
learned form of backward_propagation (src/tasks/systems.cpp:73-91).  The
analytic adjoint below is itself checked against finite differences.
"""
from __future__ import annotations

import numpy as np


def fir(x, h):
    """FIR(x, h)[n] = sum_t h[t] x[(n + t - c) mod N], c = (T-1)/2 (last axis)."""
    T = len(h)
    c = (T - 1) // 2
    y = np.zeros_like(x, dtype=np.complex128)
    for t in range(T):
        y += h[t] * np.roll(x, -(t - c), axis=-1)
    return y


def fir_adjoint(g, h):
    T = len(h)
    c = (T - 1) // 2
    out = np.zeros_like(g, dtype=np.complex128)
    for t in range(T):
        out += np.conj(h[t]) * np.roll(g, t - c, axis=-1)
    return out


def fir_tap_grad(x, g, T):
    c = (T - 1) // 2
    return np.array([np.sum(g * np.conj(np.roll(x, -(t - c), axis=-1))) for t in range(T)])


def forward(h, xi, hmf, x, span_scale, spans, steps, keep=False):
    acts = []
    x = np.asarray(x, np.complex128)
    for s in range(spans):
        x = x * span_scale
        for i in range(steps):
            k = s * steps + i
            acts.append(x)
            x = fir(x, h[k])
            acts.append(x)
            x = x * np.exp(1j * xi[k] * np.abs(x) ** 2)
    acts.append(x)
    y = fir(x, hmf)
    return (y, acts) if keep else y


def loss_grad(h, xi, hmf, x, tx, span_scale, spans, steps):
    """L = mean |y[..., 0::2] - tx|^2 and Wirtinger gradients dL/dconj(h),
    dL/dconj(hmf), real dL/dxi."""
    y, acts = forward(h, xi, hmf, x, span_scale, spans, steps, keep=True)
    d = y[..., 0::2] - tx
    M = d.size
    loss = float(np.sum(np.abs(d) ** 2) / M)
    g = np.zeros_like(y)
    g[..., 0::2] = d / M
    gh = np.zeros_like(np.asarray(h, np.complex128))
    gxi = np.zeros(len(xi))
    ghmf = fir_tap_grad(acts[-1], g, len(hmf))
    g = fir_adjoint(g, hmf)
    a = len(acts) - 1
    for s in reversed(range(spans)):
        for i in reversed(range(steps)):
            k = s * steps + i
            a -= 1
            xin = acts[a]
            p = np.abs(xin) ** 2
            e = np.exp(1j * xi[k] * p)
            yk = xin * e
            gxi[k] = np.sum(2 * np.real(np.conj(g) * 1j * p * yk))
            g = g * np.conj(e) * (1 - 1j * xi[k] * p) + np.conj(g) * 1j * xi[k] * xin ** 2 * e
            a -= 1
            gh[k] = fir_tap_grad(acts[a], g, h.shape[1])
            g = fir_adjoint(g, h[k])
        g = g * span_scale
    return loss, gh, gxi, ghmf

"""Perturbation-equalizer fit with the normal equations formed on the GPU
(focss_sino_gram) against the numpy restatement of SINO::train
(src/focss/equalizer/sino.cpp:42-159): on a synthetic link with known
coefficients both recover them, and they agree with each other."""
import numpy as np
import pytest

from focss_gb300 import sino

pytestmark = pytest.mark.gpu


def _link(rng, R, N, lw, modes=1):
    import focss_gb300 as fg
    gray = np.array([complex(a, b) for b in (-3, -1, 3, 1) for a in (-3, -1, 3, 1)]) / np.sqrt(10)
    tx = gray[rng.integers(0, 16, (modes, N))]
    mm, nn = np.meshgrid(np.arange(-R, R + 1), np.arange(-R, R + 1), indexing="ij")
    W = (rng.standard_normal(mm.shape) + 1j * rng.standard_normal(mm.shape)) * 1e-2
    W = (W + W.T) / 2
    W = (W + W[::-1, ::-1]) / 2
    W[np.abs(mm) + np.abs(nn) > R] = 0
    s = sino.SINO(R).set_weights(W, lw)
    tf = fg.Field(fg.Domain(modes, N, 1.0), data=tx[None])
    rx = lw * tx + s.cubic(tf).numpy()[0]
    rx = rx + 1e-6 * (rng.standard_normal(rx.shape) + 1j * rng.standard_normal(rx.shape))
    return tx, rx, W


def _covered(R):
    cov = np.zeros((2 * R + 1, 2 * R + 1), bool)
    for m in range(-(R // 2), R // 2 + 1):
        for n in range(abs(m), R - abs(m) + 1):
            for (a, b) in ((m, n), (n, m), (-m, -n), (-n, -m)):
                cov[a + R, b + R] = True
    return cov


def test_gpu_fit_recovers_known_coefficients(ctx):
    rng = np.random.default_rng(8)
    R, N, lw = 6, 6000, 0.8 - 0.3j
    tx, rx, W = _link(rng, R, N, lw)
    s = sino.SINO(R, 0.0, sino.SinoType.ORDINARY).train(tx, rx, solver="gpu")
    cov = _covered(R)
    assert abs(s.get_linear_weight() - lw) < 1e-4
    assert np.max(np.abs(s.weights[cov] - W[cov])) < 1e-4
    assert abs(s.get_intercept()) < 1e-4


@pytest.mark.parametrize("modes", [1, 2])
def test_gpu_fit_matches_host_fit(ctx, modes):
    rng = np.random.default_rng(9)
    R, N, lw = 16, 1 << 13, 0.9 + 0.1j
    tx, rx, _ = _link(rng, R, N, lw, modes)
    rx = rx + 1e-3 * (rng.standard_normal(rx.shape) + 1j * rng.standard_normal(rx.shape))
    g = sino.SINO(R).train(tx, rx, solver="gpu")
    h = sino.SINO(R).train(tx, rx, solver="lstsq")
    assert np.max(np.abs(g.weights - h.weights)) < 1e-4 * np.max(np.abs(h.weights)) + 1e-6
    assert abs(g.get_linear_weight() - h.get_linear_weight()) < 1e-5

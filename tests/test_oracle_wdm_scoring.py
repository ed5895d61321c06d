"""Pin the oracle's certainty-based decisions (find_certainty / sd / hd of
src/tasks/wdm_scoring.cpp:105-156).

The scoring task needs Armadillo, which is absent, so the reference cannot be
built; the C restatement is pinned against a literal pure-Python transcription
of the three functions (same loops, same expression order, complex128) and
against hand-checked cases.  CPU only.
"""
import cmath
import math

import numpy as np
import pytest

GRAY = [complex(r, i) / math.sqrt(10.0) for r, i in
        ((-3, -3), (-1, -3), (3, -3), (1, -3), (-3, -1), (-1, -1), (3, -1), (1, -1),
         (-3, 3), (-1, 3), (3, 3), (1, 3), (-3, 1), (-1, 1), (3, 1), (1, 1))]


def _demod(z):
    """demodulate_16qam (src/focss/processing/modulation.cpp:98-110)."""
    arg, mn = 0, abs(z - GRAY[0]) ** 2
    for code in range(1, 16):
        d = (z - GRAY[code]).real ** 2 + (z - GRAY[code]).imag ** 2
        if mn > d:
            mn, arg = d, code
    return arg


def _fro(a):
    return math.sqrt(sum(abs(v) ** 2 for v in a.ravel()))


def _find_certainty_loops(tx, rx):
    rows, cols = tx.shape
    scale = math.sqrt(tx.size) / _fro(tx)
    threshold = 1.0 / math.sqrt(5.0) / scale
    for s in range(cols):
        for m in range(rows):
            tc, rc = _demod(scale * tx[m, s]), _demod(scale * rx[m, s])
            if tc ^ rc:
                guess = GRAY[rc] / scale
                if threshold > abs(guess - rx[m, s]):
                    threshold = abs(guess - rx[m, s])
    return math.sqrt(5.0) * scale * threshold


def _sd_loops(field, certainty):
    rows, cols = field.shape
    amp = _fro(field) / math.sqrt(field.size)
    threshold = certainty / math.sqrt(5.0)
    result = field / amp
    for s in range(cols):
        for m in range(rows):
            guess = GRAY[_demod(result[m, s])]
            if abs(guess - result[m, s]) < threshold:
                result[m, s] = guess
    return amp * result


def _hd_loops(field):
    amp = _fro(field) / math.sqrt(field.size)
    result = field / amp
    for idx in np.ndindex(result.shape):
        result[idx] = GRAY[_demod(result[idx])]
    return amp * result


def _noisy(rng, rows, cols, sigma, power=0.7):
    codes = rng.integers(0, 16, (rows, cols))
    tx = np.array([[GRAY[c] for c in row] for row in codes]) * power
    rx = tx + sigma * (rng.standard_normal(tx.shape) + 1j * rng.standard_normal(tx.shape))
    return tx, rx


@pytest.mark.parametrize("sigma", [0.05, 0.1, 0.2])
def test_against_literal_loops(oracle_cpu, sigma):
    rng = np.random.default_rng(int(sigma * 100))
    tx, rx = _noisy(rng, 6, 300, sigma)
    want = _find_certainty_loops(tx, rx)
    got = oracle_cpu.find_certainty(tx, rx)
    assert abs(got - want) <= 1e-13 * abs(want)
    for c in (got, 0.3, 1.0):
        np.testing.assert_allclose(oracle_cpu.certainty_decision(rx, c), _sd_loops(rx.copy(), c), rtol=0, atol=1e-14)
    np.testing.assert_allclose(oracle_cpu.hd_rms(rx), _hd_loops(rx.copy()), rtol=0, atol=1e-14)


def test_hand_checked_cases(oracle_cpu):
    s10 = math.sqrt(10.0)
    # exact constellation points: no decision error, certainty = the 1/sqrt(5) cap
    tx = np.array([[complex(-3, -3), complex(1, 1), complex(3, -1), complex(-1, 3)]]) / s10
    assert abs(oracle_cpu.find_certainty(tx, tx) - 1.0) < 1e-15
    # one sample pushed across the boundary between 1/sqrt(10) and 3/sqrt(10)
    # (at 2/sqrt(10)) to 2.2/sqrt(10): its decided point 3/sqrt(10) lies
    # 0.8/sqrt(10) away; the RMS of tx is 1 (scale 1), so certainty =
    # sqrt(5) * 0.8 / sqrt(10) = 0.8 / sqrt(2)
    codes = np.arange(16)
    tx = np.array([GRAY[c] for c in codes])[None, :]
    rx = tx.copy()
    k = 15  # 1 + 1j
    rx[0, k] = complex(2.2, 1.0) / s10
    assert abs(oracle_cpu.find_certainty(tx, rx) - 0.8 / math.sqrt(2.0)) < 1e-14
    # sd at certainty 0.5 (radius 0.5/sqrt(5) = 0.224 at the RMS amplitude
    # 0.987): the samples 1.3% off a point snap to amp * point; the one half-way
    # between two points (0.32 from both) is kept
    f = np.array([[GRAY[5], complex(0.0, -1.0) / s10, GRAY[10], GRAY[0]]])
    amp = math.sqrt(np.mean(np.abs(f) ** 2))
    out = oracle_cpu.certainty_decision(f, 0.5)
    for i in (0, 2, 3):
        assert abs(out[0, i] / amp - GRAY[_demod(f[0, i] / amp)]) < 1e-15
    assert abs(out[0, 1] - f[0, 1]) < 1e-15
    # certainty 0 snaps nothing; hd snaps everything
    np.testing.assert_allclose(oracle_cpu.certainty_decision(f, 0.0), f, atol=1e-15)
    h = oracle_cpu.hd_rms(f)
    assert all(min(abs(h[0, i] / amp - g) for g in GRAY) < 1e-14 for i in range(4))
    assert cmath.isclose(h[0, 0] / amp, GRAY[_demod(f[0, 0] / amp)], abs_tol=1e-14)


def test_hd_rms_equals_hard_decision(oracle_cpu):
    """hd (RMS over rows and samples) and hard_decision_16qam (sqrt(average
    power / modes)) scale by the same amplitude."""
    rng = np.random.default_rng(3)
    _, rx = _noisy(rng, 6, 500, 0.1)
    np.testing.assert_allclose(oracle_cpu.hd_rms(rx), oracle_cpu.hard_decision(rx), rtol=0, atol=1e-14)

"""Pin the WdmPPE oracle (oracle/wdm_ppe_ref.py) against a literal
pure-Python transcription of src/focss/equalizer/wdm_sino.cpp (T, T1, T3:
:155-200; spm / xpm: :256-295; the feature loop of train: :43-81) and check
its fit on a synthetic link with known coefficients.  WdmPPE needs
Armadillo, which is absent, so the reference itself cannot be built.  CPU only.
"""
import numpy as np
import pytest

from oracle import wdm_ppe_ref as W


def _T(A, pol, k, m, n):
    term = 0j
    term += A[2, k + n] * np.conj(A[2, k + m + n])
    term += A[3, k + n] * np.conj(A[3, k + m + n])
    return A[2 + pol, k + m] * term


def _T1(A, pol, k, m, n):
    term = 0j
    if pol == 0:
        term += 2.0 * A[2, k + m] * A[0, k + n] * np.conj(A[0, k + m + n])
        term += A[2, k + m] * A[1, k + n] * np.conj(A[1, k + m + n])
        term += A[3, k + m] * A[0, k + n] * np.conj(A[1, k + m + n])
    else:
        term += 2.0 * A[3, k + m] * A[1, k + n] * np.conj(A[1, k + m + n])
        term += A[3, k + m] * A[0, k + n] * np.conj(A[0, k + m + n])
        term += A[2, k + m] * A[1, k + n] * np.conj(A[0, k + m + n])
    return term


def _T3(A, pol, k, m, n):
    term = 0j
    if pol == 0:
        term += 2.0 * A[2, k + m] * A[4, k + n] * np.conj(A[4, k + m + n])
        term += A[2, k + m] * A[5, k + n] * np.conj(A[5, k + m + n])
        term += A[3, k + m] * A[4, k + n] * np.conj(A[5, k + m + n])
    else:
        term += 2.0 * A[3, k + m] * A[5, k + n] * np.conj(A[5, k + m + n])
        term += A[3, k + m] * A[4, k + n] * np.conj(A[4, k + m + n])
        term += A[2, k + m] * A[5, k + n] * np.conj(A[4, k + m + n])
    return term


def _spm_loops(A, C, c):
    noise = np.zeros((2, A.shape[1]), complex)
    for k in range(c, A.shape[1] - c):
        for pol in range(2):
            for n in range(-c, c + 1):
                b = c - abs(n)
                for m in range(-b, b + 1):
                    noise[pol, k] += C[c + m, c + n] * _T(A, pol, k, m, n)
    return noise


def _xpm_loops(A, D, d):
    noise = np.zeros((2, A.shape[1]), complex)
    for k in range(d, A.shape[1] - d):
        for pol in range(2):
            for m in range(-d, d + 1):
                nb = d - abs(m)
                for n in range(-nb, nb + 1):
                    noise[pol, k] += D[d + m, d + n] * (_T1(A, pol, k, m, n) + _T3(A, pol, k, m, -n))
    return noise


def _features_loops(A, c, d):
    N = A.shape[1]
    R = max(c, d)
    nf = W.n_features(c, d)
    cube = np.zeros((N - 2 * R, nf, 2), complex)
    for pol in range(2):
        for s in range(R, N - R):
            i = 0
            for m in range(-(c // 2), c // 2 + 1):
                for n in range(abs(m), c - abs(m) + 1):
                    if m == 0 and n == 0:
                        v = _T(A, pol, s, 0, 0)
                    elif m == n:
                        v = _T(A, pol, s, m, n) + _T(A, pol, s, -m, -n)
                    elif m == -n:
                        v = _T(A, pol, s, m, n) + _T(A, pol, s, n, m)
                    else:
                        v = _T(A, pol, s, m, n) + _T(A, pol, s, n, m) + _T(A, pol, s, -m, -n) + _T(A, pol, s, -n, -m)
                    cube[s - R, i, pol] = v
                    i += 1
            for m in range(-d, d + 1):
                nb = d - abs(m)
                for n in range(-nb, nb + 1):
                    cube[s - R, i, pol] = _T1(A, pol, s, m, n) + _T3(A, pol, s, m, -n)
                    i += 1
            cube[s - R, i, pol] = A[2 + pol, s]
    return np.concatenate([cube[:, :, 0], cube[:, :, 1]], axis=0)


def _rand(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _tables(rng, c, d):
    ppe = W.WdmPPE(c, d)
    return ppe.install(_rand(rng, W.n_features(c, d)) * 0.01)


@pytest.mark.parametrize("c,d", [(4, 2), (3, 0), (0, 3)])
def test_against_literal_loops(c, d):
    rng = np.random.default_rng(10 * c + d)
    A = _rand(rng, (6, 40))
    ppe = _tables(rng, c, d)
    np.testing.assert_allclose(ppe.spm(A), _spm_loops(A, ppe.C, c), rtol=0, atol=1e-13)
    np.testing.assert_allclose(ppe.xpm(A), _xpm_loops(A, ppe.D, d), rtol=0, atol=1e-13)
    np.testing.assert_allclose(W.features(A, c, d), _features_loops(A, c, d), rtol=0, atol=1e-13)
    k = np.arange(5, 30)
    for pol in range(2):
        for (m, n) in ((1, 2), (-2, 1), (0, 0), (3, -2)):
            np.testing.assert_allclose(W.T1(A, pol, k, m, n), [_T1(A, pol, j, m, n) for j in k], atol=1e-13)
            np.testing.assert_allclose(W.T3(A, pol, k, m, n), [_T3(A, pol, j, m, n) for j in k], atol=1e-13)


def test_tables_are_symmetric_images():
    """install (wdm_sino.cpp:105-135): C is filled on the whole diamond with
    C(m, n) = C(n, m) = C(-m, -n) = C(-n, -m); D on the diamond only."""
    rng = np.random.default_rng(2)
    c, d = 6, 3
    ppe = _tables(rng, c, d)
    mm, nn = np.meshgrid(np.arange(-c, c + 1), np.arange(-c, c + 1), indexing="ij")
    inside = np.abs(mm) + np.abs(nn) <= c
    assert np.all(ppe.C[inside] != 0) and np.all(ppe.C[~inside] == 0)
    np.testing.assert_array_equal(ppe.C, ppe.C.T)
    np.testing.assert_array_equal(ppe.C, ppe.C[::-1, ::-1])
    md, nd = np.meshgrid(np.arange(-d, d + 1), np.arange(-d, d + 1), indexing="ij")
    assert np.all((ppe.D != 0) == (np.abs(md) + np.abs(nd) <= d))


def test_train_recovers_known_coefficients():
    rng = np.random.default_rng(5)
    c, d, N = 4, 2, 3000
    truth = _tables(rng, c, d)
    truth.linear_weight = 0.7 - 0.2j
    tx = _rand(rng, (6, N)) / np.sqrt(2)
    rx = np.zeros_like(tx)
    rx[2:4] = truth.model(tx) + 0.05 + 0.02j
    ppe = W.WdmPPE(c, d).train(tx, rx)
    assert abs(ppe.linear_weight - truth.linear_weight) < 1e-10
    assert np.max(np.abs(ppe.C - truth.C)) < 1e-10
    assert np.max(np.abs(ppe.D - truth.D)) < 1e-10
    R = max(c, d)
    assert abs(ppe.intercept - (0.05 + 0.02j)) < 1e-10
    # the equalizer inverts the model inside [R, N - R)
    eq = ppe.equalize(tx, rx - (0.05 + 0.02j))
    np.testing.assert_allclose(eq[:, R:N - R], tx[2:4, R:N - R], atol=1e-9)

"""Oracle (test infrastructure only): FP64 numpy restatement of focss::WdmPPE,
the dual-polarization WDM perturbation equalizer with SPM and XPM triplets
(src/focss/equalizer/wdm_sino.cpp, src/focss/equalizer/wdm_sino.h).

Data layout as in the reference: a (6, N) complex matrix A whose rows are
channel * 2 + polarization for the left neighbour (rows 0, 1), the centre
channel (2, 3) and the right neighbour (4, 5) (the dataset layout of
src/tasks/wdm_scoring.cpp:79-103).  Outputs are (2, N): the centre channel.

WdmPPE needs Armadillo, which is absent, so the reference cannot be built:
this restatement is pinned against a literal pure-Python transcription of
T / T1 / T3 / spm / xpm (tests/test_oracle_wdm_ppe.py) and checked on a
synthetic link with known coefficients.  Parity unpinned against a reference
run.
"""
from __future__ import annotations

import numpy as np


def n_features(c_radius: int, d_radius: int) -> int:
    """wdm_sino.cpp:32-34."""
    n_spm = 0 if c_radius < 0 else c_radius * (c_radius + 2) // 2 + 1
    n_xpm = 0 if d_radius < 0 else 2 * d_radius * d_radius + 2 * d_radius + 1
    return n_spm + n_xpm + 1


def spm_pairs(c_radius: int):
    """(m, n) of the symmetry-reduced SPM features (wdm_sino.cpp:47-71)."""
    mb = c_radius // 2
    return [(m, n) for m in range(-mb, mb + 1) for n in range(abs(m), c_radius - abs(m) + 1)] if c_radius >= 0 else []


def xpm_pairs(d_radius: int):
    """(m, n) of the XPM features, |m| + |n| <= d (wdm_sino.cpp:72-78)."""
    if d_radius < 0:
        return []
    return [(m, n) for m in range(-d_radius, d_radius + 1)
            for n in range(-(d_radius - abs(m)), d_radius - abs(m) + 1)]


def T(A, pol, k, m, n):
    """WdmPPE::T (wdm_sino.cpp:155-164), vectorized over the sample index k."""
    term = A[2, k + n] * np.conj(A[2, k + m + n]) + A[3, k + n] * np.conj(A[3, k + m + n])
    return A[2 + pol, k + m] * term


def _T13(A, pol, k, m, n, r0, r1):
    """T1 (neighbour rows r0, r1 = 0, 1) / T3 (rows 4, 5) of wdm_sino.cpp:166-200."""
    if pol == 0:
        return (2.0 * A[2, k + m] * A[r0, k + n] * np.conj(A[r0, k + m + n])
                + A[2, k + m] * A[r1, k + n] * np.conj(A[r1, k + m + n])
                + A[3, k + m] * A[r0, k + n] * np.conj(A[r1, k + m + n]))
    return (2.0 * A[3, k + m] * A[r1, k + n] * np.conj(A[r1, k + m + n])
            + A[3, k + m] * A[r0, k + n] * np.conj(A[r0, k + m + n])
            + A[2, k + m] * A[r1, k + n] * np.conj(A[r0, k + m + n]))


def T1(A, pol, k, m, n):
    return _T13(A, pol, k, m, n, 0, 1)


def T3(A, pol, k, m, n):
    return _T13(A, pol, k, m, n, 4, 5)


def features(tx, c_radius, d_radius):
    """The (2 * (N - 2R), n_features) design matrix of WdmPPE::train
    (wdm_sino.cpp:42-82): polarization-major rows, SPM features, XPM
    features, then the transmitted centre sample."""
    A = np.asarray(tx, np.complex128)
    N = A.shape[1]
    R = max(c_radius, d_radius)
    k = np.arange(R, N - R)
    cols = []
    for pol in range(2):
        fp = []
        for (m, n) in spm_pairs(c_radius):
            if m == 0 and n == 0:
                f = T(A, pol, k, 0, 0)
            elif m == n:
                f = T(A, pol, k, m, n) + T(A, pol, k, -m, -n)
            elif m == -n:
                f = T(A, pol, k, m, n) + T(A, pol, k, n, m)
            else:
                f = T(A, pol, k, m, n) + T(A, pol, k, n, m) + T(A, pol, k, -m, -n) + T(A, pol, k, -n, -m)
            fp.append(f)
        for (m, n) in xpm_pairs(d_radius):
            fp.append(T1(A, pol, k, m, n) + T3(A, pol, k, m, -n))
        fp.append(A[2 + pol, k])
        cols.append(np.stack(fp, axis=1))
    return np.concatenate(cols, axis=0)


class WdmPPE:
    """focss::WdmPPE (wdm_sino.h:8-71)."""

    def __init__(self, c_radius=0, d_radius=None):
        self.c_radius = c_radius
        self.d_radius = c_radius if d_radius is None else d_radius
        self.trained = False

    def train(self, tx, rx):
        """wdm_sino.cpp:28-142: z-scored least squares (arma stddev with
        normalization by N), then the symmetric C and diamond D tables."""
        c, d = self.c_radius, self.d_radius
        R = max(c, d)
        A, Rx = np.asarray(tx, np.complex128), np.asarray(rx, np.complex128)
        N = A.shape[1]
        resp = np.concatenate([Rx[2, R:N - R], Rx[3, R:N - R]])
        X = features(A, c, d)
        x_std = np.sqrt(np.mean(np.abs(X - X.mean(axis=0)) ** 2, axis=0))
        x_mean = X.mean(axis=0)
        y_mean = resp.mean()
        Z = (X - x_mean) / x_std
        raw = np.linalg.lstsq(Z, resp - y_mean, rcond=None)[0] / x_std
        self.install(raw, y_mean - np.sum(raw * x_mean))
        return self

    def install(self, raw, intercept=0j):
        """Coefficient tables from the raw feature weights (wdm_sino.cpp:100-139)."""
        c, d = self.c_radius, self.d_radius
        C = np.zeros((2 * c + 1, 2 * c + 1), np.complex128) if c >= 0 else np.zeros((0, 0), np.complex128)
        D = np.zeros((2 * d + 1, 2 * d + 1), np.complex128) if d >= 0 else np.zeros((0, 0), np.complex128)
        i = 0
        for (m, n) in spm_pairs(c):
            w = raw[i]
            if m == n:
                images = ((m, n), (-m, -n))
            elif m == -n:
                images = ((m, n), (n, m))
            else:
                images = ((m, n), (n, m), (-m, -n), (-n, -m))
            for (a, b) in images:
                C[c + a, c + b] = w
            i += 1
        for (m, n) in xpm_pairs(d):
            D[d + m, d + n] = raw[i]
            i += 1
        self.C, self.D = C, D
        self.linear_weight = complex(raw[i])
        self.intercept = complex(intercept)
        self.trained = True
        return self

    def spm(self, field):
        """wdm_sino.cpp:256-274: sum over |m| + |n| <= c of C(m, n) T, for
        k in [c, N - c), zero elsewhere."""
        A = np.asarray(field, np.complex128)
        c, N = self.c_radius, A.shape[1]
        out = np.zeros((2, N), np.complex128)
        if c < 0:
            return out
        k = np.arange(c, N - c)
        for pol in range(2):
            acc = np.zeros(k.size, np.complex128)
            for n in range(-c, c + 1):
                b = c - abs(n)
                for m in range(-b, b + 1):
                    acc += self.C[c + m, c + n] * T(A, pol, k, m, n)
            out[pol, k] = acc
        return out

    def xpm(self, field):
        """wdm_sino.cpp:276-295."""
        A = np.asarray(field, np.complex128)
        d, N = self.d_radius, A.shape[1]
        out = np.zeros((2, N), np.complex128)
        if d < 0:
            return out
        k = np.arange(d, N - d)
        for pol in range(2):
            acc = np.zeros(k.size, np.complex128)
            for m in range(-d, d + 1):
                b = d - abs(m)
                for n in range(-b, b + 1):
                    acc += self.D[d + m, d + n] * (T1(A, pol, k, m, n) + T3(A, pol, k, m, -n))
            out[pol, k] = acc
        return out

    def cubic(self, field):
        return self.spm(field) + self.xpm(field)

    def linear(self, field):
        return self.linear_weight * np.asarray(field, np.complex128)[2:4]

    def model(self, field):
        return self.linear(field) + self.cubic(field)

    def equalize(self, tx_spm, tx_xpm, rx=None):
        """equalize(tx, rx) = (rx[2:4] - cubic(tx)) / a; equalize(tx_spm,
        tx_xpm, rx) = (rx[2:4] - spm(tx_spm) - xpm(tx_xpm)) / a
        (wdm_sino.cpp:240-249)."""
        if rx is None:
            tx_spm, tx_xpm, rx = tx_spm, tx_spm, tx_xpm
        rx = np.asarray(rx, np.complex128)
        return (rx[2:4] - self.spm(tx_spm) - self.xpm(tx_xpm)) / self.linear_weight

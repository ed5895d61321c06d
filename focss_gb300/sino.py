"""Perturbation (triplet) equalizer: mirror of focss::SINO
(src/focss/equalizer/sino.h:10-50, sino.cpp).

`cubic` and `equalize` run on the GPU (focss_triplet_apply /
focss_sino_equalize).  `train` is the reference's least-squares fit of the
triplet coefficients restated with numpy on the host (sino.cpp:42-159): it
produces the coefficient table once, off the propagation/equalization path.
"""
from __future__ import annotations

import ctypes as C
from enum import IntEnum

import numpy as np

from ._lib import check, lib
from .api import Field

ORDINARY, FIXED, HOMOGENEOUS = 0, 1, 2  # sino.h:8


class SinoType(IntEnum):
    ORDINARY = 0
    FIXED = 1
    HOMOGENEOUS = 2


def solve_normal_equations(gram, nf, residual=None, refinements=2):
    """x = G^-1 g for the (nf+1)^2 Gram matrix [Z y]^H [Z y] returned by the
    GPU (upper triangle valid): Cholesky in FP64 on the host, then
    `refinements` steps of iterative refinement x += G^-1 residual(x) with
    residual(x) = Z^H (y - Z x) evaluated in FP64 on the GPU, which removes
    the effect of the Gram matrix's FP32 chunk sums on ill-conditioned fits."""
    Gu = np.triu(gram)
    G = Gu + np.conj(np.triu(Gu, 1)).T              # Hermitian from the upper triangle
    A, g = G[:nf, :nf], G[:nf, nf]
    try:
        from scipy.linalg import cho_factor, cho_solve
        fac = cho_factor(A)
        solve = lambda b: cho_solve(fac, b)  # noqa: E731
    except Exception:  # not positive definite to working precision, or no scipy
        solve = lambda b: np.linalg.solve(A, b)  # noqa: E731
    x = solve(g)
    if residual is not None:
        for _ in range(refinements):
            x = x + solve(residual(x))
    return x


def diamond_terms(weights, radius, prune=0.0):
    """(m, n, C) for |m| + |n| <= radius from a (2R+1)^2 matrix W[m+R, n+R]
    (the summation domain of SINO::cubic, sino.cpp:206-214); optionally drop
    |C| < prune * max|C|."""
    R = radius
    mm, nn = np.meshgrid(np.arange(-R, R + 1), np.arange(-R, R + 1), indexing="ij")
    keep = (np.abs(mm) + np.abs(nn)) <= R
    c = np.asarray(weights)[keep]
    m, n = mm[keep], nn[keep]
    if prune > 0:
        big = np.abs(c) >= prune * np.abs(c).max()
        m, n, c = m[big], n[big], c[big]
    return m.astype(np.int32), n.astype(np.int32), c.astype(np.complex128)


def box_terms(weights, radius, prune=0.0):
    """(m, n, C) over the full box |m|, |n| <= radius, pruned at prune * max|C|."""
    R = radius
    mm, nn = np.meshgrid(np.arange(-R, R + 1), np.arange(-R, R + 1), indexing="ij")
    c = np.asarray(weights).ravel()
    m, n = mm.ravel(), nn.ravel()
    keep = np.abs(c) > 0
    if prune > 0:
        keep &= np.abs(c) >= prune * np.abs(c).max()
    return m[keep].astype(np.int32), n[keep].astype(np.int32), c[keep].astype(np.complex128)


def triplet_apply(field: Field, radius: int, m, n, c) -> Field:
    """sum_i C_i A[k+m_i] A[k+n_i] conj(A[k+m_i+n_i]) for k in [R, N-R) (GPU)."""
    m = np.ascontiguousarray(m, dtype=np.int32)
    n = np.ascontiguousarray(n, dtype=np.int32)
    c = np.ascontiguousarray(c, dtype=np.complex128)
    out = Field(field.domain, batch=field.batch, ctx=field.ctx)
    check(lib().focss_triplet_apply(field.ctx.h, field.h, radius, m.size, m.ctypes.data_as(C.c_void_p),
                                    n.ctypes.data_as(C.c_void_p), c.ctypes.data_as(C.c_void_p), out.h),
          field.ctx.h)
    return out


def _term(a, k, m, n):
    """SINO::term (sino.cpp:161-171) for a vector of k; a is (modes, N)."""
    t = np.sum(a[:, k + n] * np.conj(a[:, k + m + n]), axis=0)
    return a[:, k + m] * t[None, :]


class SINO:
    def __init__(self, radius=0, lambda_=1.0, type_=SinoType.ORDINARY):
        self.radius = radius
        self.lambda_ = lambda_
        self.type = SinoType(type_)
        self.trained = False
        self.intercept = 0j
        self.linear_weight = 0j
        self.weights = None

    def set_radius(self, r):
        self.radius = r
        self.trained = False
        return self

    def set_lambda(self, x):
        self.lambda_ = x
        self.trained = False
        return self

    def set_type(self, t):
        self.type = SinoType(t)
        self.trained = False
        return self

    def set_linear_weight(self, w):
        self.linear_weight = complex(w)
        self.trained = False
        return self

    def set_weights(self, W, linear_weight=None):
        """Install a (2R+1)^2 coefficient matrix directly (e.g. analytic C_mn)."""
        self.weights = np.asarray(W, dtype=np.complex128)
        self.radius = (self.weights.shape[0] - 1) // 2
        if linear_weight is not None:
            self.linear_weight = complex(linear_weight)
        self.trained = True
        return self

    # ---- sino.cpp:42-159 with the normal equations formed on the GPU
    def _residual(self, transmitted, received, x):
        lw = complex(self.linear_weight)
        x = np.ascontiguousarray(x, np.complex128)
        r = np.zeros_like(x)
        check(lib().focss_sino_residual(transmitted.ctx.h, transmitted.h, received.h, self.radius, int(self.type),
                                        lw.real, lw.imag, x.ctypes.data_as(C.c_void_p),
                                        r.ctypes.data_as(C.c_void_p)), transmitted.ctx.h)
        return r

    def _train_gpu(self, transmitted, received):
        from .api import Domain
        if not isinstance(transmitted, Field):
            t = np.atleast_2d(np.asarray(transmitted, np.complex128))
            r = np.atleast_2d(np.asarray(received, np.complex128))
            transmitted = Field(Domain(t.shape[0], t.shape[1], 1.0), data=t[None])
            received = Field(Domain(r.shape[0], r.shape[1], 1.0), data=r[None], ctx=transmitted.ctx)
        R = self.radius
        nf = int(lib().focss_sino_num_features(R, int(self.type)))
        gram = np.zeros((nf + 1, nf + 1), np.complex128)
        mean = np.zeros(nf + 1, np.complex128)
        sd = np.zeros(nf, np.float64)
        lw = complex(self.linear_weight)
        check(lib().focss_sino_gram(transmitted.ctx.h, transmitted.h, received.h, R, int(self.type), lw.real, lw.imag,
                                    gram.ctypes.data_as(C.c_void_p), mean.ctypes.data_as(C.c_void_p),
                                    sd.ctypes.data_as(C.c_void_p)), transmitted.ctx.h)
        raw = solve_normal_equations(gram, nf, lambda x: self._residual(transmitted, received, x))
        raw = raw / sd
        x_mean, y_mean = mean[:nf], mean[nf]
        return raw, x_mean, y_mean

    # ---- sino.cpp:42-159, restated with numpy (host), or solver="gpu"
    def train(self, transmitted, received, solver="lstsq"):
        if solver == "gpu":
            raw, x_mean, y_mean = self._train_gpu(transmitted, received)
            self.intercept = y_mean - np.sum(raw * x_mean)
            return self._install(raw)
        tx = np.atleast_2d(np.asarray(transmitted.numpy()[0] if isinstance(transmitted, Field) else transmitted))
        rx = np.atleast_2d(np.asarray(received.numpy()[0] if isinstance(received, Field) else received))
        R = self.radius
        modes, N = tx.shape
        nspm = N - 2 * R
        nf = R * (R + 2) // 2 + 1 + (1 if self.type == SinoType.ORDINARY else 0)
        k = np.arange(nspm) + R
        if self.type == SinoType.FIXED:
            resp = (rx[:, k] - tx[:, k] * self.linear_weight).ravel()
        else:
            resp = rx[:, k].ravel()
        X = np.zeros((modes * nspm, nf), np.complex128)
        idx = 0
        mb = R // 2
        pairs = []
        for m in range(-mb, mb + 1):
            for n in range(abs(m), R - abs(m) + 1):
                if m == 0 and n == 0:
                    col = _term(tx, k, 0, 0)
                elif m == n:
                    col = _term(tx, k, m, n) + _term(tx, k, -m, -n)
                elif m == -n:
                    col = _term(tx, k, m, n) + _term(tx, k, n, m)
                else:
                    col = _term(tx, k, m, n) + _term(tx, k, n, m) + _term(tx, k, -m, -n) + _term(tx, k, -n, -m)
                X[:, idx] = col.ravel()
                pairs.append((m, n))
                idx += 1
        if self.type == SinoType.ORDINARY:
            X[:, idx] = tx[:, k].ravel()
        x_mean = X.mean(axis=0)
        x_std = np.sqrt(np.mean(np.abs(X - x_mean) ** 2, axis=0))  # arma stddev(.., 1, 0)
        y_mean = resp.mean()
        resp = resp - y_mean
        Z = (X - x_mean) / x_std
        if solver == "normal":
            G = Z.conj().T @ Z
            raw = np.linalg.solve(G, Z.conj().T @ resp)
        else:
            raw = np.linalg.lstsq(Z, resp, rcond=None)[0]
        raw = raw / x_std
        self.intercept = y_mean - np.sum(raw * x_mean)
        return self._install(raw)

    def _pairs(self):
        R = self.radius
        mb = R // 2
        return [(m, n) for m in range(-mb, mb + 1) for n in range(abs(m), R - abs(m) + 1)]

    def _install(self, raw):
        """Weights matrix from the raw feature weights (sino.cpp:126-153)."""
        R = self.radius
        pairs = self._pairs()
        W = np.zeros((2 * R + 1, 2 * R + 1), np.complex128)
        for i, (m, n) in enumerate(pairs):
            w = raw[i]
            if m == 0 and n == 0:
                W[R, R] = w
            elif m == n:
                W[R + m, R + n] = w
                W[R - m, R - n] = w
            elif m == -n:
                W[R + m, R + n] = w
                W[R + n, R + m] = w
            else:
                W[R + m, R + n] = w
                W[R + n, R + m] = w
                W[R - m, R - n] = w
                W[R - n, R - m] = w
        if self.type == SinoType.ORDINARY:
            self.linear_weight = raw[len(pairs)]
        elif self.type == SinoType.HOMOGENEOUS:
            self.linear_weight = 0j
        self.weights = W
        self.trained = True
        return self

    def terms(self, prune=0.0):
        return diamond_terms(self.weights, self.radius, prune)

    def get_intercept(self):
        return self.intercept

    def get_linear_weight(self):
        return self.linear_weight

    def get_coo_weight(self):
        return self.weights[self.radius, self.radius]

    def cubic(self, original: Field, prune=0.0) -> Field:
        m, n, c = self.terms(prune)
        return triplet_apply(original, self.radius, m, n, c)

    def equalize(self, rx: Field, tx: Field, prune=0.0) -> Field:
        """(rx - cubic(tx)) / linear_weight (sino.cpp:193-196), on the GPU."""
        m, n, c = self.terms(prune)
        lw = complex(self.linear_weight)
        out = Field(rx.domain, batch=rx.batch, ctx=rx.ctx)
        check(lib().focss_sino_equalize(rx.ctx.h, rx.h, tx.h, self.radius, m.size, m.ctypes.data_as(C.c_void_p),
                                        n.ctypes.data_as(C.c_void_p), c.ctypes.data_as(C.c_void_p), lw.real,
                                        lw.imag, out.h), rx.ctx.h)
        return out

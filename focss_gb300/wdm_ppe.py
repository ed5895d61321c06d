"""Dual-polarization WDM perturbation equalizer: mirror of focss::WdmPPE
(src/focss/equalizer/wdm_sino.h:8-71, wdm_sino.cpp).

Fields are 6-row realizations, rows channel * 2 + polarization: left
neighbour 0-1, centre 2-3, right neighbour 4-5 (the dataset layout of
src/tasks/wdm_scoring.cpp:79-103, see io.load_field).  Outputs are 2-row
Fields (the centre channel).

The SPM / XPM triplet sums, the equalizer and the normal equations of the fit
run on the GPU (focss_wdm_ppe_apply, focss_wdm_ppe_gram); the host solves
the small Hermitian system in FP64 and lays out the coefficient tables.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib
from .api import Domain, Field
from .sino import solve_normal_equations


def _vp(a):
    return a.ctypes.data_as(C.c_void_p)


def _field(x, ctx=None) -> Field:
    """A 6-row Field from a Field or a (6, N) / (batch, 6, N) array."""
    if isinstance(x, Field):
        return x
    a = np.asarray(x, np.complex128)
    if a.ndim == 2:
        a = a[None]
    return Field(Domain(a.shape[1], a.shape[2], 1.0), data=a, batch=a.shape[0], ctx=ctx)


def _pairs_spm(c):
    mb = c // 2
    return [(m, n) for m in range(-mb, mb + 1) for n in range(abs(m), c - abs(m) + 1)] if c >= 0 else []


def _pairs_xpm(d):
    return [(m, n) for m in range(-d, d + 1) for n in range(-(d - abs(m)), d - abs(m) + 1)] if d >= 0 else []


class WdmPPE:
    """focss::WdmPPE: WdmPPE(), WdmPPE(radii), WdmPPE(c_radius, d_radius)."""

    def __init__(self, c_radius: int = 0, d_radius: int | None = None):
        self.c_radius = int(c_radius)
        self.d_radius = int(c_radius if d_radius is None else d_radius)
        self.trained = False
        self.intercept = 0j
        self.linear_weight = 0j
        self.C = None
        self.D = None

    def set_c_radius(self, c_radius):
        self.c_radius = int(c_radius)
        self.trained = False
        return self

    def set_d_radius(self, d_radius):
        self.d_radius = int(d_radius)
        self.trained = False
        return self

    # ---- wdm_sino.cpp:28-142: the normal equations on the GPU, FP64 solve
    # with iterative refinement against the FP64 residual of the design
    def train(self, tx, rx):
        t = _field(tx)
        r = _field(rx, ctx=t.ctx)
        c, d = self.c_radius, self.d_radius
        nf = int(lib().focss_wdm_ppe_num_features(c, d))
        gram = np.zeros((nf + 1, nf + 1), np.complex128)
        mean = np.zeros(nf + 1, np.complex128)
        sd = np.zeros(nf, np.float64)
        check(lib().focss_wdm_ppe_gram(t.ctx.h, t.h, r.h, c, d, _vp(gram), _vp(mean), _vp(sd)), t.ctx.h)

        def residual(x):
            x = np.ascontiguousarray(x, np.complex128)
            out = np.zeros_like(x)
            check(lib().focss_wdm_ppe_residual(t.ctx.h, t.h, r.h, c, d, _vp(x), _vp(out)), t.ctx.h)
            return out

        raw = solve_normal_equations(gram, nf, residual) / sd
        self.intercept = complex(mean[nf] - np.sum(raw * mean[:nf]))
        return self.install(raw)

    def install(self, raw):
        """Coefficient tables from the raw feature weights (wdm_sino.cpp:100-139)."""
        c, d = self.c_radius, self.d_radius
        Cm = np.zeros((2 * c + 1, 2 * c + 1), np.complex128) if c >= 0 else None
        Dm = np.zeros((2 * d + 1, 2 * d + 1), np.complex128) if d >= 0 else None
        i = 0
        for (m, n) in _pairs_spm(c):
            w = raw[i]
            if m == n:
                images = ((m, n), (-m, -n))
            elif m == -n:
                images = ((m, n), (n, m))
            else:
                images = ((m, n), (n, m), (-m, -n), (-n, -m))
            for (a, b) in images:
                Cm[c + a, c + b] = w
            i += 1
        for (m, n) in _pairs_xpm(d):
            Dm[d + m, d + n] = raw[i]
            i += 1
        self.C, self.D = Cm, Dm
        self.linear_weight = complex(raw[i])
        self.trained = True
        return self

    def set_tables(self, C=None, D=None, linear_weight=None):
        """Install coefficient tables directly ((2c+1)^2 and (2d+1)^2)."""
        if C is not None:
            self.C = np.asarray(C, np.complex128)
            self.c_radius = (self.C.shape[0] - 1) // 2
        if D is not None:
            self.D = np.asarray(D, np.complex128)
            self.d_radius = (self.D.shape[0] - 1) // 2
        if linear_weight is not None:
            self.linear_weight = complex(linear_weight)
        self.trained = True
        return self

    def get_intercept(self):
        return self.intercept

    def get_linear_weight(self):
        return self.linear_weight

    def get_coo_weight(self):
        return self.C[self.c_radius, self.c_radius]

    # ---- wdm_sino.cpp:235-300 on the GPU
    def _apply(self, spm_in=None, xpm_in=None, rx=None, lin_in=None) -> Field:
        if not self.trained:
            raise RuntimeError("WdmPPE: not trained")
        ref = next(f for f in (spm_in, xpm_in, lin_in, rx) if f is not None)
        ctx = ref.ctx
        out = Field(Domain(2, ref.domain.samples, ref.domain.time_step, ref.domain.center_frequency),
                    batch=ref.batch, ctx=ctx)
        Cm = np.ascontiguousarray(self.C if self.C is not None else np.zeros((1, 1)), np.complex128)
        Dm = np.ascontiguousarray(self.D if self.D is not None else np.zeros((1, 1)), np.complex128)
        lw = complex(self.linear_weight)
        h = lambda f: None if f is None else f.h  # noqa: E731
        check(lib().focss_wdm_ppe_apply(ctx.h, h(spm_in), h(xpm_in), h(rx), h(lin_in), self.c_radius, _vp(Cm),
                                        self.d_radius, _vp(Dm), lw.real, lw.imag, out.h), ctx.h)
        return out

    def spm(self, field) -> Field:
        return self._apply(spm_in=_field(field))

    def xpm(self, field) -> Field:
        return self._apply(xpm_in=_field(field))

    def cubic(self, field) -> Field:
        f = _field(field)
        return self._apply(spm_in=f if self.c_radius >= 0 else None, xpm_in=f if self.d_radius >= 0 else None)

    def linear(self, field) -> Field:
        return self._apply(lin_in=_field(field))

    def model(self, field) -> Field:
        f = _field(field)
        return self._apply(spm_in=f if self.c_radius >= 0 else None, xpm_in=f if self.d_radius >= 0 else None,
                           lin_in=f)

    def equalize(self, tx_spm, tx_xpm, rx=None) -> Field:
        """equalize(tx, rx) = (rx_centre - cubic(tx)) / a and
        equalize(tx_spm, tx_xpm, rx) = (rx_centre - spm(tx_spm) - xpm(tx_xpm)) / a
        (wdm_sino.cpp:240-249)."""
        if rx is None:
            tx_spm, tx_xpm, rx = tx_spm, tx_spm, tx_xpm
        s = _field(tx_spm)
        x = s if tx_xpm is tx_spm else _field(tx_xpm, ctx=s.ctx)
        r = _field(rx, ctx=s.ctx)
        return self._apply(spm_in=s if self.c_radius >= 0 else None, xpm_in=x if self.d_radius >= 0 else None, rx=r)

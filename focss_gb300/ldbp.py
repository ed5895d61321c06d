"""Learned digital back-propagation (few learned steps per span) over the C ABI.

The model replaces backward_propagation (src/tasks/systems.cpp:73-91) with
`steps` learned [FIR dispersion filter, nonlinear phase gain] pairs per span
and a learned matched filter; all compute, including the backward pass and
the Adam update, runs in libfocss_gpu (focss_ldbp_*).  Plain split-step DBP
provides the initialisation (`init_from_dbp`).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib
from .api import Context, Field

P = C.c_void_p


def taps_from_response(H, taps):
    """Truncated FIR taps (layout FIR(x, h)[n] = sum_t h[t] x[n + t - c]) of a
    circular filter with frequency response H (numpy FFT bin order)."""
    n = H.size
    g = np.fft.fft(H) / n  # h[c + d] = fft(H)[d] / N
    c = (taps - 1) // 2
    d = np.arange(-c, c + 1)
    return g[d % n]


def dispersion_response(length, alpha, beta2, dt, n_fft):
    """A BACKWARD linear step of `length` metres: exp(+alpha L/2) exp(-i beta2/2 L w^2)
    (src/focss/solver/ssfm.cpp:142-150 with a negative step)."""
    w = 2 * np.pi * np.fft.fftfreq(n_fft, dt)
    return np.exp(0.5 * alpha * length) * np.exp(-0.5j * beta2 * length * w ** 2)


def dispersion_taps(length, alpha, beta2, dt, n_fft, taps):
    return taps_from_response(dispersion_response(length, alpha, beta2, dt, n_fft), taps)


def rrc_response(n_symbols, osf, roll_off, ctx=None):
    """Frequency response of rrc_sampling's circular filter (modulation.cpp:92-96,
    field.cpp:358-372): FFT(ifftshift(pulse)) / N."""
    from .dsp import rrc_pulse
    p = rrc_pulse(n_symbols, osf, roll_off, ctx=ctx)
    return np.fft.fft(np.fft.ifftshift(p)) / p.size


def matched_filter_taps(n_symbols, osf, roll_off, taps, ctx=None):
    """The matched filter of rrc_sampling (src/focss/processing/modulation.cpp:92-96):
    circular convolution with the full-length pulse / N, truncated to `taps`
    centred taps (pulse from the device, focss_rrc_pulse)."""
    from .dsp import rrc_pulse
    p = rrc_pulse(n_symbols, osf, roll_off, ctx=ctx)
    N = p.size
    c = (taps - 1) // 2
    return p[N // 2 - c: N // 2 + c + 1] / N


class LearnedDBP:
    def __init__(self, spans, steps, taps, mf_taps, samples, batch, span_scale, ctx=None):
        self.ctx = ctx or Context.default()
        self.spans, self.steps, self.taps, self.mf_taps = spans, steps, taps, mf_taps
        self.samples, self.batch, self.span_scale = samples, batch, span_scale
        h = C.c_void_p()
        check(lib().focss_ldbp_create(self.ctx.h, spans, steps, taps, mf_taps, samples, batch, span_scale,
                                      C.byref(h)), self.ctx.h)
        self.h = h
        self.n_params = lib().focss_ldbp_num_params(h)

    # ---- parameter layout (include/focss_gpu.h)
    @property
    def layers(self):
        return self.spans * self.steps

    def pack(self, h, xi, hmf):
        L = self.layers
        out = np.zeros(self.n_params, np.float32)
        out[: 2 * L * self.taps] = np.asarray(h, np.complex64).reshape(L, self.taps).view(np.float32).ravel()
        out[2 * L * self.taps: 2 * L * self.taps + L] = np.asarray(xi, np.float32).ravel()
        xc = (L + 1) & ~1
        out[2 * L * self.taps + xc:] = np.asarray(hmf, np.complex64).view(np.float32).ravel()
        return out

    def unpack(self, flat):
        L = self.layers
        flat = np.asarray(flat, np.float32)
        h = flat[: 2 * L * self.taps].view(np.complex64).reshape(L, self.taps).astype(np.complex128)
        xi = flat[2 * L * self.taps: 2 * L * self.taps + L].astype(np.float64)
        xc = (L + 1) & ~1
        hmf = flat[2 * L * self.taps + xc:].view(np.complex64).astype(np.complex128)
        return h, xi, hmf

    def set_params(self, h, xi, hmf):
        p = self.pack(h, xi, hmf)
        check(lib().focss_ldbp_set_params(self.h, p.ctypes.data_as(P), p.size), self.ctx.h)

    def get_params(self):
        p = np.zeros(self.n_params, np.float32)
        g = np.zeros(self.n_params, np.float32)
        check(lib().focss_ldbp_get_params(self.h, p.ctypes.data_as(P), g.ctypes.data_as(P), p.size), self.ctx.h)
        return self.unpack(p), self.unpack(g)

    def init_from_dbp(self, alpha, beta2, gamma, kappa, span_length, dt, mf_response):
        """Initialise as the reference's uniform split-step DBP
        (ssfm.cpp:62-72 run BACKWARD per span after drop_power): per span
        L(h/2) N(h) L(h) N(h) ... N(h) L(h/2), h = span/steps, Kerr phase
        -kappa gamma h (raw step, ssfm.cpp:160-164).  The trailing L(h/2) of a
        span and the leading L(h/2) of the next merge into one L(h) filter
        (drop_power is a scalar between them); the last span's trailing
        L(h/2) is folded into the matched filter, whose frequency response
        `mf_response` (e.g. rrc_response) is given at the field's length."""
        hstep = span_length / self.steps
        full = dispersion_taps(hstep, alpha, beta2, dt, self.samples, self.taps)
        half = dispersion_taps(0.5 * hstep, alpha, beta2, dt, self.samples, self.taps)
        h = np.tile(full, (self.layers, 1))
        h[0] = half
        xi = np.full(self.layers, -kappa * gamma * hstep)
        self.gain_scale = abs(kappa * gamma * hstep)
        mf = taps_from_response(np.asarray(mf_response) *
                                dispersion_response(0.5 * hstep, alpha, beta2, dt, self.samples), self.mf_taps)
        self.set_params(h, xi, mf)

    def forward(self, field: Field) -> Field:
        from .api import Domain
        out = Field(Domain(1, self.samples // 2, field.domain.time_step * 2, field.domain.center_frequency),
                    batch=self.batch, ctx=self.ctx)
        check(lib().focss_ldbp_forward(self.h, field.h, out.h), self.ctx.h)
        return out

    def loss_grad(self, field: Field, tx: Field) -> float:
        loss = C.c_double()
        check(lib().focss_ldbp_loss_grad(self.h, field.h, tx.h, C.byref(loss)), self.ctx.h)
        return loss.value

    def adam_step(self, lr=1e-3, lr_gain=None, beta1=0.9, beta2=0.999, eps=1e-8):
        """Adam; the nonlinear gains move with lr_gain (default: lr times the
        magnitude of the initial gains, so both parameter groups move by the
        same relative amount per step)."""
        if lr_gain is None:
            lr_gain = lr * getattr(self, "gain_scale", 1.0)
        check(lib().focss_ldbp_adam_step(self.h, lr, lr_gain, beta1, beta2, eps), self.ctx.h)

    def rotate_output(self, angle):
        """Multiply the matched filter by exp(i angle) (absorbs a constant
        phase, e.g. the phase-shift equalizer angle of the training data)."""
        (h, xi, hmf), _ = self.get_params()
        self.set_params(h, xi, hmf * np.exp(1j * angle))

    def fit(self, field: Field, tx: Field, iters=100, lr=1e-3, log=None):
        hist = []
        for i in range(iters):
            loss = self.loss_grad(field, tx)
            self.adam_step(lr)
            hist.append(loss)
            if log and (i % log == 0):
                print("ldbp iter %d loss %.6e" % (i, loss))
        return hist

    def close(self):
        from ._lib import alive
        if getattr(self, "h", None) and alive():
            lib().focss_ldbp_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

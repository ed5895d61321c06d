"""Transmitter / receiver DSP mirrors of src/focss/processing/modulation.h and
src/focss/equalizer/linear.h over the C ABI.  Every function returns new
device fields (or host numbers per realization) like the reference returns new
Field objects; the compute runs in libfocss_gpu.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import replace

import numpy as np

from ._lib import check, lib
from .api import Domain, Field

P = C.c_void_p


def _vp(a):
    return a.ctypes.data_as(P)


def _like(f: Field, samples=None, dt=None, batch=None):
    d = f.domain
    dom = Domain(d.modes, samples if samples is not None else d.samples,
                 dt if dt is not None else d.time_step, d.center_frequency)
    return Field(dom, batch=f.batch if batch is None else batch, ctx=f.ctx)


def qam16_map(codes, domain: Domain, batch: int = 1, ctx=None) -> Field:
    """Gray 16QAM symbols (modulation.cpp:9-17) for integer codes shaped (batch, modes, samples)."""
    out = Field(domain, batch=batch, ctx=ctx)
    c = np.ascontiguousarray(np.asarray(codes, dtype=np.int32).reshape(out.shape))
    check(lib().focss_qam16_map(out.ctx.h, _vp(c), c.size, out.h), out.ctx.h)
    return out


def upsample(f: Field, factor: int) -> Field:
    out = _like(f, f.domain.samples * factor, f.domain.time_step / factor)
    check(lib().focss_upsample(f.ctx.h, f.h, factor, out.h), f.ctx.h)
    return out


def downsample(f: Field, factor: int) -> Field:
    out = _like(f, f.domain.samples // factor, f.domain.time_step * factor)
    check(lib().focss_downsample(f.ctx.h, f.h, factor, out.h), f.ctx.h)
    return out


def decimate(f: Field, factor: int) -> Field:
    out = _like(f, f.domain.samples // factor, f.domain.time_step * factor)
    check(lib().focss_decimate(f.ctx.h, f.h, factor, out.h), f.ctx.h)
    return out


def rrc_pulse(n_symbols: int, osf: int, roll_off: float, ctx=None):
    """pulse::rrc (modulation.cpp:47-74), computed on the device; returns complex128 taps."""
    from .api import Context
    ctx = ctx or Context.default()
    out = np.zeros(n_symbols * osf, np.complex128)
    check(lib().focss_rrc_pulse(ctx.h, n_symbols, osf, roll_off, _vp(out)), ctx.h)
    return out


def filter_inplace(f: Field, impulse_response) -> Field:
    """Field::filter_inplace (field.cpp:358-372)."""
    h = np.ascontiguousarray(impulse_response, dtype=np.complex128)
    check(lib().focss_filter(f.ctx.h, f.h, _vp(h), h.size), f.ctx.h)
    return f


def rrc_shaping(symbols: Field, osf: int, roll_off: float = 0.01, gain: float = 1.0) -> Field:
    """rrc_shaping (modulation.cpp:85-90); the reference's roll-off is 0.01."""
    out = _like(symbols, symbols.domain.samples * osf, symbols.domain.time_step / osf)
    check(lib().focss_rrc_shaping(symbols.ctx.h, symbols.h, osf, roll_off, gain, out.h), symbols.ctx.h)
    return out


def rrc_sampling(signal: Field, osf: int, roll_off: float = 0.01, gain: float = 1.0) -> Field:
    """rrc_sampling (modulation.cpp:92-96)."""
    out = _like(signal, signal.domain.samples // osf, signal.domain.time_step * osf)
    check(lib().focss_rrc_sampling(signal.ctx.h, signal.h, osf, roll_off, gain, out.h), signal.ctx.h)
    return out


def frequency_shift(f: Field, frequency: float) -> Field:
    out = f.copy()
    check(lib().focss_frequency_shift(f.ctx.h, out.h, frequency), f.ctx.h)
    return out


def bandpass_filter(f: Field, frequency: float) -> Field:
    out = f.copy()
    check(lib().focss_bandpass(f.ctx.h, out.h, frequency), f.ctx.h)
    return out


def wdm_select(f: Field, channel_index: int, channel_bandwidth: float) -> Field:
    out = _like(f)
    check(lib().focss_wdm_select(f.ctx.h, f.h, channel_index, channel_bandwidth, out.h), f.ctx.h)
    return out


def wdm_mux(channels: Field, channel_bandwidth: float) -> Field:
    """channels: one realization per channel (batch = number of channels)."""
    out = _like(channels, batch=1)
    check(lib().focss_wdm_mux(channels.ctx.h, channels.h, channel_bandwidth, out.h), channels.ctx.h)
    return out


def hard_decision_16qam(f: Field) -> Field:
    out = _like(f)
    check(lib().focss_hard_decision(f.ctx.h, f.h, out.h), f.ctx.h)
    return out


def soft_decision_16qam(f: Field, uncertainty: float) -> Field:
    """soft_decision_16qam (src/focss/processing/modulation.cpp:122-146)."""
    out = _like(f)
    check(lib().focss_soft_decision(f.ctx.h, f.h, float(uncertainty), out.h), f.ctx.h)
    return out


def find_certainty(tx: Field, rx: Field):
    """find_certainty (src/tasks/wdm_scoring.cpp:105-126), one value per
    realization (each realization is one matrix: rows = modes)."""
    out = np.zeros(tx.batch)
    check(lib().focss_find_certainty(tx.ctx.h, tx.h, rx.h, _vp(out)), tx.ctx.h)
    return out


def certainty_decision(f: Field, certainty: float) -> Field:
    """sd (src/tasks/wdm_scoring.cpp:128-144): snap to the decided point when
    closer than certainty / sqrt(5) at the RMS amplitude, else keep."""
    out = _like(f)
    check(lib().focss_certainty_decision(f.ctx.h, f.h, float(certainty), out.h), f.ctx.h)
    return out


sd = certainty_decision


def hd(f: Field) -> Field:
    """hd (src/tasks/wdm_scoring.cpp:146-156): the hard decision at the RMS
    amplitude, which is hard_decision_16qam's sqrt(average power / modes)."""
    return hard_decision_16qam(f)


def hd_sequence_16qam(f: Field):
    codes = np.zeros(f.shape, np.int32)
    check(lib().focss_hd_codes(f.ctx.h, f.h, _vp(codes)), f.ctx.h)
    return codes


def error_counts(tx: Field, rx: Field, cut: int = 0):
    be = np.zeros(tx.batch, np.uint64)
    se = np.zeros(tx.batch, np.uint64)
    check(lib().focss_error_counts(tx.ctx.h, tx.h, rx.h, cut, _vp(be), _vp(se)), tx.ctx.h)
    return be, se


def bit_error_rate_16qam(tx: Field, rx: Field, cut: int = -1):
    out = np.zeros(tx.batch)
    check(lib().focss_bit_error_rate(tx.ctx.h, tx.h, rx.h, cut, _vp(out)), tx.ctx.h)
    return out


def symbol_error_rate_16qam(tx: Field, rx: Field, cut: int = 0):
    out = np.zeros(tx.batch)
    check(lib().focss_symbol_error_rate(tx.ctx.h, tx.h, rx.h, cut, _vp(out)), tx.ctx.h)
    return out


def q2_factor(tx: Field, rx: Field, cut: int = -1):
    out = np.zeros(tx.batch)
    check(lib().focss_q2_factor(tx.ctx.h, tx.h, rx.h, cut, _vp(out)), tx.ctx.h)
    return out


def rotate(f: Field, angles) -> Field:
    a = np.ascontiguousarray(np.broadcast_to(np.asarray(angles, dtype=np.float64), (f.batch,)))
    check(lib().focss_field_rotate(f.ctx.h, f.h, _vp(a)), f.ctx.h)
    return f


def scale_each(f: Field, scalars) -> Field:
    s = np.broadcast_to(np.asarray(scalars, dtype=np.complex128), (f.batch,))
    s = np.ascontiguousarray(s)
    check(lib().focss_field_scale_each(f.ctx.h, f.h, _vp(s)), f.ctx.h)
    return f


class PhaseShiftEqualizer:
    """src/focss/equalizer/linear.h:18-38, phase_shift_equalizer.cpp"""

    def __init__(self, angle_steps: int = 3600):
        self.angle_steps = angle_steps
        self.estimated_angle = None

    def estimate(self, desired: Field, actual: Field):
        out = np.zeros(desired.batch)
        check(lib().focss_pse_estimate(desired.ctx.h, desired.h, actual.h, self.angle_steps, _vp(out)),
              desired.ctx.h)
        return out

    def train(self, desired, actual):
        self.estimated_angle = self.estimate(desired, actual)

    def get_angle(self):
        return self.estimated_angle

    def equalize(self, original: Field) -> Field:
        return rotate(original.copy(), self.estimated_angle)

    def train_equalize(self, desired: Field, actual: Field) -> Field:
        return rotate(actual.copy(), self.estimate(desired, actual))


class ScalarEqualizer:
    """src/focss/equalizer/linear.h:53-66, scalar_equalizer.cpp"""

    def __init__(self):
        self.scalar = None

    def estimate(self, desired: Field, actual: Field):
        out = np.zeros(2 * desired.batch)
        check(lib().focss_scalar_estimate(desired.ctx.h, desired.h, actual.h, _vp(out)), desired.ctx.h)
        return out[0::2] + 1j * out[1::2]

    def train(self, desired, actual):
        self.scalar = self.estimate(desired, actual)

    def get_scalar(self):
        return self.scalar

    def equalize(self, original: Field) -> Field:
        return scale_each(original.copy(), self.scalar)

    def train_equalize(self, desired: Field, actual: Field) -> Field:
        return scale_each(actual.copy(), self.estimate(desired, actual))

"""numpy front end of the FP64 oracle (``libfocss_oracle.so``).

Test infrastructure only.  Arrays are complex128 numpy arrays of shape
(modes, samples) or (samples,) for single-mode fields; they are passed to the C
library as interleaved doubles in the reference's mode-major order.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

D = C.c_double
I = C.c_int
P = C.c_void_p


class Fiber(C.Structure):
    """src/focss/module/fiber.h:5-12"""

    _fields_ = [("alpha", D), ("beta2", D), ("gamma", D), ("length", D),
                ("wavelength", D), ("kappa", D)]

    def astuple(self):
        return (self.alpha, self.beta2, self.gamma, self.length, self.wavelength, self.kappa)


def lib():
    global _lib
    if _lib is None:
        path = _build.ORACLE_SO
        if not os.path.exists(path):
            path = _build.build_oracle()
        L = C.CDLL(path)
        sig = {
            "ofc_dft": (None, [I, P, I]),
            "ofc_field_fft": (None, [I, I, P]),
            "ofc_field_ifft": (None, [I, I, P]),
            "ofc_ssfm_run": (I, [I, I, D, P, C.POINTER(Fiber), I, I, D, D, D]),
            "ofc_ssfm_run_rec": (I, [I, I, D, P, C.POINTER(Fiber), I, I, D, D, D, P, I]),
            "ofc_ssfm_run_steps": (I, [I, I, D, P, C.POINTER(Fiber), P, I, D]),
            "ofc_cd_compensation": (None, [I, I, D, P, C.POINTER(Fiber), I]),
            "ofc_amplify": (None, [I, I, D, D, P, D, D, C.c_uint64, C.c_uint64, I]),
            "ofc_add_noise": (None, [I, I, D, D, P, D, D, C.c_uint64, C.c_uint64, I]),
            "ofc_drop_power": (None, [I, I, P, D]),
            "ofc_give_power": (None, [I, I, P, D]),
            "ofc_philox4x32_10": (None, [P, P, P]),
            "ofc_gray16": (None, [P]),
            "ofc_qam16_map": (None, [I, P, P]),
            "ofc_rrc_pulse": (None, [I, I, D, P]),
            "ofc_filter_inplace": (None, [I, I, P, I, P]),
            "ofc_upsample": (None, [I, I, P, I, P]),
            "ofc_downsample": (None, [I, I, P, I, P]),
            "ofc_decimate": (None, [I, I, P, I, P]),
            "ofc_rrc_shaping": (None, [I, I, P, I, D, D, P]),
            "ofc_rrc_sampling": (None, [I, I, P, I, D, D, P]),
            "ofc_demodulate16": (C.c_uint32, [D, D]),
            "ofc_hd_sequence": (None, [I, I, P, P]),
            "ofc_hard_decision": (None, [I, I, P, P]),
            "ofc_soft_decision": (None, [I, I, P, D, P]),
            "ofc_find_certainty": (D, [I, I, P, P]),
            "ofc_certainty_decision": (None, [I, I, P, D, P]),
            "ofc_hd_rms": (None, [I, I, P, P]),
            "ofc_error_counts": (None, [I, I, P, P, I, P, P]),
            "ofc_bit_error_rate": (D, [I, I, P, P, I]),
            "ofc_symbol_error_rate": (D, [I, I, P, P, I]),
            "ofc_evm2": (D, [I, I, P, P, I]),
            "ofc_q2": (D, [I, I, P, P, I]),
            "ofc_average_power": (D, [I, I, P]),
            "ofc_peak_power": (D, [I, I, P]),
            "ofc_frequency_shift": (None, [I, I, D, P, D]),
            "ofc_bandpass": (None, [I, I, D, P, D]),
            "ofc_wdm_select": (None, [I, I, D, P, I, D]),
            "ofc_wdm_mux": (None, [I, I, I, D, P, D, P]),
            "ofc_pse_estimate": (D, [I, I, P, P, I]),
            "ofc_rotate": (None, [I, I, P, D]),
            "ofc_scalar_estimate": (None, [I, I, P, P, P]),
            "ofc_sino_cubic": (None, [I, I, P, I, P, P]),
            "ofc_triplet_sparse": (None, [I, I, P, I, I, P, P, P, P]),
            "ofc_num_threads": (I, []),
            "ofc_ssfm_batch": (None, [I, I, I, D, P, C.POINTER(Fiber), I, I, D, D, D, I, P]),
            "ofc_uniform_steps_batch": (None, [I, I, I, D, P, C.POINTER(Fiber), D, I, I]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _c128(a):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    return a


def _shape(a):
    a = np.asarray(a)
    if a.ndim == 1:
        return 1, a.shape[0]
    return a.shape[-2], a.shape[-1]


def _ptr(a):
    return a.ctypes.data_as(P)


# ---- FFT -------------------------------------------------------------------
def dft(x, sign=-1):
    x = _c128(x).copy()
    lib().ofc_dft(x.size, _ptr(x), sign)
    return x


def field_fft(a):
    a = _c128(a).copy()
    m, n = _shape(a)
    lib().ofc_field_fft(m, n, _ptr(a))
    return a


def field_ifft(a):
    a = _c128(a).copy()
    m, n = _shape(a)
    lib().ofc_field_ifft(m, n, _ptr(a))
    return a


# ---- SSFM -------------------------------------------------------------------
UNIFORM, LOGARITHMIC, ADAPTIVE = 0, 1, 2
FORWARD, BACKWARD = 1.0, -1.0


def ssfm_run(a, dt, fiber, grid=UNIFORM, total_steps=1, max_phase_shift=0.0,
             max_step_size=0.0, direction=FORWARD):
    """src/focss/solver/ssfm.cpp:39-60; returns (field, steps)."""
    a = _c128(a).copy()
    m, n = _shape(a)
    steps = lib().ofc_ssfm_run(m, n, dt, _ptr(a), C.byref(fiber), grid, total_steps,
                               max_phase_shift, max_step_size, direction)
    return a, steps


def ssfm_run_recorded(a, dt, fiber, grid=UNIFORM, total_steps=1, max_phase_shift=0.0,
                      max_step_size=0.0, direction=FORWARD, capacity=1 << 16):
    """ssfm_run that also returns the step sizes |h_i| taken: (field, steps, h)."""
    a = _c128(a).copy()
    m, n = _shape(a)
    h = np.zeros(capacity)
    steps = lib().ofc_ssfm_run_rec(m, n, dt, _ptr(a), C.byref(fiber), grid, total_steps,
                                   max_phase_shift, max_step_size, direction, _ptr(h), capacity)
    if steps > capacity:
        raise ValueError("ssfm_run_recorded: %d steps exceed the capacity %d" % (steps, capacity))
    return a, steps, h[:steps].copy()


def ssfm_run_steps(a, dt, fiber, h, direction=FORWARD):
    """The ADAPTIVE loop (ssfm.cpp:92-118) on the given step sizes h."""
    a = _c128(a).copy()
    m, n = _shape(a)
    h = np.ascontiguousarray(h, dtype=np.float64)
    if h.size < 1:
        raise ValueError("ssfm_run_steps: at least one step")
    lib().ofc_ssfm_run_steps(m, n, dt, _ptr(a), C.byref(fiber), _ptr(h), h.size, direction)
    return a


def cd_compensation(a, dt, fiber, spans):
    a = _c128(a).copy()
    m, n = _shape(a)
    lib().ofc_cd_compensation(m, n, dt, _ptr(a), C.byref(fiber), spans)
    return a


def amplify(a, dt, f0, gain, noise_factor=0.0, seed=0, counter=0, realization=0):
    a = _c128(a).copy()
    m, n = _shape(a)
    lib().ofc_amplify(m, n, dt, f0, _ptr(a), gain, noise_factor, seed, counter, realization)
    return a


def add_noise(a, dt, f0, gain, noise_factor, seed=0, counter=0, realization=0):
    a = _c128(a).copy()
    m, n = _shape(a)
    lib().ofc_add_noise(m, n, dt, f0, _ptr(a), gain, noise_factor, seed, counter, realization)
    return a


def drop_power(a, gain):
    a = _c128(a).copy()
    m, n = _shape(a)
    lib().ofc_drop_power(m, n, _ptr(a), gain)
    return a


def give_power(a, gain):
    a = _c128(a).copy()
    m, n = _shape(a)
    lib().ofc_give_power(m, n, _ptr(a), gain)
    return a


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    o = np.zeros(4, np.uint32)
    lib().ofc_philox4x32_10(_ptr(c), _ptr(k), _ptr(o))
    return o


# ---- DSP --------------------------------------------------------------------
def gray16():
    t = np.zeros(16, np.complex128)
    lib().ofc_gray16(_ptr(t))
    return t


def qam16_map(codes):
    c = np.ascontiguousarray(codes, dtype=np.int32)
    out = np.zeros(c.shape, np.complex128)
    lib().ofc_qam16_map(c.size, _ptr(c), _ptr(out))
    return out


def rrc_pulse(n_symbols, osf, roll_off):
    out = np.zeros(n_symbols * osf, np.complex128)
    lib().ofc_rrc_pulse(n_symbols, osf, roll_off, _ptr(out))
    return out


def filter(a, h):
    a = _c128(a).copy()
    h = _c128(h)
    m, n = _shape(a)
    lib().ofc_filter_inplace(m, n, _ptr(a), h.size, _ptr(h))
    return a


def upsample(a, factor):
    a = _c128(a)
    m, n = _shape(a)
    out = np.zeros(a.shape[:-1] + (n * factor,), np.complex128)
    lib().ofc_upsample(m, n, _ptr(a), factor, _ptr(out))
    return out


def downsample(a, factor):
    a = _c128(a)
    m, n = _shape(a)
    out = np.zeros(a.shape[:-1] + (n // factor,), np.complex128)
    lib().ofc_downsample(m, n, _ptr(a), factor, _ptr(out))
    return out


def decimate(a, factor):
    a = _c128(a)
    m, n = _shape(a)
    out = np.zeros(a.shape[:-1] + (n // factor,), np.complex128)
    lib().ofc_decimate(m, n, _ptr(a), factor, _ptr(out))
    return out


def rrc_shaping(symbols, osf, roll_off, gain=1.0):
    s = _c128(symbols)
    m, n = _shape(s)
    out = np.zeros(s.shape[:-1] + (n * osf,), np.complex128)
    lib().ofc_rrc_shaping(m, n, _ptr(s), osf, roll_off, gain, _ptr(out))
    return out


def rrc_sampling(signal, osf, roll_off, gain=1.0):
    s = _c128(signal)
    m, n = _shape(s)
    out = np.zeros(s.shape[:-1] + (n // osf,), np.complex128)
    lib().ofc_rrc_sampling(m, n, _ptr(s), osf, roll_off, gain, _ptr(out))
    return out


def demodulate16(z):
    return int(lib().ofc_demodulate16(float(np.real(z)), float(np.imag(z))))


def hd_sequence(a):
    a = _c128(a)
    m, n = _shape(a)
    out = np.zeros(a.shape, np.int32)
    lib().ofc_hd_sequence(m, n, _ptr(a), _ptr(out))
    return out


def hard_decision(a):
    a = _c128(a)
    m, n = _shape(a)
    out = np.zeros(a.shape, np.complex128)
    lib().ofc_hard_decision(m, n, _ptr(a), _ptr(out))
    return out

def soft_decision(a, uncertainty):
    a = _c128(a)
    m, n = _shape(a)
    out = np.zeros_like(a)
    lib().ofc_soft_decision(m, n, _ptr(a), uncertainty, _ptr(out))
    return out


def find_certainty(tx, rx):
    """find_certainty (src/tasks/wdm_scoring.cpp:105-126); rows x cols arrays."""
    tx, rx = _c128(tx), _c128(rx)
    m, n = _shape(tx)
    return float(lib().ofc_find_certainty(m, n, _ptr(tx), _ptr(rx)))


def certainty_decision(a, certainty):
    """sd (src/tasks/wdm_scoring.cpp:128-144)."""
    a = _c128(a)
    m, n = _shape(a)
    out = np.zeros_like(a)
    lib().ofc_certainty_decision(m, n, _ptr(a), certainty, _ptr(out))
    return out


def hd_rms(a):
    """hd (src/tasks/wdm_scoring.cpp:146-156)."""
    a = _c128(a)
    m, n = _shape(a)
    out = np.zeros_like(a)
    lib().ofc_hd_rms(m, n, _ptr(a), _ptr(out))
    return out


def error_counts(tx, rx, cut=0):
    tx, rx = _c128(tx), _c128(rx)
    m, n = _shape(tx)
    be = np.zeros(1, np.uint64)
    se = np.zeros(1, np.uint64)
    lib().ofc_error_counts(m, n, _ptr(tx), _ptr(rx), cut, _ptr(be), _ptr(se))
    return int(be[0]), int(se[0])


def bit_error_rate(tx, rx, cut=0):
    tx, rx = _c128(tx), _c128(rx)
    m, n = _shape(tx)
    return lib().ofc_bit_error_rate(m, n, _ptr(tx), _ptr(rx), cut)


def symbol_error_rate(tx, rx, cut=0):
    tx, rx = _c128(tx), _c128(rx)
    m, n = _shape(tx)
    return lib().ofc_symbol_error_rate(m, n, _ptr(tx), _ptr(rx), cut)


def evm2(tx, rx, cut=0):
    tx, rx = _c128(tx), _c128(rx)
    m, n = _shape(tx)
    return lib().ofc_evm2(m, n, _ptr(tx), _ptr(rx), cut)


def q2(tx, rx, cut=0):
    tx, rx = _c128(tx), _c128(rx)
    m, n = _shape(tx)
    return lib().ofc_q2(m, n, _ptr(tx), _ptr(rx), cut)


def average_power(a):
    a = _c128(a)
    m, n = _shape(a)
    return lib().ofc_average_power(m, n, _ptr(a))


def peak_power(a):
    a = _c128(a)
    m, n = _shape(a)
    return lib().ofc_peak_power(m, n, _ptr(a))


def frequency_shift(a, dt, frequency):
    a = _c128(a).copy()
    m, n = _shape(a)
    lib().ofc_frequency_shift(m, n, dt, _ptr(a), frequency)
    return a


def bandpass(a, dt, frequency):
    a = _c128(a).copy()
    m, n = _shape(a)
    lib().ofc_bandpass(m, n, dt, _ptr(a), frequency)
    return a


def wdm_select(a, dt, channel_index, channel_bandwidth):
    a = _c128(a).copy()
    m, n = _shape(a)
    lib().ofc_wdm_select(m, n, dt, _ptr(a), channel_index, channel_bandwidth)
    return a


def wdm_mux(channels, dt, channel_bandwidth):
    ch = _c128(channels)
    nch = ch.shape[0]
    m, n = _shape(ch[0])
    out = np.zeros(ch.shape[1:], np.complex128)
    lib().ofc_wdm_mux(nch, m, n, dt, _ptr(ch), channel_bandwidth, _ptr(out))
    return out


def pse_estimate(desired, actual, angle_steps=3600):
    d, a = _c128(desired), _c128(actual)
    m, n = _shape(d)
    return lib().ofc_pse_estimate(m, n, _ptr(d), _ptr(a), angle_steps)


def rotate(a, angle):
    a = _c128(a).copy()
    m, n = _shape(a)
    lib().ofc_rotate(m, n, _ptr(a), angle)
    return a


def scalar_estimate(desired, actual):
    d, a = _c128(desired), _c128(actual)
    m, n = _shape(d)
    out = np.zeros(2)
    lib().ofc_scalar_estimate(m, n, _ptr(d), _ptr(a), _ptr(out))
    return complex(out[0], out[1])


def sino_cubic(a, radius, weights):
    a = _c128(a)
    w = _c128(weights)
    m, n = _shape(a)
    out = np.zeros(a.shape, np.complex128)
    lib().ofc_sino_cubic(m, n, _ptr(a), radius, _ptr(w), _ptr(out))
    return out


def triplet_sparse(a, radius, mm, nn, c):
    a = _c128(a)
    mm = np.ascontiguousarray(mm, dtype=np.int32)
    nn = np.ascontiguousarray(nn, dtype=np.int32)
    c = _c128(c)
    m, n = _shape(a)
    out = np.zeros(a.shape, np.complex128)
    lib().ofc_triplet_sparse(m, n, _ptr(a), radius, mm.size, _ptr(mm), _ptr(nn), _ptr(c), _ptr(out))
    return out


def num_threads():
    return lib().ofc_num_threads()


def ssfm_batch(a, dt, fiber, grid=UNIFORM, total_steps=1, max_phase_shift=0.0,
               max_step_size=0.0, direction=FORWARD, threads=1):
    """a: (batch, modes, samples) complex128, propagated in place (copy returned)."""
    a = _c128(a).copy()
    b, m, n = a.shape
    steps = np.zeros(b, np.int32)
    lib().ofc_ssfm_batch(b, m, n, dt, _ptr(a), C.byref(fiber), grid, total_steps,
                         max_phase_shift, max_step_size, direction, threads, _ptr(steps))
    return a, steps


def uniform_steps_batch(a, dt, fiber, step, n_steps, threads=1):
    """Timing kernel of the CPU baseline: n_steps x [N(h), L(h)] per realization, in place."""
    assert a.dtype == np.complex128 and a.flags.c_contiguous
    b, m, n = a.shape
    lib().ofc_uniform_steps_batch(b, m, n, dt, _ptr(a), C.byref(fiber), step, n_steps, threads)
    return a

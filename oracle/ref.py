"""numpy front end of the reference's own sources (``oracle/_ref/libfocss_ref.so``).

Test infrastructure only, available only where the reference tree was present
when ``oracle/build.py`` ran.  Used to pin the oracle restatement and to
generate the committed golden vectors (tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

D, I, P, U = C.c_double, C.c_int, C.c_void_p, C.c_uint
_lib = None


def available() -> bool:
    if os.path.exists(_build.REF_SO):
        return True
    try:
        return _build.build_ref() is not None
    except Exception:
        return False


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("reference build unavailable (no reference source tree)")
        L = C.CDLL(_build.REF_SO)
        sig = {
            "ref_field_fft": (None, [I, I, D, P]),
            "ref_field_ifft": (None, [I, I, D, P]),
            "ref_ssfm_run": (None, [I, I, D, P, P, I, I, D, D, D]),
            "ref_fiber_scale": (None, [P, D, P]),
            "ref_fiber_dispersive": (None, [P, P]),
            "ref_amplify": (None, [I, I, D, D, P, D, D, U]),
            "ref_drop_power": (None, [I, I, P, D]),
            "ref_give_power": (None, [I, I, P, D]),
            "ref_db_to_linear": (D, [D]),
            "ref_dbm_to_watts": (D, [D]),
            "ref_db_to_natural": (D, [D]),
            "ref_disp_to_beta2": (D, [D, D]),
            "ref_rrc_pulse": (None, [I, I, D, P]),
            "ref_filter": (None, [I, I, D, P, I, P]),
            "ref_upsample": (None, [I, I, D, P, I, P]),
            "ref_downsample": (None, [I, I, D, P, I, P]),
            "ref_decimate": (None, [I, I, D, P, I, P]),
            "ref_rrc_shaping": (None, [I, I, D, P, I, D, P]),
            "ref_rrc_sampling": (None, [I, I, D, P, I, D, P]),
            "ref_rrc_shaping_rolloff": (None, [I, I, D, P, I, D, D, P]),
            "ref_rrc_sampling_rolloff": (None, [I, I, D, P, I, D, D, P]),
            "ref_demodulate16": (U, [D, D]),
            "ref_hard_decision": (None, [I, I, P, P]),
            "ref_soft_decision": (None, [I, I, P, D, P]),
            "ref_save_transmission": (None, [I, I, P, P, C.c_char_p]),
            "ref_load_transmission": (None, [I, I, C.c_char_p, P, P]),
            "ref_ber": (D, [I, I, P, P, I]),
            "ref_ser": (D, [I, I, P, P, I]),
            "ref_q2": (D, [I, I, P, P, I]),
            "ref_pse_angle": (D, [I, I, P, P, I]),
            "ref_scalar_estimate": (None, [I, I, P, P, P]),
            "ref_frequency_shift": (None, [I, I, D, P, D]),
            "ref_bandpass": (None, [I, I, D, P, D]),
            "ref_wdm_select": (None, [I, I, D, P, I, D]),
            "ref_wdm_mux": (None, [I, I, I, D, P, D, P]),
            "ref_soliton": (None, [I, I, D, P]),
            "ref_sino_train": (None, [I, I, P, P, I, I, D, D, P, P, P]),
            "ref_sino_cubic": (None, [I, I, P, I, P, P]),
            "ref_sino_equalize": (None, [I, I, P, P, I, P, D, D, P]),
            "ref_wdm_ppe_train": (None, [I, P, P, I, I, P, P, P, P]),
            "ref_wdm_ppe_apply": (None, [I, P, P, P, I, P, I, P, D, D, I, P]),
            "ref_find_certainty": (D, [I, I, P, P]),
            "ref_certainty_sd": (None, [I, I, P, D, P]),
            "ref_hd_rms": (None, [I, I, P, P]),
            "ref_field_power": (None, [I, I, P, P, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _c(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def _shape(a):
    return (1, a.shape[0]) if a.ndim == 1 else (a.shape[-2], a.shape[-1])


def _p(a):
    return a.ctypes.data_as(P)


def field_fft(a, dt=1.0):
    a = _c(a).copy(); m, n = _shape(a); lib().ref_field_fft(m, n, dt, _p(a)); return a


def field_ifft(a, dt=1.0):
    a = _c(a).copy(); m, n = _shape(a); lib().ref_field_ifft(m, n, dt, _p(a)); return a


def ssfm_run(a, dt, fiber6, grid=0, total_steps=1, max_phase_shift=0.0, max_step_size=0.0,
             direction=1.0):
    a = _c(a).copy(); m, n = _shape(a)
    f = np.ascontiguousarray(fiber6, dtype=np.float64)
    lib().ref_ssfm_run(m, n, dt, _p(a), _p(f), grid, total_steps, max_phase_shift,
                       max_step_size, direction)
    return a


def fiber_scale(fiber6, factor):
    f = np.ascontiguousarray(fiber6, dtype=np.float64); o = np.zeros(6)
    lib().ref_fiber_scale(_p(f), factor, _p(o)); return o


def fiber_dispersive(fiber6):
    f = np.ascontiguousarray(fiber6, dtype=np.float64); o = np.zeros(6)
    lib().ref_fiber_dispersive(_p(f), _p(o)); return o


def amplify(a, dt, f0, gain, noise_factor=0.0, seed=1):
    a = _c(a).copy(); m, n = _shape(a)
    lib().ref_amplify(m, n, dt, f0, _p(a), gain, noise_factor, seed); return a


def drop_power(a, gain):
    a = _c(a).copy(); m, n = _shape(a); lib().ref_drop_power(m, n, _p(a), gain); return a


def give_power(a, gain):
    a = _c(a).copy(); m, n = _shape(a); lib().ref_give_power(m, n, _p(a), gain); return a


def db_to_linear(x): return lib().ref_db_to_linear(x)
def dbm_to_watts(x): return lib().ref_dbm_to_watts(x)
def db_to_natural(x): return lib().ref_db_to_natural(x)
def disp_to_beta2(d, wl): return lib().ref_disp_to_beta2(d, wl)


def rrc_pulse(n_symbols, osf, roll_off):
    o = np.zeros(n_symbols * osf, np.complex128)
    lib().ref_rrc_pulse(n_symbols, osf, roll_off, _p(o)); return o


def filter(a, h, dt=1.0):
    a = _c(a).copy(); h = _c(h); m, n = _shape(a)
    lib().ref_filter(m, n, dt, _p(a), h.size, _p(h)); return a


def _resample(fn, a, factor, up, dt=1.0):
    a = _c(a); m, n = _shape(a)
    o = np.zeros(a.shape[:-1] + ((n * factor) if up else (n // factor),), np.complex128)
    fn(m, n, dt, _p(a), factor, _p(o)); return o


def upsample(a, factor): return _resample(lib().ref_upsample, a, factor, True)
def downsample(a, factor): return _resample(lib().ref_downsample, a, factor, False)
def decimate(a, factor): return _resample(lib().ref_decimate, a, factor, False)


def rrc_shaping(symbols, osf, roll_off=None, gain=1.0, dt=1.0):
    s = _c(symbols); m, n = _shape(s)
    o = np.zeros(s.shape[:-1] + (n * osf,), np.complex128)
    if roll_off is None:
        lib().ref_rrc_shaping(m, n, dt, _p(s), osf, gain, _p(o))
    else:
        lib().ref_rrc_shaping_rolloff(m, n, dt, _p(s), osf, roll_off, gain, _p(o))
    return o


def rrc_sampling(signal, osf, roll_off=None, gain=1.0, dt=1.0):
    s = _c(signal); m, n = _shape(s)
    o = np.zeros(s.shape[:-1] + (n // osf,), np.complex128)
    if roll_off is None:
        lib().ref_rrc_sampling(m, n, dt, _p(s), osf, gain, _p(o))
    else:
        lib().ref_rrc_sampling_rolloff(m, n, dt, _p(s), osf, roll_off, gain, _p(o))
    return o


def demodulate16(z): return int(lib().ref_demodulate16(float(np.real(z)), float(np.imag(z))))


def hard_decision(a):
    a = _c(a); m, n = _shape(a); o = np.zeros(a.shape, np.complex128)
    lib().ref_hard_decision(m, n, _p(a), _p(o)); return o


def soft_decision(a, uncertainty):
    a = _c(a); m, n = _shape(a); o = np.zeros(a.shape, np.complex128)
    lib().ref_soft_decision(m, n, _p(a), uncertainty, _p(o)); return o


def ber(tx, rx, cut=-1):
    tx, rx = _c(tx), _c(rx); m, n = _shape(tx); return lib().ref_ber(m, n, _p(tx), _p(rx), cut)


def ser(tx, rx, cut=0):
    tx, rx = _c(tx), _c(rx); m, n = _shape(tx); return lib().ref_ser(m, n, _p(tx), _p(rx), cut)


def q2(tx, rx, cut=-1):
    tx, rx = _c(tx), _c(rx); m, n = _shape(tx); return lib().ref_q2(m, n, _p(tx), _p(rx), cut)


def pse_angle(desired, actual, angle_steps=3600):
    d, a = _c(desired), _c(actual); m, n = _shape(d)
    return lib().ref_pse_angle(m, n, _p(d), _p(a), angle_steps)


def scalar_estimate(desired, actual):
    d, a = _c(desired), _c(actual); m, n = _shape(d); o = np.zeros(2)
    lib().ref_scalar_estimate(m, n, _p(d), _p(a), _p(o)); return complex(o[0], o[1])


def frequency_shift(a, dt, f):
    a = _c(a).copy(); m, n = _shape(a); lib().ref_frequency_shift(m, n, dt, _p(a), f); return a


def bandpass(a, dt, f):
    a = _c(a).copy(); m, n = _shape(a); lib().ref_bandpass(m, n, dt, _p(a), f); return a


def wdm_select(a, dt, idx, bw):
    a = _c(a).copy(); m, n = _shape(a); lib().ref_wdm_select(m, n, dt, _p(a), idx, bw); return a


def wdm_mux(channels, dt, bw):
    ch = _c(channels); nch = ch.shape[0]; m, n = _shape(ch[0])
    o = np.zeros(ch.shape[1:], np.complex128)
    lib().ref_wdm_mux(nch, m, n, dt, _p(ch), bw, _p(o)); return o


def soliton(dark, points, z):
    o = np.zeros(points, np.complex128); lib().ref_soliton(1 if dark else 0, points, z, _p(o)); return o


def save_transmission(path, tx, rx):
    """The reference's own save_transmission (functions.cpp:174-208) on (modes, samples) arrays."""
    tx, rx = _c(tx), _c(rx)
    m, n = _shape(tx)
    lib().ref_save_transmission(m, n, _p(tx), _p(rx), str(path).encode())


def load_transmission(path, modes, samples):
    tx = np.zeros((modes, samples), np.complex128)
    rx = np.zeros((modes, samples), np.complex128)
    lib().ref_load_transmission(modes, samples, str(path).encode(), _p(tx), _p(rx))
    return tx, rx


# ---- perturbation equalizers (sino.cpp, wdm_sino.cpp) and WDM scoring decisions
def sino_train(tx, rx, radius, type_=0, linear_weight=0j):
    """SINO::train (sino.cpp:42-159): returns (weights (2R+1)^2, intercept, linear weight)."""
    tx, rx = _c(np.atleast_2d(tx)), _c(np.atleast_2d(rx))
    m, n = _shape(tx)
    W = np.zeros((2 * radius + 1, 2 * radius + 1), np.complex128)
    ic = np.zeros(1, np.complex128)
    lw = np.zeros(1, np.complex128)
    lw0 = complex(linear_weight)
    lib().ref_sino_train(m, n, _p(tx), _p(rx), radius, type_, lw0.real, lw0.imag, _p(W), _p(ic), _p(lw))
    return W, ic[0], lw[0]


def sino_cubic(a, radius, weights):
    """SINO::cubic (sino.cpp:203-220) with the weight table W[R + m, R + n]."""
    a = _c(np.atleast_2d(a))
    m, n = _shape(a)
    W = _c(weights)
    o = np.zeros_like(a)
    lib().ref_sino_cubic(m, n, _p(a), radius, _p(W), _p(o))
    return o


def sino_equalize(rx, tx, radius, weights, linear_weight):
    rx, tx = _c(np.atleast_2d(rx)), _c(np.atleast_2d(tx))
    m, n = _shape(rx)
    W = _c(weights)
    o = np.zeros_like(rx)
    lw = complex(linear_weight)
    lib().ref_sino_equalize(m, n, _p(rx), _p(tx), radius, _p(W), lw.real, lw.imag, _p(o))
    return o


def wdm_ppe_train(tx, rx, c_radius, d_radius):
    """WdmPPE::train (wdm_sino.cpp:28-142) on 6 x N datasets: (C, D, intercept, linear weight)."""
    tx, rx = _c(tx), _c(rx)
    assert tx.shape[0] == 6 and rx.shape == tx.shape
    C_ = np.zeros((2 * c_radius + 1, 2 * c_radius + 1), np.complex128)
    D_ = np.zeros((2 * d_radius + 1, 2 * d_radius + 1), np.complex128)
    ic = np.zeros(1, np.complex128)
    lw = np.zeros(1, np.complex128)
    lib().ref_wdm_ppe_train(tx.shape[1], _p(tx), _p(rx), c_radius, d_radius, _p(C_), _p(D_), _p(ic), _p(lw))
    return C_, D_, ic[0], lw[0]


WDM_SPM, WDM_XPM, WDM_CUBIC, WDM_MODEL, WDM_EQUALIZE, WDM_EQUALIZE3 = range(6)


def wdm_ppe_apply(what, a, C_, D_, linear_weight, b=None, rx=None):
    """WdmPPE spm / xpm / cubic / model / equalize (wdm_sino.cpp:235-300) with given tables."""
    a = _c(a)
    n = a.shape[1]
    b = _c(b) if b is not None else a
    rx = _c(rx) if rx is not None else a
    C_, D_ = _c(C_), _c(D_)
    o = np.zeros((2, n), np.complex128)
    lw = complex(linear_weight)
    lib().ref_wdm_ppe_apply(n, _p(a), _p(b), _p(rx), (C_.shape[0] - 1) // 2, _p(C_), (D_.shape[0] - 1) // 2,
                            _p(D_), lw.real, lw.imag, what, _p(o))
    return o


def find_certainty(tx, rx):
    tx, rx = _c(np.atleast_2d(tx)), _c(np.atleast_2d(rx))
    return lib().ref_find_certainty(tx.shape[0], tx.shape[1], _p(tx), _p(rx))


def certainty_sd(field, certainty):
    f = _c(np.atleast_2d(field))
    o = np.zeros_like(f)
    lib().ref_certainty_sd(f.shape[0], f.shape[1], _p(f), certainty, _p(o))
    return o


def hd_rms(field):
    f = _c(np.atleast_2d(field))
    o = np.zeros_like(f)
    lib().ref_hd_rms(f.shape[0], f.shape[1], _p(f), _p(o))
    return o


def field_power(a):
    """Field::average_power / peak_power (field.cpp:164-187): (average, peak)."""
    a = _c(np.atleast_2d(a))
    m, n = _shape(a)
    avg, pk = np.zeros(1), np.zeros(1)
    lib().ref_field_power(m, n, _p(a), _p(avg), _p(pk))
    return float(avg[0]), float(pk[0])

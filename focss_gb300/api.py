"""Python mirror of the focss C++ API over the GB300 C ABI.

Class and method names follow the reference (src/focss/field.h,
src/focss/module/fiber.h, src/focss/module/amplifier.h,
src/focss/solver/ssfm.h, src/tasks/systems.h) so that tests read like the
reference's usage.  Fields live on the GPU (complex64); ``numpy()`` copies
them back as complex128.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, replace

import numpy as np

from ._lib import CAmp, CDomain, CFiber, CSsfmOpts, FocssError, alive, check, lib

# src/focss/definitions.h:13-15
MATH_PI = 3.14159265358979323846264338
PLANCK = 6.62607004081818181818181e-34
LIGHT_SPEED = 299792458.0


def launch_count() -> int:
    """Kernel launches issued by libfocss_gpu in this process."""
    return int(lib().focss_launch_count())


# ---- unit conversions (src/focss/functions.cpp:82-96): plain host arithmetic
def db_to_linear(db):
    return 10.0 ** (db / 10.0)


def dbm_to_watts(dbm):
    return 1e-3 * 10.0 ** (dbm / 10.0)


def db_to_natural(db):
    return db * math.log(10) / 10.0


def disp_to_beta2(dispersion, wavelength):
    return -wavelength * wavelength * dispersion / (2 * MATH_PI * LIGHT_SPEED)


class Context:
    """One CUDA stream + plans + scratch (one per host thread)."""

    _default = None

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().focss_ctx_create(device, C.byref(h)))
        self.h = h
        self.device = device

    @classmethod
    def default(cls):
        if cls._default is None:
            cls._default = Context(0)
        return cls._default

    def sync(self):
        check(lib().focss_ctx_sync(self.h), self.h)

    @property
    def stream(self):
        return lib().focss_ctx_stream(self.h)

    def profile_enable(self, on=True):
        check(lib().focss_profile_enable(self.h, 1 if on else 0), self.h)

    def profile_read(self, reset=True):
        cm, rm = C.c_double(), C.c_double()
        cl, rl = C.c_longlong(), C.c_longlong()
        check(lib().focss_profile_read(self.h, C.byref(cm), C.byref(cl), C.byref(rm), C.byref(rl),
                                       1 if reset else 0), self.h)
        return {"col_ms": cm.value, "col_launches": cl.value, "row_ms": rm.value, "row_launches": rl.value}

    def close(self):
        if self.h and alive():
            lib().focss_ctx_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass(frozen=True)
class Domain:
    """src/focss/field.h:39-61"""

    modes: int
    samples: int
    time_step: float
    center_frequency: float = 0.0

    def size(self):
        return self.modes * self.samples


@dataclass(frozen=True)
class Fiber:
    """src/focss/module/fiber.h:5-21 and fiber.cpp:4-45"""

    alpha: float
    beta2: float
    gamma: float
    length: float
    wavelength: float = 1.55e-6
    kappa: float = 1.0

    def linear(self):
        return replace(self, gamma=0.0)

    def nonlinear(self):
        return replace(self, alpha=0.0, beta2=0.0)

    def dispersive(self):
        return replace(self, alpha=0.0, gamma=0.0)

    def __neg__(self):
        return replace(self, alpha=-self.alpha, beta2=-self.beta2, gamma=-self.gamma)

    def __mul__(self, f):
        if f >= 0:
            return replace(self, length=self.length * f)
        return replace(self, alpha=-self.alpha, beta2=-self.beta2, gamma=-self.gamma,
                       length=self.length * -f)

    def c(self):
        return CFiber(self.alpha, self.beta2, self.gamma, self.length, self.wavelength, self.kappa)


class Field:
    """Device field: `batch` realizations of one Domain (src/focss/field.h:63-181)."""

    def __init__(self, domain: Domain, data=None, batch: int = 1, ctx: Context | None = None):
        self.ctx = ctx or Context.default()
        self.domain = domain
        self.batch = batch
        h = C.c_void_p()
        d = CDomain(domain.modes, domain.samples, domain.time_step, domain.center_frequency)
        check(lib().focss_field_create(self.ctx.h, C.byref(d), batch, C.byref(h)), self.ctx.h)
        self.h = h
        if data is not None:
            self.upload(data)

    @property
    def shape(self):
        return (self.batch, self.domain.modes, self.domain.samples)

    def size(self):
        return self.batch * self.domain.modes * self.domain.samples

    def upload(self, data):
        a = np.ascontiguousarray(np.asarray(data).reshape(self.shape))
        if a.dtype == np.complex64:
            check(lib().focss_field_upload_c64(self.h, a.ctypes.data_as(C.c_void_p), a.size), self.ctx.h)
        else:
            a = np.ascontiguousarray(a, dtype=np.complex128)
            check(lib().focss_field_upload(self.h, a.ctypes.data_as(C.c_void_p), a.size), self.ctx.h)
        return self

    def numpy(self, dtype=np.complex128):
        if dtype == np.complex64:
            out = np.empty(self.shape, np.complex64)
            check(lib().focss_field_download_c64(self.h, out.ctypes.data_as(C.c_void_p), out.size), self.ctx.h)
        else:
            out = np.empty(self.shape, np.complex128)
            check(lib().focss_field_download(self.h, out.ctypes.data_as(C.c_void_p), out.size), self.ctx.h)
        return out

    def copy(self):
        f = Field(self.domain, batch=self.batch, ctx=self.ctx)
        check(lib().focss_field_copy(f.h, self.h), self.ctx.h)
        return f

    def assign(self, other: "Field"):
        check(lib().focss_field_copy(self.h, other.h), self.ctx.h)
        return self

    def device_ptr(self):
        return lib().focss_field_device_ptr(self.h)

    def copy_realizations(self, dst_first: int, src: "Field", src_first: int, count: int):
        check(lib().focss_field_copy_realizations(self.h, dst_first, src.h, src_first, count), self.ctx.h)
        return self

    def copy_modes(self, dst_first: int, src: "Field", src_first: int, count: int):
        """Copy modes src[src_first : src_first + count] into this field's
        modes [dst_first, ...), in every realization."""
        check(lib().focss_field_copy_modes(self.h, dst_first, src.h, src_first, count), self.ctx.h)
        return self

    def slice(self, first: int, count: int) -> "Field":
        out = Field(self.domain, batch=count, ctx=self.ctx)
        return out.copy_realizations(0, self, first, count)

    # src/focss/field.cpp:381-391
    def __imul__(self, s):
        s = complex(s)
        check(lib().focss_field_scale(self.h, s.real, s.imag), self.ctx.h)
        return self

    def power_stats(self):
        avg = np.zeros(self.batch)
        pk = np.zeros(self.batch)
        check(lib().focss_field_power(self.h, avg.ctypes.data_as(C.c_void_p), pk.ctypes.data_as(C.c_void_p)),
              self.ctx.h)
        return avg, pk

    def average_power(self):
        return self.power_stats()[0]

    def peak_power(self):
        return self.power_stats()[1]

    def fft_inplace(self):
        check(lib().focss_field_fft(self.h), self.ctx.h)
        return self

    def ifft_inplace(self):
        check(lib().focss_field_ifft(self.h), self.ctx.h)
        return self

    def dt(self):
        return self.domain.time_step

    def close(self):
        if getattr(self, "h", None) and alive():
            lib().focss_field_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SSFM:
    """src/focss/solver/ssfm.h:8-54"""

    UNIFORM, LOGARITHMIC, ADAPTIVE = 0, 1, 2
    FORWARD, BACKWARD = 1.0, -1.0

    def __init__(self, fiber: Fiber | None = None, total_steps: int | None = None):
        self.fiber = fiber
        self.grid = SSFM.UNIFORM if total_steps is not None else None
        self.total_steps = total_steps or 0
        self.maximum_phase_shift = 0.0
        self.maximum_step_size = 0.0

    def set_fiber(self, fiber):
        self.fiber = fiber

    def set_grid(self, grid):
        self.grid = grid

    def set_total_steps(self, n):
        self.total_steps = n

    def set_maximum_phase_shift(self, x):
        self.maximum_phase_shift = x

    def set_maximum_step_size(self, x):
        self.maximum_step_size = x

    def opts(self):
        if self.grid is None:
            raise FocssError(1, "SSFM grid not set (the reference leaves it uninitialized)")
        return CSsfmOpts(self.grid, self.total_steps, self.maximum_phase_shift, self.maximum_step_size)

    def run(self, field: Field, direction: float = FORWARD):
        steps = np.zeros(field.batch, np.int32)
        fb, op = self.fiber.c(), self.opts()
        check(lib().focss_ssfm_run(field.ctx.h, field.h, C.byref(fb), C.byref(op), direction,
                                   steps.ctypes.data_as(C.c_void_p)), field.ctx.h)
        return steps

    def run_recorded(self, field: Field, direction: float = FORWARD, capacity: int = 1 << 16):
        """run() that also returns each realization's step sizes: (steps,
        [array of |h_i| per realization]) (focss_ssfm_run_record)."""
        steps = np.zeros(field.batch, np.int32)
        hs = np.zeros((field.batch, capacity))
        fb, op = self.fiber.c(), self.opts()
        check(lib().focss_ssfm_run_record(field.ctx.h, field.h, C.byref(fb), C.byref(op), direction, capacity,
                                          hs.ctypes.data_as(C.c_void_p), steps.ctypes.data_as(C.c_void_p)),
              field.ctx.h)
        return steps, [hs[b, :steps[b]].copy() for b in range(field.batch)]

    def run_steps(self, field: Field, steps_h, direction: float = FORWARD):
        """Propagate with the given step sizes (one sequence per realization)
        instead of the grid rule (focss_ssfm_run_steps)."""
        if len(steps_h) != field.batch:
            raise FocssError(1, "run_steps: one step list per realization")
        cap = max(len(h) for h in steps_h)
        buf = np.zeros((field.batch, cap))
        n = np.zeros(field.batch, np.int32)
        for b, h in enumerate(steps_h):
            buf[b, :len(h)] = h
            n[b] = len(h)
        fb = self.fiber.c()
        check(lib().focss_ssfm_run_steps(field.ctx.h, field.h, C.byref(fb), buf.ctypes.data_as(C.c_void_p),
                                         n.ctypes.data_as(C.c_void_p), cap, direction), field.ctx.h)
        return n


class Amplifier:
    """src/focss/module/amplifier.h:7-22 (ASE from a seeded counter-based stream)."""

    AMPLIFY, ADD_NOISE, GIVE_POWER, DROP_POWER = 0, 1, 2, 3

    def __init__(self, gain: float = 1.0, noise_factor: float = 0.0, seed: int = 0):
        self.gain = gain
        self.noise_factor = noise_factor
        self.seed = seed

    def _apply(self, field, op, counter):
        check(lib().focss_amplifier_apply(field.ctx.h, field.h, self.gain, self.noise_factor, self.seed,
                                          counter, op), field.ctx.h)

    def amplify(self, field, counter=0):
        self._apply(field, Amplifier.AMPLIFY, counter)

    def add_noise(self, field, counter=0):
        self._apply(field, Amplifier.ADD_NOISE, counter)

    def give_power(self, field):
        self._apply(field, Amplifier.GIVE_POWER, 0)

    def drop_power(self, field):
        self._apply(field, Amplifier.DROP_POWER, 0)


# ---- span drivers (src/tasks/systems.cpp:26-91)
def forward_propagation(field: Field, fiber: Fiber, ssfm: SSFM, amplifier: Amplifier, spans: int, counter0=0):
    fb, op = fiber.c(), ssfm.opts()
    check(lib().focss_forward_propagation(field.ctx.h, field.h, C.byref(fb), C.byref(op), amplifier.gain,
                                          amplifier.noise_factor, amplifier.seed, counter0, spans), field.ctx.h)


def backward_propagation(field: Field, fiber: Fiber, ssfm: SSFM, gain: float, spans: int):
    fb, op = fiber.c(), ssfm.opts()
    check(lib().focss_backward_propagation(field.ctx.h, field.h, C.byref(fb), C.byref(op), gain, spans),
          field.ctx.h)


AMP_NONE = -1


def span_loop(fields, fiber: Fiber, ssfms, spans: int, direction: float = SSFM.FORWARD,
              amplifier: Amplifier | None = None, before: int = AMP_NONE, after: int = AMP_NONE,
              counter0: int = 0):
    """Span loops of forward/backward_propagation (src/tasks/systems.cpp:26-91)
    for several fields at once, as one CUDA-graph launch (focss_span_loop):
    per span, amplifier op `before`, SSFM with ssfms[i] on fields[i], op
    `after`.  `ssfms` is one SSFM or one per field.  Returns the steps per
    realization summed over spans, one array per field."""
    fields = list(fields)
    if isinstance(ssfms, SSFM):
        ssfms = [ssfms] * len(fields)
    if len(ssfms) != len(fields):
        raise FocssError(1, "span_loop: one SSFM per field")
    ctx = fields[0].ctx
    handles = (C.c_void_p * len(fields))(*[f.h.value if isinstance(f.h, C.c_void_p) else f.h for f in fields])
    opts = (CSsfmOpts * len(fields))(*[s.opts() for s in ssfms])
    amp = amplifier or Amplifier()
    ca = CAmp(amp.gain, amp.noise_factor, amp.seed, counter0, before, after)
    total = sum(f.batch for f in fields)
    steps = np.zeros(total, np.int32)
    fb = fiber.c()
    check(lib().focss_span_loop(ctx.h, len(fields), handles, C.byref(fb), opts, C.byref(ca), spans, direction,
                                steps.ctypes.data_as(C.c_void_p)), ctx.h)
    out, o = [], 0
    for f in fields:
        out.append(steps[o:o + f.batch].copy())
        o += f.batch
    return out


def autotune(samples: int, batch: int, ctx: Context | None = None):
    """Time every admissible FFT split of length `samples` (and, for
    2^12..2^14, the single-CTA kernel) on `batch` realizations and keep the
    fastest for this context's split-step runs.  Returns (log2 N1 or
    SPLIT_SINGLE_CTA, ms per step)."""
    ctx = ctx or Context.default()
    l1, ms = C.c_int(), C.c_double()
    check(lib().focss_autotune(ctx.h, samples, batch, C.byref(l1), C.byref(ms)), ctx.h)
    return l1.value, ms.value


SPLIT_SINGLE_CTA = -1  # FOCSS_SPLIT_SINGLE_CTA: one CTA per realization, field in shared memory
STAGING_LOADS, STAGING_BULK, STAGING_TMA = 0, 1, 2  # FOCSS_STAGING_*: how the passes move their data


def set_pass_staging(mode: int, ctx: Context | None = None):
    """Staging of this context's split-step passes: STAGING_LOADS
    (per-thread coalesced loads, the default), STAGING_BULK (the row pass
    by TMA bulk copies) or STAGING_TMA (as BULK, and the column pass's tiles
    by 2-D TMA tensor copies); the results are the same bit for bit."""
    ctx = ctx or Context.default()
    check(lib().focss_set_pass_staging(ctx.h, int(mode)), ctx.h)


def set_row_staging(mode: int, ctx: Context | None = None):
    """set_pass_staging restricted to STAGING_LOADS and STAGING_BULK."""
    ctx = ctx or Context.default()
    check(lib().focss_set_row_staging(ctx.h, int(mode)), ctx.h)


def set_fft_split(samples: int, log2_n1: int, ctx: Context | None = None):
    """Pin the split of length-`samples` split-step runs (0 = balanced
    default, SPLIT_SINGLE_CTA = the single-CTA kernel for 2^12..2^14)."""
    ctx = ctx or Context.default()
    check(lib().focss_set_fft_split(ctx.h, samples, log2_n1), ctx.h)


def cd_compensation(field: Field, fiber: Fiber, spans: int):
    fb = fiber.c()
    check(lib().focss_cd_compensation(field.ctx.h, field.h, C.byref(fb), spans), field.ctx.h)

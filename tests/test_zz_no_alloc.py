"""The allocation-free split-step entry point (focss_ssfm_run_noalloc).

It serves callers that cannot let a library allocate device memory (a host
framework that owns the device heap, a loop where an allocation is not
allowed, a fixed memory budget).  It must give the same fields as the
allocating entry point focss_ssfm_run, call after call, on a device buffer the
caller owns.  This file is collected last so that a failure here leaves every
other test already run.
"""
import ctypes as C

import numpy as np
import pytest

import focss_gb300 as fg
from focss_gb300._lib import CFiber, CSsfmOpts, lib
from conftest import ALPHA, BETA2, GAMMA, rel_l2

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-5


def _signal(batch, n, seed):
    rng = np.random.default_rng(seed)
    p = np.array([0.5, 1.0, 2.0, 4.0])[:batch, None] * 1e-3
    return (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))) * np.sqrt(p / 2)


@pytest.mark.parametrize("grid", [fg.SSFM.UNIFORM, fg.SSFM.ADAPTIVE])
def test_noalloc_matches_allocating_entry_point_twice(grid):
    ctx = fg.Context.default()
    n, batch, dt = 1 << 15, 4, 1 / 256e9
    fiber = fg.Fiber(ALPHA, BETA2, GAMMA, 40e3)
    ssfm = fg.SSFM(fiber, 40) if grid == fg.SSFM.UNIFORM else fg.SSFM(fiber)
    if grid == fg.SSFM.ADAPTIVE:
        ssfm.set_grid(grid)
        ssfm.set_maximum_phase_shift(0.005)
        ssfm.set_maximum_step_size(1000.0)
    for call in range(2):  # two calls in a row share the scratch array
        x = _signal(batch, n, 100 + call)
        want_f = fg.Field(fg.Domain(1, n, dt), data=x[:, None, :], batch=batch, ctx=ctx)
        want_steps = ssfm.run(want_f)
        # The caller's own device buffer (allocated by the caller, not by the entry point).
        buf = fg.Field(fg.Domain(1, n, dt), data=x[:, None, :], batch=batch, ctx=ctx)
        ctx.sync()
        steps = np.zeros(batch, np.int32)
        fb, op = fiber.c(), ssfm.opts()
        st = lib().focss_ssfm_run_noalloc(ctx.stream, buf.device_ptr(), n, batch, dt, C.byref(fb), C.byref(op),
                                          1.0, steps.ctypes.data_as(C.c_void_p))
        assert st == 0
        np.testing.assert_array_equal(steps, want_steps)
        assert rel_l2(buf.numpy(), want_f.numpy()) < FIELD_TOL


def test_noalloc_rejects_shapes_beyond_its_limits():
    ctx = fg.Context.default()
    fb = CFiber(ALPHA, BETA2, GAMMA, 1e3, 1.55e-6, 1.0)
    op = CSsfmOpts(0, 1, 0.0, 0.0)
    f = fg.Field(fg.Domain(1, 1 << 8, 1e-12), batch=1, ctx=ctx)
    too_long = lib().focss_ssfm_run_noalloc(ctx.stream, f.device_ptr(), 1 << 18, 1, 1e-12, C.byref(fb),
                                            C.byref(op), 1.0, None)
    too_many = lib().focss_ssfm_run_noalloc(ctx.stream, f.device_ptr(), 1 << 8, 257, 1e-12, C.byref(fb),
                                            C.byref(op), 1.0, None)
    assert too_long == 6 and too_many == 6  # FOCSS_ERR_UNSUPPORTED, no GPU work issued

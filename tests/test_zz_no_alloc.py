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
    p = np.resize(np.array([0.5, 1.0, 2.0, 4.0]), batch)[:, None] * 1e-3
    return (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))) * np.sqrt(p / 2)


def _noalloc(ctx, buf, n, batch, dt, fiber, ssfm, direction):
    steps = np.zeros(batch, np.int32)
    fb, op = fiber.c(), ssfm.opts()
    st = lib().focss_ssfm_run_noalloc(ctx.stream, buf.device_ptr(), n, batch, dt, C.byref(fb), C.byref(op),
                                      direction, steps.ctypes.data_as(C.c_void_p))
    return st, steps


def _ssfm(fiber, grid):
    if grid == fg.SSFM.UNIFORM:
        return fg.SSFM(fiber, 40)
    ssfm = fg.SSFM(fiber)
    ssfm.set_grid(grid)
    ssfm.set_maximum_phase_shift(0.005)
    ssfm.set_maximum_step_size(1000.0)
    return ssfm


# (log2 samples, batch, grid, direction): the documented limits 2^8 and
# 2^17 x 256 (where the fixed twiddle area and the state array are full), all
# three grids and both directions
CASES = [
    (15, 4, fg.SSFM.UNIFORM, 1.0),
    (15, 4, fg.SSFM.ADAPTIVE, 1.0),
    (12, 3, fg.SSFM.LOGARITHMIC, 1.0),
    (12, 3, fg.SSFM.UNIFORM, -1.0),
    (8, 4, fg.SSFM.ADAPTIVE, 1.0),
    (17, 256, fg.SSFM.ADAPTIVE, 1.0),
]


@pytest.mark.parametrize("lg,batch,grid,direction", CASES)
def test_noalloc_matches_allocating_entry_point_twice(lg, batch, grid, direction):
    ctx = fg.Context.default()
    n, dt = 1 << lg, 1 / 256e9
    fiber = fg.Fiber(ALPHA, BETA2, GAMMA, 40e3)
    ssfm = _ssfm(fiber, grid)
    for call in range(2):  # two calls in a row share the scratch array
        x = _signal(batch, n, 100 + call)
        want_f = fg.Field(fg.Domain(1, n, dt), data=x[:, None, :], batch=batch, ctx=ctx)
        want_steps = ssfm.run(want_f, direction)
        # The caller's own device buffer (allocated by the caller, not by the entry point).
        buf = fg.Field(fg.Domain(1, n, dt), data=x[:, None, :], batch=batch, ctx=ctx)
        ctx.sync()
        st, steps = _noalloc(ctx, buf, n, batch, dt, fiber, ssfm, direction)
        assert st == 0
        np.testing.assert_array_equal(steps, want_steps)
        assert rel_l2(buf.numpy(), want_f.numpy()) < FIELD_TOL


def test_noalloc_allocates_no_device_memory():
    """After a first call (the one-time symbol lookup), a call leaves the
    device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    ctx = fg.Context.default()
    n, batch, dt = 1 << 14, 8, 1 / 256e9
    fiber = fg.Fiber(ALPHA, BETA2, GAMMA, 20e3)
    ssfm = _ssfm(fiber, fg.SSFM.ADAPTIVE)
    buf = fg.Field(fg.Domain(1, n, dt), data=_signal(batch, n, 7)[:, None, :], batch=batch, ctx=ctx)
    ctx.sync()
    assert _noalloc(ctx, buf, n, batch, dt, fiber, ssfm, 1.0)[0] == 0
    free_before = torch.cuda.mem_get_info(0)[0]
    assert _noalloc(ctx, buf, n, batch, dt, fiber, ssfm, 1.0)[0] == 0
    assert torch.cuda.mem_get_info(0)[0] == free_before


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

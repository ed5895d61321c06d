"""The row pass with TMA bulk-copy staging (focss_set_row_staging(BULK):
rows queued by cp.async.bulk behind an mbarrier, stored back by bulk
copies) against the default per-thread loads and stores: the arithmetic is
the same, so split-step runs and plain transforms must agree bit for bit, for
every row length the plans use (2^4 .. 2^10)."""
import numpy as np
import pytest

import focss_gb300 as fg
from conftest import ALPHA, BETA2, GAMMA

pytestmark = pytest.mark.gpu


def _signal(batch, n, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((batch, 1, n)) + 1j * rng.standard_normal((batch, 1, n))) * np.sqrt(2e-3)


def _run(ctx, x, n, mode, grid):
    fg.set_row_staging(mode, ctx=ctx)
    try:
        f = fg.Field(fg.Domain(1, n, 1 / 256e9), data=x, batch=x.shape[0], ctx=ctx)
        fib = fg.Fiber(ALPHA, BETA2, GAMMA, 20e3)
        if grid == "uniform":
            steps = fg.SSFM(fib, 20).run(f)
        else:
            s = fg.SSFM(fib)
            s.set_grid(fg.SSFM.ADAPTIVE)
            s.set_maximum_phase_shift(0.005)
            s.set_maximum_step_size(1000.0)
            steps = s.run(f)
        g = fg.Field(fg.Domain(1, n, 1 / 256e9), data=x, batch=x.shape[0], ctx=ctx)
        g.fft_inplace()
        return f.numpy(), steps, g.numpy()
    finally:
        fg.set_row_staging(fg.STAGING_LOADS, ctx=ctx)


@pytest.mark.parametrize("lg,batch,grid", [(8, 3, "uniform"), (9, 2, "adaptive"), (11, 2, "adaptive"),
                                           (13, 2, "uniform"), (15, 3, "adaptive"), (17, 2, "uniform"),
                                           (19, 2, "adaptive"), (20, 1, "uniform")])
def test_bulk_staging_is_bit_identical(ctx, lg, batch, grid):
    n = 1 << lg
    x = _signal(batch, n, lg)
    a, sa, fa = _run(ctx, x, n, fg.STAGING_LOADS, grid)
    b, sb, fb = _run(ctx, x, n, fg.STAGING_BULK, grid)
    np.testing.assert_array_equal(sa, sb)
    assert np.array_equal(a, b)
    assert np.array_equal(fa, fb)


def test_staging_rejects_unknown_mode(ctx):
    with pytest.raises(fg.FocssError):
        fg.set_row_staging(7, ctx=ctx)

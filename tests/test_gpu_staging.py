"""The split-step passes with TMA staging against the default per-thread
loads and stores: focss_set_pass_staging(BULK) moves the row pass's rows by
cp.async.bulk behind an mbarrier and stores them back by bulk copies;
focss_set_pass_staging(TMA) does the same and also loads the column pass's
tiles (C columns x N1 rows, a strided block of the field) as 2-D TMA tensor
boxes.  The arithmetic is the same, so split-step runs and plain transforms
must agree bit for bit, for every row length the plans use (2^4 .. 2^10), on
one and two modes."""
import numpy as np
import pytest

import focss_gb300 as fg
from conftest import ALPHA, BETA2, GAMMA

pytestmark = pytest.mark.gpu


def _signal(batch, modes, n, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((batch, modes, n)) + 1j * rng.standard_normal((batch, modes, n))) * np.sqrt(2e-3)


def _run(ctx, x, n, mode, grid):
    modes = x.shape[1]
    fg.set_pass_staging(mode, ctx=ctx)
    try:
        f = fg.Field(fg.Domain(modes, n, 1 / 256e9), data=x, batch=x.shape[0], ctx=ctx)
        fib = fg.Fiber(ALPHA, BETA2, GAMMA, 20e3)
        if grid == "uniform":
            steps = fg.SSFM(fib, 20).run(f)
        else:
            s = fg.SSFM(fib)
            s.set_grid(fg.SSFM.ADAPTIVE)
            s.set_maximum_phase_shift(0.005)
            s.set_maximum_step_size(1000.0)
            steps = s.run(f)
        g = fg.Field(fg.Domain(modes, n, 1 / 256e9), data=x, batch=x.shape[0], ctx=ctx)
        g.fft_inplace()
        return f.numpy(), steps, g.numpy()
    finally:
        fg.set_pass_staging(fg.STAGING_LOADS, ctx=ctx)


@pytest.mark.parametrize("mode", ["bulk", "tma"])
@pytest.mark.parametrize("lg,modes,batch,grid", [(8, 1, 3, "uniform"), (9, 1, 2, "adaptive"), (11, 2, 2, "adaptive"),
                                                 (13, 1, 2, "uniform"), (15, 1, 3, "adaptive"), (17, 2, 2, "uniform"),
                                                 (19, 1, 2, "adaptive"), (20, 1, 1, "uniform")])
def test_staging_is_bit_identical(ctx, mode, lg, modes, batch, grid):
    n = 1 << lg
    x = _signal(batch, modes, n, lg)
    a, sa, fa = _run(ctx, x, n, fg.STAGING_LOADS, grid)
    b, sb, fb = _run(ctx, x, n, fg.STAGING_BULK if mode == "bulk" else fg.STAGING_TMA, grid)
    np.testing.assert_array_equal(sa, sb)
    assert np.array_equal(a, b)
    assert np.array_equal(fa, fb)


def test_staging_rejects_unknown_mode(ctx):
    with pytest.raises(fg.FocssError):
        fg.set_pass_staging(7, ctx=ctx)
    with pytest.raises(fg.FocssError):
        fg.set_row_staging(fg.STAGING_TMA, ctx=ctx)  # the row-only setter takes LOADS and BULK

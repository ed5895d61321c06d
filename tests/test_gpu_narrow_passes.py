"""The split-step passes in 64-thread CTAs against the full-width CTAs.

When a launch has fewer column (row) blocks than the GPU has SMs, the column
(row) pass runs 64-thread CTAs of fewer columns (rows) each, so that more SMs
share a small field (a single 2^17 realization: src/focss/solver/ssfm.cpp:62-72
advances one field at a time).  The per-column and per-row arithmetic does not
depend on how many columns or rows a CTA holds, so a realization run alone
(narrow launches) must equal the same realization run inside a batch large
enough for the full-width launches, bit for bit: UNIFORM and ADAPTIVE fields,
step counts and plain transforms, single and dual polarization.
"""
import numpy as np
import pytest

import focss_gb300 as fg
from conftest import ALPHA, BETA2, GAMMA

pytestmark = pytest.mark.gpu


def _signal(batch, modes, n, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((batch, modes, n)) + 1j * rng.standard_normal((batch, modes, n))) * np.sqrt(2e-3)


def _run(ctx, x, n, grid):
    modes = x.shape[1]
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
    return f.numpy(), np.asarray(steps), g.numpy()


@pytest.mark.parametrize("lg,modes,grid", [(8, 1, "uniform"), (11, 1, "adaptive"), (13, 2, "uniform"),
                                           (15, 1, "adaptive"), (17, 1, "uniform"), (17, 2, "adaptive"),
                                           (19, 1, "adaptive"), (20, 1, "uniform")])
def test_single_realization_equals_wide_batch(ctx, lg, modes, grid):
    n = 1 << lg
    wide = max(2, (1 << 22) // (n * modes))  # enough blocks for the full-width launches
    x = _signal(wide, modes, n, lg)
    a, sa, fa = _run(ctx, x[:1], n, grid)
    b, sb, fb = _run(ctx, x, n, grid)
    assert sa[0] == sb[0]
    assert np.array_equal(a[0], b[0])
    assert np.array_equal(fa[0], fb[0])

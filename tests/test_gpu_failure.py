"""Failure handling without a GPU fault: every device-side loop is bounded.

An ADAPTIVE run whose step bound is absurdly small needs more than the step
cap (2^17 column passes); the host-driven loop, the graph-captured span loop
and the single-CTA kernel must each stop at the cap and return
FOCSS_ERR_NOT_CONVERGED, and the context must stay usable: a normal run right
after matches the FP64 oracle.
"""
import numpy as np
import pytest

import focss_gb300 as fg
from focss_gb300._lib import FocssError
from conftest import ALPHA, BETA2, F0, GAMMA, rel_l2

pytestmark = pytest.mark.gpu

NOT_CONVERGED = 5


def _field(ctx, n, batch=1):
    rng = np.random.default_rng(3)
    x = (rng.standard_normal((batch, 1, n)) + 1j * rng.standard_normal((batch, 1, n))) * 0.02
    return fg.Field(fg.Domain(1, n, 1 / 256e9, F0), data=x.astype(np.complex64), batch=batch, ctx=ctx)


def _tiny_steps(fib):
    s = fg.SSFM(fib)
    s.set_grid(fg.SSFM.ADAPTIVE)
    s.set_maximum_phase_shift(1e-12)
    s.set_maximum_step_size(1000.0)
    return s


def _still_usable(ctx, oracle_cpu):
    n, dt = 1 << 12, 1 / 256e9
    fib = fg.Fiber(ALPHA, BETA2, GAMMA, 10e3)
    f = _field(ctx, n)
    x = f.numpy()[0, 0]
    fg.SSFM(fib, 10).run(f)
    want, _ = oracle_cpu.ssfm_run(x, dt, oracle_cpu.Fiber(ALPHA, BETA2, GAMMA, 10e3, 1.55e-6, 1.0),
                                  oracle_cpu.UNIFORM, 10)
    assert rel_l2(f.numpy()[0, 0], want) < 2e-6


@pytest.mark.parametrize("path", ["host", "span_loop", "single_cta"])
def test_step_cap_returns_not_converged(ctx, oracle_cpu, path):
    fib = fg.Fiber(ALPHA, BETA2, GAMMA, 80e3)
    n = 1 << 12
    f = _field(ctx, n)
    if path == "single_cta":
        fg.set_fft_split(n, fg.SPLIT_SINGLE_CTA, ctx=ctx)
    try:
        with pytest.raises(FocssError) as e:
            if path == "span_loop":
                fg.span_loop([f], fib, _tiny_steps(fib), 1)
            else:
                _tiny_steps(fib).run(f)
        assert e.value.status == NOT_CONVERGED
        assert "step cap" in str(e.value)
    finally:
        fg.set_fft_split(n, 0, ctx=ctx)
    _still_usable(ctx, oracle_cpu)

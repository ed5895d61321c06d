"""Two-mode (dual-polarization) fields through the split-step passes.

SSFM::nonlinear_step rotates every mode by kappa*gamma*h times the power
summed over modes (src/focss/solver/ssfm.cpp:160-164, Field::power
field.cpp:164-171); the adaptive grid uses the peak of that sum and the
logarithmic grid its average (ssfm.cpp:120-140).  With kappa = 8/9 (the
reference's dual-polarization coupling, src/tasks/parameters.h:7) every grid
must match the FP64 oracle: fields within 1e-5 relative L2, step counts equal,
and the graph-captured span loop must equal the host-driven one.
"""
import numpy as np
import pytest

import focss_gb300 as fg
from conftest import ALPHA, BETA2, F0, GAMMA, rel_l2

pytestmark = pytest.mark.gpu

KAPPA = 8.0 / 9.0
TOL = 1e-5


def _two_mode(rng, n, batch, powers_mw):
    x = rng.standard_normal((batch, 2, n)) + 1j * rng.standard_normal((batch, 2, n))
    X = np.fft.fft(x, axis=-1)
    X[..., np.abs(np.fft.fftfreq(n)) > 0.2] = 0
    x = np.fft.ifft(X, axis=-1)
    x /= np.sqrt(np.mean(np.abs(x) ** 2, axis=(1, 2), keepdims=True))
    return x * np.sqrt(np.asarray(powers_mw)[:, None, None] * 1e-3 / 2)


def _grid(fib, grid):
    s = fg.SSFM(fib, 25) if grid == fg.SSFM.UNIFORM else fg.SSFM(fib)
    if grid != fg.SSFM.UNIFORM:
        s.set_grid(grid)
        s.set_maximum_phase_shift(0.005)
        s.set_maximum_step_size(1000.0)
    return s


@pytest.mark.parametrize("grid", [fg.SSFM.UNIFORM, fg.SSFM.ADAPTIVE, fg.SSFM.LOGARITHMIC])
@pytest.mark.parametrize("lg", [12, 15])
def test_two_modes_match_oracle(ctx, oracle_cpu, grid, lg):
    cpu = oracle_cpu
    rng = np.random.default_rng(lg + grid)
    n, dt, L = 1 << lg, 1 / 256e9, 20e3
    x = _two_mode(rng, n, 3, [0.5, 2.0, 6.0])
    f = fg.Field(fg.Domain(2, n, dt, F0), data=x, batch=3, ctx=ctx)
    fib = fg.Fiber(ALPHA, BETA2, GAMMA, L, kappa=KAPPA)
    steps = _grid(fib, grid).run(f)
    got = f.numpy()
    ofib = cpu.Fiber(ALPHA, BETA2, GAMMA, L, 1.55e-6, KAPPA)
    for b in range(3):
        want, ws = cpu.ssfm_run(x[b], dt, ofib, grid, 25, 0.005, 1000.0)
        assert steps[b] == ws
        assert rel_l2(got[b], want) < TOL


def test_two_mode_power_is_summed(ctx, oracle_cpu):
    """All power in mode 0 vs split over both modes: the same total power
    gives the same nonlinear phase on each mode's share."""
    cpu = oracle_cpu
    rng = np.random.default_rng(3)
    n, dt = 1 << 12, 1 / 256e9
    a = _two_mode(rng, n, 1, [4.0])[0]
    x = np.stack([a[0], a[0]])       # identical modes: total power 2|a0|^2
    f = fg.Field(fg.Domain(2, n, dt, F0), data=x[None], ctx=ctx)
    fib = fg.Fiber(0.0, 0.0, GAMMA, 5e3, kappa=KAPPA)
    fg.SSFM(fib, 5).run(f)
    got = f.numpy()[0]
    want = x * np.exp(1j * KAPPA * GAMMA * 5e3 * 2 * np.abs(a[0]) ** 2)
    assert rel_l2(got, want) < TOL
    np.testing.assert_array_equal(got[0], got[1])


def test_two_mode_span_loop_matches_host_loop(ctx):
    rng = np.random.default_rng(9)
    n, dt = 1 << 13, 1 / 256e9
    x = _two_mode(rng, n, 2, [1.0, 3.0])
    fib = fg.Fiber(ALPHA, BETA2, GAMMA, 80e3, kappa=KAPPA)
    a = fg.Field(fg.Domain(2, n, dt, F0), data=x, batch=2, ctx=ctx)
    b = a.copy()
    s = _grid(fib, fg.SSFM.ADAPTIVE)
    amp = fg.Amplifier(10 ** 1.6, 10 ** 0.5, seed=3)
    steps = fg.span_loop([a], fib, s, 2, after=fg.Amplifier.AMPLIFY, amplifier=amp)
    ref = np.zeros(2, np.int64)
    for span in range(2):
        ref += s.run(b)
        amp.amplify(b, counter=span)
    np.testing.assert_array_equal(a.numpy(), b.numpy())
    np.testing.assert_array_equal(steps[0], ref)

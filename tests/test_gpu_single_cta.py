"""Single-CTA split-step kernel (N = 2^12..2^14: one CTA per realization runs
the whole SSFM with the field in shared memory).

It executes the column and row work of the two-pass kernels in the same
order, so with the same FFT split it must reproduce the two-pass results
bit for bit (fields and step counts) for UNIFORM and ADAPTIVE grids, on
its own and inside graph-captured span loops with ASE; LOGARITHMIC grids
(whose step count comes from an FP32 energy sum taken in another order) must
give the same step count and the oracle's field.  Dual-polarization fields of
those lengths keep the two-pass kernels.
"""
import numpy as np
import pytest

import focss_gb300 as fg
from conftest import ALPHA, BETA2, F0, GAMMA, rel_l2

pytestmark = pytest.mark.gpu

G = 10 ** (0.2 * 80 / 10)
NF = 10 ** 0.5
SPLIT = {1 << 12: 6, 1 << 13: 7, 1 << 14: 7}


def _field(ctx, n, batch, seed, power_dbm=4.0, modes=1, dt=1 / 256e9):
    rng = np.random.default_rng(seed)
    p = 1e-3 * 10 ** (power_dbm / 10)
    x = (rng.standard_normal((batch, modes, n)) + 1j * rng.standard_normal((batch, modes, n))) * np.sqrt(p / 2)
    X = np.fft.fft(x, axis=-1)
    X[..., np.abs(np.fft.fftfreq(n)) > 0.125] = 0
    x = np.fft.ifft(X, axis=-1) * 2.0
    return fg.Field(fg.Domain(modes, n, dt, F0), data=x.astype(np.complex64), batch=batch, ctx=ctx)


def _fiber(length=80e3):
    return fg.Fiber(ALPHA, BETA2, GAMMA, length)


def _ssfm(fib, grid):
    if grid == "uniform":
        return fg.SSFM(fib, 40)
    s = fg.SSFM(fib)
    s.set_grid(fg.SSFM.ADAPTIVE if grid == "adaptive" else fg.SSFM.LOGARITHMIC)
    s.set_maximum_phase_shift(0.005)
    s.set_maximum_step_size(1000.0)
    return s


def _both(ctx, n, fn):
    """fn() under the two-pass kernels at the single-CTA split, then under
    the single-CTA kernel."""
    fg.set_fft_split(n, SPLIT[n], ctx=ctx)
    a = fn()
    fg.set_fft_split(n, fg.SPLIT_SINGLE_CTA, ctx=ctx)
    b = fn()
    fg.set_fft_split(n, 0, ctx=ctx)
    return a, b


@pytest.mark.parametrize("n", [1 << 12, 1 << 13, 1 << 14])
@pytest.mark.parametrize("grid", ["uniform", "adaptive"])
def test_bit_identical_to_two_pass(ctx, n, grid):
    fib = _fiber()
    x = _field(ctx, n, 5, n + len(grid))

    def run():
        f = x.copy()
        steps = _ssfm(fib, grid).run(f)
        return f.numpy(), steps

    (fa, sa), (fb, sb) = _both(ctx, n, run)
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_array_equal(fa, fb)
    if grid == "adaptive":
        assert sa.min() > 40


def test_logarithmic_grid(ctx):
    n = 1 << 13
    fib = _fiber()
    x = _field(ctx, n, 3, 9)

    def run():
        f = x.copy()
        steps = _ssfm(fib, "logarithmic").run(f)
        return f.numpy(), steps

    (fa, sa), (fb, sb) = _both(ctx, n, run)
    np.testing.assert_array_equal(sa, sb)
    assert rel_l2(fb, fa) < 1e-6


def test_span_loop_with_noise(ctx):
    """Forward spans with ASE and backward DBP variants, graph-captured, with
    a single-CTA field next to a two-pass field in the same launch."""
    fib = _fiber()
    x14, x15 = _field(ctx, 1 << 14, 3, 1), _field(ctx, 1 << 15, 2, 2)

    def run():
        fs = [x14.copy(), x15.copy()]
        st = fg.span_loop(fs, fib, _ssfm(fib, "adaptive"), 3, after=fg.Amplifier.AMPLIFY,
                          amplifier=fg.Amplifier(G, NF, seed=3))
        back = [fs[0].copy() for _ in range(2)]
        fg.span_loop(back, fib, [fg.SSFM(fib, 1), fg.SSFM(fib, 4)], 3, direction=fg.SSFM.BACKWARD,
                     amplifier=fg.Amplifier(G), before=fg.Amplifier.DROP_POWER)
        return [f.numpy() for f in fs + back], st

    (fa, sa), (fb, sb) = _both(ctx, 1 << 14, run)
    for a, b in zip(sa, sb):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(fa, fb):
        np.testing.assert_array_equal(a, b)


def test_against_oracle(ctx, oracle_cpu):
    cpu = oracle_cpu
    n, dt = 1 << 14, 1 / 256e9
    x = _field(ctx, n, 1, 7, power_dbm=8.0).numpy()[0, 0]
    want, wsteps = cpu.ssfm_run(x.astype(np.complex128), dt, cpu.Fiber(ALPHA, BETA2, GAMMA, 80e3, 1.55e-6, 1.0),
                                cpu.ADAPTIVE, 1, 0.005, 1000.0)
    fg.set_fft_split(n, fg.SPLIT_SINGLE_CTA, ctx=ctx)
    f = fg.Field(fg.Domain(1, n, dt, F0), data=x[None, None], ctx=ctx)
    steps = _ssfm(_fiber(), "adaptive").run(f)
    fg.set_fft_split(n, 0, ctx=ctx)
    assert int(steps[0]) == wsteps
    assert rel_l2(f.numpy()[0, 0], want) < 1e-5


def test_dual_polarization_keeps_two_pass(ctx):
    n = 1 << 13
    fib = fg.Fiber(ALPHA, BETA2, GAMMA, 80e3, 1.55e-6, 8 / 9)
    x = _field(ctx, n, 2, 4, modes=2)

    def run():
        f = x.copy()
        _ssfm(fib, "adaptive").run(f)
        return f.numpy(), None

    (fa, _), (fb, _) = _both(ctx, n, run)
    np.testing.assert_array_equal(fa, fb)


def test_split_selection(ctx):
    with pytest.raises(fg.FocssError):
        fg.set_fft_split(1 << 15, fg.SPLIT_SINGLE_CTA, ctx=ctx)
    l1, ms = fg.autotune(1 << 12, 512, ctx=ctx)
    assert (l1 == fg.SPLIT_SINGLE_CTA or 4 <= l1 <= 8) and ms > 0
    fg.set_fft_split(1 << 12, 0, ctx=ctx)

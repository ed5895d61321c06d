"""Graph-captured span loops (focss_span_loop) and the FFT-split autotuner.

The span loop must give exactly what the host-driven span loops give
(forward_propagation / backward_propagation of src/tasks/systems.cpp:26-91,
same kernels, same order), for several fields of different lengths and
batches at once, for UNIFORM, ADAPTIVE (device-side WHILE loop) and
LOGARITHMIC grids, and on replay with new noise seeds.  Every FFT split the
autotuner may pick must match the FP64 oracle.
"""
import numpy as np
import pytest

import focss_gb300 as fg
from conftest import ALPHA, BETA2, F0, GAMMA, rel_l2

pytestmark = pytest.mark.gpu

G = 10 ** (0.2 * 80 / 10)
NF = 10 ** 0.5


def _field(ctx, n, batch, seed, power_dbm=3.0, dt=1 / 256e9):
    rng = np.random.default_rng(seed)
    p = 1e-3 * 10 ** (power_dbm / 10)
    x = (rng.standard_normal((batch, 1, n)) + 1j * rng.standard_normal((batch, 1, n))) * np.sqrt(p / 2)
    # a smooth band-limited field: keep the lowest quarter of the spectrum
    X = np.fft.fft(x, axis=-1)
    k = np.abs(np.fft.fftfreq(n)) > 0.125
    X[..., k] = 0
    x = np.fft.ifft(X, axis=-1) * 2.0
    return fg.Field(fg.Domain(1, n, dt, F0), data=x.astype(np.complex64), batch=batch, ctx=ctx)


def _fiber(length=80e3):
    return fg.Fiber(ALPHA, BETA2, GAMMA, length)


def _adaptive(fib, phase=0.01, step=2000.0):
    s = fg.SSFM(fib)
    s.set_grid(fg.SSFM.ADAPTIVE)
    s.set_maximum_phase_shift(phase)
    s.set_maximum_step_size(step)
    return s


def test_uniform_forward_matches_host_loop(ctx):
    fib = _fiber()
    a = _field(ctx, 1 << 12, 3, 1)
    b = a.copy()
    amp = fg.Amplifier(G, NF, seed=5)
    steps = fg.span_loop([a], fib, fg.SSFM(fib, 20), 3, after=fg.Amplifier.AMPLIFY, amplifier=amp, counter0=7)
    fg.forward_propagation(b, fib, fg.SSFM(fib, 20), amp, 3, counter0=7)
    np.testing.assert_array_equal(a.numpy(), b.numpy())
    np.testing.assert_array_equal(steps[0], [60, 60, 60])


def test_adaptive_forward_two_lengths_one_launch(ctx):
    fib = _fiber()
    fields = [_field(ctx, 1 << 12, 3, 2), _field(ctx, 1 << 14, 2, 3, power_dbm=6.0)]
    refs = [f.copy() for f in fields]
    ssfm = _adaptive(fib)
    amp = fg.Amplifier(G, NF, seed=11)
    n0 = fg.launch_count()
    steps = fg.span_loop(fields, fib, ssfm, 2, after=fg.Amplifier.AMPLIFY, amplifier=amp)
    assert fg.launch_count() > n0
    for i, (f, r) in enumerate(zip(fields, refs)):
        ref_steps = np.zeros(r.batch, np.int64)
        ai = fg.Amplifier(G, NF, seed=11 + i)
        for s in range(2):
            ref_steps += ssfm.run(r)
            ai.amplify(r, counter=s)
        np.testing.assert_array_equal(f.numpy(), r.numpy())
        np.testing.assert_array_equal(steps[i], ref_steps)
    # the higher-power field needs more steps
    assert steps[1].min() > steps[0].max()


def test_replay_with_new_seed(ctx):
    fib = _fiber()
    ssfm = _adaptive(fib)
    x = _field(ctx, 1 << 12, 2, 4)
    outs = []
    for seed in (21, 22):
        f = _field(ctx, 1 << 12, 2, 4)
        r = x.copy()
        fg.span_loop([f], fib, ssfm, 1, after=fg.Amplifier.AMPLIFY, amplifier=fg.Amplifier(G, NF, seed=seed))
        ssfm.run(r)
        fg.Amplifier(G, NF, seed=seed).amplify(r, counter=0)
        np.testing.assert_array_equal(f.numpy(), r.numpy())
        outs.append(f.numpy())
    assert not np.array_equal(outs[0], outs[1])


def test_backward_dbp_variants_in_one_launch(ctx):
    """DBP at 1/4/16 steps per span for one received field, one launch."""
    fib = _fiber()
    rx = _field(ctx, 1 << 13, 2, 5)
    fields = [rx.copy() for _ in range(3)]
    ks = [1, 4, 16]
    fg.span_loop(fields, fib, [fg.SSFM(fib, k) for k in ks], 2, direction=fg.SSFM.BACKWARD,
                 amplifier=fg.Amplifier(G), before=fg.Amplifier.DROP_POWER)
    for f, k in zip(fields, ks):
        r = rx.copy()
        fg.backward_propagation(r, fib, fg.SSFM(fib, k), G, 2)
        np.testing.assert_array_equal(f.numpy(), r.numpy())


def test_logarithmic_grid(ctx):
    fib = _fiber()
    s = fg.SSFM(fib)
    s.set_grid(fg.SSFM.LOGARITHMIC)
    s.set_maximum_phase_shift(0.005)
    s.set_maximum_step_size(1000.0)
    f = _field(ctx, 1 << 12, 2, 6)
    r = f.copy()
    steps = fg.span_loop([f], fib, s, 1)
    ref = s.run(r)
    np.testing.assert_array_equal(f.numpy(), r.numpy())
    np.testing.assert_array_equal(steps[0], ref)


def test_every_fft_split_matches_oracle(ctx, oracle_cpu):
    cpu = oracle_cpu
    n, dt = 1 << 14, 1 / 256e9
    fib = _fiber(10e3)
    x = _field(ctx, n, 1, 7, power_dbm=8.0).numpy()[0, 0]
    a, _ = cpu.ssfm_run(x.astype(np.complex128), dt, cpu.Fiber(ALPHA, BETA2, GAMMA, 10e3, 1.55e-6, 1.0),
                        cpu.UNIFORM, 10)
    for l1 in range(4, 11):
        fg.set_fft_split(n, l1, ctx=ctx)
        f = fg.Field(fg.Domain(1, n, dt, F0), data=x[None, None], ctx=ctx)
        fg.SSFM(fib, 10).run(f)
        assert rel_l2(f.numpy()[0, 0], a) < 2e-6, l1
    fg.set_fft_split(n, 0, ctx=ctx)
    l1, ms = fg.autotune(n, 8, ctx=ctx)
    assert (4 <= l1 <= 10 or l1 == fg.SPLIT_SINGLE_CTA) and ms > 0
    f = fg.Field(fg.Domain(1, n, dt, F0), data=x[None, None], ctx=ctx)
    fg.SSFM(fib, 10).run(f)
    assert rel_l2(f.numpy()[0, 0], a) < 2e-6
    fg.set_fft_split(n, 0, ctx=ctx)
    with pytest.raises(fg.FocssError):
        fg.set_fft_split(n, 3, ctx=ctx)

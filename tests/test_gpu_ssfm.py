"""GPU parity of the FFT, SSFM, CDC and amplifier paths (through the C ABI).

Tolerances: FP32 complex arithmetic against the FP64 reference/oracle; the
benchmark target is 1e-5 relative L2 field error, which these short runs
must meet.  Full-size cases are checked through size-independent properties
(closed forms, energy laws, forward/backward round trips).
"""
import numpy as np
import pytest

import focss_gb300 as fg
from conftest import ALPHA, BETA2, F0, GAMMA, rel_l2

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-5


def make_field(x, dt, f0=0.0, ctx=None):
    x = np.asarray(x)
    if x.ndim == 1:
        x = x[None, None, :]
    elif x.ndim == 2:
        x = x[:, None, :]
    b, m, n = x.shape
    return fg.Field(fg.Domain(m, n, dt, f0), data=x, batch=b, ctx=ctx)


@pytest.mark.parametrize("lg", [8, 9, 10, 12, 15, 16, 17, 19, 20])
def test_fft_matches_numpy(ctx, lg):
    n = 1 << lg
    rng = np.random.default_rng(lg)
    x = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
    f = make_field(x, 1.0, ctx=ctx)
    f.fft_inplace()
    want = np.fft.fft(x, axis=-1) / n
    assert rel_l2(f.numpy()[:, 0], want) < 1e-6
    f.ifft_inplace()
    assert rel_l2(f.numpy()[:, 0], x) < 1e-6


def test_fft_rejects_unsupported_length(ctx):
    f = fg.Field(fg.Domain(1, 3000, 1.0), batch=1, ctx=ctx)
    with pytest.raises(fg.FocssError) as e:
        f.fft_inplace()
    assert e.value.status == 6


def test_field_rejects_too_many_rows(ctx):
    """Realization rows (batch x modes) map to a grid dimension: at most 65535."""
    with pytest.raises(fg.FocssError) as e:
        fg.Field(fg.Domain(2, 256, 1.0), batch=40000, ctx=ctx)
    assert e.value.status == 1
    fg.Field(fg.Domain(1, 256, 1.0), batch=65535, ctx=ctx)


def test_ssfm_uniform_matches_reference(ctx, golden):
    dt = float(golden["dt"][0])
    span = fg.Fiber(*golden["ssfm_span"])
    f = make_field(golden["shaped_01"], dt, ctx=ctx)
    s = fg.SSFM(span, 20)
    steps = s.run(f, fg.SSFM.FORWARD)
    assert steps[0] == 20
    assert rel_l2(f.numpy()[0, 0], golden["ssfm_uniform"]) < FIELD_TOL
    s.run(f, fg.SSFM.BACKWARD)
    assert rel_l2(f.numpy()[0, 0], golden["ssfm_uniform_bwd"]) < FIELD_TOL


@pytest.mark.parametrize("grid,key", [(fg.SSFM.ADAPTIVE, "ssfm_adaptive"), (fg.SSFM.LOGARITHMIC, "ssfm_log")])
def test_ssfm_adaptive_and_log_match_reference(ctx, golden, oracle_cpu, grid, key):
    dt = float(golden["dt"][0])
    span = fg.Fiber(*golden["ssfm_span"])
    x = golden["shaped_01"]
    f = make_field(x, dt, ctx=ctx)
    s = fg.SSFM(span)
    s.set_grid(grid)
    s.set_maximum_phase_shift(0.005)
    s.set_maximum_step_size(1000.0)
    steps = s.run(f)
    _, want_steps = oracle_cpu.ssfm_run(x, dt, oracle_cpu.Fiber(*golden["ssfm_span"]), grid, 1, 0.005, 1000.0)
    assert steps[0] == want_steps
    assert rel_l2(f.numpy()[0, 0], golden[key]) < FIELD_TOL


def test_cdc_matches_reference(ctx, golden):
    dt = float(golden["dt"][0])
    span = fg.Fiber(*golden["ssfm_span"])
    f = make_field(golden["cdc_in"], dt, ctx=ctx)
    fg.cd_compensation(f, span, 10)
    assert rel_l2(f.numpy()[0, 0], golden["cdc_out"]) < FIELD_TOL


def test_batched_realizations_are_independent(ctx, oracle_cpu):
    """Realizations with different powers run in one launch and take different
    adaptive step counts; each must match its own oracle run."""
    rng = np.random.default_rng(7)
    n, dt = 4096, 1 / 256e9
    base = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    powers = np.array([0.2, 1.0, 3.0, 0.05]) * 1e-3
    x = np.stack([base * np.sqrt(p / 2) for p in powers])
    f = make_field(x, dt, ctx=ctx)
    fib = fg.Fiber(ALPHA, BETA2, GAMMA, 10e3)
    s = fg.SSFM(fib)
    s.set_grid(fg.SSFM.ADAPTIVE)
    s.set_maximum_phase_shift(0.005)
    s.set_maximum_step_size(1000.0)
    steps = s.run(f)
    got = f.numpy()[:, 0]
    ofib = oracle_cpu.Fiber(ALPHA, BETA2, GAMMA, 10e3, 1.55e-6, 1.0)
    for b in range(len(powers)):
        want, ws = oracle_cpu.ssfm_run(x[b], dt, ofib, oracle_cpu.ADAPTIVE, 1, 0.005, 1000.0)
        assert steps[b] == ws
        assert rel_l2(got[b], want) < FIELD_TOL
    assert len(set(steps.tolist())) > 1


def test_amplifier_gain_ops(ctx, golden):
    dt = float(golden["dt"][0])
    G = float(golden["amp_gain"][0])
    x = golden["shaped_01"]
    for op, key in (("amplify", "amp_out"), ("drop_power", "drop_out"), ("give_power", "give_out")):
        f = make_field(x, dt, F0, ctx=ctx)
        getattr(fg.Amplifier(G), op)(f)
        assert rel_l2(f.numpy()[0, 0], golden[key]) < 1e-6


def test_amplifier_noise_matches_oracle_stream(ctx, oracle_cpu):
    n, dt = 1 << 14, 1 / 256e9
    rng = np.random.default_rng(3)
    x = np.stack([(rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 1e-2 for _ in range(3)])
    G, NF = 10 ** 1.6, 10 ** 0.5
    f = make_field(x, dt, F0, ctx=ctx)
    fg.Amplifier(G, NF, seed=1234).amplify(f, counter=7)
    got = f.numpy()[:, 0]
    for b in range(3):
        want = oracle_cpu.amplify(x[b], dt, F0, G, NF, seed=1234, counter=7, realization=b)
        assert rel_l2(got[b], want) < 1e-5
    var = fg.PLANCK * F0 * NF * (G - 1) / 2 / dt / 2
    noise = got - x * np.sqrt(G)
    assert abs(np.var(noise.real) / var - 1) < 0.05


def test_bright_soliton_kat(ctx, oracle_cpu):
    """beta2 = -1, gamma = 1, P = 1: A(z, t) = sech(t) exp(i z / 2)
    (tasks/verification.cpp:10-22 form).  GPU error against the analytic
    solution must equal the FP64 oracle's own splitting error."""
    n, T = 4096, 60.0
    dt = T / n
    t = (np.arange(n) - n // 2) * dt
    a0 = 1 / np.cosh(t)
    fib = fg.Fiber(0.0, -1.0, 1.0, 2.0)
    f = make_field(a0.astype(complex), dt, ctx=ctx)
    fg.SSFM(fib, 200).run(f)
    exact = a0 * np.exp(0.5j * 2.0)
    want, _ = oracle_cpu.ssfm_run(a0.astype(complex), dt, oracle_cpu.Fiber(0, -1, 1, 2, 0, 1), 0, 200)
    got = f.numpy()[0, 0]
    assert rel_l2(got, want) < FIELD_TOL
    assert rel_l2(got, exact) < 1e-4


@pytest.mark.parametrize("lg", [19, 20])
def test_dispersion_only_closed_form_full_size(ctx, lg):
    """Linear propagation at N = 2^19 (the WDM configuration's length) and at
    the largest supported length 2^20: A_hat(L) = A_hat(0) exp(i beta2/2 L w^2)
    exactly (ssfm.cpp:142-150 sign)."""
    n = 1 << lg
    dt = 1 / 512e9
    rng = np.random.default_rng(lg)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 0.01
    L = 80e3
    f = make_field(x, dt, ctx=ctx)
    fg.SSFM(fg.Fiber(0.0, BETA2, 0.0, L), 3).run(f)
    w = 2 * np.pi * np.fft.fftfreq(n, dt)
    want = np.fft.ifft(np.fft.fft(x) * np.exp(0.5j * BETA2 * L * w ** 2))
    assert rel_l2(f.numpy()[0, 0], want) < FIELD_TOL


def test_kerr_only_and_loss_only(ctx):
    n = 1 << 16
    dt = 1 / 256e9
    rng = np.random.default_rng(2)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 0.05
    L = 50e3
    f = make_field(x, dt, ctx=ctx)
    fg.SSFM(fg.Fiber(0.0, 0.0, GAMMA, L), 10).run(f)
    want = x * np.exp(1j * GAMMA * L * np.abs(x) ** 2)
    assert rel_l2(f.numpy()[0, 0], want) < FIELD_TOL
    f = make_field(x, dt, ctx=ctx)
    fg.SSFM(fg.Fiber(ALPHA, 0.0, 0.0, L), 10).run(f)
    assert rel_l2(f.numpy()[0, 0], x * np.exp(-0.5 * ALPHA * L)) < FIELD_TOL


def test_forward_then_dbp_round_trip_full_size(ctx):
    """Noise-free link then DBP with the same fiber and steps returns the input
    (a size-independent property of the split-step pair), N = 2^17, batch 4."""
    n, dt = 1 << 17, 1 / 256e9
    rng = np.random.default_rng(17)
    x = (rng.standard_normal((4, n)) + 1j * rng.standard_normal((4, n))) * np.sqrt(1e-3 / 2)
    fib = fg.Fiber(ALPHA, BETA2, GAMMA, 80e3)
    G = fg.db_to_linear(0.2 * 80)
    f = make_field(x, dt, F0, ctx=ctx)
    s = fg.SSFM(fib, 80)
    fg.forward_propagation(f, fib, s, fg.Amplifier(G), spans=3)
    fg.backward_propagation(f, fib, s, G, spans=3)
    assert rel_l2(f.numpy()[:, 0], x) < 2e-5


@pytest.mark.parametrize("single_cta", [False, True])
def test_zero_and_mixed_power_realizations(ctx, oracle_cpu, single_cta):
    """A realization with no power takes the step bound (peak 0 => the
    maximum step: 80 steps of 1 km for 80 km) and stays zero, next to a
    powered one in the same batch that follows the FP64 oracle
    (ssfm.cpp:136-140; both passes and the single-CTA kernel)."""
    n, dt = 1 << 12, 1 / 256e9
    rng = np.random.default_rng(12)
    x = np.zeros((2, 1, n), np.complex128)
    x[1, 0] = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 0.03
    x = x.astype(np.complex64).astype(np.complex128)
    f = fg.Field(fg.Domain(1, n, dt, 193.1e12), data=x, batch=2, ctx=ctx)
    s = fg.SSFM(fg.Fiber(ALPHA, BETA2, GAMMA, 80e3))
    s.set_grid(fg.SSFM.ADAPTIVE)
    s.set_maximum_phase_shift(0.005)
    s.set_maximum_step_size(1000.0)
    if single_cta:
        fg.set_fft_split(n, fg.SPLIT_SINGLE_CTA, ctx=ctx)
    try:
        steps = s.run(f)
    finally:
        fg.set_fft_split(n, 0, ctx=ctx)
    out = f.numpy()
    assert int(steps[0]) == 80 and np.all(out[0] == 0)
    want, wsteps = oracle_cpu.ssfm_run(x[1, 0], dt, oracle_cpu.Fiber(ALPHA, BETA2, GAMMA, 80e3, 1.55e-6, 1.0),
                                       oracle_cpu.ADAPTIVE, 1, 0.005, 1000.0)
    assert int(steps[1]) == wsteps and wsteps > 80
    assert rel_l2(out[1, 0], want) < 1e-5

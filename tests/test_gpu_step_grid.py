"""Step-grid record and replay on the GPU, and the FP32 split step against
FP64 on one grid at the precision-study configuration's own size.

An ADAPTIVE grid (src/focss/solver/ssfm.cpp:92-118) takes each step size from
the current field's peak power (:136-140), so an FP32 run and an FP64 run walk
slightly different grids and their fields part by the split-step solution's
own sensitivity to its grid.  Recording the GPU run's step sizes
(focss_ssfm_run_record) and replaying them in FP64 puts both on one grid, so
the field difference measures arithmetic error only.

The full-size case is the 5-channel WDM precision study: 5 x 2^15 16QAM
symbols at 32 GBaud on a 50 GHz grid, 16 samples/symbol of the total band
(N = 2^19), 20 x 80 km SSMF, ADAPTIVE 0.005 rad / 1 km, lossless noise-free
EDFAs, at -2 and +4 dBm per channel (about 5 000 and 19 000 split steps).
The FP64 side is a complex128 restatement on the GPU (tests/fp64_ssfm.py),
pinned here against the C oracle at small sizes.

Error model (the tolerance): every split step rounds the field to FP32 in two
passes of FFT butterflies, about 2.2e-7 relative per step, and these
data-dependent roundings add like a random walk, so after K steps the field
error is about 2.2e-7 sqrt(K); the test allows 3e-7 sqrt(K) and checks the
growth along the link is a random walk's (no rounding that repeats from step
to step, which would grow linearly or faster).  FP64 runs perturbed once by
3e-8 stay within 3.3e-8 over the whole link, so the link itself does not
amplify these errors.
"""
import math

import numpy as np
import pytest

import focss_gb300 as fg
from focss_gb300 import dsp, links
from conftest import ALPHA, BETA2, GAMMA, rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _adaptive(fib):
    s = fg.SSFM(fib)
    s.set_grid(fg.SSFM.ADAPTIVE)
    s.set_maximum_phase_shift(0.005)
    s.set_maximum_step_size(1000.0)
    return s


def _signal(batch, n, seed, p_mw):
    rng = np.random.default_rng(seed)
    p = np.asarray(p_mw, float)[:, None] * 1e-3
    return (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))) * np.sqrt(p / 2)


@pytest.mark.parametrize("single_cta", [False, True])
def test_replay_of_recorded_grid_is_bit_identical(ctx, single_cta):
    n, dt = 1 << 13, 1 / 256e9
    fib = fg.Fiber(ALPHA, BETA2, GAMMA, 40e3)
    x = _signal(3, n, 11, [1.0, 4.0, 9.0])
    if single_cta:
        fg.set_fft_split(n, fg.SPLIT_SINGLE_CTA, ctx=ctx)
    try:
        ssfm = _adaptive(fib)
        f = fg.Field(fg.Domain(1, n, dt), data=x[:, None, :], batch=3, ctx=ctx)
        want_steps = ssfm.run(f)
        g = fg.Field(fg.Domain(1, n, dt), data=x[:, None, :], batch=3, ctx=ctx)
        steps, h = ssfm.run_recorded(g)
        assert np.array_equal(steps, want_steps) and [len(v) for v in h] == list(steps)
        assert np.array_equal(g.numpy(), f.numpy())
        for v in h:
            assert abs(v.sum() - 40e3) < 1e-6 and np.all(v > 0) and v.max() <= 1000.0
        r = fg.Field(fg.Domain(1, n, dt), data=x[:, None, :], batch=3, ctx=ctx)
        assert np.array_equal(ssfm.run_steps(r, h), steps)
        assert np.array_equal(r.numpy(), f.numpy())
    finally:
        fg.set_fft_split(n, 0, ctx=ctx)


def test_record_capacity_and_replay_arguments(ctx):
    n, dt = 1 << 10, 1 / 64e9
    fib = fg.Fiber(ALPHA, BETA2, GAMMA, 10e3)
    f = fg.Field(fg.Domain(1, n, dt), data=_signal(1, n, 1, [4.0])[:, None, :], ctx=ctx)
    with pytest.raises(fg.FocssError) as e:
        fg.SSFM(fib, 20).run_recorded(f, capacity=10)
    assert e.value.status == 1
    with pytest.raises(fg.FocssError):
        fg.SSFM(fib).run_steps(f, [np.array([5e3, -1.0])])
    steps, h = fg.SSFM(fib, 20).run_recorded(f, capacity=20)
    assert steps[0] == 20 and np.allclose(h[0], 500.0)


def test_fp64_restatement_matches_oracle(ctx, oracle_cpu):
    import fp64_ssfm as f64
    cpu = oracle_cpu
    ofib = cpu.Fiber(ALPHA, BETA2, GAMMA, 30e3, 1.55e-6, 1.0)
    x = _signal(1, 4096, 5, [12.0])[0]
    for d in (1.0, -1.0):
        want, steps, h = cpu.ssfm_run_recorded(x, 1 / 128e9, ofib, cpu.ADAPTIVE, 1, 0.005, 1000.0, d)
        xt = torch.from_numpy(x[None]).cuda()
        got = f64.run_steps(xt, 1 / 128e9, ofib, h, d).cpu().numpy()[0]
        free, taken = f64.run_adaptive(xt, 1 / 128e9, ofib, 0.005, 1000.0, d)
        # cuFFT and the oracle's FFT round differently: ~1e-15 per transform
        assert rel_l2(got, want) < 1e-10
        assert len(taken) == steps and np.max(np.abs(np.array(taken) - h)) < 1e-6
        assert rel_l2(free.cpu().numpy()[0], want) < 1e-10


def test_gpu_replay_against_oracle_small(ctx, oracle_cpu):
    """The GPU's recorded grid replayed by the C oracle (WDM, N = 2^13, 4 spans)."""
    cpu = oracle_cpu
    link = links.Link()
    field, _ = links.wdm_transmitter(link, 512, 1, 4.0, seed=3, ctx=ctx)
    dt = field.domain.time_step
    x = field.numpy()[0, 0]
    fib = link.fiber()
    ofib = cpu.Fiber(ALPHA, BETA2, GAMMA, 80e3, 1.55e-6, 1.0)
    g = link.gain()
    for _ in range(4):
        steps, h = _adaptive(fib).run_recorded(field)
        fg.Amplifier(g).amplify(field)
        x = cpu.amplify(cpu.ssfm_run_steps(x, dt, ofib, h[0]), dt, 0.0, g)
    assert rel_l2(field.numpy()[0, 0], x) < 1e-5


def _propagate_full(ctx, power_dbm, spans, f64):
    link = links.Link()
    fib = link.fiber()
    field, tx = links.wdm_transmitter(link, 1 << 15, 1, power_dbm, seed=7, ctx=ctx)
    dt = field.domain.time_step
    rep = torch.from_numpy(field.numpy()[0]).cuda()  # the FP32 launch field, exactly
    free = rep.clone()
    g = link.gain()
    amp = math.sqrt(g)
    ssfm = _adaptive(fib)
    gpu_steps, free_steps, errs = [], [], []
    for _ in range(spans):
        steps, h = ssfm.run_recorded(field, capacity=1 << 17)
        gpu_steps.append(int(steps[0]))
        fg.Amplifier(g).amplify(field)
        # FP64 on the GPU's grid, and FP64 free-running
        rep = f64.run_steps(rep, dt, fib, h[0]) * amp
        free, taken = f64.run_adaptive(free, dt, fib, link.max_phase, link.max_step)
        free = free * amp
        free_steps.append(len(taken))
        errs.append(rel_l2(field.numpy()[0, 0], rep.cpu().numpy()[0]))
    return link, field, tx, rep.cpu().numpy()[0], free.cpu().numpy()[0], gpu_steps, free_steps, errs


def _centre_q(cpu, link, tx, fib, dt, y, spans):
    ofib = cpu.Fiber(fib.alpha, fib.beta2, fib.gamma, fib.length, 1.55e-6, 1.0)
    a = cpu.wdm_select(cpu.cd_compensation(y, dt, ofib, spans), dt, 0, link.spacing)
    r = cpu.rrc_sampling(a, link.osf, link.roll_off)
    r = cpu.rotate(r, cpu.pse_estimate(tx, r, 720))
    return cpu.q2(tx, r, 100)


ROUNDING_WALK = 3e-7  # field error allowed per sqrt(split step)


@pytest.mark.parametrize("power_dbm", [-2.0, 4.0])
def test_wdm_precision_study_full_size(ctx, oracle_cpu, power_dbm):
    import fp64_ssfm as f64
    spans = 20
    link, field, tx, want, free, gpu_steps, free_steps, errs = _propagate_full(ctx, power_dbm, spans, f64)
    got = field.numpy()[0, 0]
    err = rel_l2(got, want)
    k = np.cumsum(gpu_steps)
    dt = field.domain.time_step
    fib = link.fiber()
    t = tx.numpy()[0, 0]
    q_gpu = _centre_q(oracle_cpu, link, t, fib, dt, got, spans)
    q_64 = _centre_q(oracle_cpu, link, t, fib, dt, want, spans)
    d_steps = [a - b for a, b in zip(gpu_steps, free_steps)]
    print("\nWDM N=2^19 %+.0f dBm/ch: %d steps, field rel L2 %.3e on the GPU grid (%.2e per sqrt(step)), "
          "Q %.4f vs %.4f dB, free-running FP64 step-count deltas per span %s, free-running field gap %.3e"
          % (power_dbm, k[-1], err, err / math.sqrt(k[-1]), q_gpu, q_64, d_steps, rel_l2(got, free)))
    assert max(abs(d) for d in d_steps) <= 1
    assert abs(q_gpu - q_64) < 0.05
    assert err < ROUNDING_WALK * math.sqrt(k[-1])
    # random-walk growth from span 5 to span 20: no repeated (systematic) rounding
    assert errs[-1] / errs[4] < 1.25 * math.sqrt(k[-1] / k[4])

"""FP32 split steps against the FP64 oracle over whole links (noise off).

Single channel: 16QAM, 32 GBaud, RRC 0.1, 4 samples/symbol, 20 x 80 km SSMF,
ADAPTIVE 0.005 rad / 1 km (about 2200 steps), lossless EDFAs; then CDC,
matched filter, phase-shift equalizer.  The field must stay within 1e-5
relative L2 of the FP64 run with the same step counts, and Q within 0.05 dB.

5-channel WDM (the precision-study link with 2^9 symbols per channel,
N = 2^13), UNIFORM (100 steps per span) and ADAPTIVE.  On the ADAPTIVE grid
every step size comes from the field's peak power, so the GPU records its
grid (focss_ssfm_run_record) and the oracle replays it (ofc_ssfm_run_steps):
both then walk one grid.  The field must stay within the FP32 rounding walk
3e-7 sqrt(K) after K split steps (see test_gpu_step_grid.py), step counts
must agree with a free-running FP64 run, and the centre channel's Q within
0.05 dB.
"""
import numpy as np
import pytest

import focss_gb300 as fg
from focss_gb300 import dsp, links
from conftest import ALPHA, BETA2, F0, GAMMA, rel_l2

pytestmark = pytest.mark.gpu

G = 10 ** 1.6


def _oracle_link(cpu, x, dt, grid, k, spans):
    ofib = cpu.Fiber(ALPHA, BETA2, GAMMA, 80e3, 1.55e-6, 1.0)
    a, steps = x.copy(), 0
    for _ in range(spans):
        a, st = cpu.ssfm_run(a, dt, ofib, grid, k, 0.005, 1000.0)
        steps += st
        a = cpu.amplify(a, dt, F0, G)
    return a, steps


def _gpu_link(field, ssfm, spans):
    steps = 0
    for _ in range(spans):
        steps += int(ssfm.run(field)[0])
        fg.Amplifier(G).amplify(field)
    return steps


def _adaptive(fib):
    s = fg.SSFM(fib)
    s.set_grid(fg.SSFM.ADAPTIVE)
    s.set_maximum_phase_shift(0.005)
    s.set_maximum_step_size(1000.0)
    return s


def test_single_channel_adaptive_link(ctx, oracle_cpu):
    cpu = oracle_cpu
    ns, osf, spans = 1024, 4, 20
    rng = np.random.default_rng(1)
    sym = dsp.qam16_map(rng.integers(0, 16, (1, 1, ns)), fg.Domain(1, ns, 1 / 32e9, F0), ctx=ctx)
    sym *= np.sqrt(fg.dbm_to_watts(2.0))
    sig = dsp.rrc_shaping(sym, osf, 0.1)
    dt = sig.domain.time_step
    x0 = sig.numpy()[0, 0]
    fib = fg.Fiber(ALPHA, BETA2, GAMMA, 80e3)
    steps = _gpu_link(sig, _adaptive(fib), spans)
    want, wsteps = _oracle_link(cpu, x0, dt, cpu.ADAPTIVE, 1, spans)
    assert steps == wsteps and steps > 2000
    assert rel_l2(sig.numpy()[0, 0], want) < 1e-5
    fg.cd_compensation(sig, fib, spans)
    r = dsp.PhaseShiftEqualizer(3600).train_equalize(sym, dsp.rrc_sampling(sig, osf, 0.1))
    q_gpu = dsp.q2_factor(sym, r, 100)[0]
    ofib = cpu.Fiber(ALPHA, BETA2, GAMMA, 80e3, 1.55e-6, 1.0)
    tx = sym.numpy()[0, 0]
    ro = cpu.rrc_sampling(cpu.cd_compensation(want, dt, ofib, spans), osf, 0.1)
    ro = cpu.rotate(ro, cpu.pse_estimate(tx, ro, 3600))
    assert abs(q_gpu - cpu.q2(tx, ro, 100)) < 0.05


@pytest.mark.parametrize("grid", ["uniform", "adaptive"])
def test_wdm_link(ctx, oracle_cpu, grid):
    cpu = oracle_cpu
    link = links.Link()
    spans = 20
    field, tx = links.wdm_transmitter(link, 512, 1, 0.0, seed=5, ctx=ctx)
    dt = field.domain.time_step
    x0 = field.numpy()[0, 0]
    fib = link.fiber()
    ofib = cpu.Fiber(ALPHA, BETA2, GAMMA, 80e3, 1.55e-6, 1.0)
    if grid == "uniform":
        steps = _gpu_link(field, fg.SSFM(fib, 100), spans)
        want, wsteps = _oracle_link(cpu, x0, dt, cpu.UNIFORM, 100, spans)
        assert steps == wsteps
    else:
        ssfm, want, steps = _adaptive(fib), x0.copy(), 0
        for _ in range(spans):
            st, h = ssfm.run_recorded(field)
            fg.Amplifier(G).amplify(field)
            want = cpu.amplify(cpu.ssfm_run_steps(want, dt, ofib, h[0]), dt, F0, G)
            steps += int(st[0])
        _, free_steps = _oracle_link(cpu, x0, dt, cpu.ADAPTIVE, 1, spans)
        assert abs(steps - free_steps) <= spans
    assert rel_l2(field.numpy()[0, 0], want) < 3e-7 * np.sqrt(steps)
    fg.cd_compensation(field, fib, spans)
    r = dsp.rrc_sampling(dsp.wdm_select(field, 0, link.spacing), link.osf, link.roll_off)
    r = dsp.PhaseShiftEqualizer(720).train_equalize(tx, r)
    q_gpu = dsp.q2_factor(tx, r, 100)[0]
    t = tx.numpy()[0, 0]
    ao = cpu.wdm_select(cpu.cd_compensation(want, dt, ofib, spans), dt, 0, link.spacing)
    ro = cpu.rrc_sampling(ao, link.osf, link.roll_off)
    ro = cpu.rotate(ro, cpu.pse_estimate(t, ro, 720))
    assert abs(q_gpu - cpu.q2(t, ro, 100)) < 0.05

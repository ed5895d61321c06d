"""FP32 against FP64 on the precision-study WDM link with ASE on, over 8 seeds.

5-channel WDM (16QAM, 32 GBaud, 50 GHz grid, RRC 0.1, 16 samples/symbol of
the total band), 2^9 symbols per channel (N = 2^13), 20 x 80 km SSMF,
ADAPTIVE 0.005 rad / 1 km, an EDFA of 16 dB gain and 5 dB noise figure after
every span (src/focss/module/amplifier.cpp:15-42, src/tasks/systems.cpp:39-56),
8 realizations with independent ASE, at -2 and +4 dBm per channel.

The reference seeds its ASE from std::random_device (non-reproducible); here
both sides draw the same counter-based stream (Philox4x32-10 keyed by the
seed, the span counter and the realization), the GPU in FP32 and the oracle
in FP64, and the oracle replays the GPU's recorded step grid, so every seed
is compared realization for realization.  The centre channel's Q (CDC,
channel select, matched filter, 720-angle phase search, cut 100) must agree
within 0.05 dB per seed and within 0.01 dB on the mean over the seeds; the
fields within the FP32 rounding walk of test_gpu_step_grid.py.
"""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import focss_gb300 as fg
from focss_gb300 import dsp, links
from conftest import ALPHA, BETA2, GAMMA, rel_l2

pytestmark = pytest.mark.gpu

SEEDS = 8
ASE_SEED = 77
ROUNDING_WALK = 3e-7  # field error allowed per sqrt(split step)


@pytest.mark.parametrize("power_dbm", [-2.0, 4.0])
def test_wdm_q_with_ase_over_seeds(ctx, oracle_cpu, power_dbm):
    cpu = oracle_cpu
    link = links.Link()
    field, tx = links.wdm_transmitter(link, 512, SEEDS, power_dbm, seed=21, ctx=ctx)
    dt, f0 = field.domain.time_step, field.domain.center_frequency
    x0 = field.numpy()[:, 0]
    fib = link.fiber()
    ssfm = fg.SSFM(fib)
    ssfm.set_grid(fg.SSFM.ADAPTIVE)
    ssfm.set_maximum_phase_shift(link.max_phase)
    ssfm.set_maximum_step_size(link.max_step)
    gain, nf = link.gain(), fg.db_to_linear(link.noise_figure_db)
    amp = fg.Amplifier(gain, nf, seed=ASE_SEED)
    grids = [[] for _ in range(SEEDS)]
    steps = np.zeros(SEEDS, int)
    for span in range(link.spans):
        st, h = ssfm.run_recorded(field)
        amp.amplify(field, counter=span)
        steps += st
        for b in range(SEEDS):
            grids[b].append(h[b])
    got = field.numpy()[:, 0]

    ofib = cpu.Fiber(ALPHA, BETA2, GAMMA, link.span_m, link.wavelength, 1.0)

    def oracle_run(b):
        a = x0[b].copy()
        for span in range(link.spans):
            a = cpu.ssfm_run_steps(a, dt, ofib, grids[b][span])
            a = cpu.amplify(a, dt, f0, gain, nf, ASE_SEED, span, b)
        return a

    with ThreadPoolExecutor(SEEDS) as ex:  # the oracle's foreign calls release the GIL
        want = list(ex.map(oracle_run, range(SEEDS)))
    for b in range(SEEDS):
        assert rel_l2(got[b], want[b]) < ROUNDING_WALK * np.sqrt(steps[b])

    fg.cd_compensation(field, fib, link.spans)
    r = dsp.rrc_sampling(dsp.wdm_select(field, 0, link.spacing), link.osf, link.roll_off)
    r = dsp.PhaseShiftEqualizer(720).train_equalize(tx, r)
    q_gpu = np.asarray(dsp.q2_factor(tx, r, 100), float)
    t = tx.numpy()[:, 0]
    q_64 = np.empty(SEEDS)
    for b in range(SEEDS):
        ao = cpu.wdm_select(cpu.cd_compensation(want[b], dt, ofib, link.spans), dt, 0, link.spacing)
        ro = cpu.rrc_sampling(ao, link.osf, link.roll_off)
        ro = cpu.rotate(ro, cpu.pse_estimate(t[b], ro, 720))
        q_64[b] = cpu.q2(t[b], ro, 100)
    d = q_gpu - q_64
    print("\nWDM N=2^13 %+.0f dBm/ch with ASE, %d seeds: Q %.3f +- %.3f dB (FP32) vs %.3f (FP64), "
          "max |dQ| %.2e dB, mean dQ %.2e dB, steps %d..%d"
          % (power_dbm, SEEDS, q_gpu.mean(), q_gpu.std(), q_64.mean(), np.abs(d).max(), d.mean(),
             steps.min(), steps.max()))
    assert np.abs(d).max() < 0.05
    assert abs(d.mean()) < 0.01

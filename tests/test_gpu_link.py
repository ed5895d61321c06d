"""End-to-end chains on the GPU.

Single channel (the single-channel configuration's chain, at 2^11 symbols
and at its own 2^14): 16QAM -> RRC 0.1 at 8 sps -> 10 x 80 km
SSMF at 1 km uniform steps with lossless EDFAs (noise off) -> CDC -> matched
filter -> phase-shift equalizer -> Q and BER, against the same chain in the
FP64 oracle: field within 1e-5 relative L2, Q within 0.05 dB, decisions equal.

Learned DBP (the WDM learned-DBP configuration reduced to 3 spans): trained
on GPU-generated fields, it must beat its split-step initialisation and run
in far less GPU time than many-step DBP.
"""
import numpy as np
import pytest

import focss_gb300 as fg
from focss_gb300 import dsp, links
from conftest import ALPHA, BETA2, F0, GAMMA, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("log2_symbols", [11, 14])
def test_single_channel_chain_matches_oracle(ctx, oracle_cpu, log2_symbols):
    """2^11 symbols, and the configuration's own 2^14 (N = 2^17; the FP64
    oracle takes a few seconds for its 800 steps)."""
    cpu = oracle_cpu
    rng = np.random.default_rng(1)
    ns, osf, spans = 1 << log2_symbols, 8, 10
    dt = 1 / (32e9 * osf)
    p = fg.dbm_to_watts(2.0)
    codes = rng.integers(0, 16, ns)
    fib = fg.Fiber(ALPHA, BETA2, GAMMA, 80e3)
    G = fg.db_to_linear(0.2 * 80)
    # GPU chain
    sym = dsp.qam16_map(codes[None, None], fg.Domain(1, ns, 1 / 32e9), ctx=ctx)
    sym *= np.sqrt(p)
    sig = dsp.rrc_shaping(sym, osf, 0.1)
    x0 = sig.numpy()[0, 0]
    fg.forward_propagation(sig, fib, fg.SSFM(fib, 80), fg.Amplifier(G), spans)
    after = sig.numpy()[0, 0]
    fg.cd_compensation(sig, fib, spans)
    rx = dsp.rrc_sampling(sig, osf, 0.1)
    rx = dsp.PhaseShiftEqualizer(3600).train_equalize(sym, rx)
    q_gpu = dsp.q2_factor(sym, rx, 100)[0]
    ber_gpu = dsp.bit_error_rate_16qam(sym, rx, 100)[0]
    codes_gpu = dsp.hd_sequence_16qam(rx)[0, 0]
    # FP64 oracle chain on the same transmitted field
    ofib = cpu.Fiber(ALPHA, BETA2, GAMMA, 80e3, 1.55e-6, 1.0)
    a = x0
    for _ in range(spans):
        a, _ = cpu.ssfm_run(a, dt, ofib, cpu.UNIFORM, 80)
        a = cpu.amplify(a, dt, F0, G)
    assert rel_l2(after, a) < 1e-5
    a = cpu.cd_compensation(a, dt, ofib, spans)
    r = cpu.rrc_sampling(a, osf, 0.1)
    tx = sym.numpy()[0, 0]
    r = cpu.rotate(r, cpu.pse_estimate(tx, r, 3600))
    assert abs(q_gpu - cpu.q2(tx, r, 100)) < 0.05
    assert ber_gpu == cpu.bit_error_rate(tx, r, 100)
    np.testing.assert_array_equal(codes_gpu, cpu.hd_sequence(r))


def test_learned_dbp_on_wdm_link(ctx):
    link = links.Link(spans=3)
    ns, B = 1 << 13, 8
    tx_train_f, tx_train = links.wdm_transmitter(link, ns, B, 3.0, seed=11, ctx=ctx)
    tx_test_f, tx_test = links.wdm_transmitter(link, ns, B, 3.0, seed=12, ctx=ctx)
    links.propagate(link, tx_train_f, seed=1)
    links.propagate(link, tx_test_f, seed=2)
    rx_train = links.centre_channel(link, tx_train_f)
    rx_test = links.centre_channel(link, tx_test_f)
    q2_plain, ms2 = links.plain_dbp_q(link, rx_test, tx_test, 2)
    q50, ms50 = links.plain_dbp_q(link, rx_test, tx_test, 50)
    # 40 km steps at 2 samples/symbol need ~63 taps (31 taps alone cap Q near 20 dB)
    r = links.learned_dbp(link, rx_train, tx_train, rx_test, tx_test, steps_per_span=2, taps=63, mf_taps=63,
                          iters=200, lr=3e-4, cnn_iters=100)
    # the split-step initialisation reproduces plain 2-step DBP
    assert abs(np.mean(r["q_init"]) - np.mean(q2_plain)) < 0.5
    assert r["loss_last"] < r["loss_first"]
    assert np.mean(r["q_learned"]) > np.mean(r["q_init"]) - 0.1
    assert np.mean(q50) > np.mean(q2_plain) - 0.05
    assert r["ms_learned"] < ms50 / 5

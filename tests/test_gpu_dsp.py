"""GPU parity of the TX/RX DSP chain (through the C ABI) against the reference's
golden vectors and the FP64 oracle.

Decisions, bit/symbol error counts and the phase-search index are integer
results and must be bit-exact on identical (FP32-representable) inputs; field
outputs are FP32 and must match to 1e-6 relative L2.
"""
import numpy as np
import pytest

import focss_gb300 as fg
from focss_gb300 import dsp
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-6


def fld(x, dt=1.0, ctx=None):
    x = np.asarray(x)
    if x.ndim == 1:
        x = x[None, None, :]
    elif x.ndim == 2:
        x = x[:, None, :]
    b, m, n = x.shape
    return fg.Field(fg.Domain(m, n, dt), data=x, batch=b, ctx=ctx)


def f32(x):
    return np.asarray(x).astype(np.complex64).astype(np.complex128)


def test_qam_map_and_rrc_pulse(ctx, golden):
    codes = golden["qam_codes"]
    s = dsp.qam16_map(codes, fg.Domain(1, codes.size, 1.0), ctx=ctx)
    assert rel_l2(s.numpy()[0, 0], golden["qam_symbols"]) < 1e-7
    assert rel_l2(dsp.rrc_pulse(512, 8, 0.1, ctx=ctx), golden["rrc_pulse_01"]) < 1e-13
    assert rel_l2(dsp.rrc_pulse(512, 8, 0.01, ctx=ctx), golden["rrc_pulse_001"]) < 1e-13


def test_rrc_shaping_and_sampling(ctx, golden):
    dt = float(golden["dt"][0])
    p = 1e-3 * 10 ** 0.2
    sym = fld(golden["qam_symbols"] * np.sqrt(p), dt * 8, ctx)
    assert rel_l2(dsp.rrc_shaping(sym, 8, 0.1).numpy()[0, 0], golden["shaped_01"]) < TOL
    assert rel_l2(dsp.rrc_shaping(sym, 8, 0.01).numpy()[0, 0], golden["shaped_ref001"]) < TOL
    sig = fld(golden["shaped_01"], dt, ctx)
    assert rel_l2(dsp.rrc_sampling(sig, 8, 0.1).numpy()[0, 0], golden["sampled_01"]) < TOL


def test_resampling(ctx, golden):
    dt = float(golden["dt"][0])
    sig = fld(golden["shaped_01"], dt, ctx)
    assert rel_l2(dsp.decimate(sig, 4).numpy()[0, 0], golden["decimate4"]) < TOL
    np.testing.assert_array_equal(dsp.downsample(sig, 4).numpy()[0, 0], f32(golden["downsample4"]))
    sym = fld(golden["qam_symbols"], 1.0, ctx)
    np.testing.assert_array_equal(dsp.upsample(sym, 2).numpy()[0, 0], f32(golden["upsample2"]))


def test_filter_matches_oracle(ctx, oracle_cpu):
    rng = np.random.default_rng(4)
    x = f32(rng.standard_normal((2, 4096)) + 1j * rng.standard_normal((2, 4096)))
    h = rng.standard_normal(33) + 1j * rng.standard_normal(33)
    f = fld(x, 1.0, ctx)
    dsp.filter_inplace(f, h)
    got = f.numpy()[:, 0]
    for b in range(2):
        assert rel_l2(got[b], oracle_cpu.filter(x[b], h)) < TOL


def test_decisions_and_metrics(ctx, golden):
    sym, noisy, rx = golden["qam_symbols"], golden["rx_noisy"], golden["rx_eq"]
    n = fld(noisy, 1.0, ctx)
    assert rel_l2(dsp.hard_decision_16qam(n).numpy()[0, 0], golden["hd_out"]) < 1e-7
    for u, key in ((0.05, "sd_out_005"), (0.02, "sd_out_002")):
        assert rel_l2(dsp.soft_decision_16qam(n, u).numpy()[0, 0], golden[key]) < 1e-7
    np.testing.assert_array_equal(dsp.hd_sequence_16qam(n)[0, 0], golden["demod_codes"])
    t, r = fld(sym, 1.0, ctx), fld(rx, 1.0, ctx)
    assert dsp.bit_error_rate_16qam(t, r, -1)[0] == golden["ber_nocut"][0]
    assert dsp.bit_error_rate_16qam(t, r, 7)[0] == golden["ber_cut7"][0]
    assert dsp.symbol_error_rate_16qam(t, r, 7)[0] == golden["ser_cut7"][0]
    assert abs(dsp.q2_factor(t, r, -1)[0] - golden["q2_nocut"][0]) < 1e-5
    assert abs(dsp.q2_factor(t, r, 7)[0] - golden["q2_cut7"][0]) < 1e-5
    assert dsp.PhaseShiftEqualizer(3600).estimate(t, n)[0] == golden["pse_angle_3600"][0]
    assert dsp.PhaseShiftEqualizer(720).estimate(t, n)[0] == golden["pse_angle_720"][0]
    assert abs(dsp.ScalarEqualizer().estimate(t, n)[0] - golden["scalar_eq"][0]) < 1e-6 * abs(golden["scalar_eq"][0])


def test_wdm(ctx, golden):
    dt = float(golden["wdm_dt"][0])
    ch = fld(golden["wdm_channels"], dt, ctx)
    mux = dsp.wdm_mux(ch, 50e9)
    assert rel_l2(mux.numpy()[0, 0], golden["wdm_mux"]) < TOL
    assert rel_l2(dsp.wdm_select(mux, -1, 50e9).numpy()[0, 0], golden["wdm_select_m1"]) < TOL
    assert rel_l2(dsp.wdm_select(mux, 0, 50e9).numpy()[0, 0], golden["wdm_select_0"]) < TOL
    c0 = fld(golden["wdm_channels"][0], dt, ctx)
    assert rel_l2(dsp.frequency_shift(c0, 12.5e9).numpy()[0, 0], golden["fshift"]) < TOL
    assert rel_l2(dsp.bandpass_filter(mux, 25e9).numpy()[0, 0], golden["bandpass"]) < TOL


def test_decisions_bit_exact_full_size(ctx, oracle_cpu):
    """2^20 noisy symbols (FP32-representable): codes, bit and symbol error
    counts with a cut equal the oracle's exactly."""
    rng = np.random.default_rng(20)
    n = 1 << 20
    tx = f32(oracle_cpu.qam16_map(rng.integers(0, 16, n)) * 0.7)
    rx = f32(tx + 0.12 * (rng.standard_normal(n) + 1j * rng.standard_normal(n)))
    t, r = fld(tx, 1.0, ctx), fld(rx, 1.0, ctx)
    np.testing.assert_array_equal(dsp.hd_sequence_16qam(r)[0, 0], oracle_cpu.hd_sequence(rx))
    be, se = dsp.error_counts(t, r, 100)
    obe, ose = oracle_cpu.error_counts(tx, rx, 100)
    assert (int(be[0]), int(se[0])) == (obe, ose) and obe > 0
    assert abs(dsp.q2_factor(t, r, 100)[0] - oracle_cpu.q2(tx, rx, 100)) < 1e-9


def test_rrc_round_trip_full_size(ctx):
    """Shaping then matched filtering at 2^14 symbols x 8 sps (the
    single-channel configuration) returns the symbols: BER 0, Q > 40 dB."""
    rng = np.random.default_rng(14)
    ns, osf = 1 << 14, 8
    codes = rng.integers(0, 16, (4, 1, ns))
    sym = dsp.qam16_map(codes, fg.Domain(1, ns, 1 / 32e9), batch=4, ctx=ctx)
    sig = dsp.rrc_shaping(sym, osf, 0.1)
    back = dsp.rrc_sampling(sig, osf, 0.1)
    assert np.all(dsp.bit_error_rate_16qam(sym, back, 0) == 0)
    assert np.all(dsp.q2_factor(sym, back, 0) > 40)
    np.testing.assert_array_equal(dsp.hd_sequence_16qam(back), codes)


def test_decisions_near_level_boundaries(ctx, oracle_cpu):
    """Samples planted on and around the level boundaries of the normalized
    coordinates (0 and +-2/sqrt 10, offsets 0 to 1e-4 on either side, on
    each axis): the kernels decide from FP32 coordinates only outside a
    guard band and take the FP64 argmin inside it, so codes, error counts,
    hard and soft decisions equal the FP64 oracle's exactly."""
    rng = np.random.default_rng(99)
    n = 1 << 16
    base = f32(oracle_cpu.qam16_map(rng.integers(0, 16, n)) * 0.7)
    b = 2 / np.sqrt(10)
    offs = np.array([0, 1e-9, 1e-7, 1e-6, 9e-6, 1.1e-5, 3e-5, 1e-4])
    offs = np.concatenate([offs, -offs[1:]])
    near = (np.array([0.0, b, -b])[:, None] + offs[None, :]).ravel()
    other = np.array([-3, -1, 1, 3]) / np.sqrt(10)
    planted = np.concatenate([(near[:, None] + 1j * other[None, :]).ravel(),
                              (other[None, :] + 1j * near[:, None]).ravel()])
    idx = rng.choice(n, planted.size, replace=False)
    x = base.copy()
    for _ in range(4):  # the planted samples move the RMS they are scaled by
        sp = np.sqrt(np.mean(np.abs(x) ** 2))
        x[idx] = planted * sp
        x = f32(x)
    r = fld(x, 1.0, ctx)
    np.testing.assert_array_equal(dsp.hd_sequence_16qam(r)[0, 0], oracle_cpu.hd_sequence(x))
    np.testing.assert_array_equal(dsp.hard_decision_16qam(r).numpy(np.complex64)[0, 0],
                                  oracle_cpu.hard_decision(x).astype(np.complex64))
    for u in (0.05, 1e-5 / np.sqrt(10), 0.0):
        np.testing.assert_array_equal(dsp.soft_decision_16qam(r, u).numpy(np.complex64)[0, 0],
                                      oracle_cpu.soft_decision(x, u).astype(np.complex64))
    be, se = dsp.error_counts(fld(base, 1.0, ctx), r, 0)
    assert (int(be[0]), int(se[0])) == oracle_cpu.error_counts(base, x, 0)


def test_certainty_decisions(ctx, oracle_cpu):
    """find_certainty / sd / hd (src/tasks/wdm_scoring.cpp:105-156) on
    3 realizations of a 6-row (3 channels x 2 modes) dataset-shaped field:
    the certainty equals the oracle's to FP64 rounding of the RMS sums, the
    snapped samples are the same (bit-exact decision pattern) and the outputs
    match to FP32 rounding."""
    rng = np.random.default_rng(105)
    rows, n, b = 6, 1 << 14, 3
    codes = rng.integers(0, 16, (b, rows, n))
    tx = f32(oracle_cpu.qam16_map(codes.ravel()).reshape(b, rows, n) * 0.8)
    rx = f32(tx + 0.11 * (rng.standard_normal(tx.shape) + 1j * rng.standard_normal(tx.shape)))
    t = fg.Field(fg.Domain(rows, n, 1.0), data=tx, batch=b, ctx=ctx)
    r = fg.Field(fg.Domain(rows, n, 1.0), data=rx, batch=b, ctx=ctx)
    cert = dsp.find_certainty(t, r)
    want = [oracle_cpu.find_certainty(tx[i], rx[i]) for i in range(b)]
    # the RMS sums run in different orders (the oracle's sequential FP64 sum of
    # 1e5 terms is off by ~1e-12), and |gray / scale - rx| amplifies the scale
    # difference by |gray / scale| / distance (~25 here)
    np.testing.assert_allclose(cert, want, rtol=1e-9)
    assert all(0 < c < 1 for c in cert)
    for c in (cert[0], 0.6):
        got = dsp.certainty_decision(r, c).numpy()
        for i in range(b):
            ref = oracle_cpu.certainty_decision(rx[i], c)
            snapped = np.abs(ref - rx[i]) > 1e-6 * np.abs(rx[i]).max()
            got_snapped = np.abs(got[i] - rx[i]) > 1e-6 * np.abs(rx[i]).max()
            np.testing.assert_array_equal(got_snapped, snapped)
            assert 0 < snapped.sum() < snapped.size
            assert rel_l2(got[i], ref) < TOL
    h = dsp.hd(r).numpy()
    for i in range(b):
        assert rel_l2(h[i], oracle_cpu.hd_rms(rx[i])) < TOL
    # a field with no decision errors sits at the 1/sqrt(5) cap: certainty 1
    assert abs(dsp.find_certainty(t, t)[0] - 1.0) < 1e-12

"""Pin the FP64 oracle restatement against the reference's own code.

Golden vectors in tests/golden/reference_golden.npz were produced by the
unmodified reference sources (tests/golden/make_golden.py).  Where the
reference build is available (this container), the oracle is also checked live
against it on fresh random inputs.  CPU only.
"""
import numpy as np
import pytest

from conftest import ALPHA, BETA2, F0, GAMMA, rel_l2

TOL = 1e-12


def test_fft_matches_reference_and_numpy(golden, oracle_cpu):
    x = golden["fft_in"]
    assert rel_l2(oracle_cpu.field_fft(x), golden["fft_out"]) < TOL
    assert rel_l2(oracle_cpu.field_ifft(x), golden["ifft_out"]) < TOL
    assert rel_l2(oracle_cpu.dft(x[0]), np.fft.fft(x[0])) < 1e-14


def test_conversions_and_fiber(golden, oracle_cpu):
    import focss_gb300 as fg
    c = golden["conv_in"]
    got = [fg.db_to_natural(c[0]), fg.dbm_to_watts(c[1]), fg.db_to_linear(c[2]), fg.disp_to_beta2(c[3], c[4])]
    np.testing.assert_allclose(got, golden["conv_out"], rtol=1e-15)
    f = fg.Fiber(*golden["fiber"])
    np.testing.assert_array_equal(
        [getattr(f * -2.0, k) for k in ("alpha", "beta2", "gamma", "length", "wavelength", "kappa")],
        golden["fiber_x_neg2"])
    np.testing.assert_array_equal(
        [getattr(f * 10.0, k) for k in ("alpha", "beta2", "gamma", "length", "wavelength", "kappa")],
        golden["fiber_x_10"])
    np.testing.assert_array_equal(
        [getattr(f.dispersive(), k) for k in ("alpha", "beta2", "gamma", "length", "wavelength", "kappa")],
        golden["fiber_dispersive"])


def test_ssfm_grids(golden, oracle_cpu):
    cpu = oracle_cpu
    span = cpu.Fiber(*golden["ssfm_span"])
    dt = float(golden["dt"][0])
    x = golden["shaped_01"]
    a, _ = cpu.ssfm_run(x, dt, span, cpu.UNIFORM, 20)
    assert rel_l2(a, golden["ssfm_uniform"]) < TOL
    b, _ = cpu.ssfm_run(a, dt, span, cpu.UNIFORM, 20, direction=cpu.BACKWARD)
    assert rel_l2(b, golden["ssfm_uniform_bwd"]) < TOL
    a, _ = cpu.ssfm_run(x, dt, span, cpu.ADAPTIVE, 1, 0.005, 1000.0)
    assert rel_l2(a, golden["ssfm_adaptive"]) < TOL
    a, _ = cpu.ssfm_run(x, dt, span, cpu.LOGARITHMIC, 1, 0.005, 1000.0)
    assert rel_l2(a, golden["ssfm_log"]) < TOL
    a = cpu.cd_compensation(golden["cdc_in"], dt, span, 10)
    assert rel_l2(a, golden["cdc_out"]) < TOL


def test_amplifier_noiseless(golden, oracle_cpu):
    cpu = oracle_cpu
    G = float(golden["amp_gain"][0])
    x = golden["shaped_01"]
    dt = float(golden["dt"][0])
    assert rel_l2(cpu.amplify(x, dt, F0, G), golden["amp_out"]) < 1e-15
    assert rel_l2(cpu.drop_power(x, G), golden["drop_out"]) < 1e-15
    assert rel_l2(cpu.give_power(x, G), golden["give_out"]) < 1e-15


def test_tx_rx_dsp(golden, oracle_cpu):
    cpu = oracle_cpu
    codes = golden["qam_codes"]
    np.testing.assert_array_equal(cpu.qam16_map(codes), golden["qam_symbols"])
    assert rel_l2(cpu.rrc_pulse(512, 8, 0.1), golden["rrc_pulse_01"]) < 1e-15
    assert rel_l2(cpu.rrc_pulse(512, 8, 0.01), golden["rrc_pulse_001"]) < 1e-15
    p = 1e-3 * 10 ** 0.2
    sh = cpu.rrc_shaping(golden["qam_symbols"] * np.sqrt(p), 8, 0.1)
    assert rel_l2(sh, golden["shaped_01"]) < TOL
    assert rel_l2(cpu.rrc_shaping(golden["qam_symbols"] * np.sqrt(p), 8, 0.01), golden["shaped_ref001"]) < TOL
    assert rel_l2(cpu.rrc_sampling(golden["shaped_01"], 8, 0.1), golden["sampled_01"]) < TOL
    assert rel_l2(cpu.decimate(golden["shaped_01"], 4), golden["decimate4"]) < TOL
    np.testing.assert_array_equal(cpu.upsample(golden["qam_symbols"], 2), golden["upsample2"])
    np.testing.assert_array_equal(cpu.downsample(golden["shaped_01"], 4), golden["downsample4"])


def test_decisions_and_metrics(golden, oracle_cpu):
    cpu = oracle_cpu
    sym, noisy, rx = golden["qam_symbols"], golden["rx_noisy"], golden["rx_eq"]
    assert rel_l2(cpu.hard_decision(noisy), golden["hd_out"]) < 1e-15
    assert rel_l2(cpu.soft_decision(noisy, 0.05), golden["sd_out_005"]) < 1e-15
    assert rel_l2(cpu.soft_decision(noisy, 0.02), golden["sd_out_002"]) < 1e-15
    np.testing.assert_array_equal(cpu.hd_sequence(noisy), golden["demod_codes"])
    assert cpu.bit_error_rate(sym, rx, 0) == golden["ber_nocut"][0]
    assert cpu.bit_error_rate(sym, rx, 7) == golden["ber_cut7"][0]
    assert cpu.symbol_error_rate(sym, rx, 7) == golden["ser_cut7"][0]
    assert abs(cpu.q2(sym, rx, 0) - golden["q2_nocut"][0]) < 1e-12
    assert abs(cpu.q2(sym, rx, 7) - golden["q2_cut7"][0]) < 1e-12
    assert cpu.pse_estimate(sym, noisy, 3600) == golden["pse_angle_3600"][0]
    assert cpu.pse_estimate(sym, noisy, 720) == golden["pse_angle_720"][0]
    assert abs(cpu.scalar_estimate(sym, noisy) - golden["scalar_eq"][0]) < 1e-14


def test_wdm(golden, oracle_cpu):
    cpu = oracle_cpu
    dt = float(golden["wdm_dt"][0])
    mux = cpu.wdm_mux(golden["wdm_channels"], dt, 50e9)
    assert rel_l2(mux, golden["wdm_mux"]) < TOL
    assert rel_l2(cpu.wdm_select(mux, dt, -1, 50e9), golden["wdm_select_m1"]) < TOL
    assert rel_l2(cpu.wdm_select(mux, dt, 0, 50e9), golden["wdm_select_0"]) < TOL
    assert rel_l2(cpu.frequency_shift(golden["wdm_channels"][0], dt, 12.5e9), golden["fshift"]) < TOL
    assert rel_l2(cpu.bandpass(mux, dt, 25e9), golden["bandpass"]) < TOL


def test_triplet_sum_against_literal_loops(oracle_cpu):
    """SINO::cubic (sino.cpp:161-171, 203-220) needs Armadillo and cannot be
    built here; pin the C restatement against a literal pure-Python loop."""
    rng = np.random.default_rng(5)
    R, N = 3, 40
    a = rng.standard_normal((1, N)) + 1j * rng.standard_normal((1, N))
    W = rng.standard_normal((2 * R + 1, 2 * R + 1)) + 1j * rng.standard_normal((2 * R + 1, 2 * R + 1))
    want = np.zeros(N, complex)
    for k in range(R, N - R):
        for m in range(-R, R + 1):
            bd = R - abs(m)
            for n in range(-bd, bd + 1):
                term = a[0, k + n] * np.conj(a[0, k + m + n])
                want[k] += W[m + R, n + R] * a[0, k + m] * term
    got = oracle_cpu.sino_cubic(a, R, W)[0]
    assert rel_l2(got, want) < 1e-14
    # sparse form over the same diamond
    mm, nn, cc = [], [], []
    for m in range(-R, R + 1):
        bd = R - abs(m)
        for n in range(-bd, bd + 1):
            mm.append(m); nn.append(n); cc.append(W[m + R, n + R])
    got2 = oracle_cpu.triplet_sparse(a, R, mm, nn, cc)[0]
    assert rel_l2(got2, want) < 1e-14


@pytest.fixture(scope="module")
def ref_live():
    from oracle import ref
    if not ref.available():
        pytest.skip("reference sources not present on this machine (golden vectors still pin the oracle)")
    return ref


def test_live_reference_random_ssfm(oracle_cpu, ref_live):
    cpu = oracle_cpu
    rng = np.random.default_rng(11)
    n = 2048
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 0.03
    fib = cpu.Fiber(ALPHA, BETA2, GAMMA, 5e3, 1.55e-6, 1.0)
    dt = 1 / 256e9
    for grid, steps in ((0, 7), (1, 1), (2, 1)):
        a, _ = cpu.ssfm_run(x, dt, fib, grid, steps, 0.01, 500.0, 1.0)
        b = ref_live.ssfm_run(x, dt, fib.astuple(), grid, steps, 0.01, 500.0, 1.0)
        assert rel_l2(a, b) < TOL


def test_live_reference_noise_statistics(oracle_cpu, ref_live):
    """ASE variance: the reference's std::normal_distribution and the oracle's
    Philox stream must give the same per-quadrature variance (amplifier.cpp:20-28)."""
    n = 1 << 16
    x = np.zeros(n, complex)
    dt = 1 / 256e9
    G, NF = 10 ** 1.6, 10 ** 0.45
    a = ref_live.amplify(x, dt, F0, G, NF, seed=3)
    b = oracle_cpu.add_noise(x, dt, F0, G, NF, seed=3)
    var = 6.62607004081818181818181e-34 * F0 * NF * (G - 1) / 2 / dt / 2
    for z in (a, b):
        assert abs(np.var(z.real) / var - 1) < 0.03
        assert abs(np.var(z.imag) / var - 1) < 0.03


def test_field_power(oracle_cpu):
    """Field::average_power / peak_power (field.cpp:164-187), golden from the reference build."""
    import os
    from conftest import ROOT
    g = dict(np.load(os.path.join(ROOT, "tests", "golden", "field_power_golden.npz")))
    for modes in (1, 2):
        a = g["power_in%d" % modes]
        avg, peak = g["power_out%d" % modes]
        assert abs(oracle_cpu.average_power(a) - avg) < 1e-15 * avg
        assert abs(oracle_cpu.peak_power(a) - peak) < 1e-15 * peak

"""Generate the golden vectors in tests/golden/*.npz from the reference's own
sources (oracle/_ref: the unmodified focss sources compiled against the
FFTW-API shim and the Armadillo stand-in).  Run where the reference tree
exists:

    python tests/golden/make_golden.py              # both files
    python tests/golden/make_golden.py --ppe-only   # ppe_golden.npz only

Inputs are seeded synthetic signals shaped like the benchmark configurations
(16QAM, RRC, SSMF) at sizes the FP64 CPU code finishes in seconds.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# SSMF per the benchmark configurations (SI units).
ALPHA = ref.db_to_natural(0.2e-3)
BETA2 = ref.disp_to_beta2(17e-6, 1.55e-6)
GAMMA = 1.3e-3
F0 = 299792458.0 / 1.55e-6


def qam_codes(rng, n):
    return rng.integers(0, 16, n).astype(np.int32)


def gray():
    s = np.sqrt(10.0)
    re = np.array([-3, -1, 3, 1, -3, -1, 3, 1, -3, -1, 3, 1, -3, -1, 3, 1]) / s
    im = np.array([-3, -3, -3, -3, -1, -1, -1, -1, 3, 3, 3, 3, 1, 1, 1, 1]) / s
    return re + 1j * im


def main():
    assert ref.available(), "reference build unavailable"
    rng = np.random.default_rng(20261203)
    g = {}

    # --- conversions and fiber transforms (functions.cpp:82-96, fiber.cpp:4-45)
    g["conv_in"] = np.array([0.2e-3, 2.0, 4.5, 17e-6, 1.55e-6])
    g["conv_out"] = np.array([ref.db_to_natural(0.2e-3), ref.dbm_to_watts(2.0), ref.db_to_linear(4.5),
                              ref.disp_to_beta2(17e-6, 1.55e-6)])
    fib = np.array([ALPHA, BETA2, GAMMA, 80e3, 1.55e-6, 1.0])
    g["fiber"] = fib
    g["fiber_x_neg2"] = ref.fiber_scale(fib, -2.0)
    g["fiber_x_10"] = ref.fiber_scale(fib, 10.0)
    g["fiber_dispersive"] = ref.fiber_dispersive(fib)

    # --- FFT (field.cpp:343-352)
    x = rng.standard_normal((2, 1024)) + 1j * rng.standard_normal((2, 1024))
    g["fft_in"] = x
    g["fft_out"] = ref.field_fft(x)
    g["ifft_out"] = ref.field_ifft(x)

    # --- TX DSP: 16QAM + RRC at 8 sps (modulation.cpp:9-17, 47-96)
    nsym, osf = 512, 8
    codes = qam_codes(rng, nsym)
    sym = gray()[codes]
    g["qam_codes"] = codes
    g["qam_symbols"] = sym
    g["rrc_pulse_01"] = ref.rrc_pulse(nsym, osf, 0.1)
    g["rrc_pulse_001"] = ref.rrc_pulse(nsym, osf, 0.01)
    dt = 1.0 / (32e9 * osf)
    p_launch = ref.dbm_to_watts(2.0)
    shaped = ref.rrc_shaping(sym * np.sqrt(p_launch), osf, roll_off=0.1, dt=dt)
    g["shaped_01"] = shaped
    g["shaped_ref001"] = ref.rrc_shaping(sym * np.sqrt(p_launch), osf, roll_off=None, dt=dt)
    g["sampled_01"] = ref.rrc_sampling(shaped, osf, roll_off=0.1, dt=dt)
    g["dt"] = np.array([dt])

    # --- SSFM on the shaped signal (ssfm.cpp:39-172): N = 4096
    n = shaped.size
    span = np.array([ALPHA, BETA2, GAMMA, 20e3, 1.55e-6, 1.0])
    g["ssfm_span"] = span
    g["ssfm_uniform"] = ref.ssfm_run(shaped, dt, span, grid=0, total_steps=20, direction=1.0)
    g["ssfm_uniform_bwd"] = ref.ssfm_run(g["ssfm_uniform"], dt, span, grid=0, total_steps=20, direction=-1.0)
    g["ssfm_adaptive"] = ref.ssfm_run(shaped, dt, span, grid=2, max_phase_shift=0.005, max_step_size=1000.0,
                                      direction=1.0)
    g["ssfm_log"] = ref.ssfm_run(shaped, dt, span, grid=1, max_phase_shift=0.005, max_step_size=1000.0,
                                 direction=1.0)
    disp = np.array([0.0, BETA2, 0.0, 10 * 80e3, 1.55e-6, 1.0])
    g["cdc_in"] = g["ssfm_uniform"]
    g["cdc_out"] = ref.ssfm_run(g["ssfm_uniform"], dt, ref.fiber_scale(ref.fiber_dispersive(span), 10.0),
                                grid=0, total_steps=1, direction=-1.0)
    del disp

    # --- amplifier without noise (amplifier.cpp:15-42)
    G = ref.db_to_linear(0.2 * 80)
    g["amp_gain"] = np.array([G])
    g["amp_out"] = ref.amplify(shaped, dt, F0, G, 0.0)
    g["drop_out"] = ref.drop_power(shaped, G)
    g["give_out"] = ref.give_power(shaped, G)

    # --- resampling (field.cpp:272-320)
    g["decimate4"] = ref.decimate(shaped, 4)
    g["upsample2"] = ref.upsample(sym, 2)
    g["downsample4"] = ref.downsample(shaped, 4)

    # --- decisions / metrics (modulation.cpp:98-223, functions.cpp:27-80)
    noisy = sym + 0.25 * (rng.standard_normal(nsym) + 1j * rng.standard_normal(nsym))
    noisy = noisy * 1.7 * np.exp(0.3j)
    g["rx_noisy"] = noisy
    g["hd_out"] = ref.hard_decision(noisy)
    g["sd_out_005"] = ref.soft_decision(noisy, 0.05)
    g["sd_out_002"] = ref.soft_decision(noisy, 0.02)
    g["demod_codes"] = np.array([ref.demodulate16(z / np.sqrt(np.mean(np.abs(noisy) ** 2))) for z in noisy],
                                np.int32)
    rx_eq = noisy / 1.7 * np.exp(-0.3j)
    g["rx_eq"] = rx_eq
    g["ber_nocut"] = np.array([ref.ber(sym, rx_eq, -1)])
    g["ber_cut7"] = np.array([ref.ber(sym, rx_eq, 7)])
    g["ser_cut7"] = np.array([ref.ser(sym, rx_eq, 7)])
    g["q2_nocut"] = np.array([ref.q2(sym, rx_eq, -1)])
    g["q2_cut7"] = np.array([ref.q2(sym, rx_eq, 7)])
    g["pse_angle_3600"] = np.array([ref.pse_angle(sym, noisy, 3600)])
    g["pse_angle_720"] = np.array([ref.pse_angle(sym, noisy, 720)])
    g["scalar_eq"] = np.array([ref.scalar_estimate(sym, noisy)])

    # --- WDM (modulation.cpp:225-277): 3 channels, 50 GHz at 16 sps
    osf_w, nsym_w = 16, 128
    dtw = 1.0 / (32e9 * osf_w)
    chans = []
    for c in range(3):
        s = gray()[qam_codes(rng, nsym_w)]
        chans.append(ref.rrc_shaping(s, osf_w, roll_off=0.1, dt=dtw))
    chans = np.array(chans)
    g["wdm_dt"] = np.array([dtw])
    g["wdm_channels"] = chans
    g["wdm_mux"] = ref.wdm_mux(chans, dtw, 50e9)
    g["wdm_select_m1"] = ref.wdm_select(g["wdm_mux"], dtw, -1, 50e9)
    g["wdm_select_0"] = ref.wdm_select(g["wdm_mux"], dtw, 0, 50e9)
    g["fshift"] = ref.frequency_shift(chans[0], dtw, 12.5e9)
    g["bandpass"] = ref.bandpass(g["wdm_mux"], dtw, 25e9)

    # --- solitons (tasks/verification.cpp:10-36)
    g["sech_1024_z0"] = ref.soliton(False, 1024, 0.0)
    g["sech_1024_z1"] = ref.soliton(False, 1024, 1.0)

    # --- dataset file written by the reference's own save_transmission (functions.cpp:174-208)
    io_rng = np.random.default_rng(31)
    scale = 10.0 ** io_rng.integers(-7, 2, (2, 40))
    g["io_tx"] = (io_rng.standard_normal((2, 40)) + 1j * io_rng.standard_normal((2, 40))) * scale
    g["io_rx"] = (io_rng.standard_normal((2, 40)) + 1j * io_rng.standard_normal((2, 40))) * scale
    ref.save_transmission(os.path.join(OUT, "transmission_ref.csv"), g["io_tx"], g["io_rx"])

    np.savez_compressed(os.path.join(OUT, "reference_golden.npz"), **g)
    print("wrote", len(g), "arrays")


def main_ppe():
    """Perturbation equalizers and certainty decisions, from the reference's own
    sino.cpp, wdm_sino.cpp and wdm_scoring.cpp (compiled against the project's
    Armadillo stand-in, whose least-squares solve is Householder QR)."""
    assert ref.available(), "reference build unavailable"
    rng = np.random.default_rng(20261204)
    g = {}
    pts = gray()

    def cn(shape, s=1.0):
        return s * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))

    # SINO::cubic (sino.cpp:203-220) with random weights, 1 and 2 modes
    R = 12
    g["cubic_R"] = np.array([R])
    g["cubic_w"] = cn((2 * R + 1, 2 * R + 1), 1e-2)
    g["cubic_in1"] = pts[rng.integers(0, 16, (1, 400))] * 0.05
    g["cubic_in2"] = pts[rng.integers(0, 16, (2, 400))] * 0.05
    g["cubic_out1"] = ref.sino_cubic(g["cubic_in1"], R, g["cubic_w"])
    g["cubic_out2"] = ref.sino_cubic(g["cubic_in2"], R, g["cubic_w"])
    g["sino_eq_lw"] = np.array([0.93 + 0.07j])
    g["sino_eq_rx"] = g["cubic_in1"] * 0.9 + cn((1, 400), 1e-3)
    g["sino_eq_out"] = ref.sino_equalize(g["sino_eq_rx"], g["cubic_in1"], R, g["cubic_w"], g["sino_eq_lw"][0])

    # SINO::train (sino.cpp:42-159): a synthetic link with known coefficients
    Rt, N = 8, 3000
    w_true = cn((2 * Rt + 1, 2 * Rt + 1), 2e-3)
    for modes in (1, 2):
        tx = pts[rng.integers(0, 16, (modes, N))]
        rx = (0.9 + 0.1j) * tx + ref.sino_cubic(tx, Rt, w_true) + cn((modes, N), 0.01)
        g["train%d_tx" % modes] = tx
        g["train%d_rx" % modes] = rx
        for t in (0, 1, 2):
            if modes == 2 and t != 0:
                continue
            W, ic, lw = ref.sino_train(tx, rx, Rt, t, 0.9 + 0.1j)
            g["train%d_t%d_w" % (modes, t)] = W
            g["train%d_t%d_ic_lw" % (modes, t)] = np.array([ic, lw])
    g["train_R"] = np.array([Rt])

    # WdmPPE::train and its operators (wdm_sino.cpp:28-300), (c, d) = (8, 2)
    c, d, N = 8, 2, 1500
    tx6 = pts[rng.integers(0, 16, (6, N))] * 0.1
    rx6 = 0.95 * tx6 + cn((6, N), 2e-3)
    rx6[2:4] += 50.0 * ref.wdm_ppe_apply(ref.WDM_CUBIC, tx6, cn((2 * c + 1, 2 * c + 1), 1e-1),
                                         cn((2 * d + 1, 2 * d + 1), 1e-1), 1.0)
    g["wdm_tx"], g["wdm_rx"] = tx6, rx6
    C_, D_, ic, lw = ref.wdm_ppe_train(tx6, rx6, c, d)
    g["wdm_C"], g["wdm_D"], g["wdm_ic_lw"] = C_, D_, np.array([ic, lw])
    test6 = pts[rng.integers(0, 16, (6, N))] * 0.1
    rxt = 0.95 * test6 + cn((6, N), 2e-3)
    g["wdm_test"], g["wdm_test_rx"] = test6, rxt
    for name, what in (("spm", ref.WDM_SPM), ("xpm", ref.WDM_XPM), ("cubic", ref.WDM_CUBIC),
                       ("model", ref.WDM_MODEL), ("eq", ref.WDM_EQUALIZE)):
        g["wdm_" + name] = ref.wdm_ppe_apply(what, test6, C_, D_, lw, rx=rxt)
    g["wdm_eq3"] = ref.wdm_ppe_apply(ref.WDM_EQUALIZE3, test6, C_, D_, lw, b=rxt, rx=rxt)

    # find_certainty / sd / hd (wdm_scoring.cpp:105-156) on a noisy 2 x N matrix
    txc = pts[rng.integers(0, 16, (2, 2000))] * 0.3
    rxc = txc + cn((2, 2000), 0.045)
    g["cert_tx"], g["cert_rx"] = txc, rxc
    cert = ref.find_certainty(txc, rxc)
    g["cert"] = np.array([cert])
    g["cert_sd"] = ref.certainty_sd(rxc, cert)
    g["cert_sd_05"] = ref.certainty_sd(rxc, 0.5)
    g["cert_hd"] = ref.hd_rms(rxc)

    np.savez_compressed(os.path.join(OUT, "ppe_golden.npz"), **g)
    print("wrote", len(g), "PPE arrays; certainty", cert)


def main_power():
    """Field::average_power / peak_power (field.cpp:164-187), 1 and 2 modes."""
    assert ref.available(), "reference build unavailable"
    rng = np.random.default_rng(20261205)
    g = {}
    for modes in (1, 2):
        a = (rng.standard_normal((modes, 4096)) + 1j * rng.standard_normal((modes, 4096))) * 0.03
        a = a.astype(np.complex64).astype(np.complex128)  # exactly representable on the GPU
        g["power_in%d" % modes] = a
        g["power_out%d" % modes] = np.array(ref.field_power(a))
    np.savez_compressed(os.path.join(OUT, "field_power_golden.npz"), **g)
    print("wrote", len(g), "power arrays")


if __name__ == "__main__":
    if "--ppe-only" not in sys.argv:
        main()
    main_ppe()
    main_power()

"""The SINO::train restatement (src/focss/equalizer/sino.cpp:42-159): on a
synthetic link rx = lw * tx + cubic_W(tx) + small noise with W in the
symmetric form the reduced basis spans, the fit recovers W and lw.  CPU only."""
import numpy as np

from focss_gb300 import sino


def test_train_recovers_known_coefficients(oracle_cpu):
    rng = np.random.default_rng(8)
    R, N = 6, 6000
    tx = oracle_cpu.qam16_map(rng.integers(0, 16, N))[None]
    mm, nn = np.meshgrid(np.arange(-R, R + 1), np.arange(-R, R + 1), indexing="ij")
    W = (rng.standard_normal(mm.shape) + 1j * rng.standard_normal(mm.shape)) * 1e-2
    W = (W + W.T) / 2
    W = (W + W[::-1, ::-1]) / 2
    W[np.abs(mm) + np.abs(nn) > R] = 0
    lw = 0.8 - 0.3j
    # features are built over |m| <= R/2, n in [|m|, R-|m|] and symmetric partners
    rx = lw * tx + oracle_cpu.sino_cubic(tx, R, W) + 1e-6 * (rng.standard_normal(N) + 1j * rng.standard_normal(N))
    s = sino.SINO(R, 0.0, sino.SinoType.ORDINARY).train(tx, rx)
    assert abs(s.get_linear_weight() - lw) < 1e-5
    covered = np.zeros_like(W, dtype=bool)
    for m in range(-(R // 2), R // 2 + 1):
        for n in range(abs(m), R - abs(m) + 1):
            for (a, b) in ((m, n), (n, m), (-m, -n), (-n, -m)):
                covered[a + R, b + R] = True
    assert np.max(np.abs(s.weights[covered] - W[covered])) < 1e-5
    assert abs(s.get_intercept()) < 1e-5

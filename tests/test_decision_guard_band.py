"""The FP32 first pass of the GPU 16QAM decisions, emulated on the CPU.

The decision kernels (hard / soft / certainty decisions, hard-decision codes,
error counts) take the nearest constellation level per axis from FP32
coordinates and hand a sample to the FP64 argmin of demodulate_16qam
(src/focss/processing/modulation.cpp:98-110) only when a coordinate lies
within 1e-5 (1 + |v|) of a level boundary (0, +-2/sqrt 10).  This checks the
argument behind that guard band with numpy's IEEE float32 arithmetic (the
same round-to-nearest products as the GPU): on random, heavy-tailed and
boundary-planted samples, every sample outside the band gets the FP64
oracle's code.
"""
import numpy as np

KB = np.float32(0.632455532)  # 2/sqrt(10) as the kernels hold it
ONE, BAND = np.float32(1.0), np.float32(1e-5)


def _levels(v):
    """Per-axis table index of the nearest level (-3, -1, 1, 3 -> 0, 1, 3, 2)."""
    return np.where(v < 0, np.where(v < -KB, 0, 1), np.where(v < KB, 3, 2))


def _near(v):
    a = np.abs(v)
    far0 = np.abs(a - np.float32(0)) > BAND * (ONE + a)
    farb = np.abs(a - KB) > BAND * (ONE + a)
    return ~(far0 & farb)


def _fast_codes(x, scale):
    s32 = np.float32(scale)
    re = (x.real.astype(np.float32) * s32).astype(np.float32)
    im = (x.imag.astype(np.float32) * s32).astype(np.float32)
    codes = _levels(re) | (_levels(im) << 2)
    return codes, _near(re) | _near(im)


def test_fp32_decisions_outside_the_band_equal_the_fp64_argmin(oracle_cpu):
    rng = np.random.default_rng(2024)
    n = 1 << 18
    gray = oracle_cpu.qam16_map(np.arange(16))
    x = gray[rng.integers(0, 16, n)] * 0.7 + 0.15 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    x[: n // 64] *= 40.0  # heavy-tailed outliers far outside the constellation
    b = 2 / np.sqrt(10)
    offs = np.array([0, 1e-9, 1e-7, 1e-6, 9e-6, 1.1e-5, 3e-5, 1e-4])
    offs = np.concatenate([offs, -offs[1:]])
    near = (np.array([0.0, b, -b])[:, None] + offs[None, :]).ravel()
    other = np.array([-3, -1, 1, 3]) / np.sqrt(10)
    planted = np.concatenate([(near[:, None] + 1j * other[None, :]).ravel(),
                              (other[None, :] + 1j * near[:, None]).ravel()])
    idx = rng.choice(np.arange(n // 64, n), planted.size, replace=False)
    for _ in range(4):  # the planted samples move the RMS they are scaled by
        x[idx] = planted * np.sqrt(np.mean(np.abs(x) ** 2))
        x = x.astype(np.complex64).astype(np.complex128)
    scale = 1.0 / np.sqrt(np.mean(np.abs(x) ** 2))  # hd_sequence's sqrt(modes / average power)
    codes, flagged = _fast_codes(x, scale)
    want = oracle_cpu.hd_sequence(x)
    assert np.array_equal(codes[~flagged], want[~flagged])
    assert flagged[idx].sum() >= planted.size // 3  # the planted boundary samples are caught
    assert flagged.mean() < 2e-3  # and the band is rare on ordinary data

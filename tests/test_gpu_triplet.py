"""GPU parity of the perturbation (triplet) sum and equalizer
(SINO::cubic / SINO::equalize, src/focss/equalizer/sino.cpp:161-220) against
the FP64 oracle.  FP32 with FP32 accumulation: tolerance 2e-6 relative L2.
"""
import numpy as np
import pytest

import focss_gb300 as fg
from focss_gb300 import sino
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 2e-6


def f32(x):
    return np.asarray(x).astype(np.complex64).astype(np.complex128)


def fld(x, ctx):
    x = np.asarray(x)
    if x.ndim == 2:
        x = x[None]
    b, m, n = x.shape
    return fg.Field(fg.Domain(m, n, 1 / 32e9), data=x, batch=b, ctx=ctx)


def symmetric_weights(R, rng, decay=0.15):
    mm, nn = np.meshgrid(np.arange(-R, R + 1), np.arange(-R, R + 1), indexing="ij")
    W = (rng.standard_normal(mm.shape) + 1j * rng.standard_normal(mm.shape)) * np.exp(-decay * (np.abs(mm) + np.abs(nn)))
    # symmetries of the reduced basis in SINO::train: W[m,n] = W[n,m] = W[-m,-n]
    W = (W + W.T) / 2
    W = (W + W[::-1, ::-1]) / 2
    return W


@pytest.mark.parametrize("modes", [1, 2])
def test_diamond_terms_match_oracle(ctx, oracle_cpu, modes):
    rng = np.random.default_rng(modes)
    R, N, B = 12, 4096, 3
    a = f32((rng.standard_normal((B, modes, N)) + 1j * rng.standard_normal((B, modes, N))) * 0.3)
    W = symmetric_weights(R, rng)
    m, n, c = sino.diamond_terms(W, R)
    got = sino.triplet_apply(fld(a, ctx), R, m, n, c).numpy()
    for b in range(B):
        want = oracle_cpu.sino_cubic(a[b], R, f32(W))
        assert rel_l2(got[b], want) < TOL


def test_pruned_box_terms_match_oracle(ctx, oracle_cpu):
    rng = np.random.default_rng(9)
    R, N = 30, 8192
    a = f32((rng.standard_normal((1, N)) + 1j * rng.standard_normal((1, N))) * 0.3)
    W = symmetric_weights(R, rng, decay=0.1)
    m, n, c = sino.box_terms(W, R, prune=1e-3)
    got = sino.triplet_apply(fld(a, ctx), R, m, n, c).numpy()[0]
    want = oracle_cpu.triplet_sparse(a, R, m, n, f32(c))
    assert rel_l2(got, want) < TOL


def test_equalize_matches_oracle(ctx, oracle_cpu):
    rng = np.random.default_rng(3)
    R, N = 10, 4096
    tx = f32(oracle_cpu.qam16_map(rng.integers(0, 16, N)))
    rx = f32(tx * (0.9 + 0.1j) + 0.05 * (rng.standard_normal(N) + 1j * rng.standard_normal(N)))
    W = symmetric_weights(R, rng) * 1e-2
    s = sino.SINO(R).set_weights(W, linear_weight=0.9 + 0.1j)
    got = s.equalize(fld(rx[None], ctx), fld(tx[None], ctx)).numpy()[0, 0]
    want = (rx - oracle_cpu.sino_cubic(tx[None], R, f32(W))[0]) / (0.9 + 0.1j)
    assert rel_l2(got, want) < TOL


def test_full_size_cubic_homogeneity_and_windows(ctx, oracle_cpu):
    """2^20 symbols with a pruned R = 75 box (the perturbation-equalizer
    configuration): y(2A) = 8 y(A), and oracle checks on windows (the output
    at k depends only on A[k-2R .. k+2R])."""
    rng = np.random.default_rng(20)
    R, N = 75, 1 << 20
    a = f32(oracle_cpu.qam16_map(rng.integers(0, 16, N)) * 0.05)
    W = symmetric_weights(R, rng, decay=0.06)
    m, n, c = sino.box_terms(W, R, prune=1e-3)
    f = fld(a[None], ctx)
    y = sino.triplet_apply(f, R, m, n, c).numpy()[0, 0]
    f2 = fld(2 * a[None], ctx)
    y2 = sino.triplet_apply(f2, R, m, n, c).numpy()[0, 0]
    assert rel_l2(y2, 8 * y) < TOL
    for k0 in (R, 500_000, N - R - 64):
        # The segment [lo, hi) holds every sample the outputs k0..k0+63 read
        # (or reaches the field's own edge, where both sides pad with zeros).
        lo, hi = max(0, k0 - 2 * R), min(N, k0 + 64 + 2 * R)
        want = oracle_cpu.triplet_sparse(a[lo:hi][None], 0, m, n, f32(c))[0]
        assert rel_l2(y[k0:k0 + 64], want[k0 - lo:k0 - lo + 64]) < 5 * TOL

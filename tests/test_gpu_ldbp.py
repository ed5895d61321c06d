"""Learned DBP on the GPU: loss and gradients of the hand-written backward
kernels against the FP64 oracle (oracle/ldbp_ref.py), and training on fields
the GPU SSFM generates.  FP32 kernels: loss to 2e-5, outputs to 2e-5 and
gradients to 2e-4 relative."""
import numpy as np
import pytest

import focss_gb300 as fg
from focss_gb300 import dsp
from focss_gb300.ldbp import LearnedDBP, rrc_response
from oracle import ldbp_ref as R
from conftest import ALPHA, BETA2, GAMMA, rel_l2

pytestmark = pytest.mark.gpu


def fld(x, dt, ctx):
    x = np.asarray(x)
    return fg.Field(fg.Domain(1, x.shape[-1], dt), data=x[:, None, :], batch=x.shape[0], ctx=ctx)


def test_loss_and_gradients_match_oracle(ctx):
    rng = np.random.default_rng(1)
    spans, steps, T, Tm, N, B = 3, 2, 15, 21, 512, 3
    L = spans * steps
    # near-unitary random filters and moderate nonlinear phases keep the
    # 6-layer network well conditioned, so FP32 vs FP64 differences stay at
    # the rounding level
    h = (rng.standard_normal((L, T)) + 1j * rng.standard_normal((L, T))) / np.sqrt(2 * T)
    xi = rng.standard_normal(L) * 0.1
    hmf = (rng.standard_normal(Tm) + 1j * rng.standard_normal(Tm)) / np.sqrt(2 * Tm)
    x = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N))) * 0.7
    tx = rng.standard_normal((B, N // 2)) + 1j * rng.standard_normal((B, N // 2))
    sc = 0.95
    m = LearnedDBP(spans, steps, T, Tm, N, B, sc, ctx=ctx)
    h32, xi32, hmf32 = [np.asarray(v).astype(np.complex64 if np.iscomplexobj(v) else np.float32) for v in (h, xi, hmf)]
    m.set_params(h32, xi32, hmf32)
    xf, tf = fld(x.astype(np.complex64), 1.0, ctx), fld(tx.astype(np.complex64), 2.0, ctx)
    loss = m.loss_grad(xf, tf)
    want_loss, gh, gxi, ghmf = R.loss_grad(h32.astype(complex), xi32.astype(float), hmf32.astype(complex),
                                           x.astype(np.complex64).astype(complex),
                                           tx.astype(np.complex64).astype(complex), sc, spans, steps)
    assert abs(loss - want_loss) < 2e-5 * want_loss
    (_, _, _), (g_h, g_xi, g_hmf) = m.get_params()
    assert rel_l2(g_h, gh) < 2e-4
    assert rel_l2(g_xi, gxi) < 2e-4
    assert rel_l2(g_hmf, ghmf) < 2e-4
    sym = m.forward(xf).numpy()[:, 0]
    y = R.forward(h32.astype(complex), xi32.astype(float), hmf32.astype(complex),
                  x.astype(np.complex64).astype(complex), sc, spans, steps)
    assert rel_l2(sym, y[..., 0::2]) < 2e-5


def test_training_on_ssfm_link_beats_its_dbp_initialisation(ctx):
    """3 x 80 km SSMF at 5 dBm, 2 samples/symbol, noise off: a 1-step/span
    learned DBP initialised from split-step DBP, trained with the GPU
    backward kernels, reaches a lower loss and a higher Q than at init."""
    rng = np.random.default_rng(5)
    ns, osf, B, spans = 4096, 2, 4, 3
    dt = 1 / (32e9 * osf)
    codes = rng.integers(0, 16, (B, 1, ns))
    p = np.sqrt(fg.dbm_to_watts(5.0))
    sym = dsp.qam16_map(codes, fg.Domain(1, ns, 1 / 32e9), batch=B, ctx=ctx)
    sym *= p
    sig = dsp.rrc_shaping(sym, osf, 0.1)
    fib = fg.Fiber(ALPHA, BETA2, GAMMA, 80e3)
    G = fg.db_to_linear(0.2 * 80)
    fg.forward_propagation(sig, fib, fg.SSFM(fib, 200), fg.Amplifier(G), spans)
    m = LearnedDBP(spans, 1, 41, 63, ns * osf, B, 1 / np.sqrt(G), ctx=ctx)
    m.init_from_dbp(ALPHA, BETA2, GAMMA, 1.0, 80e3, dt, rrc_response(ns, osf, 0.1, ctx=ctx))
    q0 = dsp.q2_factor(sym, m.forward(sig), 100)
    hist = m.fit(sig, sym, iters=150, lr=2e-3)
    q1 = dsp.q2_factor(sym, m.forward(sig), 100)
    assert hist[-1] < 0.7 * hist[0]
    assert np.all(q1 > q0 + 0.5)

"""Correction CNN on the GPU (tcgen05 BF16 implicit GEMMs with tensor-memory
accumulators): outputs, loss and gradients against the numpy restatement
with the same BF16 rounding points
(oracle/cnn_ref.py), and training on a structured distortion.  BF16 weights
and activations: 1e-3 relative on outputs and loss, 1e-2 on gradients."""
import numpy as np
import pytest

import focss_gb300 as fg
from focss_gb300.cnn import CorrectionCNN, he_init
from oracle import cnn_ref as R
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def fld(x, ctx):
    return fg.Field(fg.Domain(1, x.shape[1], 1 / 32e9), data=x[:, None, :], batch=x.shape[0], ctx=ctx)


def test_outputs_loss_and_gradients_match_reference(ctx):
    rng = np.random.default_rng(2)
    B, L, s = 2, 1000, 0.3
    y = (rng.standard_normal((B, L)) + 1j * rng.standard_normal((B, L))) * s
    tx = y + 0.05 * (rng.standard_normal((B, L)) + 1j * rng.standard_normal((B, L)))
    y = y.astype(np.complex64).astype(complex)
    tx = tx.astype(np.complex64).astype(complex)
    p = he_init(rng, zero_last=False) * 0.5
    net = CorrectionCNN(L, B, s, ctx=ctx)
    net.set_params(p)
    yf, tf = fld(y, ctx), fld(tx, ctx)
    z = net.forward(yf).numpy()[:, 0]
    loss = net.loss_grad(yf, tf)
    _, g = net.get_params()
    want_loss, want_g, want_z = R.loss_grad(p.astype(np.float64), y, tx, s)
    assert rel_l2(z, want_z) < 1e-3
    assert abs(loss - want_loss) < 1e-3 * want_loss
    off = 0
    for (cin, cout) in R.LAYERS:
        n = cout * R.KW * cin + cout
        assert rel_l2(g[off:off + n], want_g[off:off + n]) < 1e-2
        off += n


def test_triplet_inputs_match_reference(ctx):
    """The same comparison with first-order perturbation triplets of y as
    input channels 2..15 (focss_cnn_set_triplets)."""
    from focss_gb300.cnn import TRIPLETS
    rng = np.random.default_rng(5)
    B, L, s = 2, 1000, 0.3
    g = np.array([-3, -1, 1, 3]) / np.sqrt(10)
    y = (rng.choice(g, (B, L)) + 1j * rng.choice(g, (B, L))) * s * np.sqrt(5)
    y = (y + 0.05 * s * (rng.standard_normal((B, L)) + 1j * rng.standard_normal((B, L))))
    y = y.astype(np.complex64).astype(complex)
    tx = (y + 0.02 * (rng.standard_normal((B, L)) + 1j * rng.standard_normal((B, L)))).astype(np.complex64)
    tx = tx.astype(complex)
    p = he_init(rng, zero_last=False, n_triplets=len(TRIPLETS)) * 0.5
    net = CorrectionCNN(L, B, s, ctx=ctx, triplets=TRIPLETS)
    net.set_params(p)
    yf, tf = fld(y, ctx), fld(tx, ctx)
    z = net.forward(yf).numpy()[:, 0]
    loss = net.loss_grad(yf, tf)
    _, gr = net.get_params()
    want_loss, want_g, want_z = R.loss_grad(p.astype(np.float64), y, tx, s, TRIPLETS)
    assert rel_l2(z - y, want_z - y) < 1e-2
    assert abs(loss - want_loss) < 1e-3 * want_loss
    off = 0
    for (cin, cout) in R.LAYERS:
        n = cout * R.KW * cin + cout
        assert rel_l2(gr[off:off + n], want_g[off:off + n]) < 1e-2
        off += n


def test_training_learns_a_symbol_memory_distortion(ctx):
    """y_k = t_k + 0.08 t_{k-1} |t_{k+1}|^2 (a triplet-like memory term):
    the CNN trained on the GPU removes most of it (at least 60% of the loss
    in 300 Adam steps)."""
    rng = np.random.default_rng(3)
    B, L = 4, 4096
    g = np.array([-3, -1, 1, 3]) / np.sqrt(10)
    t = rng.choice(g, (B, L)) + 1j * rng.choice(g, (B, L))
    y = t + 0.08 * np.roll(t, 1, axis=1) * np.abs(np.roll(t, -1, axis=1)) ** 2
    net = CorrectionCNN(L, B, 1.0, ctx=ctx)
    net.set_params(he_init(rng))
    yf, tf = fld(y, ctx), fld(t, ctx)
    hist = net.fit(yf, tf, iters=300, lr=2e-3)
    assert hist[-1] < 0.4 * hist[0]

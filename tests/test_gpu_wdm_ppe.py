"""WdmPPE on the GPU (focss_wdm_ppe_apply / focss_wdm_ppe_gram through the C
ABI) against the FP64 oracle restatement of src/focss/equalizer/wdm_sino.cpp.

SPM / XPM sums and the equalizer: FP32 outputs within 1e-5 relative L2 of
the oracle.  The fit: on a synthetic 3-channel dual-polarization link with
known tables both the GPU fit and the oracle's least squares recover them,
and they agree with each other.
"""
import numpy as np
import pytest

import focss_gb300 as fg
from focss_gb300 import WdmPPE
from oracle import wdm_ppe_ref as W
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _qam(rng, shape, power=1.0):
    gray = np.array([complex(a, b) for b in (-3, -1, 3, 1) for a in (-3, -1, 3, 1)]) / np.sqrt(10)
    return (gray[rng.integers(0, 16, shape)] * np.sqrt(power)).astype(np.complex64).astype(np.complex128)


def _truth(rng, c, d, scale=0.01):
    t = W.WdmPPE(c, d)
    raw = (rng.standard_normal(W.n_features(c, d)) + 1j * rng.standard_normal(W.n_features(c, d))) * scale
    return t.install(raw)


def _gpu(truth):
    g = WdmPPE(truth.c_radius, truth.d_radius)
    return g.set_tables(truth.C if truth.c_radius >= 0 else None, truth.D if truth.d_radius >= 0 else None,
                        truth.linear_weight)


@pytest.mark.parametrize("c,d", [(30, 0), (8, 4), (0, 6), (12, 12)])
def test_sums_and_equalizer_match_oracle(ctx, c, d):
    rng = np.random.default_rng(c * 100 + d)
    N, B = 4096, 2
    tx = _qam(rng, (B, 6, N))
    rx = _qam(rng, (B, 6, N))
    truth = _truth(rng, c, d)
    truth.linear_weight = 0.8 + 0.1j
    g = _gpu(truth)
    t = fg.Field(fg.Domain(6, N, 1.0), data=tx, batch=B, ctx=ctx)
    r = fg.Field(fg.Domain(6, N, 1.0), data=rx, batch=B, ctx=ctx)
    spm, xpm, cub, mod = g.spm(t).numpy(), g.xpm(t).numpy(), g.cubic(t).numpy(), g.model(t).numpy()
    eq = g.equalize(t, r).numpy()
    eq2 = g.equalize(t, r, r).numpy()  # tx_spm = t, tx_xpm = r
    for b in range(B):
        s_ref, x_ref = truth.spm(tx[b]), truth.xpm(tx[b])
        assert rel_l2(spm[b], s_ref) < 1e-5
        assert rel_l2(xpm[b], x_ref) < 1e-5
        assert rel_l2(cub[b], s_ref + x_ref) < 1e-5
        assert rel_l2(mod[b], truth.model(tx[b])) < 1e-5
        assert rel_l2(eq[b], truth.equalize(tx[b], rx[b])) < 1e-5
        assert rel_l2(eq2[b], truth.equalize(tx[b], rx[b], rx[b])) < 1e-5
    # the edges [0, R) and [N - R, N) carry no triplet noise
    assert np.all(xpm[:, :, :d] == 0) and np.all(spm[:, :, N - c:] == 0)


def test_two_row_rx_equals_six_row_rx(ctx):
    rng = np.random.default_rng(3)
    N = 2048
    tx, rx = _qam(rng, (6, N)), _qam(rng, (6, N))
    g = _gpu(_truth(rng, 6, 3))
    g.linear_weight = 0.9
    a = g.equalize(tx, rx).numpy()
    r2 = fg.Field(fg.Domain(2, N, 1.0), data=rx[None, 2:4])
    t6 = fg.Field(fg.Domain(6, N, 1.0), data=tx[None], ctx=r2.ctx)
    b = g._apply(spm_in=t6, xpm_in=t6, rx=r2).numpy()
    np.testing.assert_array_equal(a, b)


def _link(rng, c, d, N, noise):
    truth = _truth(rng, c, d)
    truth.linear_weight = 0.85 - 0.25j
    tx = _qam(rng, (6, N))
    rx = np.zeros_like(tx)
    rx[2:4] = truth.model(tx) + noise * (rng.standard_normal((2, N)) + 1j * rng.standard_normal((2, N)))
    return truth, tx, rx


def test_gpu_fit_recovers_known_coefficients(ctx):
    rng = np.random.default_rng(11)
    c, d = 6, 3
    truth, tx, rx = _link(rng, c, d, 1 << 13, 1e-6)
    g = WdmPPE(c, d).train(tx, rx)
    assert abs(g.get_linear_weight() - truth.linear_weight) < 1e-4
    assert np.max(np.abs(g.C - truth.C)) < 1e-4
    assert np.max(np.abs(g.D - truth.D)) < 1e-4
    assert abs(g.get_intercept()) < 1e-4


@pytest.mark.parametrize("c,d", [(10, 0), (8, 4)])
def test_gpu_fit_matches_oracle_fit(ctx, c, d):
    rng = np.random.default_rng(12 + c)
    truth, tx, rx = _link(rng, c, d, 1 << 13, 1e-3)
    g = WdmPPE(c, d).train(tx, rx)
    h = W.WdmPPE(c, d).train(tx, rx)
    scale = np.max(np.abs(h.C))
    assert np.max(np.abs(g.C - h.C)) < 1e-4 * scale + 1e-6
    assert np.max(np.abs(g.D - h.D)) < 1e-4 * scale + 1e-6
    assert abs(g.get_linear_weight() - h.linear_weight) < 1e-5
    assert abs(g.get_intercept() - h.intercept) < 1e-5


def test_wdm_dataset_ppe_pipeline(ctx):
    """wdm_run -> wdm_scoring on the GPU (src/tasks/wdm_run.cpp:79-141,
    src/tasks/wdm_scoring.cpp:158-187): a 3-channel dual-polarization link
    (Manakov 8/9, 4 x 100 km at 4 dBm per channel, 2^12 symbols, 16
    samples/symbol).  WdmPPE trained on one realization raises the centre
    channel's Q on another, with the received symbols and with their hard
    decisions as the triplet inputs."""
    from focss_gb300 import dsp, links
    link = links.DualPolLink(spans=4)
    tx_t, rx_t, _ = links.wdm_dataset(link, 1 << 12, 4.0, seed=1, ctx=ctx)
    tx, rx, steps = links.wdm_dataset(link, 1 << 12, 4.0, seed=2, ctx=ctx)
    assert tx.domain.modes == 6 and rx.domain.samples == 1 << 12 and steps > 4
    ppe = WdmPPE(12, 1).train(tx_t, rx_t)
    cut = 36
    tc = links.centre_rows(tx)
    q_cdc = dsp.q2_factor(tc, links.centre_rows(rx), cut)[0]
    q_rx = dsp.q2_factor(tc, ppe.equalize(rx, rx), cut)[0]
    q_hd = dsp.q2_factor(tc, ppe.equalize(dsp.hd(rx), rx), cut)[0]
    print("Q cdc %.3f  ppe(rx) %.3f  ppe(hd) %.3f dB, |a| %.4f" % (q_cdc, q_rx, q_hd, abs(ppe.get_linear_weight())))
    assert q_rx > q_cdc + 0.2 and q_hd > q_cdc + 0.2


def test_copy_modes(ctx):
    """focss_field_copy_modes gathers channels' polarizations into dataset
    rows (channel * 2 + polarization) and back, in every realization."""
    rng = np.random.default_rng(4)
    n, B = 1000, 3
    chans = [_qam(rng, (B, 2, n)) for _ in range(3)]
    six = fg.Field(fg.Domain(6, n, 1.0), batch=B, ctx=ctx)
    for ch, a in enumerate(chans):
        six.copy_modes(2 * ch, fg.Field(fg.Domain(2, n, 1.0), data=a, batch=B, ctx=ctx), 0, 2)
    got = six.numpy()
    np.testing.assert_array_equal(got, np.concatenate(chans, axis=1))
    back = fg.Field(fg.Domain(2, n, 1.0), batch=B, ctx=ctx).copy_modes(0, six, 2, 2)
    np.testing.assert_array_equal(back.numpy(), chans[1])
    one = fg.Field(fg.Domain(1, n, 1.0), batch=B, ctx=ctx).copy_modes(0, six, 5, 1)
    np.testing.assert_array_equal(one.numpy()[:, 0], chans[2][:, 1])
    with pytest.raises(fg.FocssError):
        six.copy_modes(5, back, 0, 2)  # rows 5..6 of a 6-row field

"""The GPU perturbation equalizers against the reference's own outputs.

tests/golden/ppe_golden.npz holds outputs of the unmodified reference sources
sino.cpp, wdm_sino.cpp and wdm_scoring.cpp (tests/golden/make_golden.py).
Inputs are uploaded as complex64, so every comparison allows for that
rounding: sums and equalizers within 1e-5 relative L2; fitted tables within
2e-5 of their largest entry (the FP64 numpy fit on the same complex64-rounded
inputs moves by up to 2.2e-6); certainty decisions at FP32 rounding.
"""
import os

import numpy as np
import pytest

import focss_gb300 as fg
from focss_gb300 import WdmPPE, dsp, sino
from conftest import ROOT, rel_l2

pytestmark = pytest.mark.gpu

PPE = os.path.join(ROOT, "tests", "golden", "ppe_golden.npz")


@pytest.fixture(scope="module")
def gp():
    return dict(np.load(PPE))


def _field(a, ctx):
    a = np.atleast_2d(a)
    return fg.Field(fg.Domain(a.shape[0], a.shape[1], 1.0), data=a[None], ctx=ctx)


def test_triplet_sum_and_equalizer(ctx, gp):
    R = int(gp["cubic_R"][0])
    W = gp["cubic_w"]
    s = sino.SINO(R).set_weights(W, gp["sino_eq_lw"][0])
    for k in ("1", "2"):
        got = s.cubic(_field(gp["cubic_in" + k], ctx)).numpy()[0]
        assert rel_l2(got, gp["cubic_out" + k]) < 1e-5
    eq = s.equalize(_field(gp["sino_eq_rx"], ctx), _field(gp["cubic_in1"], ctx)).numpy()[0]
    assert rel_l2(eq, gp["sino_eq_out"]) < 1e-5


def test_gpu_fit_matches_reference_train(ctx, gp):
    R = int(gp["train_R"][0])
    for modes in (1, 2):
        tx, rx = gp["train%d_tx" % modes], gp["train%d_rx" % modes]
        for t in (0, 1, 2):
            key = "train%d_t%d_w" % (modes, t)
            if key not in gp:
                continue
            s = sino.SINO(R, 1.0, sino.SinoType(t))
            if t == sino.SinoType.FIXED:
                s.set_linear_weight(0.9 + 0.1j)
            s.train(_field(tx, ctx), _field(rx, ctx), solver="gpu")
            W = gp[key]
            ic, lw = gp["train%d_t%d_ic_lw" % (modes, t)]
            assert np.abs(s.weights - W).max() < 2e-5 * np.abs(W).max()
            assert abs(s.get_linear_weight() - lw) < 1e-6
            assert abs(s.get_intercept() - ic) < 1e-6


def test_wdm_ppe_fit_and_operators(ctx, gp):
    tx, rx = gp["wdm_tx"], gp["wdm_rx"]
    p = WdmPPE(8, 2).train(tx[None], rx[None])
    assert np.abs(p.C - gp["wdm_C"]).max() < 2e-5 * np.abs(gp["wdm_C"]).max()
    assert np.abs(p.D - gp["wdm_D"]).max() < 2e-5 * np.abs(gp["wdm_D"]).max()
    ic, lw = gp["wdm_ic_lw"]
    assert abs(p.get_linear_weight() - lw) < 1e-6
    q = WdmPPE(8, 2).set_tables(gp["wdm_C"], gp["wdm_D"], lw)
    t = fg.Field(fg.Domain(6, tx.shape[1], 1.0), data=gp["wdm_test"][None], ctx=ctx)
    r = fg.Field(fg.Domain(6, tx.shape[1], 1.0), data=gp["wdm_test_rx"][None], ctx=ctx)
    assert rel_l2(q.spm(t).numpy()[0], gp["wdm_spm"]) < 1e-5
    assert rel_l2(q.xpm(t).numpy()[0], gp["wdm_xpm"]) < 1e-5
    assert rel_l2(q.cubic(t).numpy()[0], gp["wdm_cubic"]) < 1e-5
    assert rel_l2(q.model(t).numpy()[0], gp["wdm_model"]) < 1e-5
    assert rel_l2(q.equalize(t, r).numpy()[0], gp["wdm_eq"]) < 1e-5
    assert rel_l2(q.equalize(t, r, r).numpy()[0], gp["wdm_eq3"]) < 1e-5


def test_certainty_decisions(ctx, gp, oracle_cpu):
    tx, rx = gp["cert_tx"], gp["cert_rx"]
    t, r = _field(tx, ctx), _field(rx, ctx)
    c = dsp.find_certainty(t, r)[0]
    # the inputs are rounded to complex64 on upload; the oracle on the same
    # rounded inputs agrees to FP64 rounding of the RMS sums
    f32 = lambda a: a.astype(np.complex64).astype(np.complex128)  # noqa: E731
    assert abs(c - oracle_cpu.find_certainty(f32(tx), f32(rx))) < 1e-9
    assert abs(c - gp["cert"][0]) < 1e-5
    assert rel_l2(dsp.certainty_decision(r, gp["cert"][0]).numpy()[0], gp["cert_sd"]) < 1e-6
    assert rel_l2(dsp.certainty_decision(r, 0.5).numpy()[0], gp["cert_sd_05"]) < 1e-6
    assert rel_l2(dsp.hd(r).numpy()[0], gp["cert_hd"]) < 1e-6

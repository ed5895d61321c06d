"""Pin the perturbation-equalizer oracles against the reference's own code.

tests/golden/ppe_golden.npz was written by the unmodified reference sources
src/focss/equalizer/sino.cpp, wdm_sino.cpp and src/tasks/wdm_scoring.cpp,
compiled against the project's Armadillo stand-in (oracle/arma_shim/armadillo:
least squares by Householder QR, the method of LAPACK's xGELS that Armadillo
calls) by tests/golden/make_golden.py.  Checked here:

* oracle/focss_oracle.c's SINO::cubic restatement (ofc_sino_cubic);
* the numpy restatement of SINO::train in focss_gb300/sino.py (solver="lstsq");
* oracle/wdm_ppe_ref.py (WdmPPE train / spm / xpm / cubic / model / equalize);
* the oracle's find_certainty / sd / hd (ofc_find_certainty, ...).

Where the reference build exists (the build container) the same checks also
run live on fresh inputs.  CPU only.
"""
import os

import numpy as np
import pytest

from conftest import ROOT, rel_l2

PPE = os.path.join(ROOT, "tests", "golden", "ppe_golden.npz")


@pytest.fixture(scope="module")
def gp():
    return dict(np.load(PPE))


def test_sino_cubic_matches_reference(gp, oracle_cpu):
    R = int(gp["cubic_R"][0])
    for k in ("1", "2"):
        got = oracle_cpu.sino_cubic(gp["cubic_in" + k], R, gp["cubic_w"])
        assert rel_l2(got, gp["cubic_out" + k]) < 1e-14


def test_sino_train_matches_reference(gp):
    from focss_gb300 import sino
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
            s.train(tx, rx, solver="lstsq")
            W = gp[key]
            ic, lw = gp["train%d_t%d_ic_lw" % (modes, t)]
            assert np.abs(s.weights - W).max() < 1e-9 * np.abs(W).max()
            assert abs(s.get_intercept() - ic) < 1e-12
            assert abs(s.get_linear_weight() - lw) < 1e-12


def test_wdm_ppe_matches_reference(gp):
    from oracle import wdm_ppe_ref as W
    p = W.WdmPPE(8, 2)
    p.train(gp["wdm_tx"], gp["wdm_rx"])
    assert np.abs(p.C - gp["wdm_C"]).max() < 1e-9 * np.abs(gp["wdm_C"]).max()
    assert np.abs(p.D - gp["wdm_D"]).max() < 1e-9 * np.abs(gp["wdm_D"]).max()
    ic, lw = gp["wdm_ic_lw"]
    assert abs(p.intercept - ic) < 1e-12 and abs(p.linear_weight - lw) < 1e-12
    # the operators with the reference's own trained tables
    q = W.WdmPPE(8, 2)
    q.C, q.D, q.linear_weight, q.trained = gp["wdm_C"], gp["wdm_D"], complex(lw), True
    t, r = gp["wdm_test"], gp["wdm_test_rx"]
    assert rel_l2(q.spm(t), gp["wdm_spm"]) < 1e-13
    assert rel_l2(q.xpm(t), gp["wdm_xpm"]) < 1e-13
    assert rel_l2(q.cubic(t), gp["wdm_cubic"]) < 1e-13
    assert rel_l2(q.model(t), gp["wdm_model"]) < 1e-13
    assert rel_l2(q.equalize(t, t, r), gp["wdm_eq"]) < 1e-13
    assert rel_l2(q.equalize(t, r, r), gp["wdm_eq3"]) < 1e-13


def test_certainty_decisions_match_reference(gp, oracle_cpu):
    tx, rx = gp["cert_tx"], gp["cert_rx"]
    c = oracle_cpu.find_certainty(tx, rx)
    assert abs(c - gp["cert"][0]) < 1e-14 and c < 1.0  # decision errors present
    np.testing.assert_allclose(oracle_cpu.certainty_decision(rx, c), gp["cert_sd"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(oracle_cpu.certainty_decision(rx, 0.5), gp["cert_sd_05"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(oracle_cpu.hd_rms(rx), gp["cert_hd"], rtol=0, atol=1e-15)


def _ref():
    from oracle import ref
    if not ref.available():
        pytest.skip("reference build unavailable (no reference source tree)")
    return ref


def test_live_against_reference_build(oracle_cpu):
    """Fresh random inputs through the reference build and the oracles."""
    ref = _ref()
    from focss_gb300 import sino
    from oracle import wdm_ppe_ref as W
    rng = np.random.default_rng(99)
    R = 5
    a = rng.standard_normal((2, 200)) + 1j * rng.standard_normal((2, 200))
    w = rng.standard_normal((2 * R + 1, 2 * R + 1)) + 1j * rng.standard_normal((2 * R + 1, 2 * R + 1))
    assert rel_l2(oracle_cpu.sino_cubic(a, R, w), ref.sino_cubic(a, R, w)) < 1e-14
    tx = a[:1] / 2
    rx = 0.8 * tx + ref.sino_cubic(tx, R, w * 1e-2) + 0.01 * rng.standard_normal(tx.shape)
    W_ref, ic, lw = ref.sino_train(tx, rx, R, 0)
    s = sino.SINO(R).train(tx, rx, solver="lstsq")
    assert np.abs(s.weights - W_ref).max() < 1e-9 * np.abs(W_ref).max() and abs(s.linear_weight - lw) < 1e-12
    t6 = rng.standard_normal((6, 300)) + 1j * rng.standard_normal((6, 300))
    r6 = t6 + 0.05 * rng.standard_normal((6, 300))
    C_, D_, ic, lw = ref.wdm_ppe_train(t6, r6, 4, 1)
    p = W.WdmPPE(4, 1)
    p.train(t6, r6)
    assert np.abs(p.C - C_).max() < 1e-9 * np.abs(C_).max() and abs(p.linear_weight - lw) < 1e-12
    assert abs(oracle_cpu.find_certainty(t6, r6) - ref.find_certainty(t6, r6)) < 1e-14

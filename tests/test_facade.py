"""C++ facade (include/focss_gpu.hpp): builds, accepts the reference's own
callers unchanged, and reproduces the single-channel chain on the GPU.

CPU: the facade example compiles and links against libfocss_gpu.so; the
reference's unmodified src/tasks/systems.cpp compiles against
include/focss_compat (only where the reference tree is present).
GPU: the facade example runs the single-channel link (10 x 80 km, 1 km
UNIFORM steps, CDC, matched filter, phase-shift equalizer) and matches the
FP64 oracle: field within 1e-5 relative L2, Q within 0.05 dB, decisions equal.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ALPHA, BETA2, F0, GAMMA, ROOT, rel_l2

INC = os.path.join(ROOT, "include")
LIB = os.path.join(ROOT, "focss_gb300", "libfocss_gpu.so")
SRC = os.path.join(ROOT, "tests", "cpp", "facade_link.cpp")
PPE_SRC = os.path.join(ROOT, "tests", "cpp", "facade_ppe.cpp")


def _cxx():
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    return cxx


def _build_example(tmp_path, src=SRC):
    if not os.path.exists(LIB):
        from focss_gb300 import build as gbuild
        gbuild.build()
    exe = str(tmp_path / os.path.splitext(os.path.basename(src))[0])
    cmd = [_cxx(), "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + INC, src, LIB,
           "-Wl,-rpath," + os.path.dirname(LIB), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_facade_example_builds(tmp_path):
    _build_example(tmp_path)
    _build_example(tmp_path, PPE_SRC)


def test_reference_caller_compiles_against_facade(tmp_path):
    from oracle import build as obuild
    tasks = os.path.join(obuild.REF_ROOT, "src", "tasks")
    if not os.path.exists(os.path.join(tasks, "systems.cpp")):
        pytest.skip("reference source tree not present")
    if not os.path.exists(LIB):
        from focss_gb300 import build as gbuild
        gbuild.build()
    main = tmp_path / "main.cpp"
    main.write_text('#include "focss/field.h"\n#include "systems.h"\n'
                    "int main() {\n"
                    "  focss::Field f(focss::Domain{1, 1024, 1.0 / 512e9, 193.4e12});\n"
                    "  forward_propagation(f, 1); backward_propagation(f, 2); cd_compensation(f, 1);\n"
                    "  return 0;\n}\n")
    exe = str(tmp_path / "systems")
    cmd = [_cxx(), "-std=c++17", "-O2", "-I" + os.path.join(INC, "focss_compat"), "-I" + tasks,
           os.path.join(tasks, "systems.cpp"), str(main), LIB, "-Wl,-rpath," + os.path.dirname(LIB), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_facade_link_matches_oracle(tmp_path, oracle_cpu):
    cpu = oracle_cpu
    exe = _build_example(tmp_path)
    rng = np.random.default_rng(7)
    ns, osf, spans = 1 << 11, 8, 10
    dt = 1 / (32e9 * osf)
    codes = rng.integers(0, 16, ns).astype(np.int32)
    cfile = tmp_path / "codes.i32"
    codes.tofile(cfile)
    prefix = str(tmp_path / "out")
    r = subprocess.run([exe, str(cfile), prefix, str(spans)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    x0 = np.fromfile(prefix + "_tx.c128", np.complex128)
    after = np.fromfile(prefix + "_after.c128", np.complex128)
    rx = np.fromfile(prefix + "_rx.c128", np.complex128)
    dec = np.fromfile(prefix + "_codes.i32", np.int32)
    q_gpu, ber_gpu, cert_gpu = map(float, open(prefix + "_metrics.txt").read().split())
    assert x0.size == ns * osf and rx.size == ns

    ofib = cpu.Fiber(ALPHA, BETA2, GAMMA, 80e3, 1.55e-6, 1.0)
    G = 10 ** (0.2 * 80 / 10)
    a = x0
    for _ in range(spans):
        a, _ = cpu.ssfm_run(a, dt, ofib, cpu.UNIFORM, 80)
        a = cpu.amplify(a, dt, F0, G)
    assert rel_l2(after, a) < 1e-5
    a = cpu.cd_compensation(a, dt, ofib, spans)
    s = cpu.rrc_sampling(a, osf, 0.1)
    tx = np.fromfile(prefix + "_sym.c128", np.complex128)
    np.testing.assert_allclose(tx, cpu.qam16_map(codes) * np.sqrt(1e-3 * 10 ** 0.2), rtol=1e-6)
    s = cpu.rotate(s, cpu.pse_estimate(tx, s, 3600))
    assert abs(q_gpu - cpu.q2(tx, s, 100)) < 0.05
    assert ber_gpu == cpu.bit_error_rate(tx, s, 100)
    np.testing.assert_array_equal(dec, cpu.hd_sequence(s))
    assert rel_l2(rx, s) < 1e-4
    assert abs(cert_gpu - cpu.find_certainty(tx, rx)) < 1e-12


@pytest.mark.gpu
def test_facade_perturbation_equalizers_match_oracle(tmp_path, oracle_cpu):
    """WdmPPE(8, 2) and SINO(6) trained through the C++ facade agree with the
    FP64 least-squares restatements (oracle/wdm_ppe_ref.py, the numpy SINO fit)
    on a synthetic 3-channel dual-polarization link with known tables, and
    their equalizer / model outputs match the oracle's to FP32 rounding."""
    from oracle import wdm_ppe_ref as W
    from focss_gb300 import sino
    exe = _build_example(tmp_path, PPE_SRC)
    rng = np.random.default_rng(17)
    n, c, d = 1 << 13, 8, 2
    gray = np.array([complex(a, b) for b in (-3, -1, 3, 1) for a in (-3, -1, 3, 1)]) / np.sqrt(10)
    tx = gray[rng.integers(0, 16, (6, n))].astype(np.complex64).astype(np.complex128)
    truth = W.WdmPPE(c, d).install((rng.standard_normal(W.n_features(c, d)) +
                                    1j * rng.standard_normal(W.n_features(c, d))) * 0.01)
    truth.linear_weight = 0.9 - 0.2j
    rx = tx.copy()
    rx[2:4] = truth.model(tx) + 1e-3 * (rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n)))
    rx = rx.astype(np.complex64).astype(np.complex128)
    tx.tofile(tmp_path / "tx.c128")
    rx.tofile(tmp_path / "rx.c128")
    prefix = str(tmp_path / "out")
    r = subprocess.run([exe, str(tmp_path / "tx.c128"), str(tmp_path / "rx.c128"), str(n), prefix],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rd = lambda k, shape: np.fromfile(prefix + k, np.complex128).reshape(shape)  # noqa: E731
    sc = np.loadtxt(prefix + "_scalars.txt")
    ref = W.WdmPPE(c, d).train(tx, rx)
    scale = np.max(np.abs(ref.C))
    assert np.max(np.abs(rd("_wdm_C.c128", ref.C.shape) - ref.C)) < 1e-4 * scale
    assert np.max(np.abs(rd("_wdm_D.c128", ref.D.shape) - ref.D)) < 1e-4 * scale
    assert abs(complex(sc[0], sc[1]) - ref.linear_weight) < 1e-5
    assert abs(complex(sc[2], sc[3]) - ref.intercept) < 1e-5
    assert rel_l2(rd("_wdm_eq.c128", (2, n)), ref.equalize(tx, rx)) < 1e-5
    assert rel_l2(rd("_wdm_model.c128", (2, n)), ref.model(tx)) < 1e-5
    s = sino.SINO(6).train(tx[2:4], rx[2:4], solver="lstsq")
    sscale = np.max(np.abs(s.weights))
    assert np.max(np.abs(rd("_sino_W.c128", s.weights.shape) - s.weights)) < 1e-4 * sscale
    assert abs(complex(sc[4], sc[5]) - s.linear_weight) < 1e-5
    assert abs(complex(sc[6], sc[7]) - s.intercept) < 1e-5
    R = 6
    k = np.arange(R, n - R)
    eq_ref = rx[2:4].copy()
    for (m, nn, cf) in zip(*s.terms()):
        eq_ref[:, k] -= cf * sino._term(tx[2:4], k, m, nn)
    eq_ref /= s.linear_weight
    assert rel_l2(rd("_sino_eq.c128", (2, n)), eq_ref) < 1e-5
    model_ref = s.linear_weight * tx[2:4] + (rx[2:4] - s.linear_weight * eq_ref)
    assert rel_l2(rd("_sino_model.c128", (2, n)), model_ref) < 1e-5
    assert abs(sc[8] - oracle_cpu.find_certainty(tx, rx)) < 1e-9

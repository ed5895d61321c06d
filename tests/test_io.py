"""Dataset files of the reference (src/focss/functions.cpp:174-221,
src/tasks/wdm_run.cpp:55-77, src/tasks/wdm_scoring.cpp:79-103).

The transmission writer must reproduce, byte for byte, the file the
reference's own save_transmission wrote (tests/golden/transmission_ref.csv),
and the reader must give back what the reference's reader gives.  The field
binary keeps the header and sample-major layout.  The C++ façade's writer is
checked on the GPU (its fields live on the device)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from focss_gb300 import io

REF_CSV = os.path.join(ROOT, "tests", "golden", "transmission_ref.csv")


def test_transmission_writer_matches_reference_file(tmp_path, golden):
    out = tmp_path / "t.csv"
    io.save_transmission(out, golden["io_tx"], golden["io_rx"])
    assert out.read_bytes() == open(REF_CSV, "rb").read()


def test_transmission_reader(golden):
    tx, rx = io.load_transmission(REF_CSV, 2, 40)
    # the file holds 15 significant digits
    np.testing.assert_allclose(tx, golden["io_tx"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(rx, golden["io_rx"], rtol=1e-14, atol=0)


def test_transmission_reader_matches_reference_reader(tmp_path):
    from oracle import build as obuild
    if not obuild.reference_available():
        pytest.skip("reference source tree not present")
    obuild.build_ref()
    from oracle import ref
    want_tx, want_rx = ref.load_transmission(REF_CSV, 2, 40)
    tx, rx = io.load_transmission(REF_CSV, 2, 40)
    np.testing.assert_array_equal(tx, want_tx)
    np.testing.assert_array_equal(rx, want_rx)


def test_field_binary_layout_and_round_trip(tmp_path):
    rng = np.random.default_rng(2)
    chans = [rng.standard_normal((2, 16)) + 1j * rng.standard_normal((2, 16)) for _ in range(3)]
    (tmp_path / "set" / "tag").mkdir(parents=True)
    path = io.save_field(chans, tmp_path / "set", "tag", 7)
    raw = open(path, "rb").read()
    hdr = np.frombuffer(raw[:16], np.int32)
    np.testing.assert_array_equal(hdr, [3, 16, 2, 0])
    vals = np.frombuffer(raw[16:], np.complex128)
    assert vals.size == 3 * 2 * 16
    # sample-major, then channel, then mode (wdm_run.cpp:73-76)
    assert vals[0] == chans[0][0, 0] and vals[1] == chans[0][1, 0] and vals[2] == chans[1][0, 0]
    assert vals[6] == chans[0][0, 1]
    back = io.load_field(tmp_path / "set", "tag", 7)
    np.testing.assert_array_equal(back, np.concatenate(chans, axis=0))


def test_facade_io_example_builds(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    src = os.path.join(ROOT, "tests", "cpp", "facade_io.cpp")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-I" + os.path.join(ROOT, "include"),
                        src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_facade_writer_matches_reference_file(tmp_path, golden):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    lib = os.path.join(ROOT, "focss_gb300", "libfocss_gpu.so")
    exe = str(tmp_path / "facade_io")
    src = os.path.join(ROOT, "tests", "cpp", "facade_io.cpp")
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), src, lib,
                        "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    inp = tmp_path / "in.c128"
    np.concatenate([golden["io_tx"].ravel(), golden["io_rx"].ravel()]).astype(np.complex128).tofile(inp)
    out = tmp_path / "out.csv"
    r = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    # the device holds complex64: compare through the reader at FP32 precision
    tx, rx = io.load_transmission(out, 2, 40)
    np.testing.assert_allclose(tx, golden["io_tx"].astype(np.complex64), rtol=1e-7, atol=0)
    np.testing.assert_allclose(rx, golden["io_rx"].astype(np.complex64), rtol=1e-7, atol=0)
    ref_tx, ref_rx = io.load_transmission(str(out) + ".back", 2, 40)
    np.testing.assert_array_equal(ref_tx, tx)
    np.testing.assert_array_equal(ref_rx, rx)

"""Build recipe for the test oracle (test infrastructure only).

* ``build_oracle()`` compiles the FP64 C restatement ``focss_oracle.c`` into
  ``oracle/libfocss_oracle.so`` (gcc, portable flags, OpenMP over realizations).
  It runs on every machine that runs the tests or the CPU baseline.
* ``build_ref()`` compiles the reference's own unmodified sources, where they
  lie, together with the FFTW-API shim (``fftw_shim/``), the Armadillo
  stand-in (``arma_shim/``) and the C bridges (``ref_bridge.cpp``,
  ``ref_ppe_bridge.cpp``) into ``oracle/_ref/libfocss_ref.so``.  It needs the
  reference source tree, so it only runs where that tree exists; the outputs
  are git-ignored.  Reference sources are read in place, never copied.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference tree: FOCSS_REFERENCE_ROOT, else a `reference` directory beside
# this repository's root.
REF_ROOT = os.environ.get("FOCSS_REFERENCE_ROOT",
                          os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
ORACLE_SO = os.path.join(HERE, "libfocss_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libfocss_ref.so")

# Reference translation units on the path (relative to the reference's src/).
REF_SOURCES = [
    "focss/field.cpp",
    "focss/functions.cpp",
    "focss/solver/ssfm.cpp",
    "focss/module/fiber.cpp",
    "focss/module/amplifier.cpp",
    "focss/processing/modulation.cpp",
    "focss/equalizer/phase_shift_equalizer.cpp",
    "focss/equalizer/scalar_equalizer.cpp",
    "tasks/verification.cpp",
    # perturbation equalizers and the WDM scoring task's decision helpers,
    # against the project's Armadillo stand-in (arma_shim/)
    "focss/equalizer/sino.cpp",
    "focss/equalizer/wdm_sino.cpp",
    "tasks/wdm_scoring.cpp",
]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, "focss_oracle.c"), os.path.join(HERE, "focss_oracle.h")]
    if force or _stale(ORACLE_SO, srcs):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-fno-fast-math",
              "-ffp-contract=off", "-o", ORACLE_SO + ".tmp", srcs[0], "-lm", "-lpthread"])
        os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def reference_available() -> bool:
    return os.path.isfile(os.path.join(REF_ROOT, "src", "focss", "solver", "ssfm.cpp"))


def build_ref(force: bool = False) -> str | None:
    """Compile the reference's own sources into oracle/_ref (this container only)."""
    if not reference_available():
        return None
    src_root = os.path.join(REF_ROOT, "src")
    sources = [os.path.join(src_root, s) for s in REF_SOURCES]
    own = [os.path.join(HERE, "ref_bridge.cpp"), os.path.join(HERE, "fftw_shim", "fftw_shim.c"),
           os.path.join(HERE, "fftw_shim", "fftw3.h"), os.path.join(HERE, "focss_oracle.c"),
           os.path.join(HERE, "ref_ppe_bridge.cpp"), os.path.join(HERE, "arma_shim", "armadillo")]
    if not (force or _stale(REF_SO, sources + own)):
        return REF_SO
    os.makedirs(REF_DIR, exist_ok=True)
    obj_dir = os.path.join(REF_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    cxx = ["g++", "-std=c++11", "-O2", "-DNDEBUG", "-fPIC", "-ffp-contract=off",
           "-I", src_root, "-I", os.path.join(HERE, "fftw_shim"), "-I", os.path.join(HERE, "arma_shim")]
    jobs = []
    for s in sources + [own[0], own[4]]:
        o = os.path.join(obj_dir, os.path.basename(s).replace(".cpp", ".o"))
        jobs.append(cxx + ["-c", s, "-o", o])
    for s in (own[1], own[3]):
        o = os.path.join(obj_dir, os.path.basename(s).replace(".c", ".c.o"))
        jobs.append(["gcc", "-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    objs = [j[j.index("-o") + 1] for j in jobs]
    _run(["g++", "-shared", "-o", REF_SO + ".tmp"] + objs + ["-lm", "-lpthread"])
    os.replace(REF_SO + ".tmp", REF_SO)
    shutil.rmtree(obj_dir, ignore_errors=True)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))

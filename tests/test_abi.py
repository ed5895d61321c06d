"""The C-ABI library loads and exports exactly what include/*.h declares (CPU only)."""
import ctypes as C
import glob
import os
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        for m in re.finditer(r"FOCSS_API\s+[^;(]*?\b(focss_\w+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_header_declares_symbols():
    names = declared_symbols()
    assert "focss_ssfm_run" in names and "focss_ctx_create" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    from focss_gb300 import _lib
    L = _lib.lib()
    missing = [n for n in sorted(declared_symbols()) if not hasattr(L, n)]
    assert not missing, missing


def test_binding_table_covers_header():
    from focss_gb300 import _lib
    assert set(_lib.SIGNATURES) == declared_symbols()


def test_status_strings_and_version():
    from focss_gb300 import _lib
    L = _lib.lib()
    assert L.focss_abi_version() >= 1
    assert L.focss_status_string(0) == b"ok"
    assert L.focss_status_string(7) == b"no CUDA device"


def test_invalid_arguments_are_rejected_without_a_device():
    from focss_gb300 import _lib
    L = _lib.lib()
    assert L.focss_ctx_create(0, None) == 1  # null out-pointer
    h = C.c_void_p()
    st = L.focss_ctx_create(-1, C.byref(h))
    assert st in (1, 7)  # invalid device index, or no device at all
    assert L.focss_field_destroy(None) == 0
    assert L.focss_ctx_destroy(None) == 0


def test_product_path_does_not_touch_the_oracle():
    """No product source may import, link or load anything under oracle/."""
    pkg = os.path.join(ROOT, "focss_gb300")
    for path in glob.glob(os.path.join(pkg, "**", "*"), recursive=True):
        if os.path.isdir(path) or path.endswith((".so", ".o", ".pyc")):
            continue
        text = open(path, errors="ignore").read()
        assert "import oracle" not in text and "from oracle" not in text, path
        assert "focss_oracle" not in text and "libfocss_ref" not in text, path

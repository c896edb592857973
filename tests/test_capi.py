"""CPU tests of the C ABI: the library builds, loads and exports every symbol
declared in include/glass_gb300.h (no compute calls without a GPU)."""

from __future__ import annotations

import ctypes
import re

from tests.conftest import ROOT


def _declared_symbols() -> set[str]:
    text = (ROOT / "include" / "glass_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(glg_[a-z0-9_]+)\s*\(", text))


def test_library_builds_and_exports_header_symbols():
    from glass_gb300.build import build

    path = build()
    lib = ctypes.CDLL(str(path))
    declared = _declared_symbols()
    assert len(declared) >= 15
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, f"symbols declared but not exported: {missing}"
    assert lib.glg_version
    lib.glg_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.glg_version()


def test_python_binding_covers_header():
    from glass_gb300 import _lib

    declared = _declared_symbols()
    assert declared <= set(_lib.EXPORTED) | {"glg_version", "glg_last_error"}


def test_invalid_arguments_report_errors_without_gpu():
    """Argument checks run on the host and return GLG_ERR_INVALID."""
    from glass_gb300 import _lib

    lib = _lib.load_library(require_gpu=False)
    rc = lib.glg_plan_create(3, 10, None, ctypes.byref(ctypes.c_void_p()))
    assert rc == _lib.GLG_ERR_INVALID
    assert "power of two" in _lib.last_error()
    rc = lib.glg_iternorm(None, 1, 1, 0, None, None, None)
    assert rc == _lib.GLG_ERR_INVALID
    rc = lib.glg_iternorm(ctypes.c_void_p(8), 1, 1, 200, ctypes.c_void_p(8), ctypes.c_void_p(8), None)
    assert rc == _lib.GLG_ERR_INVALID
    assert "126" in _lib.last_error()
    rc = lib.glg_alm2map_host(None, None, 1, None, None, None, 0, None)
    assert rc == _lib.GLG_ERR_INVALID
    assert "null plan" in _lib.last_error()
    assert lib.glg_alm2map_host_workspace(None, 3) == 0

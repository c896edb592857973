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
    assert "120" in _lib.last_error()
    rc = lib.glg_alm2map_host(None, None, 1, None, None, None, 0, None)
    assert rc == _lib.GLG_ERR_INVALID
    assert "null plan" in _lib.last_error()
    assert lib.glg_alm2map_host_workspace(None, 3) == 0


def test_host_output_runs_tile_the_rings_and_pixels():
    """The runs of glg_alm2map_host (host arithmetic of the C library): tiles
    and ring pairs from the equator end down to pair 0, and pixel bands that
    hold exactly each run's rings and together cover every pixel once."""
    import numpy as np

    from glass_gb300 import _lib

    lib = _lib.load_library(require_gpu=False)
    out = np.zeros(8 * 8, dtype=np.int64)
    for nside in [2 ** e for e in range(14)]:
        n = lib.glg_host_output_runs(nside, out.ctypes.data, 8)
        npairs, npix = 2 * nside, 12 * nside * nside
        ntiles = (npairs + 127) // 128
        assert n == min(ntiles, 8)
        runs = out[:8 * n].reshape(n, 8)
        nph = np.array([4 * (p + 1) if p + 1 < nside else 4 * nside for p in range(npairs)], dtype=np.int64)
        assert runs[0, 1] == ntiles and runs[-1, 0] == 0 and runs[0, 3] == npairs and runs[-1, 2] == 0
        bands = []
        for k, (t0, t1, p0, p1, n0, n1, s0, s1) in enumerate(runs):
            assert t0 < t1 and p0 == 128 * t0 and p1 == min(128 * t1, npairs)
            if k:
                assert t1 == runs[k - 1, 0] and p1 == runs[k - 1, 2]
            q1 = p1 if p1 < npairs else npairs - 1  # the equator has no separate south ring
            assert n1 - n0 == nph[p0:p1].sum() and s1 - s0 == nph[p0:q1].sum()
            bands += [(n0, n1)] + ([(s0, s1)] if s1 > s0 else [])
        bands.sort()
        assert bands[0][0] == 0 and bands[-1][1] == npix
        assert all(a[1] == b[0] for a, b in zip(bands, bands[1:]))
    assert lib.glg_host_output_runs(0, out.ctypes.data, 8) == _lib.GLG_ERR_INVALID
    assert lib.glg_host_output_runs(2048, out.ctypes.data, 7) == _lib.GLG_ERR_INVALID


def test_gather_host_concatenates_in_order():
    """glg_gather_host (host memcpy split over threads, no device call) equals
    numpy's concatenation, for thread counts whose byte ranges start and end
    inside pieces, with empty pieces, and rejects bad arguments."""
    import numpy as np

    from glass_gb300 import _lib

    lib = _lib.load_library(require_gpu=False)
    rng = np.random.default_rng(0)
    for sizes in ([4097] * 820, [0, 5, 0, 300_000, 1, 0, 700_001, 3], [1_000_003]):
        parts = [rng.standard_normal(n) for n in sizes]
        ref = np.concatenate(parts)
        for nt in (1, 3, 8, 64):
            out = np.full(ref.size, np.nan)
            src = (ctypes.c_void_p * len(parts))(*[p.ctypes.data for p in parts])
            nb = (ctypes.c_int64 * len(parts))(*[p.nbytes for p in parts])
            assert lib.glg_gather_host(src, nb, len(parts), out.ctypes.data, nt) == _lib.GLG_OK
            np.testing.assert_array_equal(out, ref)
    assert lib.glg_gather_host(None, None, 0, None, 4) == _lib.GLG_OK
    assert lib.glg_gather_host(None, None, 2, None, 4) == _lib.GLG_ERR_INVALID
    bad = (ctypes.c_int64 * 1)(-8)
    src = (ctypes.c_void_p * 1)(8)
    assert lib.glg_gather_host(src, bad, 1, ctypes.c_void_p(8), 1) == _lib.GLG_ERR_INVALID

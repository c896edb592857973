"""CPU tests of the host-side logic mirroring glass/fields.py (no GPU calls)."""

from __future__ import annotations

import numpy as np
import pytest

import glass_gb300 as g
from glass_gb300 import fields


def test_cls2cov_values_and_buffer_reuse():
    # glass tests/core/test_fields.py:166-252 semantics
    gen = g.cls2cov([np.asarray([1.0, 0.5, 0.3]), None, np.asarray([0.7, 0.6, 0.1])], 3, 2, 2)
    cov = next(gen)
    assert cov.shape == (3, 3)
    np.testing.assert_array_equal(cov[:, 0], [0.5, 0.25, 0.15])
    np.testing.assert_array_equal(cov[:, 1:], 0.0)
    with pytest.raises(ValueError, match="negative values in cl"):
        next(g.cls2cov([np.asarray([-1.0, 0.5, 0.3]), np.ones(3), np.ones(3)], 3, 3, 2))
    cls = [np.asarray(a) for a in ([1.0, 0.5, 0.3], [0.8, 0.4, 0.2], [0.7, 0.6, 0.1],
                                   [0.9, 0.5, 0.3], [0.6, 0.3, 0.2], [0.8, 0.7, 0.4])]
    gen = g.cls2cov(cls, 3, 3, 2)
    c1 = next(gen)
    c1c = c1.copy()
    c2 = next(gen)
    c3 = next(gen)
    np.testing.assert_array_equal(c1[:, 0], [0.45, 0.25, 0.15])
    np.testing.assert_array_equal(c1, c3)
    np.testing.assert_array_equal(c2, c3)
    np.testing.assert_array_equal(c1c[:, 0], [0.5, 0.25, 0.15])


def test_cls2cov_matches_golden(golden):
    gls6 = [golden[f"gls6_{i}"] for i in range(21)]
    got = np.stack([c.copy() for c in g.cls2cov(gls6, 41, 6, 5)])
    np.testing.assert_array_equal(got, golden["cls2cov_cfg2_nc5"])


def test_triangle_numbers():
    for n in range(2000):
        assert g.nfields_from_nspectra(n * (n + 1) // 2) == n
    for t in [2, 4, 5, 7, 8, 9, 11]:
        with pytest.raises(ValueError, match=f"invalid number of spectra: {t}"):
            g.nfields_from_nspectra(t)
        with pytest.raises(ValueError, match=f"not a triangle number: {t}"):
            fields._inv_triangle_number(t)


def test_getcl_and_enumerate():
    cls = [np.asarray([i, j], dtype=float) for i in range(6) for j in range(i, -1, -1)]
    for i in range(6):
        for j in range(6):
            np.testing.assert_array_equal(np.sort(g.getcl(cls, i, j)), [min(i, j), max(i, j)])
            assert g.getcl(cls, i, j, lmax=0).shape == (1,)
            r = g.getcl(cls, i, j, lmax=20)
            assert r.shape == (21,)
            np.testing.assert_array_equal(r[2:], 0)
    idx = [(i, j) for i in range(5) for j in range(i, -1, -1)]
    assert [(a, b) for a, b, _ in g.enumerate_spectra(range(15))] == idx
    np.testing.assert_array_equal(g.spectra_indices(3), [[0, 0], [1, 1], [1, 0], [2, 2], [2, 1], [2, 0]])


def test_glass_to_healpix_alm_numpy():
    inp = np.asarray([0, 10, 11, 20, 21, 22, 30, 31, 32, 33], dtype=np.complex128)
    np.testing.assert_array_equal(fields._glass_to_healpix_alm(inp),
                                  [0, 10, 20, 30, 11, 21, 31, 22, 32, 33])


def test_generate_field_count_error():
    fs = [lambda x, v: x, lambda x, v: x]
    with pytest.raises(ValueError, match="mismatch between number of fields and gls"):
        list(g.generate(fs, [np.ones(10), np.ones(10)], nside=16))


def test_iternorm_empty_error():
    with pytest.raises(ValueError, match="empty covariance"):
        list(g.iternorm([np.ones(0)]))


def test_transformations():
    x = np.linspace(-2, 2, 11)
    np.testing.assert_array_equal(g.grf.Normal()(x, 1.0), x)
    np.testing.assert_array_equal(g.grf.Lognormal(1.0)(x, 0.3), np.expm1(x - 0.15))
    np.testing.assert_array_equal(g.grf.Lognormal(0.7)(x, 0.3), 0.7 * np.expm1(x - 0.15))
    np.testing.assert_array_equal(g.grf.SquaredNormal(0.5, 2.0)(x, 0.3), 2.0 * ((x - 0.5) ** 2 - 1))
    assert g.grf.fused_kind(g.grf.Lognormal(0.7)) == ("lognormal", 0.7)
    assert g.grf.fused_kind(g.grf.Normal()) == ("normal", 1.0)
    assert g.grf.fused_kind(lambda x, v: x) is None


def test_no_cpu_fallback_without_gpu():
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from glass_gb300 import _lib

    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.lib()


def test_serving_memory_model():
    from glass_gb300 import serving

    a = serving.request_bytes(128, 256, 3)
    b = serving.request_bytes(128, 256, 6)
    assert 0 < a < b
    assert serving.request_bytes(1024, 2048, 20) > 20 * 12 * 1024 * 1024 * 4
    r = serving.Request(gls=[np.ones(9)], nside=4, shifts=[1.0], arrival=1.0)
    r.finished = 3.5
    assert r.latency == 2.5 and r.nshell == 1 and r.lmax == 8


def test_cls_files_interchange_with_reference(tmp_path):
    """save_cls / load_cls use the reference's .npz layout (glass/user.py:42-86):
    a file written by the reference's own save_cls (tests/golden/make_golden_cls.py)
    loads here, and the file written here holds the same arrays under the same
    keys."""
    import numpy as np

    import glass_gb300 as g
    from tests.conftest import ROOT
    from tests.golden.make_golden_cls import spectra

    cls = spectra()
    ref = ROOT / "tests" / "golden" / "glass_cls_ref.npz"
    back = g.load_cls(ref)
    assert len(back) == 4 and all(np.array_equal(a, b) for a, b in zip(cls, back))
    g.save_cls(tmp_path / "mine.npz", cls)
    with np.load(tmp_path / "mine.npz") as mine, np.load(ref) as theirs:
        assert sorted(mine.files) == sorted(theirs.files)
        for k in theirs.files:
            np.testing.assert_array_equal(mine[k], theirs[k])
            assert mine[k].dtype == theirs[k].dtype


def test_fft_radix_constants_exact():
    """The FP32 ring FFT's radix constants, written as (hi, lo) float pairs in
    glass_gb300/csrc/ringfft32.cu: hi the nearest float of the exact value and
    hi + lo within 1e-15 of it (products with them round once)."""
    import re
    from pathlib import Path

    src = (Path(__file__).resolve().parent.parent / "glass_gb300" / "csrc" / "ringfft32.cu").read_text()

    def table(name):
        body = re.search(name + r"\[\] = \{(.*?)\n\};", src, re.S).group(1)
        vals = [float(v) for v in re.findall(r"(-?[0-9.]+(?:e-?[0-9]+)?)f", body)]
        return np.asarray(vals, dtype=np.float32).astype(np.float64).reshape(-1, 2)

    hi, lo = table("kOddHi"), table("kOddLo")
    k = 0
    for r in (3, 5, 7, 11, 13):
        for j in range(r):
            ex = np.array([np.cos(2 * np.pi * j / r), np.sin(2 * np.pi * j / r)])
            assert np.all(hi[k] == ex.astype(np.float32))
            assert np.all(np.abs(hi[k] + lo[k] - ex) < 1e-15)
            k += 1
    assert k == hi.shape[0]
    for name, val in (("R2", np.sqrt(0.5)), ("C8", np.cos(np.pi / 8)), ("S8", np.sin(np.pi / 8))):
        h = np.float32(val)
        lval = float(np.float32(re.search(name + r"L = (-?[0-9.]+(?:e-?[0-9]+)?)f", src).group(1)))
        assert abs(float(h) + lval - val) < 1e-15


def test_pinned_output_buffers_reused_only_when_dropped(monkeypatch):
    """The host-output synthesis hands out rows of a pooled page-locked
    buffer: a buffer is reused only once every map of the earlier call that
    wrote into it has been dropped (pinning 8 GB anew costs more than a
    step)."""
    import torch

    import glass_gb300.fields as f

    real_empty = torch.empty

    def empty(*a, **k):  # no page-locked memory without a GPU
        k.pop("pin_memory", None)
        return real_empty(*a, **k)

    monkeypatch.setattr(f.torch, "empty", empty)
    monkeypatch.setattr(f, "_PINNED", [])
    e = f._pinned_maps(3, 5)
    rows = list(e[1])
    first = id(e[1])
    del e
    e = f._pinned_maps(3, 5)
    assert id(e[1]) != first  # the first call's maps are alive
    second = id(e[1])
    del e
    keep = rows[1]
    del rows
    e = f._pinned_maps(3, 5)
    assert id(e[1]) == second  # the first buffer is still viewed by `keep`
    del e, keep
    e = f._pinned_maps(3, 5)
    assert id(e[1]) in (first, second) and len(f._PINNED) == 2

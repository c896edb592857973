"""GPU parity tests: the CUDA path (through the C ABI) against the oracle.

Tolerances: plain form (FP64 throughout) <= 1e-12 relative to the largest
oracle value; iternorm and the Philox integer stream bit-exact; the
glass-side glue (alm assembly) to 1e-15 absolute against the reference's own
fixtures.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import oracle.fields as of
import oracle.rng as orng
import oracle.sht as osht
from tests.conftest import random_alm, rel_err, spectra_powerlaw15, spectra_damped12

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def g(cuda_lib):
    import glass_gb300

    return glass_gb300


# ------------------------------------------------------------- iternorm


def _iternorm_gpu(cov):
    import torch

    from glass_gb300 import fields

    w, status = fields._iternorm_device(torch.as_tensor(cov, device="cuda").contiguous())
    return w.cpu().numpy(), fields._first_bad(status)


def test_iternorm_bit_exact_vs_oracle(g, golden):
    for nc in (5, 2):
        cov = golden[f"cls2cov_cfg2_nc{nc}"]
        w, bad = _iternorm_gpu(cov)
        wo, bado = of.iternorm_stack(cov)
        assert bad == bado == -1
        np.testing.assert_array_equal(w, wo)
        np.testing.assert_allclose(w, golden[f"iternorm_cfg2_nc{nc}"], rtol=1e-13, atol=1e-16)


def test_iternorm_bit_exact_large_k(g):
    gls, _ = spectra_damped12(40, 300, seed=4)
    cov = np.stack([c.copy() for c in of.cls2cov(gls, 301, 40, 39)])
    w, bad = _iternorm_gpu(cov)
    wo, bado = of.iternorm_stack(cov)
    assert bad == bado == -1
    np.testing.assert_array_equal(w, wo)


def test_iternorm_generator_api(g, golden):
    for k in (0, 1, 2):
        for nd in ("0d", "nd"):
            rows = [golden[f"iternorm_k{k}_{nd}_in{i}"] for i in range(3)]
            ws = list(g.iternorm(iter(rows)))
            for i, w in enumerate(ws):
                np.testing.assert_allclose(w, golden[f"iternorm_k{k}_{nd}_row{i}"], rtol=1e-13, atol=1e-16)


def test_iternorm_errors(g):
    with pytest.raises(ValueError, match="shape mismatch"):
        list(g.iternorm([np.ones(1), np.ones((5, 2))]))
    gen = g.iternorm([np.asarray([1.0]), np.asarray([0.1, 1.0])])
    assert next(gen).shape == (1,)
    with pytest.raises(ValueError, match="not positive definite"):
        next(gen)


# -------------------------------------------------------------- variates


def test_philox_normals_vs_oracle(g):
    import torch

    r = g.rng.Generator(1234)
    z = r.complex_normal(50_000, sid=7, offset=100).cpu().numpy()
    zo = orng.complex_normals(1234, 7, 100, 50_000)
    assert rel_err(z, zo) < 1e-13
    z32 = r.complex_normal(50_000, sid=7, offset=100, dtype=torch.complex64).cpu().numpy()
    # FP32 Box-Muller of the same 53-bit uniforms: about an FP32 ulp
    assert np.max(np.abs(z32 - zo) / (1.0 + np.abs(zo))) < 2e-6
    assert np.sqrt(np.mean(np.abs(z32 - zo) ** 2) / np.mean(np.abs(zo) ** 2)) < 1.5e-7


# --------------------------------------------------------- transforms


@pytest.mark.parametrize(("nside", "lmax"), [(1, 2), (2, 3), (4, 11), (8, 7), (16, 40), (32, 64),
                                             (64, 128), (64, 200)])
def test_alm2map_plain_vs_oracle(g, nside, lmax):
    alm = random_alm(lmax, seed=lmax, nmaps=3)
    got = g.healpix.alm2map(list(alm), nside, pol=False)
    ref = osht.alm2map(alm, nside, lmax)
    assert rel_err(got, ref) < TOL


def test_alm2map_plain_vs_direct_sum(g):
    nside, lmax = 8, 20
    alm = random_alm(lmax, seed=5)
    assert rel_err(g.healpix.alm2map(alm, nside), osht.alm2map_direct(alm, nside, lmax)) < TOL


def test_alm2map_extended_range(g):
    """lmax >> nside: high-m, near-pole values need the scaled recurrence."""
    nside, lmax = 32, 1000
    alm = random_alm(lmax, seed=9)
    got = g.healpix.alm2map(alm, nside)
    ref = osht.alm2map(alm, nside, lmax)
    assert rel_err(got, ref) < TOL


@pytest.mark.parametrize("spin", [1, 2])
@pytest.mark.parametrize(("nside", "lmax"), [(4, 11), (16, 40), (32, 95)])
def test_alm2map_spin_vs_oracle(g, spin, nside, lmax):
    e = random_alm(lmax, seed=1)
    b = random_alm(lmax, seed=2)
    q, u = g.healpix.alm2map_spin([e, b], nside, spin, lmax)
    qo, uo = osht.alm2map_spin([e, b], nside, spin, lmax)
    assert rel_err(q, qo) < 1e-11
    assert rel_err(u, uo) < 1e-11


@pytest.mark.parametrize("niter", [0, 3])
def test_map2alm_vs_oracle(g, niter):
    nside, lmax = 16, 47
    rng = np.random.default_rng(3)
    m = rng.standard_normal(12 * nside * nside)
    got = g.healpix.map2alm(m, lmax=lmax, iter=niter)
    ref = osht.map2alm(m, lmax, iter=niter)
    assert rel_err(got, ref) < 1e-11


def test_map2alm_roundtrip(g):
    nside, lmax = 32, 40
    alm = random_alm(lmax, seed=11)
    m = g.healpix.alm2map(alm, nside)
    back = g.healpix.map2alm(m, lmax=lmax, iter=3)
    # uniform-weight quadrature with 3 refinements (healpy's default iter)
    assert rel_err(back, alm) < 1e-5
    assert rel_err(back, osht.map2alm(osht.alm2map(alm, nside, lmax), lmax, iter=3)) < 1e-11


def test_almxfl_and_multalm(g, golden):
    np.testing.assert_array_equal(g.multalm(golden["multalm_alm"], golden["multalm_bl"]),
                                  golden["multalm_out"])
    # reference test values (tests/core/test_harmonics.py:15-52)
    np.testing.assert_array_equal(g.multalm(np.array([1.0, 2, 3, 4, 5, 6]), np.array([2.0, 0.5, 1.0])),
                                  [2.0, 1.0, 1.5, 4.0, 5.0, 6.0])
    np.testing.assert_array_equal(g.multalm(np.array([1.0, 2, 3, 4, 5, 6]), np.array([0.0, 1.0, 0.0])),
                                  [0.0, 2.0, 3.0, 0.0, 0.0, 0.0])
    assert g.multalm(np.array([]), np.array([])).shape == (0,)
    alm = random_alm(30, seed=4)
    fl = np.random.default_rng(0).standard_normal(25)
    np.testing.assert_array_equal(g.healpix.almxfl(alm, fl), osht.almxfl(alm, fl))


# ------------------------------------------------------- field generation


@pytest.mark.parametrize("tag,ncorr", [("all", None), ("nc1", 1)])
def test_generate_vs_reference_fixture(g, golden, tag, ncorr):
    gls3 = [golden[f"gls3_{i}"] for i in range(6)]
    fields = [g.grf.Lognormal(1.0), g.grf.Lognormal(0.7), g.grf.Normal()]
    maps = np.stack(list(g.generate(fields, gls3, 8, ncorr=ncorr, rng=np.random.default_rng(42))))
    assert rel_err(maps, golden[f"generate_maps_{tag}"]) < TOL


def test_generate_lognormal_vs_reference_fixture(g, golden):
    gls4 = [golden[f"gls4_{i}"] for i in range(10)]
    with pytest.deprecated_call():
        maps = np.stack(list(g.generate_lognormal(gls4, 4, rng=np.random.default_rng(7))))
    assert rel_err(maps, golden["lognormal4_maps"]) < TOL


def test_correlated_alm_vs_reference_fixture(g, golden):
    from glass_gb300 import fields

    gls3 = [golden[f"gls3_{i}"] for i in range(6)]
    b = fields._FieldBatcher(gls3, 8, None, np.random.default_rng(42), "plain")
    alm = np.stack([b.alm(t, 1)[0].cpu().numpy() for t in range(3)])
    np.testing.assert_allclose(alm, golden["generate_alm_all"], rtol=0, atol=1e-15)


def _correlate(g, w, nshell, lmax, k, t0, z, z_first, dtype, out):
    import torch

    from glass_gb300._lib import c_p, check, lib, ptr, stream_ptr

    check(lib().glg_alm_correlate(c_p(ptr(w)), nshell, lmax, k, t0, None if z is None else c_p(ptr(z)), z_first,
                                  ctypes.c_uint64(42), ctypes.c_uint64(7), dtype, c_p(ptr(out)),
                                  c_p(stream_ptr(torch.device("cuda", 0)))), "glg_alm_correlate")


@pytest.mark.parametrize(("nshell", "lmax", "k", "split", "hostz"),
                         [(12, 300, 5, 5, False), (12, 300, 5, 7, True), (50, 200, 39, 23, False),
                          (30, 130, 0, 11, False), (9, 64, 39, 4, True), (9, 64, 47, 4, True), (20, 70, 60, 9, False)])
def test_alm_correlate_fast_window(g, nshell, lmax, k, split, hostz):
    """The fast form's correlated alm (register window for k + 1 <= 40, the
    shared-memory window above): within FP32 rounding of the FP64 sums, and a
    call split into two groups of shells (the second drawing its window of
    earlier variates again) gives the same bits as one call."""
    import torch

    from glass_gb300 import _lib

    kp, nalm = k + 1, (lmax + 1) * (lmax + 2) // 2
    gen = torch.Generator().manual_seed(nshell + k)
    w64 = (torch.randn((nshell, lmax + 1, kp), generator=gen, dtype=torch.float64) * 0.3).cuda()
    w32 = w64.float()
    z64 = torch.randn((nshell, nalm), generator=gen, dtype=torch.complex128).cuda() if hostz else None
    z32 = z64.to(torch.complex64) if hostz else None
    ref = torch.empty((nshell, nalm), dtype=torch.complex128, device="cuda")
    _correlate(g, w64, nshell, lmax, k, 0, z64, 0, _lib.GLG_F64, ref)
    one = torch.empty((nshell, nalm), dtype=torch.complex64, device="cuda")
    _correlate(g, w32, nshell, lmax, k, 0, z32, 0, _lib.GLG_F32, one)
    two = torch.empty_like(one)
    _correlate(g, w32[:split].contiguous(), split, lmax, k, 0, z32[:split].contiguous() if hostz else None, 0,
               _lib.GLG_F32, two[:split])
    zlo = max(0, split - k)
    _correlate(g, w32[split:].contiguous(), nshell - split, lmax, k, split,
               z32[zlo:].contiguous() if hostz else None, zlo, _lib.GLG_F32, two[split:])
    torch.cuda.synchronize()
    assert torch.equal(torch.view_as_real(one), torch.view_as_real(two))
    d = (one.to(torch.complex128) - ref).abs()
    assert float(d.max()) < 1e-5 * float(ref.abs().max())
    assert float(torch.sqrt((d * d).mean() / (ref.abs() ** 2).mean())) < 1e-6


def test_generate_philox_vs_oracle(g):
    """3 shells at nside 64 / lmax 128 with the device stream."""
    gls = spectra_powerlaw15(3, 128)
    r = g.rng.Generator(42)
    maps = np.stack(list(g.generate_lognormal(gls, 64, rng=r)))
    sid0 = 0
    ref = np.stack(list(of.generate_lognormal(
        gls, 64, [1.0] * 3, z_of_shell=lambda t, s: orng.complex_normals(42, sid0 + t, 0, s))))
    assert rel_err(maps, ref) < TOL


def test_generate_batched_matches_per_shell(g):
    """Batched shells (one SHT launch) equal shell-by-shell results."""
    gls, lam = spectra_damped12(6, 64, seed=2)
    fields = [g.grf.Lognormal(float(x)) for x in lam]
    a = np.stack(list(g.generate(fields, gls, 32, rng=g.rng.Generator(5))))
    import os

    os.environ["GLASS_GB300_BATCH_BYTES"] = "1"
    try:
        b = np.stack(list(g.generate(fields, gls, 32, rng=g.rng.Generator(5))))
    finally:
        del os.environ["GLASS_GB300_BATCH_BYTES"]
    assert rel_err(a, b) < 1e-14


def test_generate_custom_callables(g):
    """glass tests/core/test_fields.py:403-438: x and x**2 of the same field."""
    fields = [lambda x, var: x, lambda x, var: x**2]
    gls = [np.ones(10), np.ones(10), np.ones(10)]
    res = list(g.generate(fields, gls, nside=16))
    assert len(res) == 2 and all(r.shape == (12 * 16 * 16,) for r in res)
    np.testing.assert_allclose(res[1], res[0] ** 2, atol=1e-5)
    assert len(list(g.generate(fields, gls, nside=16, ncorr=1))) == 2


def test_generate_grf_ncorr_invariance(g):
    from glass_gb300 import fields

    gls = [np.asarray([1.0, 0.5, 0.1])]
    a = list(fields._generate_grf(gls, 4, rng=np.random.default_rng(42)))
    b = list(fields._generate_grf(gls, 4, ncorr=1, rng=np.random.default_rng(42)))
    np.testing.assert_array_equal(a[0], b[0])
    with pytest.raises(ValueError, match="all gls are empty"):
        list(fields._generate_grf([np.asarray([])], 4))


def test_generate_not_posdef_raises_at_shell(g):
    gls = [np.ones(4), np.ones(4), np.ones(4) * 5.0]  # C10 > sqrt(C00 C11)
    gen = g.generate([g.grf.Normal(), g.grf.Normal()], gls, 4, rng=np.random.default_rng(1))
    first = next(gen)
    assert first.shape == (192,)
    with pytest.raises(ValueError, match="not positive definite"):
        next(gen)


def test_torch_in_torch_out(g):
    import torch

    gls = [torch.as_tensor(c, device="cuda") for c in spectra_powerlaw15(2, 16)]
    maps = list(g.generate([g.grf.Lognormal(), g.grf.Lognormal()], gls, 8))
    assert all(isinstance(m, torch.Tensor) and m.is_cuda for m in maps)


# --------------------------------------------------------------- lensing


def test_from_convergence_vs_oracle(g):
    nside = 16
    rng = np.random.default_rng(0)
    kappa = rng.random(12 * nside * nside) * 10
    assert g.from_convergence(kappa) == ()
    psi, alpha, gamma = g.from_convergence(kappa, potential=True, deflection=True, shear=True,
                                           discretized=False)
    lmax = 3 * nside - 1
    alm = osht.map2alm(kappa, lmax, iter=3)
    ell = np.arange(lmax + 1, dtype=float)
    fl = np.zeros_like(ell)
    fl[1:] = -2 / (ell[1:] * (ell[1:] + 1))
    alm = osht.almxfl(alm, fl)
    np.testing.assert_allclose(psi, osht.alm2map(alm, nside, lmax), rtol=0, atol=1e-10 * np.abs(psi).max())
    alm = osht.almxfl(alm, np.sqrt(ell * (ell + 1)))
    a0, a1 = osht.alm2map_spin([alm, None], nside, 1, lmax)
    assert rel_err(alpha, a0 + 1j * a1) < 1e-10
    fl = np.zeros_like(ell)
    fl[1:] = np.sqrt((ell[1:] - 1) * (ell[1:] + 2)) / 2
    alm = osht.almxfl(alm, fl)
    g0, g1 = osht.alm2map_spin([alm, None], nside, 2, lmax)
    assert rel_err(gamma, g0 + 1j * g1) < 1e-10
    for combo in ((True, False, False), (False, True, False), (False, False, True),
                  (True, True, False), (True, False, True), (False, True, True)):
        res = g.from_convergence(kappa, potential=combo[0], deflection=combo[1], shear=combo[2],
                                 discretized=False)
        assert len(res) == sum(combo)


# -------------------------------------------------------------- fast form
# Tolerance: relative RMS map error <= 1e-6 against the FP64 oracle (FP32
# maps, split-precision 3xTF32 Legendre contraction, FP32 ring FFTs).
FAST_RMS = 1e-6


def rel_rms(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b**2)))


def _fast_synth(alm, nside, lmax):
    import torch

    from glass_gb300 import healpix as hp

    a = torch.as_tensor(np.atleast_2d(alm), device="cuda").to(torch.complex64)
    return hp.synth(a, nside, lmax, form="fast").cpu().numpy()


@pytest.mark.parametrize(("nside", "lmax", "nmaps"), [(4, 11, 1), (16, 40, 3), (32, 64, 8),
                                                      (64, 128, 40), (32, 300, 5), (128, 256, 2),
                                                      (1, 2, 1), (2, 5, 2), (8, 31, 2), (16, 47, 3),
                                                      (64, 63, 4)])
def test_alm2map_fast_vs_oracle(g, nside, lmax, nmaps):
    ell = np.concatenate([np.arange(m, lmax + 1) for m in range(lmax + 1)])
    alm = random_alm(lmax, seed=7, nmaps=nmaps) * (ell + 1.0) ** -0.65
    got = _fast_synth(alm, nside, lmax)
    ref = osht.alm2map(alm, nside, lmax)
    assert rel_rms(got, ref) < FAST_RMS
    assert rel_err(got, ref) < 2e-5


def test_alm2map_fast_table_and_recurrence_paths(g):
    """The fast form with the resident P_lm table (default) and, with the
    table budget at 0, with lambda from the FP32 recurrence and its seeds."""
    from glass_gb300 import _lib

    lib = _lib.lib()
    cases = [(32, 64, 3), (64, 128, 8), (32, 300, 2)]
    for budget, table in ((160 << 30, True), (0, False)):
        lib.glg_set_plm_table_budget(budget)
        _lib.clear_plans()
        try:
            for nside, lmax, nmaps in cases:
                ell = np.concatenate([np.arange(m, lmax + 1) for m in range(lmax + 1)])
                alm = random_alm(lmax, seed=8, nmaps=nmaps) * (ell + 1.0) ** -0.65
                got = _fast_synth(alm, nside, lmax)
                assert _lib.get_plan(nside, lmax).has_plm_table == table
                assert rel_rms(got, osht.alm2map(alm, nside, lmax)) < FAST_RMS
        finally:
            lib.glg_set_plm_table_budget(160 << 30)
            _lib.clear_plans()


def test_generate_fast_vs_plain(g):
    """Same Philox stream: fast form within 1e-6 RMS of the FP64 plain form."""
    gls, lam = spectra_damped12(6, 128, seed=1)
    fields = [g.grf.Lognormal(float(x)) for x in lam]
    plain = np.stack(list(g.generate(fields, gls, 64, rng=g.rng.Generator(3), form="plain")))
    fast = np.stack(list(g.generate(fields, gls, 64, rng=g.rng.Generator(3), form="fast")))
    assert fast.dtype == np.float32
    for s in range(6):
        assert rel_rms(fast[s], plain[s]) < FAST_RMS


# ------------------------------------------------------- Poisson counts


def test_poisson_counts_bit_exact_vs_oracle(g):
    """Counts of glass/points.py:252-348 from the Philox stream: bit-exact
    with the host restatement, for float64 and float32 delta (same values),
    with bias, visibility, clipped and NaN pixels and means far above 256."""
    import torch

    rng = np.random.default_rng(11)
    npix = 12 * 64 * 64
    d = np.exp(rng.normal(0.0, 1.2, npix)) - 1.0
    d[:50] = -5.0
    d[50:60] = np.nan
    d[60:80] = 2000.0  # expected counts of ~10^4: forty pieces
    vis = rng.uniform(0.0, 1.0, npix)
    ngal = 5.0 * npix / g.points.ARCMIN2_SPHERE  # 5 per pixel
    scale = g.points.ARCMIN2_SPHERE / npix * ngal
    got = g.points.counts_from_delta(ngal, d, 1.3, vis, rng=g.rng.Generator(7))
    ref = orng.poisson_counts(d, bias=1.3, scale=scale, vis=vis, seed=7, stream=0)
    assert got.dtype == np.int64
    np.testing.assert_array_equal(got, ref)
    assert np.all(got[:60] == 0)
    lam_big = (1.3 * 2000.0 + 1.0) * scale * vis[60:80]  # up to ~1.3e4: many 256-mean pieces
    assert np.all(np.abs(got[60:80] - lam_big) < 6 * np.sqrt(lam_big) + 1)
    d32 = d.astype(np.float32)
    got32 = g.points.counts_from_delta(ngal, torch.as_tensor(d32, device="cuda"), rng=g.rng.Generator(7))
    assert isinstance(got32, torch.Tensor) and got32.dtype == torch.int64
    np.testing.assert_array_equal(got32.cpu().numpy(),
                                  orng.poisson_counts(d32.astype(np.float64), scale=scale, seed=7, stream=0))
    # remove_monopole subtracts the mean of the biased delta
    got_m = g.points.counts_from_delta(ngal, d[80:], remove_monopole=True, rng=g.rng.Generator(2))
    n2 = d.size - 80
    ref_m = orng.poisson_counts(d[80:], offset=float(np.mean(d[80:])), scale=g.points.ARCMIN2_SPHERE / n2 * ngal,
                                seed=2, stream=0)
    assert np.mean(got_m == ref_m) > 0.999  # the offset is a device mean: may differ in the last bit
    assert g.points.counts_from_delta(ngal, np.zeros(0)).size == 0


# ------------------------------------------------- map-level lensing (8f)


@pytest.fixture(scope="module")
def lensing_golden():
    from tests.conftest import ROOT

    return np.load(ROOT / "tests" / "golden" / "glass_lensing.npz")


def _cosmo():
    import sys

    from tests.conftest import ROOT

    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    from cosmo_stub import FlatLCDM

    return FlatLCDM()


@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_multiplane_convergence_vs_reference(g, lensing_golden, tag):
    """Device convergence planes equal the reference's, bit for bit."""
    import torch

    gd = lensing_golden
    mpc = g.MultiPlaneConvergence(_cosmo())
    mpc_t = g.MultiPlaneConvergence(_cosmo())
    for z, w, d, ref in zip(gd[f"mpc_{tag}_z"], gd[f"mpc_{tag}_w"], gd[f"mpc_{tag}_delta"], gd[f"mpc_{tag}_kappa"]):
        mpc.add_plane(d.copy(), float(z), float(w))
        mpc_t.add_plane(torch.as_tensor(d, device="cuda"), float(z), float(w))
        assert mpc.kappa.dtype == ref.dtype
        np.testing.assert_array_equal(mpc.kappa, ref)
        assert isinstance(mpc_t.kappa, torch.Tensor) and mpc_t.kappa.is_cuda
        np.testing.assert_array_equal(mpc_t.kappa.cpu().numpy(), ref)
    with pytest.raises(ValueError, match="source redshift must be increasing"):
        mpc.add_plane(gd[f"mpc_{tag}_delta"][0], 0.1)


def test_ang2pix_vs_oracle(g):
    import oracle.lensing as olens

    rng = np.random.default_rng(5)
    for nside in (1, 16, 256, 2048):
        lon = rng.uniform(-400, 400, 200_000)
        lat = np.degrees(np.arcsin(rng.uniform(-1, 1, lon.size)))
        lat[:4] = [90.0, -90.0, 0.0, 41.8103148958]  # poles, equator, z = 2/3
        np.testing.assert_array_equal(g.healpix.ang2pix(nside, lon, lat, lonlat=True),
                                      olens.ang2pix_lonlat(nside, lon, lat))
        theta, phi = olens.lonlat_to_thetaphi(lon, lat)
        np.testing.assert_array_equal(g.healpix.ang2pix(nside, theta, phi), olens.ang2pix_ring(nside, theta, phi))


@pytest.mark.parametrize("reduced", [True, False])
def test_galaxy_shear_vs_reference(g, lensing_golden, reduced):
    gd = lensing_golden
    got = g.galaxy_shear(gd["shear_lon"], gd["shear_lat"], gd["shear_eps"], gd["shear_kappa"], gd["shear_g1"],
                         gd["shear_g2"], reduced_shear=reduced)
    assert got.dtype == np.complex128
    np.testing.assert_allclose(got, gd[f"shear_{int(reduced)}"], rtol=1e-15, atol=0)


def test_positions_in_their_pixels_vs_oracle(g):
    """positions_from_delta (glass/points.py:443-540): every position lies in
    its pixel (pixels in order, as many as the Poisson count), batches end at
    pixel boundaries, positions do not depend on the batch size, and inside
    the pixels they follow the oracle's uniform sampler (two-sample KS)."""
    import torch
    from scipy import stats

    import oracle.lensing as olens

    nside = 64
    npix = 12 * nside * nside
    rng = np.random.default_rng(4)
    delta = np.exp(rng.normal(0.0, 0.8, npix) - 0.32) - 1.0
    delta[:100] = -1.0  # empty pixels
    ngal = 20.0 * npix / g.points.ARCMIN2_SPHERE
    out = list(g.points.positions_from_delta(ngal, torch.as_tensor(delta, device="cuda"), 1.1, batch=100_000,
                                             rng=g.rng.Generator(9)))
    counts = g.points.counts_from_delta(ngal, delta, 1.1, rng=g.points._Keyed(9, 0))
    lon = torch.cat([b[0] for b in out]).cpu().numpy()
    lat = torch.cat([b[1] for b in out]).cpu().numpy()
    sizes = np.array([b[2] for b in out])
    assert sizes.sum() == counts.sum() == lon.size and np.all(sizes <= 100_000)
    assert np.all(np.isin(np.cumsum(sizes), np.cumsum(counts)))  # batches end at pixel boundaries
    ipix = np.repeat(np.arange(npix), counts)
    np.testing.assert_array_equal(olens.ang2pix_lonlat(nside, lon, lat), ipix)
    assert lon.min() >= 0 and lon.max() < 360 and lat.min() >= -90 and lat.max() <= 90
    # the galaxy's counter, not its batch, keys its draws
    again = list(g.points.positions_from_delta(ngal, delta, 1.1, batch=7_777, rng=g.rng.Generator(9)))
    np.testing.assert_array_equal(np.concatenate([b[0] for b in again]), lon)
    np.testing.assert_array_equal(np.concatenate([b[1] for b in again]), lat)
    # distribution within the pixels: position in the pixel's box vs the oracle sampler
    lon_o, lat_o = olens.randang_lonlat(nside, ipix, np.random.default_rng(1))
    zlo, zhi, phic, dphi = olens.pixel_box(nside, ipix)

    def box_coords(lo, la):
        z = np.sin(np.radians(la))
        dp = np.mod(np.radians(lo) - phic + np.pi, 2 * np.pi) - np.pi
        return (z - zlo) / (zhi - zlo), dp / dphi

    u, v = box_coords(lon, lat)
    uo, vo = box_coords(lon_o, lat_o)
    assert np.all((u >= 0) & (u <= 1) & (np.abs(v) <= 0.5))
    assert stats.ks_2samp(u, uo).pvalue > 1e-4
    assert stats.ks_2samp(v, vo).pvalue > 1e-4


def test_positions_from_delta_reference_cases(g):
    """The cases of the reference's test_positions_from_delta: scalar and
    broadcast populations, count shapes, negative delta, no vis, the
    TypeError, and numpy in / numpy out."""
    import torch

    import oracle.lensing as olens

    def cat(gen):
        lon, lat, cnt = [], [], 0
        for a, b, c in gen:
            lon.append(np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a))
            lat.append(np.asarray(b.cpu() if isinstance(b, torch.Tensor) else b))
            cnt = cnt + c
        return (np.concatenate(lon) if lon else np.zeros(0)), (np.concatenate(lat) if lat else np.zeros(0)), cnt

    pts = g.points
    nside = 128
    npix = 12 * nside * nside
    for kw in ({"bias": 0.8, "vis": np.ones(npix)}, {"bias": None, "vis": np.ones(npix), "bias_model": lambda x: x},
               {"bias": 0.8, "vis": None}, {"bias": 0.8, "vis": np.ones(npix), "remove_monopole": True}):
        kw = dict(kw)
        lon, lat, count = cat(pts.positions_from_delta(1e-3, np.zeros(npix), kw.pop("bias"), kw.pop("vis"), **kw))
        assert int(count) == count and lon.shape == lat.shape == (count,)
        assert abs(count - 1e-3 * pts.ARCMIN2_SPHERE) < 6 * np.sqrt(1e-3 * pts.ARCMIN2_SPHERE)
    lon, lat, count = cat(pts.positions_from_delta(1e-3, np.full(npix, -1.0), None, np.ones(npix)))
    assert count == 0 and lon.size == 0 and lat.size == 0
    lon, lat, count = cat(pts.positions_from_delta(1e-3, np.random.default_rng(0).normal(100, 1, npix), 0.8,
                                                   np.ones(npix)))
    assert lon.shape == lat.shape == (count,)
    lon, lat, count = cat(pts.positions_from_delta(np.array([1e-3, 2e-3]), np.zeros(12), 0.8, np.ones(12)))
    assert count.shape == (2,) and lon.shape == lat.shape == (count.sum(),)
    assert count[1] > 1.8 * count[0]
    lon, lat, count = cat(pts.positions_from_delta(1e-3, np.zeros((3, 2, 12)), 0.8, np.ones(12)))
    assert count.shape == (3, 2) and lon.shape == (count.sum(),)
    vis = np.ones(12)
    lon, lat, count = cat(pts.positions_from_delta(np.array([1e-3, 2e-3]), np.zeros((3, 1, 12)), 0.8, vis))
    assert count.shape == (3, 2) and lon.shape == (count.sum(),)
    vis[:6] = 0.0  # only the southern hemisphere is visible
    lon, lat, count = cat(pts.positions_from_delta(np.array([1e-3, 2e-3]), np.zeros((3, 1, 12)), 0.8, vis))
    assert count.shape == (3, 2) and lon.shape == (count.sum(),)
    assert olens.ang2pix_lonlat(1, lon, lat).min() >= 6
    with pytest.raises(TypeError, match="bias_model must be callable"):
        next(pts.positions_from_delta(1e-3, np.zeros(12), 0.8, vis, bias_model=0))
    one = next(pts.positions_from_delta(1e-3, np.zeros(12)))
    assert isinstance(one[0], np.ndarray) and one[0].dtype == np.float64
    one = next(pts.positions_from_delta(1e-3, torch.zeros(12, device="cuda", dtype=torch.float64)))
    assert isinstance(one[0], torch.Tensor) and one[0].is_cuda


def test_autotuner_picks_block_sizes(g):
    """The first fast transform of a plan times every ring-FFT bucket and
    keeps a block size per bucket; results stay within the fast tolerance."""
    import torch

    from glass_gb300 import healpix as hp

    nside, lmax = 64, 150
    ell = np.concatenate([np.arange(m, lmax + 1) for m in range(lmax + 1)])
    alm = random_alm(lmax, seed=3, nmaps=5) * (ell + 1.0) ** -0.65
    got = hp.synth(torch.as_tensor(alm, device="cuda").to(torch.complex64), nside, lmax, form="fast")
    b = hp.buckets(nside, lmax)
    assert b and all(x["threads"] in (128, 256, 512, 1024) for x in b)
    assert sum(x["pairs"] for x in b) == 2 * nside
    assert rel_rms(got.cpu().numpy(), osht.alm2map(alm, nside, lmax)) < FAST_RMS


@pytest.mark.parametrize(("nside", "lmax"), [(64, 128), (256, 512), (512, 1024)])
def test_fast_maps_written_to_host_memory(g, nside, lmax):
    """Fast synthesis into host memory (glg_alm2map_host: ring-tile runs from
    the equator to the poles, each copied while the next computes; 1, 4 and
    8 runs here) gives the same bits as into device memory, pinned or
    pageable, with a fused epilogue; generate with numpy spectra (which takes
    that route) equals it with torch spectra."""
    import torch

    from glass_gb300 import healpix as hp

    nm = 3
    epi = ([g._lib.EPI_LOGNORMAL, g._lib.EPI_NONE, g._lib.EPI_LOGNORMAL], [0.2, 0.0, 0.5], [1.0, 1.0, 2.0])
    alm = torch.as_tensor(random_alm(lmax, seed=8, nmaps=nm) * 0.1, device="cuda").to(torch.complex64)
    ref = hp.synth(alm, nside, lmax, epilogue=epi, form="fast").cpu()
    for pinned in (True, False):
        host = torch.full((nm, 12 * nside * nside), float("nan"), dtype=torch.float32, pin_memory=pinned)
        got = hp.synth(alm, nside, lmax, epilogue=epi, form="fast", out=host)
        torch.cuda.synchronize()
        assert got is host
        torch.testing.assert_close(host, ref, rtol=0, atol=0)
    if nside != 64:
        return
    pinned = torch.empty((nm, 12 * nside * nside), dtype=torch.float32, pin_memory=True)
    g._lib.host_device_pointer(pinned)  # mapped pinned memory has a device address
    with pytest.raises(ValueError):
        g._lib.host_device_pointer(torch.empty(4))  # pageable memory has none
    gls, lam = spectra_damped12(4, 2 * nside)
    fields = [g.grf.Lognormal(float(x)) for x in lam]
    a = list(g.generate(fields, gls, nside, rng=g.rng.Generator(3), form="fast"))
    b = list(g.generate(fields, [torch.as_tensor(c, device="cuda") for c in gls], nside, rng=g.rng.Generator(3),
                        form="fast"))
    assert all(isinstance(x, np.ndarray) and x.dtype == np.float32 for x in a)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y.cpu().numpy())


def test_synth_graph_replays_equal_direct_calls(g):
    """A captured fast synthesis replays to the same maps as direct calls,
    for new inputs written into its static buffer, with a fused epilogue."""
    import torch

    from glass_gb300 import healpix as hp

    nside, lmax, nm = 32, 64, 3
    epi = ([g._lib.EPI_LOGNORMAL, g._lib.EPI_NONE, g._lib.EPI_LOGNORMAL], [0.2, 0.0, 0.5], [1.0, 1.0, 2.0])
    graph = hp.SynthGraph(nside, lmax, nm, epilogue=epi)
    for seed in (1, 2):
        alm = torch.as_tensor(random_alm(lmax, seed=seed, nmaps=nm) * 0.1, device="cuda").to(torch.complex64)
        got = graph(alm).clone()
        graph.status()
        ref = hp.synth(alm, nside, lmax, epilogue=epi, form="fast")
        torch.testing.assert_close(got, ref, rtol=0, atol=0)


def test_synth_graph_device_epilogue(g):
    """One captured graph, its epilogue read from device memory: replays
    with different epilogues (Gaussian, lognormal, and a lognormal of
    variance >= 4 that takes the FP64 tail refinement) equal direct calls
    with those epilogues, bit for bit."""
    import torch

    from glass_gb300 import healpix as hp

    nside, lmax, nm = 64, 128, 3
    graph = hp.SynthGraph(nside, lmax, nm, device_epilogue=True)
    L = g._lib.EPI_LOGNORMAL
    # maps of standard deviation ~2.2 (variance ~5): a few pixels of the
    # variance-5 lognormal maps cross the tail threshold, far fewer than the
    # list holds, so the refined set does not depend on the listing order
    alm = torch.as_tensor(random_alm(lmax, seed=9, nmaps=nm) * 0.043, device="cuda").to(torch.complex64)
    epis = [None,
            ([L, g._lib.EPI_NONE, L], [0.2, 0.0, 0.5], [1.0, 1.0, 2.0]),
            ([L, L, L], [5.0, 0.3, 4.5], [0.7, 1.0, 1.5])]
    for epi in epis:
        got = graph(alm, epilogue=epi).clone()
        graph.status()
        ref = hp.synth(alm, nside, lmax, epilogue=epi, form="fast")
        torch.testing.assert_close(got, ref, rtol=0, atol=0)

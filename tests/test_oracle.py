"""CPU tests of the oracle: pinned against brute force, KATs and the reference."""

from __future__ import annotations

import numpy as np
import pytest

import oracle.fields as of
import oracle.rng as orng
import oracle.sht as osht
from tests.conftest import random_alm, rel_err


@pytest.mark.parametrize(("nside", "lmax"), [(1, 2), (2, 5), (4, 11), (8, 20), (8, 30)])
def test_alm2map_matches_direct_sum(nside, lmax):
    alm = random_alm(lmax, seed=nside + lmax)
    assert rel_err(osht.alm2map(alm, nside, lmax), osht.alm2map_direct(alm, nside, lmax)) < 1e-13


@pytest.mark.parametrize("spin", [1, 2])
@pytest.mark.parametrize(("nside", "lmax"), [(2, 6), (4, 11), (8, 16)])
def test_spin_matches_goldberg(spin, nside, lmax):
    e = random_alm(lmax, seed=1)
    b = random_alm(lmax, seed=2)
    q, u = osht.alm2map_spin([e, b], nside, spin, lmax)
    qd, ud = osht.alm2map_spin_direct(e, b, nside, spin, lmax)
    assert rel_err(q, qd) < 1e-11
    assert rel_err(u, ud) < 1e-11


def test_known_answers():
    nside, lmax = 8, 4
    theta, _ = osht.pix_angles(nside)
    a = np.zeros(osht.nalm(lmax), complex)
    a[0] = 2.0
    np.testing.assert_allclose(osht.alm2map(a, nside, lmax), 2 / np.sqrt(4 * np.pi), rtol=1e-14)
    a[:] = 0
    a[osht.alm_index(1, 0, lmax)] = 1.5
    np.testing.assert_allclose(osht.alm2map(a, nside, lmax),
                               1.5 * np.sqrt(3 / (4 * np.pi)) * np.cos(theta), atol=1e-14)


def test_map2alm_roundtrip():
    nside, lmax = 16, 16
    alm = random_alm(lmax, seed=3)
    m = osht.alm2map(alm, nside, lmax)
    assert rel_err(osht.map2alm(m, lmax, iter=3), alm) < 1e-6


def test_extended_range_large_m():
    """High-m modes on near-polar rings underflow FP64 without the exponent scale."""
    nside, lmax = 64, 400
    alm = np.zeros(osht.nalm(lmax), complex)
    for m in (300, 350, 399):
        alm[osht.alm_index(lmax, m, lmax)] = 1.0
    F = osht.alm2ring(alm, nside, lmax)
    assert np.all(np.isfinite(F))
    assert np.abs(F).max() > 1e-3  # non-negligible near the equator


def _lambda_mp(l, m, z):  # noqa: E741
    """Normalised lambda_lm(z) (Condon-Shortley phase) in 50-digit arithmetic:
    the closed form of lambda_mm from sqrt(1 - z^2), then the three-term
    recurrence in l."""
    mp = pytest.importorskip("mpmath").mp
    mp.dps = 50
    z = mp.mpf(z)
    v = mp.mpf(1) / (4 * mp.pi)
    for k in range(1, m + 1):
        v *= mp.mpf(2 * k - 1) / (2 * k)
    p2 = (-1) ** m * mp.sqrt((2 * m + 1) * v) * mp.sqrt(1 - z * z) ** m
    if l == m:
        return p2
    p1 = mp.sqrt(2 * m + 3) * z * p2
    for n in range(m + 2, l + 1):
        a = mp.sqrt(mp.mpf(4 * n * n - 1) / (n * n - m * m))
        b = mp.sqrt(mp.mpf((n - 1) ** 2 - m * m) / (4 * (n - 1) ** 2 - 1))
        p2, p1 = p1, a * (z * p1 - b * p2)
    return p1


def test_legendre_at_benchmark_degrees_vs_50_digit_values():
    """The oracle's FP64 Legendre sums at the benchmark's nside 2048 / lmax 4096
    against 50-digit values at the same ring heights z (one unit alm per map,
    so F_m(ring) = lambda_lm(z_ring)).  The 50-digit recurrence agrees with
    mpmath's hypergeometric spherical harmonics to 20 digits.  Away from the
    poles the FP64 values are within 1e-12 of the scale sqrt((2l+1)/4pi); on
    the two rings nearest each pole (z = 1 - 8e-8), where the recurrence at
    l = 4096 loses more to rounding, within 1e-9."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 50
    for ell, m, th in [(4096, 2048, 0.7), (4096, 10, 0.01)]:
        ref = mpmath.re(mpmath.spherharm(ell, m, th, 0))
        assert abs(_lambda_mp(ell, m, mpmath.cos(th)) - ref) < mpmath.mpf(10) ** -20
    nside, lmax = 2048, 4096
    z = osht.ring_info(nside)[0]
    rings = np.array([1, 2, 64, 700, 2048, 4096, 6000, 8190], dtype=np.intc)  # 1-based ring numbers
    pairs = [(4096, 0), (4096, 1), (4096, 2048), (4096, 4096), (3001, 1500), (100, 7)]
    alm = np.zeros((len(pairs), osht.nalm(lmax)), complex)
    for k, (ell, m) in enumerate(pairs):
        alm[k, osht.alm_index(ell, m, lmax)] = 1.0
    F = osht.alm2ring(alm, nside, lmax, rings)
    for k, (ell, m) in enumerate(pairs):
        scale = np.sqrt((2 * ell + 1) / (4 * np.pi))
        for j, r in enumerate(rings):
            ref = float(_lambda_mp(ell, m, float(z[r - 1])))
            tol = 1e-9 if r in (1, 2, 8190) else 1e-12
            assert abs(F[k, j, m].real - ref) < tol * scale, (ell, m, r, F[k, j, m].real, ref)
            assert F[k, j, m].imag == 0.0


def test_philox_known_answers():
    # Random123 Philox4x32-10 published known-answer vectors
    np.testing.assert_array_equal(orng.philox4x32_10([0, 0, 0, 0], [0, 0]),
                                  [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8])
    np.testing.assert_array_equal(orng.philox4x32_10([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2),
                                  [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD])
    np.testing.assert_array_equal(
        orng.philox4x32_10([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]),
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1])


def test_philox_normals_moments():
    z = orng.complex_normals(42, 3, 0, 100_000)
    assert abs(z.real.mean()) < 0.02 and abs(z.imag.mean()) < 0.02
    assert abs(z.real.std() - 1) < 0.02 and abs(z.imag.std() - 1) < 0.02
    z2 = orng.complex_normals(42, 3, 500, 10)
    np.testing.assert_array_equal(z2, z[500:510])


# ------------------------------------------------- pinned to the reference


def test_iternorm_matches_reference(golden):
    for nc in (5, 2):
        w, bad = of.iternorm_stack(golden[f"cls2cov_cfg2_nc{nc}"])
        assert bad == -1
        np.testing.assert_allclose(w, golden[f"iternorm_cfg2_nc{nc}"], rtol=1e-13, atol=1e-16)


def test_iternorm_ulp_distance_to_reference(golden):
    """The oracle's iternorm rows -- bit-exact with the GPU kernel
    (tests/test_gpu_parity.py) -- against the reference's numpy rows on the
    the 10-shell covariances: at most 2 ulp apart and about 87 % of the entries
    identical (the sums run in another order than numpy's matmuls)."""
    for nc in (5, 2):
        wo, bad = of.iternorm_stack(golden[f"cls2cov_cfg2_nc{nc}"])
        ref = golden[f"iternorm_cfg2_nc{nc}"]
        big = np.maximum(np.abs(wo), np.abs(ref))
        ulp = np.where(wo == ref, 0.0, np.abs(wo - ref) / np.spacing(np.where(big > 0, big, 1.0)))
        assert bad == -1
        assert ulp.max() <= 2.0
        assert np.mean(ulp == 0) > 0.85


@pytest.mark.parametrize("k", [0, 1, 2])
@pytest.mark.parametrize("nd", ["0d", "nd"])
def test_iternorm_reference_test_matrices(golden, k, nd):
    rows = [golden[f"iternorm_k{k}_{nd}_in{i}"] for i in range(3)]
    kmax = max(r.shape[-1] for r in rows) - 1
    stack = np.zeros((3,) + rows[0].shape[:-1] + (kmax + 1,))
    for i, r in enumerate(rows):
        stack[i, ..., : r.shape[-1]] = r
    stack = stack.reshape(3, -1, kmax + 1)
    w, bad = of.iternorm_stack(stack)
    for i, r in enumerate(rows):
        kk = r.shape[-1] - 1
        ref = golden[f"iternorm_k{k}_{nd}_row{i}"].reshape(-1, kk + 1)
        np.testing.assert_allclose(w[i][:, kmax - kk:], ref, rtol=1e-13, atol=1e-16)


def test_iternorm_block_sums_equal_dense_sums(golden):
    """The sums over the non-zero block of m (what the GPU kernel does) give
    the same bits as sums over all k indices: the skipped terms are exact
    zeros.  Correlated spectra with k up to 59, perturbed into
    non-positive-definite cases too."""
    rng = np.random.default_rng(0)
    for nshell, k, nl in [(1, 0, 5), (3, 2, 7), (10, 9, 33), (10, 3, 33), (40, 39, 40), (60, 59, 12)]:
        ell = np.arange(nl)
        amp = 10 ** rng.uniform(-3, -1, nshell)
        auto = [a * (ell + 1.0) ** -1.3 for a in amp]
        gls = [np.exp(-abs(i - j) / 3.0) * np.sqrt(auto[i] * auto[j]) for i in range(nshell) for j in range(i, -1, -1)]
        cov = np.stack(list(of.cls2cov(gls, nl, nshell, k)))
        for c in (cov, cov * rng.uniform(0.5, 1.5, cov.shape)):
            w1, b1 = of.iternorm_stack(c)
            w2, b2 = of.iternorm_stack(c, dense=True)
            assert b1 == b2
            np.testing.assert_array_equal(w1.view(np.uint64), w2.view(np.uint64))


def test_iternorm_not_posdef():
    cov = np.array([[[1.0, 0.0]], [[0.1, 1.0]]])  # second row: var 0.1 < corr^2
    _, bad = of.iternorm_stack(cov)
    assert bad == 1


def test_cls2cov_matches_reference(golden):
    gls6 = [golden[f"gls6_{i}"] for i in range(21)]
    for nc in (5, 2):
        got = np.stack([c.copy() for c in of.cls2cov(gls6, 41, 6, nc)])
        np.testing.assert_array_equal(got, golden[f"cls2cov_cfg2_nc{nc}"])


@pytest.mark.parametrize("tag,ncorr", [("all", None), ("nc1", 1)])
def test_generate_alm_matches_reference(golden, tag, ncorr):
    gls3 = [golden[f"gls3_{i}"] for i in range(6)]
    alm = np.stack(list(of.generate_grf_alm(gls3, ncorr=ncorr)))
    np.testing.assert_allclose(alm, golden[f"generate_alm_{tag}"], rtol=0, atol=1e-15)


def test_generate_lognormal_matches_reference(golden):
    gls4 = [golden[f"gls4_{i}"] for i in range(10)]
    rng = np.random.default_rng(7)
    maps = np.stack(list(of.generate_lognormal(
        gls4, 4, [1.0] * 4, z_of_shell=lambda t, s: rng.standard_normal((s, 2)) @ np.asarray([1, 1j]))))
    np.testing.assert_allclose(maps, golden["lognormal4_maps"], rtol=1e-13, atol=1e-15)


def test_multalm_and_reorder_match_reference(golden):
    np.testing.assert_array_equal(of.multalm(golden["multalm_alm"], golden["multalm_bl"]),
                                  golden["multalm_out"])
    np.testing.assert_array_equal(of.glass_to_healpix_alm(golden["reorder_in"]), golden["reorder_out"])
    # the reference's own permutation test (tests/core/test_fields.py:649-655)
    inp = np.array([0, 10, 11, 20, 21, 22, 30, 31, 32, 33], dtype=complex)
    np.testing.assert_array_equal(of.glass_to_healpix_alm(inp),
                                  np.array([0, 10, 20, 30, 11, 21, 31, 22, 32, 33], dtype=complex))


def test_poisson_exp_accuracy():
    """The library-free e^{-x} of the count sampler is within a few ulp of exp."""
    from oracle import lib

    xs = np.concatenate([np.linspace(0.0, 256.0, 20001), [1e-300, 0.5 * np.log(2.0), 255.999]])
    got = np.array([lib().orc_exp_neg(float(x)) for x in xs])
    ref = np.exp(-xs)
    assert np.max(np.abs(got - ref) / ref) < 5e-16


def test_poisson_counts_statistics_and_streams():
    rng = np.random.default_rng(0)
    d = rng.normal(0.0, 0.4, 400_000)
    c1 = orng.poisson_counts(d, scale=5.0, seed=1, stream=2)
    assert c1.dtype == np.int64
    np.testing.assert_array_equal(c1, orng.poisson_counts(d, scale=5.0, seed=1, stream=2))
    assert np.mean(c1 != orng.poisson_counts(d, scale=5.0, seed=1, stream=3)) > 0.5
    lam = np.clip((d + 1.0) * 5.0, 0.0, None)
    n = d.size
    assert abs(c1.mean() - lam.mean()) < 5 * np.sqrt(lam.mean() / n)
    # Var[N] = E[lam] + Var[lam] for a Poisson mixture
    assert abs(c1.var() / (lam.mean() + lam.var()) - 1.0) < 0.02
    # pieces of mean 256: large means keep mean and variance
    big = orng.poisson_counts(np.zeros(100_000), scale=1000.0, seed=5)
    assert abs(big.mean() - 1000.0) < 5 * np.sqrt(1000.0 / 1e5)
    assert abs(big.var() / 1000.0 - 1.0) < 0.03
    # clipping, NaN and the visibility / bias / offset arithmetic
    z = orng.poisson_counts(np.array([-3.0, np.nan, -1.0]), scale=5.0)
    np.testing.assert_array_equal(z, [0, 0, 0])
    vis = rng.uniform(0.0, 1.0, 1000)
    a = orng.poisson_counts(d[:1000], bias=1.5, offset=0.1, scale=2.0, vis=vis, seed=9)
    b = orng.poisson_counts(((1.5 * d[:1000] - 0.1) + 1.0) * 2.0 * vis, scale=1.0, bias=1.0, offset=1.0, seed=9)
    assert np.mean(a == b) > 0.99  # same uniforms, expected counts equal up to rounding


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
def test_multiplane_convergence_matches_reference(lensing_golden, tag):
    import oracle.lensing as olens

    g = lensing_golden
    mpc = olens.MultiPlaneConvergence(_cosmo())
    for z, w, d, ref in zip(g[f"mpc_{tag}_z"], g[f"mpc_{tag}_w"], g[f"mpc_{tag}_delta"], g[f"mpc_{tag}_kappa"]):
        mpc.add_plane(d.copy(), float(z), float(w))
        assert mpc.kappa.dtype == ref.dtype
        np.testing.assert_array_equal(mpc.kappa, ref)


def test_ang2pix_ring_pixel_centres_and_offsets():
    import oracle.lensing as olens

    for nside in (1, 2, 4, 16, 64):
        z, _, nph, phi0, start = osht.ring_info(nside)
        theta = np.repeat(np.arccos(z), nph)
        j = np.concatenate([np.arange(n) for n in nph])
        phi = np.repeat(phi0, nph) + 2 * np.pi * j / np.repeat(nph, nph)
        ref = np.repeat(start, nph) + j
        np.testing.assert_array_equal(olens.ang2pix_ring(nside, theta, phi), ref)
        # small offsets inside the pixel keep it; longitudes wrap
        rng = np.random.default_rng(nside)
        d = 0.05 * np.pi / (4 * nside)
        np.testing.assert_array_equal(
            olens.ang2pix_ring(nside, theta + rng.uniform(-d, d, theta.size) * 0.2,
                               phi + 2 * np.pi * rng.integers(-2, 3, phi.size)), ref)


def test_pixel_box_holds_each_pixel():
    """Ring geometry of RING pixels agrees with the SHT ring table, and the
    (z, phi) box of a pixel holds every point that ang2pix puts in it; the
    pixel fills half the box (the acceptance rate of the position sampler)."""
    import oracle.lensing as olens

    rng = np.random.default_rng(3)
    for nside in (1, 2, 4, 16, 64):
        z, _, nph, phi0, start = osht.ring_info(nside)
        p = np.arange(12 * nside * nside)
        r, j, n = olens.pix_ring(nside, p)
        np.testing.assert_array_equal(start[r - 1] + j, p)
        np.testing.assert_array_equal(nph[r - 1], n)
        np.testing.assert_allclose(olens.ring_z(nside, r), z[r - 1], rtol=0, atol=1e-15)
        zlo, zhi, phic, dphi = olens.pixel_box(nside, p)
        np.testing.assert_allclose(phic, phi0[r - 1] + 2 * np.pi * j / n, rtol=1e-15, atol=1e-15)
        zz = rng.uniform(-1, 1, 400_000)
        pp = rng.uniform(0, 2 * np.pi, zz.size)
        q = olens.ang2pix_ring(nside, np.arccos(zz), pp)
        zlo, zhi, phic, dphi = olens.pixel_box(nside, q)
        assert np.all((zz >= zlo) & (zz <= zhi))
        assert np.all(np.abs(np.mod(pp - phic + np.pi, 2 * np.pi) - np.pi) <= 0.5 * dphi)
        # a pixel (area 4 pi / npix) fills at least half of its box, and draws
        # in the box land in the pixel at that rate
        zlo, zhi, phic, dphi = olens.pixel_box(nside, p)
        fill = 4 * np.pi / p.size / ((zhi - zlo) * dphi)
        assert fill.min() > 0.5 - 1e-12 and fill.max() <= 1.0
        for pix in (0, 6 * nside * nside):
            zlo, zhi, phic, dphi = olens.pixel_box(nside, np.full(200_000, pix))
            hit = olens.ang2pix_ring(nside, np.arccos(zlo + rng.random(zlo.size) * (zhi - zlo)),
                                     phic + (rng.random(zlo.size) - 0.5) * dphi) == pix
            assert abs(hit.mean() - fill[pix]) < 0.01
    lon, lat = olens.randang_lonlat(4, np.repeat(np.arange(192), 50), rng)
    np.testing.assert_array_equal(olens.ang2pix_lonlat(4, lon, lat), np.repeat(np.arange(192), 50))
    assert lon.min() >= 0 and lon.max() < 360 and lat.min() >= -90 and lat.max() <= 90


def test_galaxy_shear_matches_reference(lensing_golden):
    import oracle.lensing as olens

    g = lensing_golden
    for red in (True, False):
        got = olens.galaxy_shear(g["shear_lon"], g["shear_lat"], g["shear_eps"], g["shear_kappa"],
                                 g["shear_g1"], g["shear_g2"], reduced_shear=red)
        np.testing.assert_array_equal(got, g[f"shear_{int(red)}"])

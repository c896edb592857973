"""Pixel window functions (healpy.pixwin, glass/healpix.py:313-356) and the
discretized shear of from_convergence (glass/lensing.py:360-362).

healpy's tables are data files that are not available offline, so parity
with them is unpinned.  The oracle (``oracle.pixwin``) restates the
definition -- the pixel-averaged harmonics' power, spin 0 and spin 2 -- and
evaluates it by direct pair sums of P_l and d^l_22 (scipy); the GPU evaluates
the same definition through pair moments and the kernels' power series in
sin^2(gamma/2).  CPU tests pin the oracle's series form against its direct
sums and its pixel quadrature against a finer one; GPU tests compare the
library with the oracle (1e-13) and check the known behaviour of the window
(1 at l = 0, the exact dipole identity, self-similarity in l / nside).
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle.pixwin as opw
import oracle.sht as osht
from tests.conftest import random_alm, rel_err

TOL = 1e-13


# ------------------------------------------------------------- oracle (CPU)


@pytest.mark.parametrize("nside", [1, 2, 4])
def test_oracle_series_matches_direct_sums(nside):
    lmax = 4 * nside
    d0, d2 = opw.pixwin_direct(nside, lmax)
    s0, s2 = opw.pixwin_series(nside, lmax)
    assert np.max(np.abs(d0 - s0)) < 1e-14
    assert np.max(np.abs(d2 - s2)) < 1e-14


@pytest.mark.parametrize("nside", [2, 8])
def test_oracle_quadrature_converged(nside):
    lmax = 4 * nside
    a0, a2 = opw.pixwin_series(nside, lmax)
    b0, b2 = opw.pixwin_series(nside, lmax, q=12)
    assert np.max(np.abs(a0 - b0)) < 2e-11
    assert np.max(np.abs(a2 - b2)) < 2e-11


def test_oracle_pixel_classes_cover_the_sphere():
    for nside in (1, 2, 3, 8, 16):
        assert sum(w for _, _, w in opw.pixel_classes(nside)) == 12 * nside * nside


def test_oracle_known_answers():
    nside = 4
    pw0, pw2 = opw.pixwin_series(nside, 4 * nside)
    assert pw0[0] == 1.0 and pw2[0] == 0.0 and pw2[1] == 0.0
    # l = 1: P_1(cos g) = cos g, so pw0_1^2 is the mean squared length of the
    # pixels' mean position vectors
    tot = 0.0
    for i, jj, w in opw.pixel_classes(nside):
        n, wt = opw.pixel_nodes(nside, i, jj)
        tot += w * np.sum((wt[:, None] * n).sum(axis=0) ** 2)
    assert abs(pw0[1] ** 2 - tot / (12 * nside * nside)) < 1e-15
    assert np.all(np.diff(pw0) < 0) and np.all(np.diff(pw2[2:]) < 0)


# ----------------------------------------------------------------- GPU


@pytest.fixture(scope="module")
def g(cuda_lib):
    import glass_gb300

    return glass_gb300


@pytest.mark.gpu
@pytest.mark.parametrize("nside", [1, 2, 4, 8])
def test_pixwin_vs_oracle_direct(g, nside):
    lmax = 4 * nside
    pw0, pw2 = g.healpix.pixwin(nside, lmax=lmax, pol=True)
    d0, d2 = opw.pixwin_direct(nside, lmax)
    assert np.max(np.abs(pw0 - d0)) < TOL
    assert np.max(np.abs(pw2 - d2)) < TOL


@pytest.mark.gpu
def test_pixwin_vs_oracle_series_nside32(g):
    pw0, pw2 = g.healpix.pixwin(32, pol=True)
    assert pw0.shape == (96,) and pw2.shape == (96,)
    s0, s2 = opw.pixwin_series(32, 95)
    assert np.max(np.abs(pw0 - s0)) < TOL
    assert np.max(np.abs(pw2 - s2)) < TOL
    assert np.array_equal(g.healpix.pixwin(32), pw0)


@pytest.mark.gpu
def test_pixwin_self_similar(g):
    # the window depends on l times the pixel size: nside 128 and 256 agree
    # at the same l / nside to the pixels' residual shape change
    a = g.healpix.pixwin(128, lmax=512)
    b = g.healpix.pixwin(256, lmax=1024)
    assert a[0] == 1.0 and b[0] == 1.0
    assert np.max(np.abs(a[::4] - b[::8][: a[::4].size])) < 2e-3
    assert np.all(np.diff(b) < 0)


@pytest.mark.gpu
def test_pixwin_limits(g):
    with pytest.raises(ValueError):
        g.healpix.pixwin(8, lmax=33)
    with pytest.raises(ValueError):
        g.healpix.pixwin(16384)


@pytest.mark.gpu
def test_alm2map_pixwin(g):
    nside, lmax = 16, 40
    alm = random_alm(lmax, seed=3)
    got = g.healpix.alm2map(alm, nside, lmax=lmax, pixwin=True)
    s0, _ = opw.pixwin_series(nside, lmax)
    ref = osht.alm2map(osht.almxfl(alm, s0), nside, lmax)
    assert rel_err(got, ref) < 1e-12


@pytest.mark.gpu
def test_from_convergence_discretized_default(g):
    nside = 16
    lmax = 3 * nside - 1
    rng = np.random.default_rng(5)
    kappa = rng.standard_normal(12 * nside * nside) * 0.01
    (gamma,) = g.from_convergence(kappa, shear=True)  # discretized=True by default
    alm = osht.map2alm(kappa, lmax, iter=3)
    ell = np.arange(lmax + 1, dtype=float)
    fl = np.zeros_like(ell)
    fl[1:] = -2 / (ell[1:] * (ell[1:] + 1))
    fl *= np.sqrt(ell * (ell + 1))
    f2 = np.zeros_like(ell)
    f2[1:] = np.sqrt((ell[1:] - 1) * (ell[1:] + 2)) / 2
    s0, s2 = opw.pixwin_series(nside, lmax)
    alm = osht.almxfl(osht.almxfl(alm, fl), f2 * s2 / s0)
    g0, g1 = osht.alm2map_spin([alm, None], nside, 2, lmax)
    assert rel_err(gamma, g0 + 1j * g1) < 1e-10
    (plain,) = g.from_convergence(kappa, shear=True, discretized=False)
    assert rel_err(gamma, plain) > 1e-4  # the window does change the shear
    g1s, g2s = g.lensing.shear_from_convergence(kappa)
    g1n, g2n = g.lensing.shear_from_convergence(kappa, discretized=False)
    assert rel_err(g1s, g1n) > 1e-4 and np.all(np.isfinite(g1s)) and np.all(np.isfinite(g2s))

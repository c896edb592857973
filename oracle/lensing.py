"""Map-level lensing restatements -- TEST INFRASTRUCTURE ONLY.

numpy restatements, in the reference's own operation order, of

* the multi-plane convergence update of ``MultiPlaneConvergence.add_plane``
  (glass/lensing.py:577-581),
* the HEALPix RING-scheme ``ang2pix`` (Gorski et al. 2005, ApJ 622, 759;
  healpy.ang2pix is what glass/healpix.py calls; healpy itself is not
  installed here, so the pixelisation is pinned by its published formulas,
  pix2ang round trips and known pixels),
* ``galaxy_shear`` (glass/galaxies.py:271-347) on top of it,
* the pixel geometry behind sampling positions inside pixels (the
  healpy.randang step of glass/points.py:426-430): ring, position in the
  ring and the (z, phi) box that holds each RING pixel.
"""

from __future__ import annotations

import numpy as np


def convergence_step(kappa3, kappa2, delta2, t: float, f: float):
    """kappa3 (in place): *= 1 - t; += t * kappa2; += f * delta2."""
    t = np.asarray(t)
    kappa3 *= 1 - t
    kappa3 += t * kappa2
    kappa3 += np.asarray(f) * delta2
    return kappa3


def ang2pix_ring(nside: int, theta, phi) -> np.ndarray:
    theta = np.asarray(theta, dtype=np.float64)
    phi = np.asarray(phi, dtype=np.float64)
    z = np.cos(theta)
    za = np.abs(z)
    ph = np.fmod(phi, 2 * np.pi)
    ph = np.where(ph < 0, ph + 2 * np.pi, ph)
    tt = ph * 0.63661977236758134308
    ncap = 2 * nside * (nside - 1)
    npix = 12 * nside * nside
    out = np.empty(theta.shape, dtype=np.int64)
    eq = za <= 2.0 / 3.0
    # equatorial belt
    t1 = nside * (0.5 + tt[eq])
    t2 = nside * (z[eq] * 0.75)
    jp = (t1 - t2).astype(np.int64)
    jm = (t1 + t2).astype(np.int64)
    ir = nside + 1 + jp - jm
    kshift = 1 - (ir & 1)
    ip = (jp + jm - nside + kshift + 1) // 2
    ip = np.mod(ip, 4 * nside)
    out[eq] = ncap + (ir - 1) * 4 * nside + ip
    # polar caps
    pc = ~eq
    ttp = tt[pc]
    tp = ttp - ttp.astype(np.int64)
    zp, zap = z[pc], za[pc]
    tmp = np.where(zap < 0.99, nside * np.sqrt(3.0 * (1.0 - zap)),
                   nside * np.sin(theta[pc]) / np.sqrt((1.0 + zap) / 3.0))
    jp = (tp * tmp).astype(np.int64)
    jm = ((1.0 - tp) * tmp).astype(np.int64)
    ir = jp + jm + 1
    ip = np.mod((ttp * ir).astype(np.int64), 4 * ir)
    out[pc] = np.where(zp > 0, 2 * ir * (ir - 1) + ip, npix - 2 * ir * (ir + 1) + ip)
    return out


def lonlat_to_thetaphi(lon, lat):
    d2r = np.pi / 180
    return np.pi / 2 - np.asarray(lat, dtype=np.float64) * d2r, np.asarray(lon, dtype=np.float64) * d2r


def ang2pix_lonlat(nside: int, lon, lat) -> np.ndarray:
    return ang2pix_ring(nside, *lonlat_to_thetaphi(lon, lat))


def galaxy_shear(lon, lat, eps, kappa, gamma1, gamma2, *, reduced_shear: bool = True):
    npix = np.asarray(kappa).shape[-1]
    nside = int(round((npix // 12) ** 0.5))
    ipix = ang2pix_lonlat(nside, lon, lat)
    k = np.asarray(kappa, dtype=np.float64)[ipix]
    g = np.asarray(gamma1)[ipix] + 1j * np.asarray(gamma2)[ipix]
    if reduced_shear:
        g /= 1 - k
        g = (eps + g) / (1 + np.conj(g) * eps)
    else:
        g += eps
    return g


class MultiPlaneConvergence:
    """Restatement of glass/lensing.py:430-586 (host arithmetic and the
    in-place plane update in the reference's order)."""

    def __init__(self, cosmo):
        self.cosmo = cosmo
        self.z2 = self.z3 = self.x3 = self.w3 = 0.0
        self.r23 = 1.0
        self.delta3 = np.asarray(0.0)
        self.kappa2 = self.kappa3 = None

    def add_plane(self, delta, zsrc, wlens=1.0):
        if zsrc <= self.z3:
            raise ValueError("source redshift must be increasing")
        delta2, self.delta3 = self.delta3, delta
        z1, self.z2, self.z3 = self.z2, self.z3, zsrc
        w2, self.w3 = self.w3, wlens
        x2, self.x3 = self.x3, self.cosmo.transverse_comoving_distance(self.z3) / self.cosmo.hubble_distance
        r12 = self.r23
        r13, self.r23 = self.cosmo.transverse_comoving_distance([z1, self.z2], self.z3) / (
            self.cosmo.hubble_distance * self.x3)
        t = r13 / r12
        f = 3 * self.cosmo.Omega_m0 / 2
        f *= x2 * self.r23
        f *= (1 + self.z2) / self.cosmo.H_over_H0(self.z2)
        f *= w2
        if self.kappa2 is None:
            self.kappa2 = np.zeros_like(delta)
            self.kappa3 = np.zeros_like(delta)
        self.kappa2, self.kappa3 = self.kappa3, self.kappa2
        convergence_step(self.kappa3, self.kappa2, delta2, t, f)

    @property
    def kappa(self):
        return self.kappa3


def ring_z(nside: int, r):
    """z = cos(theta) of the centres of ring r (1 .. 4 nside - 1)."""
    r = np.asarray(r, dtype=np.int64)
    ns = float(nside)
    q = 4 * nside - r
    return np.where(r < nside, 1.0 - (r * r) / (3.0 * ns * ns),
                    np.where(r <= 3 * nside, 4.0 / 3.0 - 2.0 * r / (3.0 * ns), (q * q) / (3.0 * ns * ns) - 1.0))


def pix_ring(nside: int, p):
    """(ring r, position j in the ring, ring length) of RING pixels p."""
    p = np.asarray(p, dtype=np.int64)
    ncap = 2 * nside * (nside - 1)
    npix = 12 * nside * nside
    r = np.empty_like(p)
    j = np.empty_like(p)
    nph = np.empty_like(p)
    a = p < ncap
    r[a] = (1 + np.floor(np.sqrt(1.0 + 2.0 * p[a])).astype(np.int64)) // 2
    j[a] = p[a] - 2 * r[a] * (r[a] - 1)
    nph[a] = 4 * r[a]
    b = (p >= ncap) & (p < npix - ncap)
    q = p[b] - ncap
    r[b] = q // (4 * nside) + nside
    j[b] = q % (4 * nside)
    nph[b] = 4 * nside
    c = p >= npix - ncap
    q = npix - 1 - p[c]
    rs = (1 + np.floor(np.sqrt(1.0 + 2.0 * q)).astype(np.int64)) // 2
    r[c] = 4 * nside - rs
    nph[c] = 4 * rs
    j[c] = nph[c] - 1 - (q - 2 * rs * (rs - 1))
    return r, j, nph


def pixel_box(nside: int, p):
    """(zlo, zhi, phi centre, phi width) of the box that holds RING pixel p.

    A pixel of ring r lies between the centres of rings r+1 and r-1 in z and
    within half a pixel width of its centre in phi; it fills half the box.
    """
    r, j, nph = pix_ring(nside, p)
    zhi = np.where(r == 1, 1.0, ring_z(nside, np.maximum(r - 1, 1)))
    zlo = np.where(r == 4 * nside - 1, -1.0, ring_z(nside, np.minimum(r + 1, 4 * nside - 1)))
    shifted = (r < nside) | (r > 3 * nside) | (((r - nside) & 1) == 0)
    dphi = 2 * np.pi / nph
    return zlo, zhi, (j + np.where(shifted, 0.5, 0.0)) * dphi, dphi


def randang_lonlat(nside: int, ipix, rng) -> tuple[np.ndarray, np.ndarray]:
    """Uniform positions inside RING pixels ipix by rejection from pixel_box."""
    ipix = np.asarray(ipix, dtype=np.int64)
    zlo, zhi, phic, dphi = pixel_box(nside, ipix)
    z = np.empty(ipix.shape)
    phi = np.empty(ipix.shape)
    todo = np.arange(ipix.size)
    while todo.size:
        zz = zlo[todo] + rng.random(todo.size) * (zhi[todo] - zlo[todo])
        pp = phic[todo] + (rng.random(todo.size) - 0.5) * dphi[todo]
        ok = ang2pix_ring(nside, np.arccos(zz), pp) == ipix[todo]
        z[todo[ok]] = zz[ok]
        phi[todo[ok]] = pp[ok]
        todo = todo[~ok]
    return np.degrees(np.mod(phi, 2 * np.pi)), np.degrees(np.arcsin(z))

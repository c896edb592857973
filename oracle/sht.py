"""FP64 CPU restatement of the HEALPix ring SHT (TEST INFRASTRUCTURE ONLY).

Stands in for healpy, which the reference calls at ``glass/healpix.py:71``
(alm2map), ``:107`` (alm2map_spin), ``:136`` (almxfl) and ``:270`` (map2alm).
Legendre sums run in C (``orc_sht.c``, OpenMP); the ring Fourier sums use
numpy's FFT.  ``alm2map_direct`` evaluates the same sums pixel by pixel with
``scipy.special.sph_harm_y`` and pins the fast restatement at small sizes.

Conventions: HEALPix RING order, alm in HEALPix m-major order with
mmax = lmax, ``map = sum_l a_l0 Y_l0 + 2 Re sum_{m>0} a_lm Y_lm`` (the
imaginary part of a_l0 is ignored), and for spin s:
``Q + iU = -sum_lm (E_lm + i B_lm) sY_lm``.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np

from . import lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def nalm(lmax: int) -> int:
    return (lmax + 1) * (lmax + 2) // 2


def lmax_from_nalm(n: int) -> int:
    lmax = (math.isqrt(8 * n + 1) - 3) // 2
    if nalm(lmax) != n:
        raise ValueError(f"alm size {n} is not (lmax+1)(lmax+2)/2")
    return lmax


def alm_index(l, m, lmax):  # noqa: E741
    return m * (2 * lmax + 1 - m) // 2 + l


def ring_info(nside: int):
    """Arrays (z, sin theta, nph, phi0, startpix) for rings 1..4 nside - 1."""
    L = lib()
    nr = 4 * nside - 1
    z = np.empty(nr)
    sth = np.empty(nr)
    nph = np.empty(nr, dtype=np.int64)
    phi0 = np.empty(nr)
    start = np.empty(nr, dtype=np.int64)
    zz, ss, pp = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    nn = ctypes.c_int()
    st = ctypes.c_int64()
    for i in range(1, nr + 1):
        L.orc_ring_info(nside, i, ctypes.byref(zz), ctypes.byref(ss), ctypes.byref(nn),
                        ctypes.byref(pp), ctypes.byref(st))
        z[i - 1], sth[i - 1], nph[i - 1], phi0[i - 1], start[i - 1] = zz.value, ss.value, nn.value, pp.value, st.value
    return z, sth, nph, phi0, start


def pix_angles(nside: int):
    """(theta, phi) of every pixel centre, RING order."""
    z, sth, nph, phi0, start = ring_info(nside)
    npix = 12 * nside * nside
    theta = np.empty(npix)
    phi = np.empty(npix)
    for r in range(z.size):
        n = int(nph[r])
        s = int(start[r])
        theta[s:s + n] = np.arctan2(sth[r], z[r])
        phi[s:s + n] = phi0[r] + 2 * np.pi * np.arange(n) / n
    return theta, phi


def alm2ring(alm: np.ndarray, nside: int, lmax: int, rings=None) -> np.ndarray:
    """Legendre sums F_m(ring) = sum_l a_lm lambda_lm(z_ring): [nmaps][nring][lmax+1]."""
    alm = np.ascontiguousarray(np.atleast_2d(alm), dtype=np.complex128)
    nmaps = alm.shape[0]
    if rings is None:
        F = np.empty((nmaps, 4 * nside - 1, lmax + 1), dtype=np.complex128)
        lib().orc_alm2ring_all(_dp(alm.view(np.float64)), nmaps, lmax, nside, _dp(F.view(np.float64)))
        return F
    rings = np.ascontiguousarray(rings, dtype=np.intc)
    F = np.empty((nmaps, rings.size, lmax + 1), dtype=np.complex128)
    lib().orc_alm2ring(_dp(alm.view(np.float64)), nmaps, lmax, nside, _ip(rings), rings.size,
                       _dp(F.view(np.float64)))
    return F


def ring_synthesis(F: np.ndarray, nside: int) -> np.ndarray:
    """Real ring maps from per-ring Fourier coefficients F[..., ring, m]."""
    z, sth, nph, phi0, start = ring_info(nside)
    lead = F.shape[:-2]
    mmax = F.shape[-1] - 1
    out = np.empty(lead + (12 * nside * nside,))
    m = np.arange(mmax + 1)
    c = np.where(m == 0, 1.0, 2.0)
    for r in range(z.size):
        n = int(nph[r])
        s = int(start[r])
        G = F[..., r, :] * (c * np.exp(1j * m * phi0[r]))
        H = np.zeros(lead + (n,), dtype=np.complex128)
        # fold m into n bins
        for k0 in range(0, mmax + 1, n):
            seg = G[..., k0:k0 + n]
            H[..., : seg.shape[-1]] += seg
        out[..., s:s + n] = (np.fft.ifft(H, axis=-1) * n).real
    return out


def ring_analysis(maps: np.ndarray, nside: int, mmax: int) -> np.ndarray:
    """Weighted ring Fourier coefficients G[..., ring, m] = w sum_j f_j e^{-i m phi_j}."""
    z, sth, nph, phi0, start = ring_info(nside)
    lead = maps.shape[:-1]
    npix = 12 * nside * nside
    w = 4 * np.pi / npix
    G = np.empty(lead + (z.size, mmax + 1), dtype=np.complex128)
    m = np.arange(mmax + 1)
    for r in range(z.size):
        n = int(nph[r])
        s = int(start[r])
        X = np.fft.fft(maps[..., s:s + n], axis=-1)
        G[..., r, :] = w * X[..., m % n] * np.exp(-1j * m * phi0[r])
    return G


def alm2map(alm: np.ndarray, nside: int, lmax: int | None = None) -> np.ndarray:
    """Spin-0 synthesis, FP64 (healpy.alm2map with pol=False, pixwin=False)."""
    alm = np.asarray(alm)
    single = alm.ndim == 1
    alm2 = np.atleast_2d(alm)
    if lmax is None:
        lmax = lmax_from_nalm(alm2.shape[-1])
    F = alm2ring(alm2, nside, lmax)
    out = ring_synthesis(F, nside)
    return out[0] if single else out


def ring2alm(G: np.ndarray, nside: int, lmax: int) -> np.ndarray:
    G = np.ascontiguousarray(np.atleast_3d(G) if G.ndim == 2 else G, dtype=np.complex128)
    if G.ndim == 2:
        G = G[None]
    nmaps = G.shape[0]
    rings = np.arange(1, 4 * nside, dtype=np.intc)
    alm = np.empty((nmaps, nalm(lmax)), dtype=np.complex128)
    lib().orc_ring2alm(_dp(G.view(np.float64)), nmaps, lmax, nside, _ip(rings), rings.size,
                       _dp(alm.view(np.float64)))
    return alm


def map2alm(maps: np.ndarray, lmax: int, iter: int = 3) -> np.ndarray:  # noqa: A002
    """Spin-0 analysis with uniform pixel weights and `iter` Jacobi refinements."""
    maps = np.asarray(maps, dtype=np.float64)
    single = maps.ndim == 1
    m2 = np.atleast_2d(maps)
    nside = math.isqrt(m2.shape[-1] // 12)
    alm = ring2alm(ring_analysis(m2, nside, lmax), nside, lmax)
    for _ in range(iter):
        resid = m2 - ring_synthesis(alm2ring(alm, nside, lmax), nside)
        alm = alm + ring2alm(ring_analysis(resid, nside, lmax), nside, lmax)
    return alm[0] if single else alm


def alm2map_spin(alms, nside: int, spin: int, lmax: int) -> list[np.ndarray]:
    """Spin-s synthesis (s = 1, 2): returns [Q, U]."""
    if spin not in (1, 2):
        raise ValueError("spin must be 1 or 2")
    elm = np.ascontiguousarray(alms[0], dtype=np.complex128)
    blm = None if alms[1] is None else np.ascontiguousarray(alms[1], dtype=np.complex128)
    rings = np.arange(1, 4 * nside, dtype=np.intc)
    QU = np.empty((2, rings.size, lmax + 1), dtype=np.complex128)
    lib().orc_alm2ring_spin(_dp(elm.view(np.float64)),
                            None if blm is None else _dp(blm.view(np.float64)),
                            spin, lmax, nside, _ip(rings), rings.size, _dp(QU.view(np.float64)))
    out = ring_synthesis(QU, nside)
    return [out[0], out[1]]


def almxfl(alm: np.ndarray, fl: np.ndarray) -> np.ndarray:
    alm = np.asarray(alm)
    lmax = lmax_from_nalm(alm.shape[-1])
    ell = np.concatenate([np.arange(m, lmax + 1) for m in range(lmax + 1)])
    f = np.zeros(lmax + 1)
    n = min(len(fl), lmax + 1)
    f[:n] = np.asarray(fl)[:n]
    return alm * f[ell]


# -------------------------------------------------------------- independent pin


def alm2map_direct(alm: np.ndarray, nside: int, lmax: int) -> np.ndarray:
    """Brute-force pixel-by-pixel synthesis with scipy's Y_lm (small sizes)."""
    from scipy.special import sph_harm_y

    theta, phi = pix_angles(nside)
    out = np.zeros(theta.size)
    for m in range(lmax + 1):
        for ell in range(m, lmax + 1):
            a = alm[alm_index(ell, m, lmax)]
            y = sph_harm_y(ell, m, theta, phi)
            out += (a * y).real if m == 0 else 2 * (a * y).real
    return out


def spin_ylm_goldberg(s: int, ell: int, m: int, theta: np.ndarray, phi: np.ndarray) -> np.ndarray:
    """Spin-weighted harmonic sY_lm from the explicit Goldberg et al. (1967) sum."""
    from math import comb, factorial

    if ell < abs(s) or ell < abs(m):
        return np.zeros_like(theta, dtype=complex)
    pref = (-1.0) ** m * math.sqrt(
        (2 * ell + 1) / (4 * math.pi)
        * factorial(ell + m) * factorial(ell - m) / (factorial(ell + s) * factorial(ell - s))
    )
    half = theta / 2
    tot = np.zeros_like(theta, dtype=complex)
    for r in range(0, ell - s + 1):
        k = r + s - m
        if k < 0 or k > ell + s:
            continue
        c = comb(ell - s, r) * comb(ell + s, k) * (-1.0) ** (ell - r - s)
        tot += c * np.cos(half) ** (2 * r + s - m) * np.sin(half) ** (2 * ell - 2 * r - s + m)
    return pref * tot * np.exp(1j * m * phi)


def alm2map_spin_direct(elm, blm, nside: int, spin: int, lmax: int):
    """Brute-force spin synthesis over m = -l..l with Goldberg's sY_lm."""
    theta, phi = pix_angles(nside)
    tot = np.zeros(theta.size, dtype=complex)
    for ell in range(spin, lmax + 1):
        for m in range(-ell, ell + 1):
            ix = alm_index(ell, abs(m), lmax)
            if m == 0:
                # a real field has real m = 0 coefficients; the imaginary part is ignored
                e, b = elm[ix].real, (0 if blm is None else blm[ix].real)
            elif m > 0:
                e, b = elm[ix], (0 if blm is None else blm[ix])
            else:
                e = (-1) ** m * np.conj(elm[ix])
                b = 0 if blm is None else (-1) ** m * np.conj(blm[ix])
            tot += -(e + 1j * b) * spin_ylm_goldberg(spin, ell, m, theta, phi)
    return [tot.real, tot.imag]

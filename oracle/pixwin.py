"""HEALPix pixel window functions from their definition (TEST INFRASTRUCTURE ONLY).

Stands in for ``healpy.pixwin`` as called by ``glass/healpix.py:313-356``
(``pixwin(nside, lmax=, pol=)``) and used by ``glass/lensing.py:360-362``
(``from_convergence(..., discretized=True)``: the shear alm are scaled by
pw2 / pw0).  healpy reads these windows from data files that are not
available offline, so parity with healpy's tables is UNPINNED; this module
restates the definition of the windows and evaluates it by direct pair sums:

* temperature (spin 0): the window of pixel p at l is
  ``w_l(p)^2 = (4 pi / (2l+1)) sum_m |(1/A) int_p Y_lm|^2``, which the
  addition theorem turns into the pixel's pair average
  ``<< P_l(cos gamma) >>_p`` over two independent uniform points of the pixel;
  ``pw0_l = sqrt(mean_p w_l(p)^2)`` (Gorski et al. 2005, the pixel window
  averaged over the sphere);
* polarisation (spin 2): the same with ``d^l_22(gamma) = cos^4(gamma/2)
  P^(0,4)_{l-2}(cos gamma)``, the spin-2 addition kernel; the frames of the
  two points are parallel-transported to the pixel centre, which leaves a
  phase of twice the spherical excess of a triangle inside the pixel
  (below 1e-6 radians for nside >= 512, so cos of it differs from 1 by less
  than 1e-12) -- it is neglected.  pw2_l = 0 for l < 2.

Pixel quadrature (shared with the GPU kernel, part of the definition here):
every HEALPix pixel is the diamond ``|x - xc| + |y - yc| <= h``,
``h = pi / (4 nside)``, of the equal-area HEALPix projection (Calabretta &
Roukema 2007): ``x = phi, y = 3 pi z / 8`` for ``|z| <= 2/3``, and
``y = (pi/4)(2 - s)``, ``x = phic + (phi - phic) s``, ``s = sqrt(3 (1-|z|))``
in the polar caps (``phic`` the centre of the quadrant).  The diamond is cut
at ``y = yc`` (where the projection's second derivative jumps for the rings
next to |z| = 2/3) and each half is integrated with a Q-point Gauss-Legendre
rule in y times a Q-point rule across the half-diamond's width: 2 Q^2 nodes of
equal-area weight per pixel.

Only one pixel per congruence class is evaluated: a quadrant of each polar
ring (rings 1..nside; weight 8 for the four quadrants and the south mirror)
and one pixel of each belt ring nside+1..2 nside (all its pixels are
rotations of one another; weight 2 nph, nph for the equator).
"""

from __future__ import annotations

import math

import numpy as np
from scipy import special

Q_DEFAULT = 8


def _gauss(q: int):
    u, w = np.polynomial.legendre.leggauss(q)
    return u, w


def pixel_classes(nside: int):
    """(ring i, index jj within the ring, weight) of one pixel per class."""
    out = []
    for i in range(1, nside + 1):
        for jj in range(i):
            out.append((i, jj, 8.0))
    for i in range(nside + 1, 2 * nside + 1):
        out.append((i, 0, (8.0 if i < 2 * nside else 4.0) * nside))
    return out


def pixel_nodes(nside: int, i: int, jj: int, q: int = Q_DEFAULT):
    """Unit vectors [2 q^2, 3] and weights (sum 1) of pixel jj of north ring i
    (polar rings: jj-th pixel of the first quadrant)."""
    h = math.pi / (4 * nside)
    if i <= nside:
        yc = (math.pi / 4) * (2 - i / nside)
        phic = math.pi / 4
        xc = phic + (math.pi / (2 * nside)) * (jj - (i - 1) / 2)
    else:
        yc = math.pi / 2 - i * math.pi / (4 * nside)
        half = 1 if (i - nside) % 2 == 0 else 0
        phic = math.pi / 4
        xc = (math.pi / (2 * nside)) * (jj + half / 2)
    u, w = _gauss(q)
    xs, ys, ws = [], [], []
    for sgn in (-1.0, 1.0):  # lower and upper half of the diamond
        yp = sgn * (h / 2) * (1 + u)  # |yp| in [0, h]
        width = h - np.abs(yp)
        for a in range(q):
            xs.append(xc + width[a] * u)
            ys.append(np.full(q, yc + yp[a]))
            ws.append((h / 2) * w[a] * width[a] * w)
    x = np.concatenate(xs)
    y = np.concatenate(ys)
    wt = np.concatenate(ws)
    wt = wt / wt.sum()
    z = np.empty_like(y)
    phi = np.empty_like(x)
    eq = np.abs(y) <= math.pi / 4
    z[eq] = 8 * y[eq] / (3 * math.pi)
    phi[eq] = x[eq]
    s = 2 - 4 * np.abs(y[~eq]) / math.pi
    z[~eq] = np.sign(y[~eq]) * (1 - s * s / 3)
    phi[~eq] = phic + (x[~eq] - phic) / s
    st = np.sqrt((1 - z) * (1 + z))
    n = np.stack([st * np.cos(phi), st * np.sin(phi), z], axis=1)
    return n, wt


def _pair_t(n: np.ndarray):
    d = n[:, None, :] - n[None, :, :]
    return 0.25 * np.sum(d * d, axis=-1)  # sin^2(gamma / 2)


def pixwin_direct(nside: int, lmax: int, q: int = Q_DEFAULT):
    """(pw0, pw2) float64 [lmax+1] by direct pair sums of P_l and d^l_22."""
    acc0 = np.zeros(lmax + 1)
    acc2 = np.zeros(lmax + 1)
    tot = 0.0
    ell = np.arange(lmax + 1)
    for i, jj, wgt in pixel_classes(nside):
        n, w = pixel_nodes(nside, i, jj, q)
        t = _pair_t(n).ravel()
        ww = np.outer(w, w).ravel()
        x = 1 - 2 * t
        for l in range(lmax + 1):
            acc0[l] += wgt * np.dot(ww, special.eval_legendre(l, x))
            if l >= 2:
                d22 = (1 - t) ** 2 * special.eval_jacobi(l - 2, 0, 4, x)
                acc2[l] += wgt * np.dot(ww, d22)
        tot += wgt
    assert abs(tot - 12 * nside * nside) < 1e-6
    # normalised by the pair-weight total (acc0[0], = npix up to rounding)
    pw0 = np.sqrt(acc0 / acc0[0])
    pw2 = np.sqrt(np.maximum(acc2 / acc0[0], 0.0))
    pw2[ell < 2] = 0.0
    return pw0, pw2


def pair_moments(nside: int, kmax: int, q: int = Q_DEFAULT, scale: float | None = None):
    """Scaled pair moments M_k = mean_p <<t^k>> / scale^k, k = 0 .. kmax."""
    scale = 1.0 / (nside * nside) if scale is None else scale
    acc = np.zeros(kmax + 1)
    tot = 0.0
    for i, jj, wgt in pixel_classes(nside):
        n, w = pixel_nodes(nside, i, jj, q)
        t = _pair_t(n).ravel() / scale
        ww = np.outer(w, w).ravel()
        tk = np.ones_like(t)
        for k in range(kmax + 1):
            acc[k] += wgt * np.dot(ww, tk)
            tk = tk * t
        tot += wgt
    return acc / acc[0]


def pixwin_series(nside: int, lmax: int, kmax: int = 40, q: int = Q_DEFAULT):
    """(pw0, pw2) from the pair moments and the hypergeometric series
    P_l(1-2t) = sum_k (-1)^k C(l,k) C(l+k,k) t^k,
    P^(0,4)_n(1-2t) = sum_k (-1)^k C(n,k) C(n+k+4,k) t^k (the GPU's method)."""
    s = 1.0 / (nside * nside)
    M = pair_moments(nside, kmax + 2, q, s)
    pw0 = np.zeros(lmax + 1)
    pw2 = np.zeros(lmax + 1)
    for l in range(lmax + 1):
        c, acc = 1.0, 0.0
        for k in range(kmax + 1):
            if k > l:
                break
            acc += c * M[k]
            c *= -(l - k) * (l + k + 1) / ((k + 1) ** 2) * s
        pw0[l] = math.sqrt(acc)
        if l >= 2:
            n = l - 2
            c, acc = 1.0, 0.0
            for k in range(kmax + 1):
                if k > n:
                    break
                acc += c * (M[k] - 2 * s * M[k + 1] + s * s * M[k + 2])
                c *= -(n - k) * (n + k + 5) / ((k + 1) ** 2) * s
            pw2[l] = math.sqrt(max(acc, 0.0))
    return pw0, pw2

"""Restatement of the reference's field-generation glue (TEST INFRASTRUCTURE ONLY).

Follows, function by function:

* ``cls2cov``            -- glass/fields.py:191-236
* ``iternorm``           -- glass/fields.py:101-188 (C, fixed order: orc_iternorm)
* ``glass_to_healpix_alm`` -- glass/fields.py:943-962
* ``multalm``            -- glass/harmonics.py:17-47
* ``generate_grf_alm``   -- glass/fields.py:334-425 (everything before the SHT)
* ``generate``           -- glass/fields.py:839-894 with the SHT of ``oracle.sht``
* ``lognormal``          -- glass/grf/_transformations.py:83-89
* ``cltovar``            -- transformcl.cltovar (variance sum (2l+1)/(4 pi) C_l)

The pinned golden fixtures in ``tests/golden/`` come from running the
reference's own Python (``tests/golden/make_golden.py``); the CPU tests check
this module against them.
"""

from __future__ import annotations

import collections
import ctypes
import math

import numpy as np

from . import lib
from . import sht


def nfields_from_nspectra(nspectra: int) -> int:
    n = math.floor(math.sqrt(2 * nspectra))
    if n * (n + 1) // 2 != nspectra:
        raise ValueError(f"invalid number of spectra: {nspectra}")
    return n


def cls2cov(cls, nl: int, nf: int, nc: int):
    """Yield, per field j, the (nl, nc+1) matrix [C_jj, C_j,j-1, ...] / 2."""
    for j in range(nf):
        cov = np.zeros((nl, nc + 1))
        begin = j * (j + 1) // 2
        for i, cl in enumerate(cls[begin:begin + j + 1][: nc + 1]):
            cl = np.asarray(cl, dtype=np.float64)
            if i == 0 and np.any(cl < 0):
                raise ValueError("negative values in cl")
            n = min(cl.shape[0], nl)
            cov[:n, i] = cl[:n]
        yield cov / 2


def iternorm_stack(cov: np.ndarray, dense: bool = False) -> tuple[np.ndarray, int]:
    """cov [nrows][nl][k+1] -> (w same shape, first bad row or -1).

    ``dense``: every sum over all k indices (orc_iternorm_dense) instead of
    over the non-zero block only; the two agree bit for bit."""
    cov = np.ascontiguousarray(cov, dtype=np.float64)
    nrows, nl, kp = cov.shape
    w = np.empty_like(cov)
    dp = ctypes.POINTER(ctypes.c_double)
    fn = lib().orc_iternorm_dense if dense else lib().orc_iternorm
    bad = fn(cov.ctypes.data_as(dp), nrows, nl, kp - 1, w.ctypes.data_as(dp))
    return w, int(bad)


def cltovar(cl) -> float:
    cl = np.asarray(cl, dtype=np.float64)
    ell = np.arange(cl.shape[0])
    return float(np.sum((2 * ell + 1) / (4 * np.pi) * cl))


def getcl(cls, i: int, j: int, lmax: int | None = None):
    if j > i:
        i, j = j, i
    cl = np.asarray(cls[i * (i + 1) // 2 + i - j])
    if lmax is not None:
        cl = cl[: lmax + 1] if cl.shape[0] > lmax + 1 else np.pad(cl, (0, lmax + 1 - cl.shape[0]))
    return cl


def multalm(alm: np.ndarray, bl: np.ndarray) -> np.ndarray:
    bl = np.asarray(bl)
    return alm * np.repeat(bl, np.arange(bl.size) + 1)


def glass_to_healpix_alm(alm: np.ndarray) -> np.ndarray:
    n = (math.isqrt(8 * alm.size + 1) - 1) // 2
    ell = np.arange(n)
    return np.concatenate([alm[ell[m:] * (ell[m:] + 1) // 2 + m] for m in range(n)])


def generate_grf_alm(gls, ncorr=None, z_of_shell=None):
    """Yield HEALPix-order alm per shell, exactly as handed to alm2map.

    ``z_of_shell(t, z_size)`` returns the complex standard normals of shell t
    in GLASS order (default: numpy ``default_rng(42)``, drawn as the
    reference does).
    """
    ngrf = nfields_from_nspectra(len(gls))
    if ncorr is None:
        ncorr = ngrf - 1
    n = max((np.asarray(gl).shape[0] for gl in gls), default=0)
    if n == 0:
        raise ValueError("all gls are empty")
    if z_of_shell is None:
        rng = np.random.default_rng(42)

        def z_of_shell(t, size):
            return rng.standard_normal((size, 2)) @ np.asarray([1, 1j])

    z_size = n * (n + 1) // 2
    covs = np.stack(list(cls2cov(gls, n, ngrf, ncorr)))
    w_all, bad = iternorm_stack(covs)
    y = collections.deque()
    for t in range(ngrf):
        if bad >= 0 and t >= bad:
            raise ValueError("covariance matrix is not positive definite")
        w = w_all[t]
        y.append(z_of_shell(t, z_size))
        while len(y) > w.shape[-1]:
            y.popleft()
        mis = w.shape[-1] - len(y)
        alm = sum(multalm(z, w[..., i + mis]) for i, z in enumerate(y))
        alm = glass_to_healpix_alm(alm)
        alm[:n] = alm[:n].real + alm[:n].imag + 0j
        yield alm


def lognormal(x: np.ndarray, var: float, lamda: float = 1.0) -> np.ndarray:
    x = np.expm1(x - var / 2)
    if lamda != 1.0:
        x = lamda * x
    return x


def generate_lognormal(gls, nside: int, shifts, ncorr=None, z_of_shell=None):
    """Lognormal shell maps: SHT of generate_grf_alm, then lambda expm1(x - var/2)."""
    n = nfields_from_nspectra(len(gls))
    for i, alm in enumerate(generate_grf_alm(gls, ncorr=ncorr, z_of_shell=z_of_shell)):
        lmax = sht.lmax_from_nalm(alm.size)
        x = sht.alm2map(alm, nside, lmax)
        var = cltovar(getcl(gls, i, i))
        yield lognormal(x, var, shifts[i] if n else 1.0)

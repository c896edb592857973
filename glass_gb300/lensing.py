"""Weak-lensing maps from the convergence (glass/lensing.py:185-428).

``from_convergence`` follows the reference step by step: analysis of kappa
(map2alm), multiplication by the harmonic kernels with almxfl, and spin-0,
spin-1 and spin-2 synthesis, all on the GPU.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from . import healpix as hp


def _ell(lmax: int, like) -> np.ndarray:
    return np.arange(lmax + 1, dtype=np.float64)


def from_convergence(kappa, lmax: int | None = None, *, potential: bool = False,
                     deflection: bool = False, shear: bool = False, discretized: bool = True):
    """Potential, deflection and/or shear from a convergence map (glass/lensing.py:185-371).

    ``discretized=True`` needs the HEALPix pixel-window tables (pw2 / pw0),
    which are not available: pass ``discretized=False``.
    """
    if not (potential or deflection or shear):
        return ()
    numpy_out = _lib.is_numpy_like(kappa)
    k = _lib.to_device(kappa, torch.float64)
    nside = hp.get_nside(k)
    if lmax is None:
        lmax = 3 * nside - 1
    if shear and discretized:
        hp.pixwin(nside, lmax=lmax, pol=True)  # raises: tables unavailable
    alm = hp.analysis(k.reshape(1, -1), lmax, 3)[0]
    ell = _ell(lmax, k)
    results: tuple = ()

    def out(x):
        return x.cpu().numpy() if numpy_out else x

    # convergence -> potential: -2 / (l (l+1)), 0 at l = 0
    fl = np.zeros_like(ell)
    fl[1:] = -2.0 / (ell[1:] * (ell[1:] + 1))
    alm = hp.almxfl(alm, torch.as_tensor(fl, device=alm.device))
    if potential:
        psi = hp.synth(alm.reshape(1, -1), nside, lmax)[0]
        results += (out(psi),)
    if not (deflection or shear):
        return results
    # potential -> deflection: sqrt(l (l+1))
    fl = np.sqrt(ell * (ell + 1))
    alm = hp.almxfl(alm, torch.as_tensor(fl, device=alm.device))
    if deflection:
        q, u = hp._spin_synth(alm, None, nside, 1, lmax)
        results += (out(torch.complex(q, u)),)
    if not shear:
        return results
    # deflection -> shear: sqrt((l-1)(l+2)) / 2, 0 at l = 0
    fl = np.zeros_like(ell)
    fl[1:] = np.sqrt((ell[1:] - 1) * (ell[1:] + 2)) / 2
    alm = hp.almxfl(alm, torch.as_tensor(fl, device=alm.device))
    q, u = hp._spin_synth(alm, None, nside, 2, lmax)
    results += (out(torch.complex(q, u)),)
    return results


def shear_from_convergence(kappa, lmax: int | None = None, *, discretized: bool = True):
    """Shear maps [g1, g2] from convergence (glass/lensing.py:374-428; deprecated upstream)."""
    numpy_out = _lib.is_numpy_like(kappa)
    k = _lib.to_device(kappa, torch.float64)
    nside = hp.get_nside(k)
    if lmax is None:
        lmax = 3 * nside - 1
    if discretized:
        hp.pixwin(nside, lmax=lmax, pol=True)
    alm = hp.analysis(k.reshape(1, -1), lmax, 3)[0]
    ell = np.arange(lmax + 1)
    fl = np.sqrt((ell + 2.0) * (ell + 1) * ell * (ell - 1))
    fl /= np.clip(ell * (ell + 1), 1, None)
    fl *= -1
    alm = hp.almxfl(alm, torch.as_tensor(fl, device=alm.device))
    q, u = hp._spin_synth(alm, None, nside, 2, lmax)
    return [q.cpu().numpy(), u.cpu().numpy()] if numpy_out else [q, u]

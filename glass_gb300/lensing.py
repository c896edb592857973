"""Weak-lensing maps from the convergence (glass/lensing.py:185-586).

``from_convergence`` follows the reference step by step: analysis of kappa
(map2alm), multiplication by the harmonic kernels with almxfl, and spin-0,
spin-1 and spin-2 synthesis, all on the GPU.  ``MultiPlaneConvergence``
keeps its convergence planes on the device and advances them with one fused
kernel per plane.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from . import healpix as hp


def _ell(lmax: int, like) -> np.ndarray:
    return np.arange(lmax + 1, dtype=np.float64)


def from_convergence(kappa, lmax: int | None = None, *, potential: bool = False,
                     deflection: bool = False, shear: bool = False, discretized: bool = True,
                     form: str | None = None):
    """Potential, deflection and/or shear from a convergence map (glass/lensing.py:185-371).

    ``discretized=True`` (the default) scales the shear's harmonic kernel by
    the ratio of the spin-2 and spin-0 pixel windows pw2 / pw0
    (glass/lensing.py:360-362), computed on the GPU by ``healpix.pixwin``.
    ``form="plain"`` (default unless ``GLASS_GB300_FORM`` says otherwise):
    FP64 throughout.  ``form="fast"``: the analysis of kappa and the harmonic
    kernels stay FP64; the syntheses of the potential, deflection and shear
    run in the fast form (split-precision TF32 contractions, FP32 ring FFTs)
    and return float32 / complex64 maps.
    """
    if not (potential or deflection or shear):
        return ()
    form = _lib.default_form() if form is None else form
    if form not in ("plain", "fast"):
        raise ValueError(f"form must be 'plain' or 'fast', not {form!r}")
    fast = form == "fast"
    numpy_out = _lib.is_numpy_like(kappa)
    k = _lib.to_device(kappa, torch.float64)
    nside = hp.get_nside(k)
    if lmax is None:
        lmax = 3 * nside - 1
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
        psi = hp.synth(alm.reshape(1, -1), nside, lmax, form="fast")[0] if fast else \
            hp.synth(alm.reshape(1, -1), nside, lmax)[0]
        results += (out(psi),)
    if not (deflection or shear):
        return results
    # potential -> deflection: sqrt(l (l+1))
    fl = np.sqrt(ell * (ell + 1))
    alm = hp.almxfl(alm, torch.as_tensor(fl, device=alm.device))
    spin_synth = hp._spin_synth_fast if fast else hp._spin_synth
    if deflection:
        q, u = spin_synth(alm, None, nside, 1, lmax)
        results += (out(torch.complex(q, u)),)
    if not shear:
        return results
    # deflection -> shear: sqrt((l-1)(l+2)) / 2, 0 at l = 0
    fl = np.zeros_like(ell)
    fl[1:] = np.sqrt((ell[1:] - 1) * (ell[1:] + 2)) / 2
    flt = torch.as_tensor(fl, device=alm.device)
    if discretized:  # factor out the spin-0 pixel window, apply the spin-2 one
        pw0, pw2 = hp.pixwin_device(nside, lmax, alm.device)
        flt = flt * (pw2 / pw0)
    alm = hp.almxfl(alm, flt)
    q, u = spin_synth(alm, None, nside, 2, lmax)
    results += (out(torch.complex(q, u)),)
    return results


def shear_from_convergence(kappa, lmax: int | None = None, *, discretized: bool = True):
    """Shear maps [g1, g2] from convergence (glass/lensing.py:374-428; deprecated upstream)."""
    numpy_out = _lib.is_numpy_like(kappa)
    k = _lib.to_device(kappa, torch.float64)
    nside = hp.get_nside(k)
    if lmax is None:
        lmax = 3 * nside - 1
    alm = hp.analysis(k.reshape(1, -1), lmax, 3)[0]
    ell = np.arange(lmax + 1)
    fl = np.sqrt((ell + 2.0) * (ell + 1) * ell * (ell - 1))
    fl /= np.clip(ell * (ell + 1), 1, None)
    fl *= -1
    flt = torch.as_tensor(fl, device=alm.device)
    if discretized:
        pw0, pw2 = hp.pixwin_device(nside, lmax, alm.device)
        flt = flt * (pw2 / pw0)
    alm = hp.almxfl(alm, flt)
    q, u = hp._spin_synth(alm, None, nside, 2, lmax)
    return [q.cpu().numpy(), u.cpu().numpy()] if numpy_out else [q, u]


class MultiPlaneConvergence:
    """Convergence from multiple matter planes (glass/lensing.py:430-598).

    Same state and recurrence as the reference: the host computes the
    distance ratios t and the lensing weight f from ``cosmo`` exactly as the
    reference does, and one kernel per plane applies
    kappa3 <- kappa1 (1 - t) + t kappa2 + f delta2 to the device planes.
    numpy planes in give numpy planes out (``kappa`` / ``delta`` copy to the
    host on access); torch planes stay on the device.
    """

    def __init__(self, cosmo) -> None:
        self.cosmo = cosmo
        self.z2 = 0.0
        self.z3 = 0.0
        self.x3 = 0.0
        self.w3 = 0.0
        self.r23 = 1.0
        self._delta3 = None
        self._kappa2 = None
        self._kappa3 = None
        self._numpy = True

    def add_window(self, delta, w) -> None:
        """Add a mass plane with the weight and redshift of window ``w``."""
        zsrc = w.zeff
        lens_weight = float(np.trapezoid(w.wa, w.za) / np.interp(zsrc, w.za, w.wa))
        self.add_plane(delta, zsrc, lens_weight)

    def add_plane(self, delta, zsrc, wlens: float = 1.0) -> None:
        """Add a mass plane at redshift ``zsrc`` (glass/lensing.py:512-581)."""
        if zsrc <= self.z3:
            raise ValueError("source redshift must be increasing")
        self._numpy = _lib.is_numpy_like(delta)
        d = _lib.to_device(delta, torch.float64 if np.asarray(delta).dtype != np.float32 else torch.float32) \
            if self._numpy else delta.contiguous()
        if d.dtype not in (torch.float32, torch.float64):
            d = d.to(torch.float64)
        delta2, self._delta3 = self._delta3, d
        z1, self.z2, self.z3 = self.z2, self.z3, zsrc
        w2, self.w3 = self.w3, wlens
        x2, self.x3 = (self.x3,
                       self.cosmo.transverse_comoving_distance(self.z3) / self.cosmo.hubble_distance)
        r12 = self.r23
        r13, self.r23 = self.cosmo.transverse_comoving_distance([z1, self.z2], self.z3) / (
            self.cosmo.hubble_distance * self.x3)
        t = r13 / r12
        f = 3 * self.cosmo.Omega_m0 / 2
        f *= x2 * self.r23
        f *= (1 + self.z2) / self.cosmo.H_over_H0(self.z2)
        f *= w2
        if self._kappa2 is None:
            self._kappa2 = torch.zeros_like(d)
            self._kappa3 = torch.zeros_like(d)
        self._kappa2, self._kappa3 = self._kappa3, self._kappa2
        k3 = self._kappa3
        if delta2 is not None and (delta2.dtype != k3.dtype or delta2.shape != k3.shape):
            raise ValueError("mass planes must share their shape and dtype")
        code = _lib.GLG_F64 if k3.dtype == torch.float64 else _lib.GLG_F32
        _lib.check(_lib.lib().glg_convergence_step(
            _lib.c_p(_lib.ptr(k3)), _lib.c_p(_lib.ptr(self._kappa2)), _lib.c_p(_lib.ptr(delta2)), code,
            k3.numel(), float(t), float(f), _lib.c_p(_lib.stream_ptr(k3.device))), "glg_convergence_step")

    def _out(self, t):
        if t is None:
            return None
        return t.cpu().numpy() if self._numpy else t

    @property
    def zsrc(self):
        """The redshift of the current convergence plane."""
        return self.z3

    @property
    def kappa(self):
        """The current convergence plane."""
        return self._out(self._kappa3)

    @property
    def delta(self):
        """The current matter plane."""
        return self._out(self._delta3)

    @property
    def wlens(self) -> float:
        """The weight of the current matter plane."""
        return self.w3

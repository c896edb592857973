"""A flat LambdaCDM stand-in for the ``cosmology`` objects GLASS takes.

Test infrastructure: the golden generator and the tests hand the same
object to the reference's MultiPlaneConvergence and to glass_gb300's, so the
host-side scalars of both agree.  Comoving distance by a fixed 2000-point
Gauss-Legendre rule (deterministic)."""

from __future__ import annotations

import numpy as np


class FlatLCDM:
    def __init__(self, omega_m: float = 0.3, h: float = 0.7):
        self.Omega_m0 = omega_m
        self.hubble_distance = 2997.92458 / h  # Mpc
        self._x, self._w = np.polynomial.legendre.leggauss(2000)

    def H_over_H0(self, z):
        z = np.asarray(z, dtype=np.float64)
        return np.sqrt(self.Omega_m0 * (1 + z) ** 3 + 1 - self.Omega_m0)

    def _dc(self, z):
        z = np.asarray(z, dtype=np.float64)
        zz = 0.5 * z[..., None] * (self._x + 1)
        return self.hubble_distance * 0.5 * z * np.sum(self._w / self.H_over_H0(zz), axis=-1)

    def transverse_comoving_distance(self, z1, z2=None):
        if z2 is None:
            return self._dc(z1)
        return self._dc(z2) - self._dc(z1)

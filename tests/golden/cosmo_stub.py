"""A flat LambdaCDM stand-in for the ``cosmology`` objects GLASS takes.

Test infrastructure: the golden generator and the tests hand the same
object to the reference's MultiPlaneConvergence and to glass_gb300's, so the
host-side scalars of both agree.  Every number comes from correctly rounded
scalar operations (math.sqrt, math.fsum), so it is the same on every
platform; comoving distance by a 4096-point midpoint rule."""

from __future__ import annotations

import math

import numpy as np

_N = 4096


class FlatLCDM:
    def __init__(self, omega_m: float = 0.3, h: float = 0.7):
        self.Omega_m0 = omega_m
        self.hubble_distance = 2997.92458 / h  # Mpc

    def _e(self, z: float) -> float:
        a = 1.0 + z
        return math.sqrt(self.Omega_m0 * (a * a * a) + (1.0 - self.Omega_m0))

    def H_over_H0(self, z):
        if np.ndim(z) == 0:
            return self._e(float(z))
        return np.array([self._e(float(x)) for x in np.ravel(z)]).reshape(np.shape(z))

    def _dc(self, z: float) -> float:
        dz = z / _N
        return self.hubble_distance * dz * math.fsum(1.0 / self._e((k + 0.5) * dz) for k in range(_N))

    def transverse_comoving_distance(self, z1, z2=None):
        if z2 is None:
            if np.ndim(z1) == 0:
                return self._dc(float(z1))
            return np.array([self._dc(float(x)) for x in np.ravel(z1)]).reshape(np.shape(z1))
        d2 = self._dc(float(z2))
        if np.ndim(z1) == 0:
            return d2 - self._dc(float(z1))
        return np.array([d2 - self._dc(float(x)) for x in np.ravel(z1)]).reshape(np.shape(z1))

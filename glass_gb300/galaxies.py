"""Observed galaxy shears (glass/galaxies.py:271-347).

``galaxy_shear`` gathers convergence and shear at each galaxy's HEALPix RING
pixel and applies the reduced-shear transformation in one kernel; the
arithmetic follows the reference's numpy expressions step by step.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from . import healpix as hp

__all__ = ["galaxy_shear"]


def galaxy_shear(lon, lat, eps, kappa, gamma1, gamma2, *, reduced_shear: bool = True):
    """Lensed ellipticities of galaxies at (lon, lat) in degrees (complex128)."""
    numpy_out = _lib.is_numpy_like(lon)
    dev = torch.device("cuda", torch.cuda.current_device()) if numpy_out else lon.device
    maps = [k if isinstance(k, torch.Tensor) else torch.as_tensor(np.asarray(k)) for k in (kappa, gamma1, gamma2)]
    mdt = torch.float32 if all(m.dtype == torch.float32 for m in maps) else torch.float64
    maps = [m.to(dev, mdt).contiguous().reshape(-1) for m in maps]
    nside = hp.npix2nside(maps[0].numel())
    lo = _lib.to_device(lon, torch.float64, dev).reshape(-1)
    la = _lib.to_device(lat, torch.float64, dev).reshape(-1)
    e = _lib.to_device(eps, torch.complex128, dev).reshape(-1)
    n = lo.numel()
    if la.numel() != n or e.numel() != n:
        raise ValueError("lon, lat and eps must have the same size")
    out = torch.empty(n, dtype=torch.complex128, device=dev)
    code = _lib.GLG_F64 if mdt == torch.float64 else _lib.GLG_F32
    c = _lib.c_p
    _lib.check(_lib.lib().glg_galaxy_shear(c(_lib.ptr(lo)), c(_lib.ptr(la)), c(_lib.ptr(e)), n,
                                           c(_lib.ptr(maps[0])), c(_lib.ptr(maps[1])), c(_lib.ptr(maps[2])),
                                           code, nside, 1 if reduced_shear else 0, c(_lib.ptr(out)),
                                           c(_lib.stream_ptr(dev))), "glg_galaxy_shear")
    return out.cpu().numpy() if numpy_out else out

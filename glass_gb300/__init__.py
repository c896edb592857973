"""glass_gb300: GB300-native field generation for GLASS.

A drop-in for the field-generation path of GLASS (glass-dev/glass):
``generate``, ``generate_gaussian``, ``generate_lognormal``, ``iternorm``,
``cls2cov`` (glass/fields.py), ``from_convergence`` and
``shear_from_convergence`` (glass/lensing.py), ``multalm``
(glass/harmonics.py) and the HEALPix transform façade (glass/healpix.py),
computed by hand-written CUDA kernels for sm_103a behind the C ABI of
``include/glass_gb300.h``.  There is no CPU fallback.
"""

from __future__ import annotations

from . import galaxies, grf, harmonics, healpix, points, rng, user
from .fields import (
    accuracy_report,
    cls2cov,
    enumerate_spectra,
    generate,
    generate_gaussian,
    generate_lognormal,
    getcl,
    iternorm,
    nfields_from_nspectra,
    spectra_indices,
)
from .harmonics import multalm
from .galaxies import galaxy_shear
from .user import load_cls, save_cls
from .lensing import MultiPlaneConvergence, from_convergence, shear_from_convergence

__all__ = [
    "MultiPlaneConvergence",
    "accuracy_report",
    "cls2cov",
    "enumerate_spectra",
    "from_convergence",
    "galaxies",
    "galaxy_shear",
    "generate",
    "generate_gaussian",
    "generate_lognormal",
    "getcl",
    "grf",
    "harmonics",
    "healpix",
    "points",
    "iternorm",
    "load_cls",
    "multalm",
    "nfields_from_nspectra",
    "rng",
    "save_cls",
    "shear_from_convergence",
    "spectra_indices",
]

__version__ = "0.1.0"

"""Transformations of Gaussian random fields (glass/grf/_transformations.py).

Only ``__call__`` is on the field-generation path.  ``generate`` fuses the
transforms it recognises (:class:`Normal`, :class:`Lognormal`, and the
reference's own classes of the same names) into the map store of the
transform kernel; any other callable is applied to the finished map.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch


def _expm1(x):
    return torch.expm1(x) if isinstance(x, torch.Tensor) else np.expm1(x)


@dataclass
class Normal:
    """t(X) = X (glass/grf/_transformations.py:14-28)."""

    def __call__(self, x, _var: float, /):
        return x


@dataclass
class Lognormal:
    """t(X) = lamda [exp(X - var/2) - 1] (glass/grf/_transformations.py:62-89)."""

    lamda: float = 1.0

    def __call__(self, x, var: float, /):
        x = _expm1(x - var / 2)
        if self.lamda != 1.0:
            x = self.lamda * x
        return x


@dataclass
class SquaredNormal:
    """t(X) = lamda [(X - a)^2 - 1] (glass/grf/_transformations.py:141-...)."""

    a: float
    lamda: float = 1.0

    def __call__(self, x, _var: float, /):
        return self.lamda * ((x - self.a) ** 2 - 1)


def fused_kind(t) -> tuple[str, float] | None:
    """('normal', 1) / ('lognormal', lamda) for transforms the kernel fuses."""
    name = type(t).__name__
    if name == "Normal" and not hasattr(t, "lamda"):
        return ("normal", 1.0)
    if name == "Lognormal" and hasattr(t, "lamda"):
        return ("lognormal", float(t.lamda))
    return None

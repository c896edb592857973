"""Spherical-harmonic utilities (glass/harmonics.py)."""

from __future__ import annotations

import math

import torch

from . import _lib
from ._lib import c_p, check, lib, ptr, stream_ptr


def multalm(alm, bl):
    """alm * repeat(bl, l+1) for alm in GLASS order (glass/harmonics.py:17-47).

    GLASS order is l-major: [00, 10, 11, 20, 21, 22, ...].  Computed by the
    CUDA library; numpy in, numpy out.
    """
    numpy_out = _lib.is_numpy_like(alm)
    a = _lib.to_device(alm, torch.complex128)
    b = _lib.to_device(bl, torch.float64, a.device).reshape(-1)
    n = b.numel()
    if a.numel() != n * (n + 1) // 2:
        raise ValueError(f"alm of size {a.numel()} does not match bl of size {n}")
    real_in = not torch.is_complex(torch.as_tensor(alm)) if numpy_out else not torch.is_complex(alm)
    out = torch.empty_like(a)
    if n:
        check(lib().glg_multalm(c_p(ptr(a)), c_p(ptr(b)), n - 1, _lib.GLG_F64, c_p(ptr(out)),
                                c_p(stream_ptr(a.device))), "glg_multalm")
    if real_in:
        out = out.real
    return out.cpu().numpy() if numpy_out else out


def lmax_from_glass_size(n: int) -> int:
    L = (math.isqrt(8 * n + 1) - 1) // 2
    if L * (L + 1) // 2 != n:
        raise ValueError(f"not a triangle number: {n}")
    return L - 1

"""Poisson galaxy counts per pixel (GLASS glass/points.py:252-348).

``positions_from_delta`` (glass/points.py:443-540) turns a density contrast
into an expected number of galaxies per pixel and draws the actual number
from a Poisson distribution before it samples positions inside the pixels.
:func:`counts_from_delta` is that count map on the device: the expected
count (``_compute_expected_count``, ``_apply_visibility``) and the clipped
Poisson draw (``_sample_number_galaxies``) in one kernel, from the Philox
stream of :mod:`glass_gb300.rng`.  Given the same delta values the counts are
identical whatever form produced delta (plain FP64 or fast FP32 maps).
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from ._lib import c_p, check, lib, ptr, stream_ptr
from . import rng as grng

__all__ = ["ARCMIN2_SPHERE", "counts_from_delta", "linear_bias", "loglinear_bias"]

ARCMIN2_SPHERE = 60**6 // 100 / math.pi  # glass/points.py:72


def linear_bias(delta, b):
    """Linear bias model delta_g = b delta (glass/points.py:115-134)."""
    return b * delta


def loglinear_bias(delta, b):
    """Log-linear bias model ln(1 + delta_g) = b ln(1 + delta) (glass/points.py:137-160)."""
    if isinstance(delta, torch.Tensor):
        return torch.expm1(b * torch.log1p(delta))
    return np.expm1(b * np.log1p(delta))


def _stream_of(rng) -> tuple[int, int]:
    """(seed, stream id) for one count map."""
    if rng is None:
        rng = grng.default_rng()
    if isinstance(rng, grng.Generator):
        return rng.seed, rng.reserve_streams(1) & 0xFFFFFFFF
    if isinstance(rng, np.random.Generator):
        # the reference's numpy stream cannot run on the device: key the
        # Philox stream with a seed drawn from the caller's generator
        return int(rng.integers(0, 2**63)), 0
    raise TypeError("rng must be a numpy Generator or a glass_gb300.rng.Generator")


def counts_from_delta(ngal: float, delta, bias: float | None = None, vis=None, *,
                      bias_model=linear_bias, remove_monopole: bool = False, rng=None):
    """Poisson-sampled galaxy counts per pixel of one delta map.

    ``n = (bias_model(delta, bias) [- mean] + 1) * ARCMIN2_SPHERE / npix * ngal``,
    times ``vis`` when given, clipped at zero, then one Poisson draw per pixel
    (glass/points.py:252-348).  ``delta`` is a float64 or float32 map (numpy
    or CUDA torch); the result is int64 in the same namespace.
    """
    if not callable(bias_model):
        raise TypeError("bias_model must be callable")
    numpy_in = not isinstance(delta, torch.Tensor)
    dev = torch.device("cuda", torch.cuda.current_device()) if numpy_in else delta.device
    d = torch.as_tensor(np.asarray(delta)) if numpy_in else delta
    if d.dtype not in (torch.float32, torch.float64):
        d = d.to(torch.float64)
    d = d.to(dev).contiguous().reshape(-1)
    b = 1.0
    if bias is not None:
        if bias_model is linear_bias:
            b = float(bias)  # fused into the kernel
        else:
            d = bias_model(d.double(), bias).contiguous()
    npix = d.numel()
    if npix == 0:
        empty = torch.empty(0, dtype=torch.int64, device=dev)
        return empty.cpu().numpy() if numpy_in else empty
    offset = 0.0
    if remove_monopole:
        offset = float((b * d.double()).mean())
    scale = ARCMIN2_SPHERE / npix * float(ngal)
    v = None
    if vis is not None:
        v = _lib.to_device(vis, torch.float64, dev).reshape(-1)
        if v.numel() != npix:
            raise ValueError("vis must have the shape of delta")
    seed, sid = _stream_of(rng)
    counts = torch.empty(npix, dtype=torch.int64, device=dev)
    code = _lib.GLG_F64 if d.dtype == torch.float64 else _lib.GLG_F32
    with torch.cuda.device(dev):
        check(lib().glg_poisson_counts(c_p(ptr(d)), code, npix, b, offset, scale, c_p(ptr(v)),
                                       ctypes.c_uint64(seed), ctypes.c_uint64(sid), c_p(ptr(counts)),
                                       c_p(stream_ptr(dev))), "glg_poisson_counts")
    return counts.cpu().numpy() if numpy_in else counts

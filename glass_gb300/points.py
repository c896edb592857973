"""Poisson galaxy counts per pixel and galaxy positions (glass/points.py:252-540).

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

__all__ = ["ARCMIN2_SPHERE", "counts_from_delta", "linear_bias", "loglinear_bias", "positions_from_delta"]

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
    if isinstance(rng, _Keyed):
        return rng.seed, rng.sid
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


def _leading(x, dims, k, core: int):
    """Entry k of x broadcast to leading axes ``dims`` (``core`` trailing axes kept)."""
    if x is None:
        return None
    if isinstance(x, torch.Tensor):
        return x.expand(*dims, *x.shape[x.dim() - core:])[k] if dims else x
    a = np.asarray(x)
    return np.broadcast_to(a, (*dims, *a.shape[a.ndim - core:]))[k] if dims else a


def positions_from_delta(ngal, delta, bias=None, vis=None, *, bias_model=linear_bias,
                         remove_monopole: bool = False, batch: int = 1_000_000, rng=None):
    """Positions tracing a density contrast (glass/points.py:443-540).

    Poisson counts per pixel as :func:`counts_from_delta`, then every galaxy
    placed uniformly on its pixel's area (the healpy.randang step), all on
    the device.  Yields ``(lon, lat, count)`` batches of at most ``batch``
    positions, each batch ending at a pixel boundary (a pixel with more
    points than ``batch`` is one batch), in pixel order like the reference
    (glass/points.py:351-440).  Leading axes of ``ngal``, ``delta``, ``bias``
    and ``vis`` broadcast together into separate populations, sampled in
    turn, with ``count`` an array in the shape of those axes that marks the
    population (glass/points.py:163-211).
    """
    if not callable(bias_model):
        raise TypeError("bias_model must be callable")
    numpy_in = not isinstance(delta, torch.Tensor)
    d = torch.as_tensor(np.asarray(delta)) if numpy_in else delta
    shapes = [np.shape(ngal), tuple(d.shape[:-1])]
    if bias is not None:
        shapes.append(np.shape(bias))
    if vis is not None:
        shapes.append(tuple(vis.shape[:-1]))
    dims = tuple(np.broadcast_shapes(*shapes))
    dev = torch.device("cuda", torch.cuda.current_device()) if numpy_in else d.device
    d = d.to(dev)
    nflat = int(np.prod(dims)) if dims else 1
    if rng is None:
        rng = grng.default_rng()
    if isinstance(rng, grng.Generator):  # two streams per population: counts, positions
        seed, sid0 = rng.seed, rng.reserve_streams(2 * nflat)
    else:
        seed, sid0 = _stream_of(rng)
    for k_flat in range(nflat):
        k = tuple(int(i) for i in np.unravel_index(k_flat, dims)) if dims else ()
        ng = float(_leading(ngal, dims, k, 0))
        b = None if bias is None else float(_leading(bias, dims, k, 0))
        counts = counts_from_delta(ng, _leading(d, dims, k, 1), b, _leading(vis, dims, k, 1),
                                   bias_model=bias_model, remove_monopole=remove_monopole,
                                   rng=_Keyed(seed, (sid0 + 2 * k_flat) & 0xFFFFFFFF))
        counts = torch.as_tensor(counts).to(dev)
        npix = counts.numel()
        nside = int(round((npix // 12) ** 0.5))
        if npix == 0 or 12 * nside * nside != npix:
            raise ValueError("delta must be a HEALPix map")
        cum = torch.cumsum(counts, 0)
        off = cum - counts  # exclusive prefix sums
        total = int(cum[-1])
        if dims:
            cmask = np.zeros(dims, dtype=np.int64)
            cmask[k] = 1
        else:
            cmask = 1
        miss = torch.zeros(1, dtype=torch.int64, device=dev)
        start = 0
        while start < total:
            # the batch ends at the last pixel boundary within `batch` points
            stop = int(torch.searchsorted(cum, torch.tensor(start + batch, device=dev), right=True))
            end = int(cum[stop - 1]) if stop > 0 else 0
            if end <= start:  # the next pixel alone holds more than `batch`
                end = int(cum[int(torch.searchsorted(cum, torch.tensor(start, device=dev), right=True))])
            n = end - start
            lon = torch.empty(n, dtype=torch.float64, device=dev)
            lat = torch.empty(n, dtype=torch.float64, device=dev)
            with torch.cuda.device(dev):
                check(lib().glg_positions(nside, c_p(ptr(off)), start, n, ctypes.c_uint64(seed),
                                          ctypes.c_uint64((sid0 + 2 * k_flat + 1) & 0xFFFFFFFF), c_p(ptr(lon)),
                                          c_p(ptr(lat)), c_p(ptr(miss)), c_p(stream_ptr(dev))), "glg_positions")
            if numpy_in:
                yield lon.cpu().numpy(), lat.cpu().numpy(), n * cmask
            else:
                yield lon, lat, n * cmask
            start = end
        if total and int(miss) != 0:
            # 64 draws from a box that the pixel fills half of: never in practice
            raise RuntimeError(f"positions_from_delta: {int(miss)} positions were not placed in their pixel")


class _Keyed:
    """A fixed (seed, stream) pair for counts_from_delta."""

    def __init__(self, seed: int, sid: int):
        self.seed, self.sid = seed, sid

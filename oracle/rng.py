"""Philox4x32-10 + Box-Muller restatement of the GPU variate stream.

TEST INFRASTRUCTURE ONLY.  The reference draws its Gaussian variates from
numpy's PCG64 (``glass/fields.py:407`` via ``glass/rng.py:176-197``); the GPU
path draws them from a counter-based Philox4x32-10 stream instead, so any
shell's variates can be regenerated independently.  This module is the CPU
checker for that stream: integer outputs are bit-exact, normals agree to a
few ulp (host libm vs CUDA math).
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import lib


def philox4x32_10(counter, key) -> np.ndarray:
    c = (ctypes.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in counter])
    k = (ctypes.c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    o = (ctypes.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return np.array(list(o), dtype=np.uint32)


def complex_normals(seed: int, stream: int, offset: int, n: int, raw: bool = False):
    """Elements offset..offset+n-1 of complex stream `stream` under key `seed`."""
    z = np.empty(n, dtype=np.complex128)
    r = np.empty((n, 4), dtype=np.uint32) if raw else None
    lib().orc_philox_normals(
        ctypes.c_uint64(seed), ctypes.c_uint64(stream), ctypes.c_int64(offset), ctypes.c_int64(n),
        z.view(np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
        None if r is None else r.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
    )
    return (z, r) if raw else z


def poisson_counts(delta, *, bias: float = 1.0, offset: float = 0.0, scale: float = 1.0, vis=None,
                   seed: int = 42, stream: int = 0) -> np.ndarray:
    """Per-pixel Poisson counts of the GPU stream (bit-exact restatement)."""
    d = np.ascontiguousarray(delta, dtype=np.float64)
    v = None if vis is None else np.ascontiguousarray(vis, dtype=np.float64)
    out = np.empty(d.size, dtype=np.int64)
    dp = ctypes.POINTER(ctypes.c_double)
    lib().orc_poisson_counts(
        d.ctypes.data_as(dp), ctypes.c_int64(d.size), ctypes.c_double(bias), ctypes.c_double(offset),
        ctypes.c_double(scale), None if v is None else v.ctypes.data_as(dp), ctypes.c_uint64(seed),
        ctypes.c_uint32(stream), out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    return out

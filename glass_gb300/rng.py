"""Random-number seam of the GPU path (replaces glass/rng.py:21-247 for fields).

The reference draws its Gaussian variates from numpy's PCG64 stream.  A
counter-based stream lets every shell's variates be generated independently
on the device, so this module provides :class:`Generator`, a Philox4x32-10
generator: stream ``sid`` element ``e`` under key ``seed`` is one Philox block
mapped by Box-Muller.  Passing a numpy ``Generator`` to the field functions
instead reproduces the reference's own draws exactly (they are then made on
the host, in the reference's order, and uploaded).
"""

from __future__ import annotations

import ctypes
import threading

import torch

from . import _lib
from ._lib import c_p, check, lib, ptr, stream_ptr

SEED = 42  # glass/rng.py:18


class Generator:
    """Philox4x32-10 generator of complex standard normals on the device."""

    def __init__(self, seed: int = SEED):
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self._next_stream = 0
        self._lock = threading.Lock()

    def reserve_streams(self, n: int) -> int:
        """Reserve n consecutive stream ids; returns the first."""
        with self._lock:
            s = self._next_stream
            self._next_stream += int(n)
        return s

    def complex_normal(self, n: int, *, sid: int | None = None, offset: int = 0,
                       dtype: torch.dtype = torch.complex128,
                       device: torch.device | None = None) -> torch.Tensor:
        """n complex standard normals (real and imaginary parts each N(0, 1))."""
        if sid is None:
            sid = self.reserve_streams(1)
        device = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        out = torch.empty(int(n), dtype=dtype, device=device)
        code = _lib.GLG_F64 if dtype == torch.complex128 else _lib.GLG_F32
        check(lib().glg_philox_normals(ctypes.c_uint64(self.seed), ctypes.c_uint64(sid), int(offset),
                                       int(n), code, c_p(ptr(out)), c_p(stream_ptr(device))),
              "glg_philox_normals")
        return out

    def standard_normal(self, size=None, dtype: torch.dtype = torch.float64,
                        device: torch.device | None = None) -> torch.Tensor:
        """Real standard normals of the given shape (pairs of one complex draw)."""
        shape = () if size is None else (tuple(size) if isinstance(size, (tuple, list)) else (int(size),))
        n = 1
        for s in shape:
            n *= s
        cdt = torch.complex128 if dtype == torch.float64 else torch.complex64
        z = self.complex_normal((n + 1) // 2, dtype=cdt, device=device)
        return torch.view_as_real(z).reshape(-1)[:n].reshape(shape).to(dtype)


def default_rng(seed: int = SEED) -> Generator:
    """Default GPU generator (seeded like glass.rng.default_rng)."""
    return Generator(seed)

"""HEALPix spherical-harmonic transforms on the GPU.

Drop-in for the transform façade of ``glass/healpix.py`` (``alm2map``
:38-78, ``alm2map_spin`` :81-108, ``almxfl`` :111-140, ``get_nside``
:214-229, ``map2alm`` :232-276, ``nside2npix`` :296, ``npix2nside``), which
the reference delegates to healpy.  Inputs may be numpy arrays (results come
back as numpy) or torch tensors (results stay on the device).  Everything is
computed by the CUDA library; nothing falls back to the CPU.

Conventions (HEALPix): RING ordering, alm in m-major order with mmax = lmax,
Condon-Shortley phase; spin-s maps ``Q + iU = -sum_lm (E_lm + i B_lm) sY_lm``.
"""

from __future__ import annotations

import ctypes
import math
import os
import warnings
from collections.abc import Sequence

import numpy as np
import torch

from . import _lib
from ._lib import c_p, check, get_plan, lib, ptr, stream_ptr

__all__ = [
    "SynthGraph",
    "alm2map",
    "ang2pix",
    "alm2map_spin",
    "almxfl",
    "get_nside",
    "map2alm",
    "npix2nside",
    "nside2npix",
    "pixwin",
]


def nside2npix(nside: int) -> int:
    return 12 * int(nside) * int(nside)


def npix2nside(npix: int) -> int:
    nside = math.isqrt(int(npix) // 12)
    if 12 * nside * nside != int(npix):
        raise ValueError(f"{npix} is not a valid number of HEALPix pixels")
    return nside


def ang2pix(nside: int, theta, phi, *, lonlat: bool = False):
    """RING-scheme pixel indices of positions (healpy.ang2pix, as called
    through glass/healpix.py at glass/galaxies.py:329).  With ``lonlat``,
    ``theta`` / ``phi`` are longitude / latitude in degrees."""
    numpy_out = _lib.is_numpy_like(theta)
    a = _lib.to_device(theta, torch.float64).reshape(-1)
    b = _lib.to_device(phi, torch.float64).reshape(-1)
    if a.numel() != b.numel():
        raise ValueError("theta and phi must have the same size")
    out = torch.empty(a.numel(), dtype=torch.int64, device=a.device)
    _lib.check(_lib.lib().glg_ang2pix(int(nside), _lib.c_p(_lib.ptr(a)), _lib.c_p(_lib.ptr(b)), a.numel(),
                                      1 if lonlat else 0, _lib.c_p(_lib.ptr(out)),
                                      _lib.c_p(_lib.stream_ptr(a.device))), "glg_ang2pix")
    shape = np.shape(theta) if numpy_out else tuple(theta.shape)
    return _finish(out.reshape(shape), numpy_out)


def get_nside(m) -> int:
    n = m.shape[-1]
    return npix2nside(n)


def _lmax_from_size(n: int) -> int:
    lmax = (math.isqrt(8 * n + 1) - 3) // 2
    if (lmax + 1) * (lmax + 2) // 2 != n:
        raise ValueError(f"wrong alm size {n}: not (lmax+1)(lmax+2)/2 for any lmax")
    return lmax


def _as_device_alm(a) -> torch.Tensor:
    return _lib.to_device(a, torch.complex128)


def _finish(t: torch.Tensor, numpy_out: bool):
    return t.cpu().numpy() if numpy_out else t


def _resize_alm(alm: torch.Tensor, lmax_in: int, lmax_out: int) -> torch.Tensor:
    """Truncate or zero-pad HEALPix-order alm (mmax = lmax) to another lmax."""
    if lmax_in == lmax_out:
        return alm
    out = torch.zeros(alm.shape[:-1] + ((lmax_out + 1) * (lmax_out + 2) // 2,), dtype=alm.dtype,
                      device=alm.device)
    lm = min(lmax_in, lmax_out)
    for m in range(lm + 1):
        si = m * (2 * lmax_in + 1 - m) // 2
        so = m * (2 * lmax_out + 1 - m) // 2
        out[..., so + m:so + lm + 1] = alm[..., si + m:si + lm + 1]
    return out


FAST_MAX_MAPS = 40  # maps per fast-form launch (N = 80 tensor-core columns)


def synth(alm: torch.Tensor, nside: int, lmax: int, *, epilogue=None, form: str = "plain",
          out: torch.Tensor | None = None, ws: torch.Tensor | None = None,
          status: torch.Tensor | None = None) -> torch.Tensor:
    """Spin-0 synthesis of alm [nmaps, nalm] -> maps [nmaps, npix].

    ``form="plain"``: complex128 alm, float64 maps (FP64 throughout).
    ``form="fast"``: complex64 alm, float32 maps (tensor-core Legendre sums);
    ``out`` may be a float32 [nmaps, npix] device tensor or pinned host
    tensor to write the maps into.
    ``ws``: a caller-owned uint8 device workspace of at least
    ``workspace_bytes(...)`` bytes (allocated per call otherwise).
    ``status`` (fast form, device maps): a pinned int32 host tensor of one
    element that receives the call's device-wait status asynchronously
    instead of the call synchronising to check it (the caller reads it once
    the stream has passed the call; non-zero = a bounded wait timed out).
    """
    if form == "fast":
        return _synth_fast(alm, nside, lmax, epilogue, out, ws, status)
    if out is not None:
        raise ValueError("out is supported by the fast form only")
    plan = get_plan(nside, lmax, alm.device)
    nmaps = alm.shape[0]
    maps = torch.empty((nmaps, plan.npix), dtype=torch.float64, device=alm.device)
    ws_bytes = int(lib().glg_alm2map_workspace(plan.handle, nmaps, _lib.FORM_PLAIN))
    if ws is None or ws.numel() < ws_bytes:
        ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=alm.device)
    epi = _make_epilogue(epilogue, nmaps)
    check(lib().glg_alm2map(plan.handle, c_p(ptr(alm)), nmaps, _lib.FORM_PLAIN, c_p(ptr(maps)),
                            ctypes.byref(epi) if epi is not None else None, c_p(ptr(ws)), ws_bytes,
                            c_p(stream_ptr(alm.device))), "glg_alm2map")
    return maps


def autotune(plan, nmaps: int, maps: torch.Tensor, ws: torch.Tensor) -> None:
    """Pick the ring-FFT block sizes of ``plan`` by timing (glg_autotune_fast).

    Runs once per plan (on its first fast transform) unless the environment
    sets ``GLASS_GB300_AUTOTUNE=0``; ``buckets`` reports the choice."""
    if getattr(plan, "tuned", False) or os.environ.get("GLASS_GB300_AUTOTUNE", "1") == "0":
        return
    check(lib().glg_autotune_fast(plan.handle, nmaps, c_p(ptr(maps)), c_p(ptr(ws)), ws.numel(),
                                  c_p(stream_ptr(maps.device))), "glg_autotune_fast")
    plan.tuned = True


def buckets(nside: int, lmax: int) -> list[dict]:
    """The fast-form ring-FFT launch buckets of a plan: kind (0 mixed radix,
    1 Bluestein, 2 power-of-two equatorial length), transform size, ring
    pairs, threads per block and the autotuner's time of one launch (ms, for
    the map count it was tuned on)."""
    plan = get_plan(nside, lmax)
    out = (ctypes.c_int * (4 * 64))()
    n = lib().glg_plan_buckets(plan.handle, out, 64)
    ms = (ctypes.c_float * 64)()
    lib().glg_plan_bucket_times(plan.handle, ms, 64)
    return [dict(kind=out[4 * i], size=out[4 * i + 1], pairs=out[4 * i + 2], threads=out[4 * i + 3],
                 ms=float(ms[i])) for i in range(n)]


def workspace_bytes(nside: int, lmax: int, nmaps: int, form: str = "fast", device=None) -> int:
    """Device workspace of one synthesis call of ``nmaps`` maps (device maps)."""
    plan = get_plan(nside, lmax, device)
    f = _lib.FORM_FAST if form == "fast" else _lib.FORM_PLAIN
    return int(lib().glg_alm2map_workspace(plan.handle, min(nmaps, FAST_MAX_MAPS) if form == "fast" else nmaps, f))


def _synth_fast(alm: torch.Tensor, nside: int, lmax: int, epilogue, out: torch.Tensor | None = None,
                ws: torch.Tensor | None = None, status: torch.Tensor | None = None) -> torch.Tensor:
    """Fast-form synthesis into new device maps, or into ``out``: float32
    [nmaps, npix] on the device, or in host memory (pinned, for the copies to
    overlap), which glg_alm2map_host fills run by run while the next run of
    ring tiles computes."""
    plan = get_plan(nside, lmax, alm.device)
    alm = alm.to(torch.complex64).contiguous()
    nmaps = alm.shape[0]
    if out is None:
        maps = torch.empty((nmaps, plan.npix), dtype=torch.float32, device=alm.device)
    else:
        if out.dtype != torch.float32 or tuple(out.shape) != (nmaps, plan.npix) or not out.is_contiguous():
            raise ValueError("out must be a contiguous float32 [nmaps, npix] tensor")
        if not (out.is_cuda or out.device.type == "cpu"):
            raise ValueError("out must be a CUDA or CPU tensor")
        maps = out
    to_host = not maps.is_cuda
    base = ptr(maps) if maps.is_cuda else maps.data_ptr()
    step = min(nmaps, FAST_MAX_MAPS)
    ws_bytes = int(lib().glg_alm2map_host_workspace(plan.handle, step) if to_host else
                   lib().glg_alm2map_workspace(plan.handle, step, _lib.FORM_FAST))
    if ws is None or ws.numel() < ws_bytes:
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device=alm.device)
    else:
        ws_bytes = ws.numel()
    stream = c_p(stream_ptr(alm.device))
    if not getattr(plan, "tuned", False):  # time the FFT buckets on device maps
        autotune(plan, step, maps[:step] if maps.is_cuda else
                 torch.empty((step, plan.npix), dtype=torch.float32, device=alm.device), ws)
    for m0 in range(0, nmaps, step):
        cnt = min(step, nmaps - m0)
        epi = None
        if epilogue is not None:
            kind, var, lam = epilogue
            kinds = list(kind) if isinstance(kind, (list, tuple)) else [int(kind)] * nmaps
            epi = _make_epilogue((kinds[m0:m0 + cnt], var[m0:m0 + cnt], lam[m0:m0 + cnt]), cnt)
        epi_p = ctypes.byref(epi) if epi is not None else None
        if to_host:
            check(lib().glg_alm2map_host(plan.handle, c_p(ptr(alm[m0:m0 + cnt])), cnt, c_p(base + 4 * m0 * plan.npix),
                                         epi_p, c_p(ptr(ws)), ws_bytes, stream), "glg_alm2map_host")
        else:
            check(lib().glg_alm2map(plan.handle, c_p(ptr(alm[m0:m0 + cnt])), cnt, _lib.FORM_FAST,
                                    c_p(base + 4 * m0 * plan.npix), epi_p, c_p(ptr(ws)), ws_bytes, stream),
                  "glg_alm2map (fast)")
    if status is not None and not to_host and nmaps <= step:  # one call: one status word
        status.copy_(ws[:4].view(torch.int32), non_blocking=True)
    else:
        check(lib().glg_workspace_status(c_p(ptr(ws)), stream), "glg_alm2map (fast)")
    return maps


class SynthGraph:
    """A fast-form synthesis captured once into a CUDA graph and replayed.

    Static buffers: ``alm`` (complex64 [nmaps, nalm], HEALPix order) and
    ``maps`` (float32 [nmaps, npix]), allocated here or passed in (``alm``,
    ``maps``, ``ws``: a caller's launch buffers).  ``__call__(alm)`` copies
    its argument into the static input (or pass ``None`` after writing
    ``self.alm`` in place), replays the ~30 launches of the transform (status
    reset, B packing, tensor-core contraction, transposes, one launch per
    ring-FFT size bucket, tail refinement) as one graph launch and returns
    ``self.maps`` (overwritten by the next replay).

    The epilogue (kinds, variances, shifts) is fixed at capture, or, with
    ``device_epilogue=True``, given per call: the kernels then read it from
    a small device buffer that each call refills from page-locked host memory
    on the replay's stream just before the replay (glg_alm2map_fast_devepi).
    """

    _SLOTS = 256  # page-locked epilogue images in flight (a slot is reused only after its copy ran)

    def __init__(self, nside: int, lmax: int, nmaps: int, *, epilogue=None,
                 device: torch.device | None = None, device_epilogue: bool = False,
                 alm: torch.Tensor | None = None, maps: torch.Tensor | None = None,
                 ws: torch.Tensor | None = None):
        if not 1 <= nmaps <= FAST_MAX_MAPS:
            raise ValueError(f"nmaps must be in [1, {FAST_MAX_MAPS}]")
        device = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        self.plan = get_plan(nside, lmax, device)
        self.nside, self.lmax, self.nmaps = nside, lmax, nmaps
        self.alm = alm[:nmaps] if alm is not None else \
            torch.zeros((nmaps, self.plan.nalm), dtype=torch.complex64, device=device)
        self.maps = maps[:nmaps] if maps is not None else \
            torch.empty((nmaps, self.plan.npix), dtype=torch.float32, device=device)
        if self.alm.dtype != torch.complex64 or tuple(self.alm.shape) != (nmaps, self.plan.nalm) or \
                not self.alm.is_contiguous():
            raise ValueError("alm must be a contiguous complex64 [nmaps, nalm] device tensor")
        if self.maps.dtype != torch.float32 or tuple(self.maps.shape) != (nmaps, self.plan.npix) or \
                not self.maps.is_contiguous():
            raise ValueError("maps must be a contiguous float32 [nmaps, npix] device tensor")
        ws_bytes = int(lib().glg_alm2map_workspace(self.plan.handle, nmaps, _lib.FORM_FAST))
        self.ws = ws if ws is not None and ws.numel() >= ws_bytes else \
            torch.empty(ws_bytes, dtype=torch.uint8, device=device)
        self.device_epilogue = bool(device_epilogue)
        self._epi = _make_epilogue(epilogue, nmaps) if epilogue is not None else None
        if self.device_epilogue:
            nb = int(lib().glg_epilogue_dev_bytes())
            self.epi_dev = torch.empty(nb, dtype=torch.uint8, device=device)
            self._slots = torch.empty((self._SLOTS, nb), dtype=torch.uint8, pin_memory=True)
            self._slot_ev = [None] * self._SLOTS
            self._slot = 0
        side = torch.cuda.Stream(device)
        side.wait_stream(torch.cuda.current_stream(device))
        with torch.cuda.stream(side):
            if not getattr(self.plan, "tuned", False):  # the plan's fast tables and FFT block sizes
                autotune(self.plan, nmaps, self.maps, self.ws)
                self._launch(host_epilogue=True)  # builds whatever the capture must not
            if self.device_epilogue:
                self.set_epilogue(epilogue)
            side.synchronize()
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph, stream=side):
                self._launch()
        torch.cuda.current_stream(device).wait_stream(side)

    def _launch(self, host_epilogue: bool = False) -> None:
        stream = c_p(stream_ptr(self.alm.device))
        if self.device_epilogue and not host_epilogue:
            check(lib().glg_alm2map_fast_devepi(self.plan.handle, c_p(ptr(self.alm)), self.nmaps,
                                                c_p(ptr(self.maps)), c_p(ptr(self.epi_dev)), c_p(ptr(self.ws)),
                                                self.ws.numel(), stream), "glg_alm2map_fast_devepi (graph)")
            return
        epi = ctypes.byref(self._epi) if self._epi is not None else None
        check(lib().glg_alm2map(self.plan.handle, c_p(ptr(self.alm)), self.nmaps, _lib.FORM_FAST,
                                c_p(ptr(self.maps)), epi, c_p(ptr(self.ws)), self.ws.numel(), stream),
              "glg_alm2map (graph)")

    def set_epilogue(self, epilogue) -> None:
        """Stage the epilogue of the next replay (device-epilogue graphs):
        its image goes into the next page-locked slot and is copied to the
        device buffer on the current stream."""
        if not self.device_epilogue:
            raise ValueError("this graph's epilogue was fixed at capture")
        k = self._slot % self._SLOTS
        self._slot += 1
        if self._slot_ev[k] is not None:
            self._slot_ev[k].synchronize()  # that slot's previous copy has been read
        epi = _make_epilogue(epilogue, self.nmaps) if epilogue is not None else None
        check(lib().glg_epilogue_dev_fill(ctypes.byref(epi) if epi is not None else None, self.nmaps,
                                          c_p(self._slots[k].data_ptr())), "glg_epilogue_dev_fill")
        self.epi_dev.copy_(self._slots[k], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.alm.device))
        self._slot_ev[k] = ev

    def __call__(self, alm=None, epilogue=None) -> torch.Tensor:
        if alm is not None:
            self.alm.copy_(torch.as_tensor(alm).reshape(self.alm.shape))
        if self.device_epilogue:
            self.set_epilogue(epilogue)
        elif epilogue is not None:
            raise ValueError("this graph's epilogue was fixed at capture (device_epilogue=False)")
        self.graph.replay()
        return self.maps

    def status(self) -> None:
        """Raise if a bounded device wait of the last replay timed out."""
        check(lib().glg_workspace_status(c_p(ptr(self.ws)), c_p(stream_ptr(self.alm.device))), "SynthGraph")


def _make_epilogue(epilogue, nmaps):
    if epilogue is None:
        return None
    kind, var, lam = epilogue
    kinds = list(kind) if isinstance(kind, (list, tuple)) else [int(kind)] * nmaps
    kinds_a = (ctypes.c_int * nmaps)(*kinds)
    var_a = (ctypes.c_double * nmaps)(*var)
    lam_a = (ctypes.c_double * nmaps)(*lam)
    epi = _lib.Epilogue(_lib.EPI_NONE, kinds_a, var_a, lam_a)
    epi._keep = (kinds_a, var_a, lam_a)
    return epi


def alm2map(alms, nside: int, *, inplace: bool = False, lmax: int | None = None,
            pixwin: bool = False, pol: bool = True):
    """HEALPix map(s) from alm (glass/healpix.py:38-78).

    ``alms`` is one complex array, or a sequence of them; with ``pol=True``
    and three arrays they are (T, E, B) and (T, Q, U) maps are returned.
    ``pixwin=True`` multiplies the alm by the pixel window (temperature
    window for spin 0, polarisation window for E and B), as healpy does.
    """
    seq = isinstance(alms, (list, tuple))
    items = list(alms) if seq else [alms]
    numpy_out = all(_lib.is_numpy_like(a) for a in items)
    dev = [_as_device_alm(a) for a in items]
    if any(d.ndim != 1 for d in dev) and not (not seq and dev[0].ndim == 2):
        raise ValueError("alm must be one-dimensional")
    if not seq and dev[0].ndim == 2:
        dev = list(dev[0])
        seq = True
    n = dev[0].shape[-1]
    lmax_in = _lmax_from_size(n)
    lmax = lmax_in if lmax is None else int(lmax)
    if pixwin:
        pw0, pw2 = pixwin_device(nside, lmax, dev[0].device)
        pw0 = pw0[: min(lmax, lmax_in) + 1]
        pw2 = pw2[: min(lmax, lmax_in) + 1]
        pols = seq and pol and len(dev) == 3
        dev = [almxfl(d, pw2 if (pols and i > 0) else pw0) for i, d in enumerate(dev)]
    if seq and pol and len(dev) == 3:
        t = synth(_resize_alm(dev[0], lmax_in, lmax)[None], nside, lmax)[0]
        q, u = _spin_synth(_resize_alm(dev[1], lmax_in, lmax), _resize_alm(dev[2], lmax_in, lmax),
                           nside, 2, lmax)
        out = [t, q, u]
        return [_finish(o, numpy_out) for o in out] if not numpy_out else np.stack([o.cpu().numpy() for o in out])
    stack = torch.stack([_resize_alm(d, lmax_in, lmax) for d in dev])
    maps = synth(stack, nside, lmax)
    if not seq:
        return _finish(maps[0], numpy_out)
    return maps.cpu().numpy() if numpy_out else list(maps)


def _spin_synth(elm: torch.Tensor, blm: torch.Tensor | None, nside: int, spin: int, lmax: int):
    plan = get_plan(nside, lmax, elm.device)
    q = torch.empty(plan.npix, dtype=torch.float64, device=elm.device)
    u = torch.empty_like(q)
    ws_bytes = int(lib().glg_alm2map_spin_workspace(plan.handle))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=elm.device)
    check(lib().glg_alm2map_spin(plan.handle, c_p(ptr(elm)), c_p(ptr(blm)) if blm is not None else None,
                                 spin, c_p(ptr(q)), c_p(ptr(u)), c_p(ptr(ws)), ws_bytes,
                                 c_p(stream_ptr(elm.device))), "glg_alm2map_spin")
    return q, u


def _spin_synth_fast(elm: torch.Tensor, blm: torch.Tensor | None, nside: int, spin: int, lmax: int):
    """Fast-form spin synthesis of nf fields: E (and B) alm [nf, nalm] (or
    [nalm]) -> float32 Q, U maps [nf, npix] (or [npix]).  The spin tables
    are built with the plan on first use (NotImplementedError when they do
    not fit the P_lm table budget)."""
    plan = get_plan(nside, lmax, elm.device)
    single = elm.ndim == 1
    e = elm.reshape(-1, plan.nalm).to(torch.complex64).contiguous()
    b = None if blm is None else blm.reshape(-1, plan.nalm).to(torch.complex64).contiguous()
    nf = e.shape[0]
    stream = c_p(stream_ptr(e.device))
    if not getattr(plan, "tuned", False):
        n = min(2 * nf, FAST_MAX_MAPS)
        tws = torch.empty(int(lib().glg_alm2map_workspace(plan.handle, n, _lib.FORM_FAST)), dtype=torch.uint8,
                          device=e.device)
        autotune(plan, n, torch.empty((n, plan.npix), dtype=torch.float32, device=e.device), tws)
        del tws
    step = min(nf, 20)
    ws_bytes = int(lib().glg_alm2map_spin_fast_workspace(plan.handle, step, int(b is not None)))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=e.device)
    q = torch.empty((nf, plan.npix), dtype=torch.float32, device=e.device)
    u = torch.empty_like(q)
    for f0 in range(0, nf, step):
        cnt = min(step, nf - f0)
        qu = torch.empty((2, cnt, plan.npix), dtype=torch.float32, device=e.device)
        check(lib().glg_alm2map_spin_fast(plan.handle, c_p(ptr(e[f0:f0 + cnt])),
                                          c_p(ptr(b[f0:f0 + cnt])) if b is not None else None, cnt, int(spin),
                                          c_p(ptr(qu)), c_p(ptr(ws)), ws_bytes, stream), "glg_alm2map_spin_fast")
        check(lib().glg_workspace_status(c_p(ptr(ws)), stream), "glg_alm2map_spin_fast")
        q[f0:f0 + cnt] = qu[0]
        u[f0:f0 + cnt] = qu[1]
    return (q[0], u[0]) if single else (q, u)


def alm2map_spin(alms: Sequence, nside: int, spin: int, lmax: int, *, form: str | None = None):
    """Spin-weighted maps [Q, U] from [E, B] alm (glass/healpix.py:81-108).

    ``form="plain"`` (the default unless ``GLASS_GB300_FORM`` says otherwise):
    FP64, float64 maps.  ``form="fast"``: split-precision TF32 contraction
    and FP32 ring FFTs, float32 maps."""
    if len(alms) != 2:
        raise ValueError("alm2map_spin needs exactly two alm arrays")
    form = _lib.default_form() if form is None else form
    if form not in ("plain", "fast"):
        raise ValueError(f"form must be 'plain' or 'fast', not {form!r}")
    numpy_out = all(_lib.is_numpy_like(a) for a in alms)
    e = _as_device_alm(alms[0])
    b = _as_device_alm(alms[1])
    lmax_in = _lmax_from_size(e.shape[-1])
    e = _resize_alm(e, lmax_in, lmax)
    b = _resize_alm(b, lmax_in, lmax)
    if not bool(torch.any(b != 0)):
        b = None
    if form == "fast":
        q, u = _spin_synth_fast(e, b, nside, int(spin), int(lmax))
    else:
        q, u = _spin_synth(e, b, nside, int(spin), int(lmax))
    return [_finish(q, numpy_out), _finish(u, numpy_out)]


def analysis(maps: torch.Tensor, lmax: int, niter: int = 3) -> torch.Tensor:
    """float64 maps [nmaps, npix] -> complex128 alm [nmaps, nalm]."""
    nside = npix2nside(maps.shape[-1])
    plan = get_plan(nside, lmax, maps.device)
    nmaps = maps.shape[0]
    alm = torch.empty((nmaps, plan.nalm), dtype=torch.complex128, device=maps.device)
    ws_bytes = int(lib().glg_map2alm_workspace(plan.handle, nmaps))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=maps.device)
    check(lib().glg_map2alm(plan.handle, c_p(ptr(maps)), nmaps, int(niter), c_p(ptr(alm)),
                            c_p(ptr(ws)), ws_bytes, c_p(stream_ptr(maps.device))), "glg_map2alm")
    return alm


_WARNED_WEIGHTS = False


def map2alm(maps, *, lmax: int | None = None, pol: bool = True,
            use_pixel_weights: bool = False, iter: int = 3):  # noqa: A002
    """alm of RING-ordered map(s) (glass/healpix.py:232-276).

    Uses uniform pixel weights and ``iter`` Jacobi refinements (healpy's
    default of 3).  HEALPix pixel-weight files are not available, so
    ``use_pixel_weights=True`` falls back to the same iterated quadrature.
    """
    global _WARNED_WEIGHTS
    if use_pixel_weights and not _WARNED_WEIGHTS:
        warnings.warn("pixel-weight files are not available: using uniform weights with "
                      f"{iter} refinement iterations", RuntimeWarning, stacklevel=2)
        _WARNED_WEIGHTS = True
    seq = isinstance(maps, (list, tuple))
    items = list(maps) if seq else [maps]
    numpy_out = all(_lib.is_numpy_like(m) for m in items)
    dev = torch.stack([_lib.to_device(m, torch.float64).reshape(-1) for m in items]) if seq else \
        _lib.to_device(maps, torch.float64)
    if dev.ndim == 1:
        dev = dev[None]
        single = True
    else:
        single = False
    nside = npix2nside(dev.shape[-1])
    lmax = 3 * nside - 1 if lmax is None else int(lmax)
    if seq and pol and len(items) == 3:
        raise NotImplementedError("polarised map2alm (TQU -> TEB) is not part of this path")
    alm = analysis(dev, lmax, iter)
    if single:
        return _finish(alm[0], numpy_out)
    return alm.cpu().numpy() if numpy_out else list(alm)


def almxfl(alm, fl, *, inplace: bool = False):
    """alm[l, m] * fl[l] in HEALPix order (glass/healpix.py:111-140)."""
    numpy_out = _lib.is_numpy_like(alm)
    a = _as_device_alm(alm)
    f = _lib.to_device(fl, torch.float64, a.device).reshape(-1)
    single = a.ndim == 1
    a2 = a.reshape(-1, a.shape[-1])
    lmax = _lmax_from_size(a2.shape[-1])
    out = a2 if (inplace and not numpy_out and isinstance(alm, torch.Tensor) and alm.dtype == torch.complex128) \
        else torch.empty_like(a2)
    check(lib().glg_almxfl(c_p(ptr(a2)), c_p(ptr(f)) if f.numel() else None, int(f.numel()), lmax,
                           a2.shape[0], _lib.GLG_F64, c_p(ptr(out)), c_p(stream_ptr(a.device))),
          "glg_almxfl")
    res = out[0] if single else out
    if numpy_out:
        r = res.cpu().numpy()
        if inplace and isinstance(alm, np.ndarray):
            alm[...] = r
            return alm
        return r
    return res


_PIXWIN: dict[tuple[int, int, int], tuple[torch.Tensor, torch.Tensor]] = {}


def pixwin_device(nside: int, lmax: int, device: torch.device | None = None):
    """(pw0, pw2) float64 [lmax+1] device tensors, computed once per
    (device, nside, lmax) by glg_pixwin and cached."""
    device = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    key = (device.index if device.index is not None else torch.cuda.current_device(), int(nside), int(lmax))
    hit = _PIXWIN.get(key)
    if hit is not None:
        return hit
    pw0 = torch.empty(lmax + 1, dtype=torch.float64, device=device)
    pw2 = torch.empty_like(pw0)
    ws_bytes = int(lib().glg_pixwin_workspace(int(nside)))
    if ws_bytes == 0:
        raise ValueError("pixwin: nside must be in [1, 8192]")
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=device)
    check(lib().glg_pixwin(int(nside), int(lmax), c_p(ptr(pw0)), c_p(ptr(pw2)), c_p(ptr(ws)), ws_bytes,
                           c_p(stream_ptr(device))), "glg_pixwin")
    _PIXWIN[key] = (pw0, pw2)
    return pw0, pw2


def pixwin(nside: int, *, lmax: int | None = None, pol: bool = False, xp=None):
    """Pixel window function(s) of HEALPix pixels at ``nside``
    (glass/healpix.py:313-356, healpy.pixwin): the temperature window, or
    (temperature, polarisation) with ``pol=True``; ``lmax`` defaults to
    3 nside - 1.

    healpy reads these from data files that are not available offline; they
    are computed on the GPU from their definition instead (the pixel-averaged
    harmonics' power, spin 0 and spin 2), see ``glg_pixwin`` in
    include/glass_gb300.h.  ``xp``: the array namespace of the result
    (numpy by default; ``torch`` gives CUDA tensors).
    """
    lmax = 3 * int(nside) - 1 if lmax is None else int(lmax)
    pw0, pw2 = pixwin_device(nside, lmax)
    if xp is not None and xp is torch:
        return (pw0.clone(), pw2.clone()) if pol else pw0.clone()
    a0 = pw0.cpu().numpy()
    if not pol:
        return a0 if xp is None else xp.asarray(a0, dtype=xp.float64)
    a2 = pw2.cpu().numpy()
    return (a0, a2) if xp is None else (xp.asarray(a0, dtype=xp.float64), xp.asarray(a2, dtype=xp.float64))

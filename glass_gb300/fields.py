"""Random fields on the GPU: drop-in for the field-generation path of GLASS.

Mirrors ``glass/fields.py``: ``iternorm`` (:101-188), ``cls2cov``
(:191-236), ``_generate_grf`` (:334-429), ``generate_gaussian`` (:432-482),
``generate_lognormal`` (:485-522), ``getcl`` (:525-560), ``generate``
(:839-894) and the alm reordering of :943-962, with the same signatures,
generator semantics and error messages.

All numerical work runs in the CUDA library (``include/glass_gb300.h``):
iternorm, the variate draws (Philox stream) or their upload (numpy stream),
the correlated alm sum with its reordering, the spherical-harmonic transform
and the fused lognormal transform.  Inputs given as numpy arrays produce
numpy maps; torch inputs produce CUDA tensors.

Extra keyword ``form``: ``"plain"`` (default; FP64 throughout, the drop-in)
or ``"fast"`` (float32 maps, split-precision Legendre contraction).  The
environment variable ``GLASS_GB300_FORM`` sets the default.
"""

from __future__ import annotations

import collections
import ctypes
import math
import os
import sys
import warnings
from collections.abc import Iterable, Iterator, Sequence

import numpy as np
import torch

from . import _lib, grf
from . import healpix as hp
from . import rng as grng
from ._lib import c_p, check, lib, ptr, stream_ptr

__all__ = [
    "accuracy_report",
    "cls2cov",
    "enumerate_spectra",
    "generate",
    "generate_gaussian",
    "generate_lognormal",
    "getcl",
    "iternorm",
    "nfields_from_nspectra",
    "spectra_indices",
]


def _deprecated(msg: str):
    def deco(func):
        import functools  # noqa: PLC0415

        @functools.wraps(func)
        def wrapper(*args, **kwargs):
            warnings.warn(msg, category=DeprecationWarning, stacklevel=2)
            return func(*args, **kwargs)

        return wrapper

    return deco


def _inv_triangle_number(triangle_number: int) -> int:
    n = math.floor(math.sqrt(2 * triangle_number))
    if n * (n + 1) // 2 != triangle_number:
        raise ValueError(f"not a triangle number: {triangle_number}")
    return n


def nfields_from_nspectra(nspectra: int) -> int:
    """Number of fields n with n (n+1) / 2 == nspectra (glass/fields.py:83-98)."""
    try:
        return _inv_triangle_number(nspectra)
    except ValueError:
        raise ValueError(f"invalid number of spectra: {nspectra}") from None


def enumerate_spectra(entries):
    """Yield (i, j, cl) in GLASS standard order."""
    for k, cl in enumerate(entries):
        i = int((2 * k + 0.25) ** 0.5 - 0.5)
        j = i * (i + 3) // 2 - k
        yield i, j, cl


def spectra_indices(n: int, *, xp=None):
    i, j = np.tril_indices(n)
    return np.stack([i, i - j]).T


def _to_np(x) -> np.ndarray:
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def getcl(cls, i: int, j: int, lmax: int | None = None):
    """Spectrum (i, j) from GLASS-ordered spectra (glass/fields.py:525-560)."""
    if j > i:
        i, j = j, i
    cl = cls[i * (i + 1) // 2 + i - j]
    if lmax is not None:
        if cl.shape[0] > lmax + 1:
            cl = cl[: lmax + 1]
        elif isinstance(cl, torch.Tensor):
            cl = torch.nn.functional.pad(cl, (0, lmax + 1 - cl.shape[0]))
        else:
            cl = np.pad(cl, (0, lmax + 1 - cl.shape[0]))
    return cl


def cls2cov(cls, nl: int, nf: int, nc: int):
    """Covariance rows for iterative sampling (glass/fields.py:191-236).

    Like the reference, every yielded matrix is the same buffer, updated in
    place for the next field.
    """
    use_torch = any(isinstance(c, torch.Tensor) for c in cls if c is not None)
    if use_torch:
        dev = next(c.device for c in cls if isinstance(c, torch.Tensor))
        cov = torch.zeros((nl, nc + 1), dtype=torch.float64, device=dev)
    else:
        cov = np.zeros((nl, nc + 1))
    end = 0
    for j in range(nf):
        begin, end = end, end + j + 1
        for i, cl in enumerate(cls[begin:end][: nc + 1]):
            if i == 0 and bool((cl < 0).any()):
                raise ValueError("negative values in cl")
            n = cl.shape[0]
            if use_torch:
                cov[:n, i] = torch.as_tensor(cl, dtype=torch.float64, device=cov.device)
            else:
                cov[:n, i] = cl
            cov[n:, i] = 0.0
        cov /= 2
        yield cov


# ---------------------------------------------------------------- iternorm


def _iternorm_device(rows: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    """rows float64 [nrows][nl][k+1] on the device -> (w, status uint64)."""
    nrows, nl, kp = rows.shape
    w = torch.empty_like(rows)
    status = torch.empty(1, dtype=torch.int64, device=rows.device)
    check(lib().glg_iternorm(c_p(ptr(rows)), nrows, nl, kp - 1, c_p(ptr(w)), c_p(ptr(status)),
                             c_p(stream_ptr(rows.device))), "glg_iternorm")
    return w, status


def _first_bad(status: torch.Tensor) -> int:
    v = int(status.item())
    return -1 if v == -1 else v  # UINT64_MAX reads as -1 in int64


def iternorm(cov: Iterable) -> Iterator:
    """Scaling vectors for iterative normal sampling (glass/fields.py:101-188).

    The rows are collected, computed together on the device (one warp per
    mode), and yielded one by one; errors are raised at the row where the
    reference raises them.  Rows whose number of correlations k varies are
    zero-padded to the largest k, which leaves the retained entries unchanged.
    """
    raw = []
    err = None
    shape = None
    numpy_out = True
    for i, row in enumerate(cov):
        if isinstance(row, torch.Tensor):
            numpy_out = False
            r = row.detach().clone()
        else:
            r = np.array(row, dtype=np.float64, copy=True)
        k = r.shape[-1] - 1
        if k < 0:
            err = ValueError("empty covariance matrix")
            break
        if i == 0:
            shape = tuple(r.shape[:-1])
        elif tuple(r.shape[:-1]) != shape:
            err = ValueError("shape mismatch in covariance")
            break
        raw.append(r)
    rows = [_lib.to_device(r, torch.float64).reshape(-1, r.shape[-1]) for r in raw]
    if rows:
        kmax = max(r.shape[-1] for r in rows) - 1
        nl = rows[0].shape[0]
        stack = torch.zeros((len(rows), nl, kmax + 1), dtype=torch.float64, device=rows[0].device)
        for i, r in enumerate(rows):
            stack[i, :, : r.shape[-1]] = r
        w, status = _iternorm_device(stack)
        bad = _first_bad(status)
        for i, r in enumerate(rows):
            if bad == i:
                raise ValueError("covariance matrix is not positive definite")
            k = r.shape[-1] - 1
            wi = w[i, :, kmax - k:].reshape(shape + (k + 1,))
            yield wi.cpu().numpy() if numpy_out else wi
    if err is not None:
        raise err


# ------------------------------------------------------------ generation


def _glass_to_healpix_alm(alm):
    """Reorder alm from GLASS (l-major) to HEALPix (m-major) order (glass/fields.py:943-962)."""
    numpy_out = _lib.is_numpy_like(alm)
    a = np.asarray(alm) if numpy_out else alm
    n = _inv_triangle_number(a.shape[-1])
    ell = np.arange(n)
    idx = np.concatenate([ell[m:] * (ell[m:] + 1) // 2 + m for m in range(n)])
    if numpy_out:
        return a[..., idx]
    return a[..., torch.as_tensor(idx, device=a.device)]


def _default_form() -> str:
    return _lib.default_form()


class _FieldBatcher:
    """Shared machinery of _generate_grf / generate: w, variates, alm, maps."""

    def __init__(self, gls, nside: int, ncorr, rng, form: str, device=None):
        self.numpy_out = all(_lib.is_numpy_like(g) for g in gls)
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        self.ngrf = nfields_from_nspectra(len(gls))
        self.ncorr = self.ngrf - 1 if ncorr is None else int(ncorr)
        lens = [0 if g is None else int(g.shape[0]) for g in gls]
        n = max(lens, default=0)
        if n == 0:
            raise ValueError("all gls are empty")
        self.n = n
        self.lmax = n - 1
        self.nside = int(nside)
        self.form = form
        if form not in ("plain", "fast"):
            raise ValueError(f"form must be 'plain' or 'fast', not {form!r}")
        self.cdtype = torch.complex128 if form == "plain" else torch.complex64
        self.code = _lib.GLG_F64 if form == "plain" else _lib.GLG_F32
        self.z_size = n * (n + 1) // 2
        k = self.ncorr
        self.k = k
        # cls2cov + variances of every field in one launch from the
        # concatenated spectra, then iternorm of every field in one launch
        offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
        if self.numpy_out:
            # concatenated straight into pinned memory: one asynchronous copy
            # (the caching host allocator keeps the buffer until it is done)
            parts = [g if (isinstance(g, np.ndarray) and g.dtype == np.float64 and g.ndim == 1
                           and g.flags.c_contiguous) else np.ascontiguousarray(g, dtype=np.float64).reshape(-1)
                     for g in gls if g is not None]
            flat_h = torch.empty(int(offs[-1]), dtype=torch.float64, pin_memory=True)
            # one host copy split over threads (glg_gather_host), then one upload
            src = (ctypes.c_void_p * len(parts))(*[q.ctypes.data for q in parts])
            nb = (ctypes.c_int64 * len(parts))(*[q.nbytes for q in parts])
            check(lib().glg_gather_host(src, nb, len(parts), c_p(flat_h.data_ptr()), 8), "glg_gather_host")
            flat = flat_h.to(self.device, non_blocking=True)
        else:
            dev, f64 = self.device, torch.float64
            flat = torch.cat([g if (isinstance(g, torch.Tensor) and g.dtype == f64 and g.device == dev
                                    and g.dim() == 1) else _lib.to_device(g, f64, dev).reshape(-1)
                              for g in gls if g is not None])
        offs_d = torch.from_numpy(offs).to(self.device)
        cov = torch.empty((self.ngrf, n, k + 1), dtype=torch.float64, device=self.device)
        self.var_dev = torch.empty(self.ngrf, dtype=torch.float64, device=self.device)
        status = torch.empty(2, dtype=torch.int64, device=self.device)
        check(lib().glg_cls2cov(c_p(ptr(flat)), c_p(ptr(offs_d)), self.ngrf, n, k, c_p(ptr(cov)),
                                c_p(ptr(self.var_dev)), c_p(ptr(status)), c_p(stream_ptr(self.device))),
              "glg_cls2cov")
        self.w, st_it = _iternorm_device(cov)
        status[1:2].copy_(st_it)
        host = torch.cat([status.double(), self.var_dev]).cpu().numpy()  # one sync
        neg, nonpd = int(host[0]), int(host[1])
        self.variances = [float(v) for v in host[2:]]
        # the reference raises at the first failing field, after the earlier maps
        self.bad_msg = None
        self.bad = -1
        if neg >= 0:
            self.bad, self.bad_msg = neg, "negative values in cl"
        if nonpd >= 0 and (self.bad < 0 or nonpd < self.bad):
            self.bad, self.bad_msg = nonpd, "covariance matrix is not positive definite"
        # variate source
        if rng is None:
            rng = grng.default_rng()
        self.np_rng = rng if isinstance(rng, np.random.Generator) else None
        if self.np_rng is None and not isinstance(rng, grng.Generator):
            raise TypeError("rng must be a numpy Generator or a glass_gb300.rng.Generator")
        self.g_rng = rng if self.np_rng is None else None
        self.sid0 = self.g_rng.reserve_streams(self.ngrf) if self.g_rng is not None else 0
        self.zwin: collections.deque[torch.Tensor] = collections.deque()

    def _host_variates(self, t: int) -> torch.Tensor:
        z = self.np_rng.standard_normal((self.z_size, 2)) @ np.asarray([1, 1j])
        return torch.as_tensor(z, dtype=self.cdtype).to(self.device)

    def alm(self, t0: int, nshell: int) -> torch.Tensor:
        """Correlated alm of shells t0..t0+nshell-1 (HEALPix order) [nshell][nalm]."""
        alm = torch.empty((nshell, self.z_size), dtype=self.cdtype, device=self.device)
        w = self.w[t0:t0 + nshell].to(torch.float64 if self.form == "plain" else torch.float32).contiguous()
        zlo = max(0, t0 - self.k)
        if self.np_rng is not None:
            for t in range(t0, t0 + nshell):
                self.zwin.append(self._host_variates(t))
            while len(self.zwin) > t0 + nshell - zlo:
                self.zwin.popleft()
            z = torch.stack(list(self.zwin))
            check(lib().glg_alm_correlate(c_p(ptr(w)), nshell, self.lmax, self.k, t0, c_p(ptr(z)),
                                          zlo, 0, 0, self.code, c_p(ptr(alm)),
                                          c_p(stream_ptr(self.device))), "glg_alm_correlate")
        else:
            # shell t draws Philox stream sid0 + t (streams reserved per generate call)
            check(lib().glg_alm_correlate(c_p(ptr(w)), nshell, self.lmax, self.k, t0, None, zlo,
                                          ctypes.c_uint64(self.g_rng.seed), ctypes.c_uint64(self.sid0),
                                          self.code, c_p(ptr(alm)), c_p(stream_ptr(self.device))),
                  "glg_alm_correlate")
        return alm

    def maps(self, t0: int, nshell: int, epi=None, out=None) -> torch.Tensor:
        alm = self.alm(t0, nshell)
        return hp.synth(alm, self.nside, self.lmax, epilogue=epi, form=self.form, out=out)


def _group_size(ngrf: int, nside: int, lmax: int, form: str, host_rng: bool = False) -> int:
    """Shells per batched transform, bounded by a workspace budget
    (``GLASS_GB300_BATCH_BYTES``, 48 GB by default).  Larger groups measured
    slower at nside 4096 (17 shells a group: 4.9 s for 60 shells against
    2.6 s with 11).

    With a numpy generator the variates are drawn shell by shell, exactly when
    the reference draws them, so the caller may share that generator.
    """
    if host_rng:
        return 1
    budget = int(os.environ.get("GLASS_GB300_BATCH_BYTES", str(48 << 30)))
    per = 16 * (4 * nside - 1) * (lmax + 1) + 8 * 12 * nside * nside + 16 * (lmax + 1) * (lmax + 2) // 2
    return max(1, min(ngrf, budget // max(per, 1)))


def _generate_grf(gls, nside: int, *, ncorr=None, rng=None, form: str | None = None):
    """Gaussian random field maps, one per shell (glass/fields.py:334-429)."""
    form = _default_form() if form is None else form
    b = _FieldBatcher(gls, nside, ncorr, rng, form)
    g = _group_size(b.ngrf, nside, b.lmax, form, b.np_rng is not None)
    for t0 in range(0, b.ngrf, g):
        cnt = min(g, b.ngrf - t0)
        if b.bad >= 0 and b.bad < t0 + cnt:
            cnt = b.bad - t0
        maps = b.maps(t0, cnt) if cnt > 0 else None
        if b.numpy_out and cnt > 0:
            maps = _to_host(maps)
        for s in range(cnt):
            yield maps[s]
        maps = None
        if b.bad >= 0 and b.bad < t0 + g:
            raise ValueError(b.bad_msg)


# Page-locked output buffers of the host-output synthesis, kept for reuse.
# Each is held as (tensor, numpy view of the whole buffer); the maps handed
# to a caller are rows of that numpy view, so its reference count says
# whether any map of an earlier call is still alive.  Pinning 8 GB anew
# costs 0.3-0.6 s, more than a whole 40-shell step.
_PINNED: list[tuple[torch.Tensor, np.ndarray]] = []
_PINNED_KEEP = 2  # buffers of one shape kept when every one is in use


def _pinned_maps(nmaps: int, npix: int) -> tuple[torch.Tensor, np.ndarray]:
    """Pinned float32 [nmaps, npix] host buffer for the fast form's
    host-output synthesis, and its numpy view (hand out its rows), reused
    once the caller has dropped every map of an earlier call into it."""
    for i in range(len(_PINNED)):
        # references to the view: the pool entry and getrefcount's argument;
        # any more are maps of an earlier call still alive
        if _PINNED[i][1].shape == (nmaps, npix) and sys.getrefcount(_PINNED[i][1]) <= 2:
            return _PINNED[i]
    t = torch.empty((nmaps, npix), dtype=torch.float32, pin_memory=True)
    entry = (t, t.numpy())
    same = [i for i in range(len(_PINNED)) if _PINNED[i][1].shape == (nmaps, npix)]
    if len(same) >= _PINNED_KEEP:
        del _PINNED[same[0]]  # the oldest goes back to torch once its maps are dropped
    _PINNED.append(entry)
    return entry


def _to_host(maps: torch.Tensor) -> list[np.ndarray]:
    """Device maps -> numpy arrays backed by page-locked host memory.

    One asynchronous copy per map into pinned buffers (recycled by torch's
    caching host allocator) and a single synchronisation.
    """
    out = [torch.empty(m.shape, dtype=m.dtype, pin_memory=True) for m in maps]
    for h, m in zip(out, maps):
        h.copy_(m, non_blocking=True)
    torch.cuda.current_stream(maps.device).synchronize()
    return [h.numpy() for h in out]


def _cltovar(cl) -> float:
    c = _to_np(cl).astype(np.float64)
    ell = np.arange(c.shape[0])
    return float(np.sum((2 * ell + 1) / (4 * np.pi) * c))


def generate(fields: Sequence, gls, nside: int, *, ncorr: int | None = None, rng=None,
             form: str | None = None) -> Iterator:
    """Sample transformed Gaussian random fields (glass/fields.py:839-894).

    Known transformations (Normal, Lognormal) are fused into the transform
    kernel; other callables are applied to each finished map.
    """
    n = len(fields)
    if len(gls) != n * (n + 1) // 2:
        raise ValueError("mismatch between number of fields and gls")
    return _generate(list(fields), gls, nside, ncorr, rng,
                     _default_form() if form is None else form)


def _generate(fields, gls, nside, ncorr, rng, form):
    b = _FieldBatcher(gls, nside, ncorr, rng, form)
    variances = b.variances
    kinds = [grf.fused_kind(t) for t in fields]
    g = _group_size(b.ngrf, nside, b.lmax, form, b.np_rng is not None)
    for t0 in range(0, b.ngrf, g):
        cnt = min(g, b.ngrf - t0)
        if b.bad >= 0 and b.bad < t0 + cnt:
            cnt = b.bad - t0
        if cnt > 0:
            fused = [kinds[t] is not None and kinds[t][0] == "lognormal" for t in range(t0, t0 + cnt)]
            epi_kind = [_lib.EPI_LOGNORMAL if f else _lib.EPI_NONE for f in fused]
            epi = (epi_kind, [variances[t] for t in range(t0, t0 + cnt)],
                   [kinds[t][1] if fused[s] else 1.0 for s, t in enumerate(range(t0, t0 + cnt))])
            pinned = _pinned_maps(cnt, 12 * b.nside * b.nside) if b.numpy_out and form == "fast" else None
            if pinned is not None:
                # each run of ring tiles is copied to the pinned buffer while
                # the next run computes: little copying is left after the last
                b.maps(t0, cnt, epi=epi, out=pinned[0])
                torch.cuda.current_stream(b.device).synchronize()
                maps = list(pinned[1])
                del pinned
            else:
                maps = b.maps(t0, cnt, epi=epi)
                if b.numpy_out:
                    maps = _to_host(maps)
        for s in range(cnt):
            t = t0 + s
            x = maps[s]
            if kinds[t] is None:
                x = fields[t](x, variances[t])
            yield x
        # the next group's maps are made with this group's released (unless the caller keeps them)
        maps = x = None
        if b.bad >= 0 and b.bad < t0 + g:
            raise ValueError(b.bad_msg)


def accuracy_report(fields: Sequence, gls, nside: int, *, ncorr: int | None = None, seed: int = 42,
                    ref_form: str = "plain") -> list[dict]:
    """Per-output error of the fast form against the FP64 form.

    Generates the same shells twice from the same Philox stream (key
    ``seed``): with ``form="fast"`` and with ``ref_form`` (the FP64 plain
    form, which matches the oracle to 1e-12), and returns one record per
    shell: relative RMS error (RMS of the difference over the RMS of the
    FP64 map), relative maximum error (largest difference over the largest
    FP64 value) and the largest absolute difference.  Costs one FP64 run.
    """
    dev = torch.device("cuda", torch.cuda.current_device())
    gls_d = [None if c is None else _lib.to_device(c, torch.float64, dev).reshape(-1) for c in gls]
    out = []
    fast = generate(fields, gls_d, nside, ncorr=ncorr, rng=grng.Generator(seed), form="fast")
    ref = generate(fields, gls_d, nside, ncorr=ncorr, rng=grng.Generator(seed), form=ref_form)
    for t, (a, b) in enumerate(zip(fast, ref)):
        d = a.double() - b
        out.append({"shell": t,
                    "rms_rel": float(torch.sqrt(torch.mean(d * d)) / torch.sqrt(torch.mean(b * b))),
                    "max_rel": float(d.abs().max() / b.abs().max()),
                    "max_abs": float(d.abs().max())})
    return out


@_deprecated("use glass.generate() instead")
def generate_gaussian(gls, nside: int, *, ncorr: int | None = None, rng=None,
                      form: str | None = None):
    """Gaussian random fields (glass/fields.py:432-482; deprecated upstream)."""
    n = nfields_from_nspectra(len(gls))
    fields = [grf.Normal() for _ in range(n)]
    yield from generate(fields, gls, nside, ncorr=ncorr, rng=rng, form=form)


@_deprecated("use glass.generate() instead")
def generate_lognormal(gls, nside: int, shift: float = 1.0, *, ncorr: int | None = None, rng=None,
                       form: str | None = None):
    """Lognormal random fields (glass/fields.py:485-522; deprecated upstream)."""
    n = nfields_from_nspectra(len(gls))
    fields = [grf.Lognormal(shift) for _ in range(n)]
    yield from generate(fields, gls, nside, ncorr=ncorr, rng=rng, form=form)

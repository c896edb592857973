"""Continuous-batching request loop for field simulations on one GPU.

A request is one call's worth of ``generate``: Gaussian spectra of
``nshell`` correlated shells at one (nside, lmax), lognormal shifts and a
seed.  The server admits requests while their device-memory estimate fits
an HBM budget, keeps their alm, maps and the per-(nside, lmax) plans
resident on the device, and forms every launch of the fast spherical-harmonic
transform from the shells that are ready at that moment, across requests of
the same (nside, lmax).  Different (nside, lmax) groups run on their own CUDA
streams, so their kernels overlap on the device.  Requests that arrive while
others are running are admitted as memory frees up.

Each result equals the result of the same request served alone: every map
is computed from its own alm column, its own Philox stream and its own
epilogue, independent of what it is batched with.
"""

from __future__ import annotations

import collections
import dataclasses
import threading
import time

import numpy as np
import torch

from . import _lib, grf
from . import healpix as hp
from .fields import _FieldBatcher
from .rng import Generator

__all__ = ["Request", "Server"]


@dataclasses.dataclass
class Request:
    """One simulation request (spectra in GLASS order, one shift per shell)."""

    gls: list
    nside: int
    shifts: list[float]
    seed: int = 42
    ncorr: int | None = None
    arrival: float = 0.0
    id: int = -1
    # filled by the server
    maps: list = dataclasses.field(default_factory=list)
    admitted: float | None = None
    finished: float | None = None
    reserved: int = 0

    @classmethod
    def from_cls_file(cls, filename, nside: int, shifts, seed: int = 42, **kw) -> "Request":
        """A request whose spectra come from a GLASS ``.npz`` spectra file."""
        from .user import load_cls

        return cls(gls=load_cls(filename), nside=nside, shifts=[float(x) for x in shifts], seed=seed, **kw)

    @property
    def nshell(self) -> int:
        return len(self.shifts)

    @property
    def lmax(self) -> int:
        return max(np.asarray(g).shape[0] for g in self.gls) - 1

    @property
    def latency(self) -> float | None:
        return None if self.finished is None else self.finished - self.arrival


def request_bytes(nside: int, lmax: int, nshell: int, form: str = "fast") -> int:
    """Device bytes a request holds: alm, maps and w/cov (twice as many alm
    and map bytes in the FP64 form)."""
    nalm = (lmax + 1) * (lmax + 2) // 2
    npix = 12 * nside * nside
    f = 2 if form == "plain" else 1
    return nshell * f * (8 * nalm + 4 * npix) + 2 * 8 * nshell * (lmax + 1) * nshell


def launch_bytes(nside: int, lmax: int, nmaps: int) -> int:
    """Workspace of one fast transform launch (B pack + Legendre sums)."""
    nalm = (lmax + 1) * (lmax + 2) // 2
    ngroups = nalm // 16 + lmax + 1
    n = ((2 * nmaps + 15) // 16) * 16
    return ngroups * 128 * n + 8 * nmaps * (4 * nside - 1) * (lmax + 1) + nmaps * (lmax + 1) * 8


class _Active:
    """Per-request state while it is being served."""

    def __init__(self, req: Request, device: torch.device, form: str = "fast"):
        self.req = req
        fields = [grf.Lognormal(float(s)) for s in req.shifts]
        self.kinds = [_lib.EPI_LOGNORMAL] * req.nshell
        self.lam = [f.lamda for f in fields]
        self.batcher = _FieldBatcher(req.gls, req.nside, req.ncorr, Generator(req.seed), form,
                                     device=device)
        if self.batcher.bad >= 0:
            raise ValueError(f"request {req.id}: {self.batcher.bad_msg}")
        self.var = self.batcher.variances
        self.alm = self.batcher.alm(0, req.nshell)  # [nshell][nalm] complex64, device
        self.next_shell = 0
        self.maps: list[torch.Tensor | None] = [None] * req.nshell
        self.done_event: torch.cuda.Event | None = None


class Server:
    """Continuous batching of simulation requests within an HBM budget.

    ``form="fast"`` with ``batching=True`` is the serving configuration;
    ``form="plain", batching=False`` (one map per transform launch, no
    sharing across requests) is the comparison point of the FP64 form.
    """

    def __init__(self, hbm_budget: int = 120 << 30, max_maps_per_launch: int = 40,
                 device: torch.device | None = None, form: str = "fast", batching: bool = True):
        if form not in ("fast", "plain"):
            raise ValueError(f"form must be 'plain' or 'fast', not {form!r}")
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        self.budget = int(hbm_budget)
        self.form = form
        self.batching = bool(batching)
        self.max_maps = int(max_maps_per_launch) if batching else 1
        self.used = 0
        self.queue: collections.deque[Request] = collections.deque()
        self.active: list[_Active] = []
        self.finished: list[Request] = []
        self.streams: dict[tuple[int, int], torch.cuda.Stream] = {}
        self.lock = threading.Lock()
        self._next_id = 0

    # ------------------------------------------------------------- intake

    def submit(self, req: Request) -> Request:
        with self.lock:
            req.id = self._next_id
            self._next_id += 1
            if req.arrival == 0.0:
                req.arrival = time.perf_counter()
            need = request_bytes(req.nside, req.lmax, req.nshell, self.form)
            if need > self.budget:
                raise MemoryError(f"request {req.id} needs {need} bytes, over the HBM budget {self.budget}")
            self.queue.append(req)
        return req

    def _admit(self) -> None:
        while self.queue:
            req = self.queue[0]
            need = request_bytes(req.nside, req.lmax, req.nshell, self.form)
            if self.used + need > self.budget:
                break
            self.queue.popleft()
            self.used += need
            req.reserved = need
            req.admitted = time.perf_counter()
            stream = self._stream(req.nside, req.lmax)
            with torch.cuda.stream(stream):
                self.active.append(_Active(req, self.device, self.form))

    def _stream(self, nside: int, lmax: int) -> torch.cuda.Stream:
        key = (nside, lmax)
        if key not in self.streams:
            self.streams[key] = torch.cuda.Stream(self.device)
        return self.streams[key]

    # ------------------------------------------------------------ batching

    def _launch_batches(self) -> bool:
        """One launch per (nside, lmax) group from the shells ready now."""
        groups: dict[tuple, list[tuple[_Active, int]]] = collections.defaultdict(list)
        for a in self.active:
            key = (a.req.nside, a.req.lmax) if self.batching else (a.req.nside, a.req.lmax, a.req.id)
            for s in range(a.next_shell, a.req.nshell):
                groups[key].append((a, s))
        launched = False
        for key, items in groups.items():
            nside, lmax = key[0], key[1]
            stream = self._stream(nside, lmax)
            for c0 in range(0, len(items), self.max_maps):
                chunk = items[c0:c0 + self.max_maps]
                with torch.cuda.stream(stream):
                    alm = torch.stack([a.alm[s] for a, s in chunk])
                    epi = ([a.kinds[s] for a, s in chunk], [a.var[s] for a, s in chunk],
                           [a.lam[s] for a, s in chunk])
                    maps = hp.synth(alm, nside, lmax, epilogue=epi, form=self.form)
                for k, (a, s) in enumerate(chunk):
                    a.maps[s] = maps[k]
                    a.next_shell = max(a.next_shell, s + 1)
                launched = True
            for a in {id(x[0]): x[0] for x in items}.values():
                if a.next_shell == a.req.nshell and a.done_event is None:
                    ev = torch.cuda.Event()
                    ev.record(stream)
                    a.done_event = ev
        return launched

    def _retire(self) -> None:
        keep = []
        for a in self.active:
            if a.done_event is not None and a.done_event.query():
                a.req.maps = a.maps
                a.req.finished = time.perf_counter()
                self.used -= a.req.reserved
                self.finished.append(a.req)
            else:
                keep.append(a)
        self.active = keep

    def step(self) -> None:
        """Admit, launch what is ready, retire what finished."""
        with self.lock:
            self._admit()
        self._launch_batches()
        self._retire()

    def drain(self, timeout: float = 600.0) -> list[Request]:
        """Serve until the queue and the active set are empty."""
        t0 = time.perf_counter()
        while True:
            with self.lock:
                idle = not self.queue and not self.active
            if idle:
                return self.finished
            self.step()
            if time.perf_counter() - t0 > timeout:
                raise TimeoutError("server did not drain in time")
            if self.active and not self.queue:
                time.sleep(0.0005)


def latency_summary(reqs: list[Request]) -> dict:
    lat = np.array([r.latency for r in reqs if r.latency is not None])
    shells = sum(r.nshell for r in reqs)
    span = max(r.finished for r in reqs) - min(r.arrival for r in reqs)
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "requests": len(reqs), "shell_maps": shells,
            "shell_maps_per_s": shells / span}

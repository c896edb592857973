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
import os
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


def _ngroups(lmax: int) -> int:
    """16-l groups of the fast contraction's B operand: sum_m ceil((lmax-m+1)/16)."""
    return sum((lmax - m + 16) // 16 for m in range(lmax + 1))


def request_bytes(nside: int, lmax: int, nshell: int, form: str = "fast") -> int:
    """Device bytes a request holds while it is served: its spectra, cls2cov
    rows, iternorm rows (and their float32 copy), alm and maps (alm complex128
    and maps float64 in the FP64 form)."""
    n = lmax + 1
    nalm = n * (n + 1) // 2
    npix = 12 * nside * nside
    f = 2 if form == "plain" else 1
    nspec = nshell * (nshell + 1) // 2
    return (8 * nspec * n + 2 * 8 * nshell * n * nshell + 4 * nshell * n * nshell
            + nshell * f * (8 * nalm + 4 * npix))


def launch_bytes(nside: int, lmax: int, nmaps: int, form: str = "fast") -> int:
    """Device bytes of one (nside, lmax) group's launch buffers for up to
    ``nmaps`` maps: the transform workspace (fast: status block, B pack and two
    copies of the Legendre sums; plain: the FP64 sums), the staged alm and the
    staged maps."""
    n = lmax + 1
    nalm = n * (n + 1) // 2
    nrings = 4 * nside - 1
    npix = 12 * nside * nside
    if form == "fast":
        nn = ((2 * nmaps + 15) // 16) * 16
        up = lambda b: (b + 255) // 256 * 256  # noqa: E731 - 256-byte aligned blocks
        ws = (256 + up(_ngroups(lmax) * 128 * nn) + 2 * up(8 * nmaps * nrings * n) + 256
              + up(16 * 65536 * nmaps))  # + tail-refinement list
        return ws + nmaps * (8 * nalm + 4 * npix)
    return 16 * nmaps * nrings * n + nmaps * (16 * nalm + 8 * npix)


PLM_TABLE_BUDGET = int(os.environ.get("GLASS_GB300_PLM_TABLE_BYTES", str(160 << 30)))


def plm_table_bytes(nside: int, lmax: int) -> int:
    """Bytes of a plan's P_lm table (FP32 lambda per (l, m, ring pair),
    in 8 KB tiles of 16 l x 128 ring pairs)."""
    return 8192 * _ngroups(lmax) * ((2 * nside + 127) // 128)


def plan_bytes(nside: int, lmax: int, fast: bool = True) -> int:
    """Upper bound of the device bytes of a transform plan (glg_plan_create)
    and of its fast-form tables (built on the first fast transform): ring
    geometry, recurrence tables, lambda_mm starts, FFT twiddles; seeds,
    FP32 coefficients, first-l tables and the FP32 ring-FFT tables (each
    Bluestein length M < 16 i for a ring of 4 i pixels)."""
    n = lmax + 1
    nalm = n * (n + 1) // 2
    npairs = 2 * nside
    ntw = 4 * nside * (nside + 1)
    b = (npairs * 40 + 8 * (n + 1) + 16 * nalm + 12 * n * npairs + 84 * (nside + 1) + 8 * (nside + 2)
         + 16 * ntw)
    if fast:
        tiles = (npairs + 127) // 128
        plm = plm_table_bytes(nside, lmax)
        lam = plm if plm <= PLM_TABLE_BUDGET else 8 * _ngroups(lmax) * tiles * 128  # table or seeds
        b += (8 * npairs + 8 * ntw + 16 * (nalm + 16) + 8 * (n + 1) + lam
              + 4 * n * npairs + 4 * n * tiles)
        b += (4 * npairs + 8 * (nside + 2) + 2 * ntw + 20 * (nside + 1) + 8 * 8 * ntw + 8 * ntw
              + 8 * (16 * nside + 1))
    return b


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
        mdt = torch.float32 if form == "fast" else torch.float64
        self.out = torch.empty((req.nshell, 12 * req.nside * req.nside), dtype=mdt, device=device)
        self.done_event: torch.cuda.Event | None = None


class _Group:
    """Launch buffers of one (nside, lmax): the plan, a stream, the transform
    workspace and the staged alm / maps of one launch, reused by every
    launch of the group (launches on one stream run in order)."""

    def __init__(self, nside: int, lmax: int, nmaps: int, form: str, device: torch.device):
        self.nside, self.lmax, self.nmaps, self.form = nside, lmax, nmaps, form
        self.plan = _lib.get_plan(nside, lmax, device)
        self.stream = torch.cuda.Stream(device)
        n = lmax + 1
        nalm = n * (n + 1) // 2
        npix = 12 * nside * nside
        cdt = torch.complex64 if form == "fast" else torch.complex128
        self.alm = torch.empty((nmaps, nalm), dtype=cdt, device=device)
        self.maps = torch.empty((nmaps, npix), dtype=torch.float32, device=device) if form == "fast" else None
        self.ws = torch.empty(hp.workspace_bytes(nside, lmax, nmaps, form, device), dtype=torch.uint8,
                              device=device)
        self.bytes = launch_bytes(nside, lmax, nmaps, form)
        self.plan_bytes = plan_bytes(nside, lmax, form == "fast")  # until the fast tables exist
        self.active = 0
        self.last_used = 0.0
        # device-wait status of each launch, copied asynchronously (one slot
        # per launch in flight, checked when the launch's requests retire)
        self.status = torch.zeros(64, dtype=torch.int32, pin_memory=True)
        self.slot = 0
        self.graphs: dict[int, hp.SynthGraph] = {}  # fast form: captured launches by map count

    def graph(self, cnt: int) -> hp.SynthGraph:
        """The captured fast synthesis of `cnt` maps on this group's buffers,
        its epilogue read from device memory (captured on first use)."""
        gr = self.graphs.get(cnt)
        if gr is None:
            gr = self.graphs[cnt] = hp.SynthGraph(self.nside, self.lmax, cnt, device_epilogue=True,
                                                  alm=self.alm, maps=self.maps, ws=self.ws,
                                                  device=self.alm.device)
        return gr


class Server:
    """Continuous batching of simulation requests within an HBM budget.

    ``form="fast"`` with ``batching=True`` is the serving configuration;
    ``form="plain", batching=False`` (one map per transform launch, no
    sharing across requests) is the comparison point of the FP64 form.

    Device memory: the budget covers every device byte the server causes --
    the requests' spectra, iternorm rows, alm and maps (``request_bytes``),
    each (nside, lmax) group's launch buffers (``launch_bytes``: transform
    workspace, staged alm and maps) and the cached plans with their fast
    tables (``plan_bytes`` until a plan's tables exist, its measured size
    after).  A request waits in the queue until all of that fits; idle
    groups (no request in service) give up their buffers and plans, least
    recently used first, when a new request needs the room.

    Launches: with ``graphs=True`` (or ``GLASS_GB300_SERVING_GRAPHS=1``),
    each fast (nside, lmax, map count) launch of a small transform (nside <=
    ``GLASS_GB300_SERVING_GRAPH_NSIDE``, 256 by default) replays a CUDA graph
    captured on first use over the group's buffers, its epilogue (kinds,
    variances, shifts of the launch's shells) read from device memory
    (``healpix.SynthGraph(device_epilogue=True)``); otherwise the kernels
    are launched one by one (the default: measured no slower).
    """

    def __init__(self, hbm_budget: int = 120 << 30, max_maps_per_launch: int = 40,
                 device: torch.device | None = None, form: str = "fast", batching: bool = True,
                 graphs: bool | None = None):
        if form not in ("fast", "plain"):
            raise ValueError(f"form must be 'plain' or 'fast', not {form!r}")
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        self.budget = int(hbm_budget)
        self.form = form
        self.batching = bool(batching)
        # fast form: each (nside, lmax, map count) launch replays a captured
        # CUDA graph whose epilogue comes from device memory
        if graphs is None:
            graphs = os.environ.get("GLASS_GB300_SERVING_GRAPHS", "0") == "1"
        self.graphs = bool(graphs) and form == "fast"
        # graphs for the small transforms only, where the ~30 launches cost
        # as much as the work.  Off by default: on the GB300 the serving
        # workload measured no gain from them (capacity 529-577 req/s with
        # and without, p99 higher with), its latency being set by the
        # device work queued behind the large requests, not by launches
        self.graph_nside = int(os.environ.get("GLASS_GB300_SERVING_GRAPH_NSIDE", "256"))
        self.max_maps = min(int(max_maps_per_launch), hp.FAST_MAX_MAPS) if batching else 1
        self.queue: collections.deque[Request] = collections.deque()
        self.active: list[_Active] = []
        self.finished: list[Request] = []
        self.groups: dict[tuple[int, int], _Group] = {}
        self.lock = threading.Lock()
        self._next_id = 0
        self._req_bytes = 0
        self.peak_active = 0  # most requests in service at once

    @property
    def used(self) -> int:
        """Device bytes currently accounted: requests + group buffers + plans."""
        return self._req_bytes + sum(g.bytes + g.plan_bytes for g in self.groups.values())

    # ------------------------------------------------------------- intake

    def _fixed_bytes(self, nside: int, lmax: int) -> int:
        return launch_bytes(nside, lmax, self.max_maps, self.form) + plan_bytes(nside, lmax, self.form == "fast")

    def submit(self, req: Request) -> Request:
        with self.lock:
            req.id = self._next_id
            self._next_id += 1
            if req.arrival == 0.0:
                req.arrival = time.perf_counter()
            need = request_bytes(req.nside, req.lmax, req.nshell, self.form) + self._fixed_bytes(req.nside, req.lmax)
            if need > self.budget:
                raise MemoryError(f"request {req.id} needs {need} bytes, over the HBM budget {self.budget}")
            self.queue.append(req)
        return req

    def _evict_idle(self, need: int, keep: tuple[int, int]) -> None:
        """Free idle groups (least recently used first) until `need` fits."""
        idle = sorted((g.last_used, k) for k, g in self.groups.items() if g.active == 0 and k != keep)
        for _, k in idle:
            if self.used + need <= self.budget:
                break
            g = self.groups.pop(k)
            g.stream.synchronize()  # its last launch has left the buffers
            _lib.drop_plan(g.nside, g.lmax, self.device)
            del g

    def _admit(self) -> None:
        while self.queue:
            req = self.queue[0]
            key = (req.nside, req.lmax)
            need = request_bytes(req.nside, req.lmax, req.nshell, self.form)
            if key not in self.groups:
                need += self._fixed_bytes(req.nside, req.lmax)
            if self.used + need > self.budget:
                self._evict_idle(need, key)
                if self.used + need > self.budget:
                    break
            self.queue.popleft()
            g = self.groups.get(key)
            if g is None:
                g = self.groups[key] = _Group(req.nside, req.lmax, self.max_maps, self.form, self.device)
            req.reserved = request_bytes(req.nside, req.lmax, req.nshell, self.form)
            self._req_bytes += req.reserved
            g.active += 1
            req.admitted = time.perf_counter()
            with torch.cuda.stream(g.stream):
                self.active.append(_Active(req, self.device, self.form))
            self.peak_active = max(self.peak_active, len(self.active))

    def _stream(self, nside: int, lmax: int) -> torch.cuda.Stream:
        return self.groups[(nside, lmax)].stream

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
            g = self.groups[(nside, lmax)]
            for c0 in range(0, len(items), self.max_maps):
                chunk = items[c0:c0 + self.max_maps]
                cnt = len(chunk)
                with torch.cuda.stream(g.stream):
                    torch.stack([a.alm[s] for a, s in chunk], out=g.alm[:cnt])
                    epi = ([a.kinds[s] for a, s in chunk], [a.var[s] for a, s in chunk],
                           [a.lam[s] for a, s in chunk])
                    if self.form == "fast":
                        st = g.status[g.slot % g.status.numel():][:1]
                        g.slot += 1
                        if self.graphs and nside <= self.graph_nside:
                            # one graph launch instead of ~30 kernel launches
                            maps = g.graph(cnt)(None, epilogue=epi)
                            st.copy_(g.ws[:4].view(torch.int32), non_blocking=True)
                        else:
                            maps = hp.synth(g.alm[:cnt], nside, lmax, epilogue=epi, form="fast",
                                            out=g.maps[:cnt], ws=g.ws, status=st)
                    else:
                        maps = hp.synth(g.alm[:cnt], nside, lmax, epilogue=epi, form="plain", ws=g.ws)
                    for k, (a, s) in enumerate(chunk):
                        a.out[s].copy_(maps[k])
                for a, s in chunk:
                    a.next_shell = max(a.next_shell, s + 1)
                g.last_used = time.perf_counter()
                launched = True
            if self.form == "fast" and g.plan_bytes and getattr(g.plan, "tuned", False):
                g.plan_bytes = int(_lib.lib().glg_plan_device_bytes(g.plan.handle))  # measured now
            for a in {id(x[0]): x[0] for x in items}.values():
                if a.next_shell == a.req.nshell and a.done_event is None:
                    ev = torch.cuda.Event()
                    ev.record(g.stream)
                    a.done_event = ev
        return launched

    def _retire(self) -> None:
        keep = []
        for a in self.active:
            if a.done_event is not None and a.done_event.query():
                g = self.groups[(a.req.nside, a.req.lmax)]
                if self.form == "fast" and bool(torch.any(g.status != 0)):
                    raise RuntimeError("a bounded device wait of the fast Legendre contraction timed out")
                a.req.maps = list(a.out)
                a.req.finished = time.perf_counter()
                self._req_bytes -= a.req.reserved
                g.active -= 1
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

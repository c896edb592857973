"""ctypes binding of ``libglassgb300.so`` (the C ABI of include/glass_gb300.h).

The product path has no CPU fallback: if the library or a CUDA device is
missing, :func:`lib` raises instead of computing anything on the host.
"""

from __future__ import annotations

import ctypes
import os
import pathlib
import threading

import numpy as np
import torch

_HERE = pathlib.Path(__file__).resolve().parent
_LIBPATH = _HERE / "_build" / "libglassgb300.so"
_LIB = None
_LOCK = threading.Lock()

GLG_OK = 0
GLG_ERR_INVALID = -1
GLG_ERR_NOT_POSDEF = -2
GLG_ERR_CUDA = -3
GLG_ERR_NOMEM = -4
GLG_ERR_UNSUPPORTED = -5
GLG_ERR_TIMEOUT = -6

GLG_F64 = 0
GLG_F32 = 1
FORM_PLAIN = 0
FORM_FAST = 1
EPI_NONE = 0
EPI_LOGNORMAL = 1

c_p = ctypes.c_void_p
c_i = ctypes.c_int
c_i64 = ctypes.c_int64
c_u64 = ctypes.c_uint64
c_sz = ctypes.c_size_t


class Epilogue(ctypes.Structure):
    _fields_ = [("kind", c_i), ("kinds", ctypes.POINTER(c_i)),
                ("var", ctypes.POINTER(ctypes.c_double)),
                ("lamda", ctypes.POINTER(ctypes.c_double))]


_SIGNATURES = {
    "glg_version": ([], ctypes.c_char_p),
    "glg_last_error": ([], ctypes.c_char_p),
    "glg_plan_create": ([c_i, c_i, c_p, ctypes.POINTER(c_p)], c_i),
    "glg_plan_destroy": ([c_p], None),
    "glg_plan_device_bytes": ([c_p], c_sz),
    "glg_set_plm_table_budget": ([c_sz], c_i),
    "glg_plan_has_plm_table": ([c_p], c_i),
    "glg_plan_info": ([c_p, ctypes.POINTER(c_i), ctypes.POINTER(c_i), ctypes.POINTER(c_i),
                       ctypes.POINTER(c_i64), ctypes.POINTER(c_i64)], c_i),
    "glg_iternorm": ([c_p, c_i64, c_i64, c_i, c_p, c_p, c_p], c_i),
    "glg_philox_normals": ([c_u64, c_u64, c_i64, c_i64, c_i, c_p, c_p], c_i),
    "glg_cls2cov": ([c_p, c_p, c_i, c_i, c_i, c_p, c_p, c_p, c_p], c_i),
    "glg_alm_correlate": ([c_p, c_i, c_i, c_i, c_i64, c_p, c_i64, c_u64, c_u64, c_i, c_p, c_p], c_i),
    "glg_gather_host": ([c_p, c_p, c_i, c_p, c_i], c_i),
    "glg_multalm": ([c_p, c_p, c_i, c_i, c_p, c_p], c_i),
    "glg_almxfl": ([c_p, c_p, c_i, c_i, c_i, c_i, c_p, c_p], c_i),
    "glg_autotune_fast": ([c_p, c_i, c_p, c_p, c_sz, c_p], c_i),
    "glg_plan_buckets": ([c_p, c_p, c_i], c_i),
    "glg_plan_bucket_times": ([c_p, c_p, c_i], c_i),
    "glg_convergence_step": ([c_p, c_p, c_p, c_i, c_i64, ctypes.c_double, ctypes.c_double, c_p], c_i),
    "glg_ang2pix": ([c_i, c_p, c_p, c_i64, c_i, c_p, c_p], c_i),
    "glg_galaxy_shear": ([c_p, c_p, c_p, c_i64, c_p, c_p, c_p, c_i, c_i, c_i, c_p, c_p], c_i),
    "glg_positions": ([c_i, c_p, c_i64, c_i64, c_u64, c_u64, c_p, c_p, c_p, c_p], c_i),
    "glg_poisson_counts": ([c_p, c_i, c_i64, ctypes.c_double, ctypes.c_double, ctypes.c_double, c_p,
                            c_u64, c_u64, c_p, c_p], c_i),
    "glg_alm2map_workspace": ([c_p, c_i, c_i], c_sz),
    "glg_alm2map": ([c_p, c_p, c_i, c_i, c_p, ctypes.POINTER(Epilogue), c_p, c_sz, c_p], c_i),
    "glg_alm2map_host_workspace": ([c_p, c_i], c_sz),
    "glg_alm2map_host": ([c_p, c_p, c_i, c_p, ctypes.POINTER(Epilogue), c_p, c_sz, c_p], c_i),
    "glg_host_output_runs": ([c_i, c_p, c_i], c_i),
    "glg_workspace_status": ([c_p, c_p], c_i),
    "glg_alm2map_noalloc": ([c_i, c_i, c_p, c_i, c_p, c_p], c_i),
    "glg_pixwin_workspace": ([c_i], c_sz),
    "glg_pixwin": ([c_i, c_i, c_p, c_p, c_p, c_sz, c_p], c_i),
    "glg_test_fail_plan_alloc": ([c_i], c_i),
    "glg_test_stall_contraction": ([c_i, ctypes.c_uint], c_i),
    "glg_peak_tf32": ([c_i, c_i, c_p, c_p], c_i),
    "glg_host_device_pointer": ([c_p, ctypes.POINTER(c_p)], c_i),
    "glg_peak_fma": ([c_i, c_i, c_i, c_p, c_p], c_i),
    "glg_alm2map_spin_workspace": ([c_p], c_sz),
    "glg_alm2map_spin": ([c_p, c_p, c_p, c_i, c_p, c_p, c_p, c_sz, c_p], c_i),
    "glg_alm2map_spin_fast_workspace": ([c_p, c_i, c_i], c_sz),
    "glg_epilogue_dev_bytes": ([], c_sz),
    "glg_epilogue_dev_fill": ([c_p, c_i, c_p], c_i),
    "glg_alm2map_fast_devepi": ([c_p, c_p, c_i, c_p, c_p, c_p, c_sz, c_p], c_i),
    "glg_alm2map_spin_fast": ([c_p, c_p, c_p, c_i, c_i, c_p, c_p, c_sz, c_p], c_i),
    "glg_map2alm_workspace": ([c_p, c_i], c_sz),
    "glg_map2alm": ([c_p, c_p, c_i, c_i, c_p, c_p, c_sz, c_p], c_i),
    "glg_timing_enable": ([c_i], c_i),
    "glg_timing_reset": ([], c_i),
    "glg_launch_count": ([], c_i64),
    "glg_timing_query": ([ctypes.c_char_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(c_i64)], c_i),
}

# Exported symbols declared in include/glass_gb300.h (checked by the tests).
EXPORTED = tuple(_SIGNATURES)


def library_path() -> pathlib.Path:
    return _LIBPATH


def load_library(require_gpu: bool = True) -> ctypes.CDLL:
    """Load the CUDA library; raise if it is missing (no host fallback)."""
    global _LIB
    with _LOCK:
        if _LIB is None:
            if not _LIBPATH.exists():
                raise ImportError(
                    f"glass_gb300 CUDA library not built ({_LIBPATH}); run "
                    "`python -m glass_gb300.build` (needs nvcc) -- there is no CPU fallback"
                )
            L = ctypes.CDLL(str(_LIBPATH))
            for name, (args, res) in _SIGNATURES.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = res
            if "GLASS_GB300_PLM_TABLE_BYTES" in os.environ:  # P_lm table budget of the fast form
                L.glg_set_plm_table_budget(int(os.environ["GLASS_GB300_PLM_TABLE_BYTES"]))
            _LIB = L
    if require_gpu and not torch.cuda.is_available():
        raise RuntimeError("glass_gb300 needs a CUDA device; none is available (no CPU fallback)")
    return _LIB


def lib() -> ctypes.CDLL:
    return load_library(require_gpu=True)


def last_error() -> str:
    msg = load_library(require_gpu=False).glg_last_error()
    return msg.decode() if msg else ""


def check(rc: int, what: str) -> None:
    """Map a C status to the reference's exception types."""
    if rc == GLG_OK:
        return
    msg = f"{what}: {last_error()}"
    if rc in (GLG_ERR_INVALID, GLG_ERR_NOT_POSDEF):
        raise ValueError(msg)
    if rc == GLG_ERR_NOMEM:
        raise MemoryError(msg)
    if rc == GLG_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise RuntimeError(msg)


def stream_ptr(device: torch.device | None = None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t: torch.Tensor | None) -> int | None:
    if t is None:
        return None
    return t.data_ptr()


def timing_enable(on: bool = True) -> None:
    lib().glg_timing_enable(1 if on else 0)


def timing_reset() -> None:
    lib().glg_timing_reset()


def launch_count() -> int:
    return int(lib().glg_launch_count())


def host_device_pointer(t: torch.Tensor) -> int:
    """Device address of a page-locked (pinned) CPU tensor's memory, for
    kernels that write straight into host buffers; raises ValueError when the
    memory is not pinned and mapped into the device."""
    dev = c_p()
    check(lib().glg_host_device_pointer(c_p(t.data_ptr()), ctypes.byref(dev)), "glg_host_device_pointer")
    return int(dev.value)


def kernel_time(name: str) -> tuple[float, int]:
    """(total ms, launches) of one kernel since the last reset (timing enabled)."""
    ms = ctypes.c_double()
    n = c_i64()
    check(lib().glg_timing_query(name.encode(), ctypes.byref(ms), ctypes.byref(n)), "glg_timing_query")
    return ms.value, n.value


# ------------------------------------------------------------------ plans


class Plan:
    """Device tables of one (nside, lmax): geometry, recurrence, FFT twiddles."""

    def __init__(self, nside: int, lmax: int, device: torch.device):
        self.nside, self.lmax, self.device = nside, lmax, device
        h = c_p()
        with torch.cuda.device(device):
            check(lib().glg_plan_create(nside, lmax, c_p(stream_ptr(device)), ctypes.byref(h)),
                  "glg_plan_create")
        self.handle = h
        self.nrings = 4 * nside - 1
        self.npix = 12 * nside * nside
        self.nalm = (lmax + 1) * (lmax + 2) // 2

    @property
    def bytes(self) -> int:
        """Device bytes of the plan's tables (grows when the fast tables are built)."""
        return int(lib().glg_plan_device_bytes(self.handle))

    @property
    def has_plm_table(self) -> bool:
        return bool(lib().glg_plan_has_plm_table(self.handle))

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _LIB is not None:
            try:
                torch.cuda.synchronize(self.device)
                _LIB.glg_plan_destroy(h)
            except Exception:  # noqa: BLE001 - interpreter shutdown
                pass
            self.handle = None


_PLANS: dict[tuple[int, int, int], Plan] = {}
_PLAN_LOCK = threading.Lock()
_PLAN_BUDGET = int(os.environ.get("GLASS_GB300_PLAN_BYTES", str(200 << 30)))


def get_plan(nside: int, lmax: int, device: torch.device | None = None) -> Plan:
    """Cached plan for (nside, lmax) on `device` (LRU within a byte budget)."""
    device = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    key = (device.index if device.index is not None else torch.cuda.current_device(), nside, lmax)
    with _PLAN_LOCK:
        p = _PLANS.pop(key, None)
        if p is None:
            p = Plan(nside, lmax, torch.device("cuda", key[0]))
        _PLANS[key] = p
        total = sum(q.bytes for q in _PLANS.values())
        while total > _PLAN_BUDGET and len(_PLANS) > 1:
            k0 = next(iter(_PLANS))
            total -= _PLANS.pop(k0).bytes
    return p


def clear_plans() -> None:
    with _PLAN_LOCK:
        _PLANS.clear()


def drop_plan(nside: int, lmax: int, device: torch.device | None = None) -> None:
    """Remove one plan from the cache (its device memory is freed once no
    caller holds the Plan object any more)."""
    device = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    key = (device.index if device.index is not None else torch.cuda.current_device(), nside, lmax)
    with _PLAN_LOCK:
        _PLANS.pop(key, None)


# -------------------------------------------------------------- conversion


def to_device(x, dtype: torch.dtype, device: torch.device | None = None) -> torch.Tensor:
    """numpy / torch / sequence -> contiguous CUDA tensor of `dtype`."""
    device = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    if isinstance(x, torch.Tensor):
        t = x.to(device=device, dtype=dtype)
    else:
        t = torch.as_tensor(np.asarray(x), dtype=dtype).to(device, non_blocking=False)
    return t.contiguous()


def default_form() -> str:
    """The transform form when a call names none: ``GLASS_GB300_FORM``
    ("plain", the FP64 drop-in, by default; or "fast")."""
    f = os.environ.get("GLASS_GB300_FORM", "plain").lower()
    if f not in ("plain", "fast"):
        raise ValueError(f"GLASS_GB300_FORM must be 'plain' or 'fast', not {f!r}")
    return f


def is_numpy_like(x) -> bool:
    return not isinstance(x, torch.Tensor)

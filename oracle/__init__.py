"""CPU oracle for the GLASS field-generation path -- TEST INFRASTRUCTURE ONLY.

Nothing in the product (``glass_gb300``) imports this package.  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its ``cpu_baseline``
leg and its ``--impl reference`` arm) use it, as the checker and as the timed
CPU baseline.

Contents
--------
``oracle.sht``
    FP64 restatement of the HEALPix ring spherical-harmonic transform that
    the reference calls through healpy (``glass/healpix.py:38-108``,
    ``:232-276``): C Legendre sums (``orc_sht.c``) plus numpy ring FFTs,
    and a brute-force ``scipy.special.sph_harm_y`` direct sum that pins it.
``oracle.fields``
    Restatement of the reference's field-generation glue
    (``glass/fields.py:191-236`` cls2cov, ``:101-188`` iternorm,
    ``:334-429`` _generate_grf, ``:839-894`` generate,
    ``glass/harmonics.py:17-47`` multalm, ``glass/fields.py:943-962``
    alm reordering, ``glass/grf/_transformations.py:83-89`` Lognormal).
``oracle.rng``
    Philox4x32-10 + Box-Muller restatement of the GPU variate stream.

Parity status: the field-generation glue is pinned against fixtures made by
running the reference's own Python under import shims
(``tests/golden/make_golden.py``).  The SHT restatement is pinned against the
brute-force direct sum and analytic known answers; parity with healpy itself
is unpinned (healpy is not installed here or on the GPU host).
"""

from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess
import threading

_HERE = pathlib.Path(__file__).resolve().parent
_LIB = None
_LOCK = threading.Lock()


def build() -> pathlib.Path:
    """Compile ``orc_sht.c`` into ``oracle/_build/liborc.so`` (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", str(_HERE)], check=True)
    return _HERE / "_build" / "liborc.so"


def lib() -> ctypes.CDLL:
    """Load (building if needed) the oracle's C library."""
    global _LIB
    with _LOCK:
        if _LIB is None:
            path = _HERE / "_build" / "liborc.so"
            src = _HERE / "orc_sht.c"
            if not path.exists() or path.stat().st_mtime < src.stat().st_mtime:
                build()
            _LIB = ctypes.CDLL(str(path))
            _declare(_LIB)
    return _LIB


def _declare(L: ctypes.CDLL) -> None:
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    u32p = ctypes.POINTER(ctypes.c_uint32)
    i64p = ctypes.POINTER(ctypes.c_int64)
    L.orc_ring_info.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, ip, dp, i64p]
    L.orc_ring_info.restype = None
    L.orc_alm2ring.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip, ctypes.c_int, dp]
    L.orc_alm2ring.restype = None
    L.orc_alm2ring_all.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
    L.orc_alm2ring_all.restype = None
    L.orc_ring2alm.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip, ctypes.c_int, dp]
    L.orc_ring2alm.restype = None
    L.orc_alm2ring_spin.argtypes = [dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip, ctypes.c_int, dp]
    L.orc_alm2ring_spin.restype = None
    L.orc_iternorm.argtypes = [dp, ctypes.c_long, ctypes.c_long, ctypes.c_int, dp]
    L.orc_iternorm.restype = ctypes.c_long
    L.orc_iternorm_dense.argtypes = [dp, ctypes.c_long, ctypes.c_long, ctypes.c_int, dp]
    L.orc_iternorm_dense.restype = ctypes.c_long
    L.orc_philox4x32_10.argtypes = [u32p, u32p, u32p]
    L.orc_philox4x32_10.restype = None
    L.orc_philox_normals.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64, dp, u32p]
    L.orc_philox_normals.restype = None
    L.orc_poisson_counts.argtypes = [dp, ctypes.c_int64, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                     dp, ctypes.c_uint64, ctypes.c_uint32, i64p]
    L.orc_poisson_counts.restype = None
    L.orc_exp_neg.argtypes = [ctypes.c_double]
    L.orc_exp_neg.restype = ctypes.c_double
    L.orc_num_threads.argtypes = []
    L.orc_num_threads.restype = ctypes.c_int


def num_threads() -> int:
    return int(lib().orc_num_threads())


def set_threads(n: int) -> None:
    """Set the OpenMP thread count for subsequent oracle calls."""
    os.environ["OMP_NUM_THREADS"] = str(n)

"""Failure paths of the CUDA library, made to happen without a GPU fault.

* An allocation failure during plan creation (injected on the host by
  glg_test_fail_plan_alloc, the n-th plan allocation reporting
  cudaErrorMemoryAllocation) surfaces as MemoryError, leaks nothing the next
  plan needs and leaves plan creation working.
* A bounded device wait that runs out: glg_test_stall_contraction makes the
  fast contraction's B streamer issue no copies, so the MMA warps' waits end
  after a few thousand polls; the kernel records GLG_ERR_TIMEOUT in the
  workspace status word, retires what it started, frees its tensor memory and
  returns.  The caller sees RuntimeError ("timed out"), and the next call on
  the same context is correct.

The error contract mirrors the reference's: errors are raised as Python
exceptions at the call (glass/fields.py:125-126, :140-141, :180-181 raise
ValueError for bad input; allocation failures are MemoryError).
"""

from __future__ import annotations

import time

import numpy as np
import pytest

import oracle.sht as osht
from tests.conftest import random_alm

pytestmark = pytest.mark.gpu


def test_plan_alloc_failure_is_memory_error(cuda_lib):
    from glass_gb300 import _lib

    for nth in (1, 5, 12):
        assert cuda_lib.glg_test_fail_plan_alloc(nth) == 0
        with pytest.raises(MemoryError, match="injected"):
            _lib.Plan(16, 20, __import__("torch").device("cuda", 0))
    cuda_lib.glg_test_fail_plan_alloc(0)
    p = _lib.Plan(16, 20, __import__("torch").device("cuda", 0))  # creation works again
    assert p.npix == 12 * 16 * 16


def test_contraction_wait_timeout_then_recovers(cuda_lib):
    import torch

    from glass_gb300 import _lib
    from glass_gb300 import healpix as hp

    nside, lmax = 32, 64
    alm = torch.as_tensor(random_alm(lmax, seed=9, nmaps=3), device="cuda")
    ref = osht.alm2map(random_alm(lmax, seed=9, nmaps=3), nside, lmax)
    hp.synth(alm, nside, lmax, form="fast")  # tables and autotuning outside the stall
    torch.cuda.synchronize()
    assert cuda_lib.glg_test_stall_contraction(1, 4000) == 0
    try:
        t = time.perf_counter()
        with pytest.raises(RuntimeError, match="timed out"):
            hp.synth(alm, nside, lmax, form="fast")
        torch.cuda.synchronize()
        assert time.perf_counter() - t < 60
    finally:
        cuda_lib.glg_test_stall_contraction(0, 0)
    got = hp.synth(alm, nside, lmax, form="fast").cpu().numpy()
    err = np.sqrt(np.mean((got - ref) ** 2)) / np.sqrt(np.mean(ref ** 2))
    assert err < 1e-6
    assert torch.cuda.synchronize() is None  # the context is still usable
    assert _lib.last_error() != ""

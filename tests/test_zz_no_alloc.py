"""GPU test of glg_alm2map_noalloc, the synthesis entry point that allocates nothing.

It serves callers that cannot call cudaMalloc where they need a map (loops
whose device memory is fixed at start-up, programs whose device memory belongs
to another allocator).  This test calls it through the C ABI and checks it
against the plan-and-workspace entry point glg_alm2map (plain FP64 form) to
the plain form's tolerance, 1e-12 relative, on two calls in a row with
different inputs -- the second call must not see the first call's scratch
contents -- and on a small call right after a large one.  The file is
collected last so that a run stopping at the first failure has already run
every other test.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from tests.conftest import random_alm, rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _plain(alm, nside, lmax):
    import torch

    from glass_gb300 import healpix as hp

    a = torch.as_tensor(alm, device="cuda", dtype=torch.complex128)
    return hp.synth(a, nside, lmax).cpu().numpy()


def _noalloc(lib, alm, nside, lmax):
    import torch

    from glass_gb300 import _lib

    a = torch.as_tensor(alm, device="cuda", dtype=torch.complex128).contiguous()
    out = torch.empty((a.shape[0], 12 * nside * nside), dtype=torch.float64, device="cuda")
    rc = lib.glg_alm2map_noalloc(nside, lmax, ctypes.c_void_p(a.data_ptr()), a.shape[0],
                                 ctypes.c_void_p(out.data_ptr()),
                                 ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, _lib.last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize(("nside", "lmax", "nmaps"), [(16, 40, 2), (64, 150, 3)])
def test_noalloc_matches_alm2map_twice(cuda_lib, nside, lmax, nmaps):
    for seed in (1, 2):  # two calls in a row, different inputs
        alm = random_alm(lmax, seed=seed + nside, nmaps=nmaps)
        got = _noalloc(cuda_lib, alm, nside, lmax)
        ref = _plain(alm, nside, lmax)
        assert rel_err(got, ref) < TOL


def test_noalloc_small_after_large(cuda_lib):
    # the large call fills more of the shared scratch array than the small
    # one writes: the small call must read only entries it wrote itself
    big = random_alm(150, seed=11, nmaps=3)
    assert rel_err(_noalloc(cuda_lib, big, 64, 150), _plain(big, 64, 150)) < TOL
    small = random_alm(20, seed=12, nmaps=1)
    assert rel_err(_noalloc(cuda_lib, small, 16, 20), _plain(small, 16, 20)) < TOL


def test_noalloc_rejects_oversize(cuda_lib):
    import torch

    from glass_gb300 import _lib

    a = torch.zeros(10, dtype=torch.complex128, device="cuda")
    out = torch.zeros(10, dtype=torch.float64, device="cuda")
    rc = cuda_lib.glg_alm2map_noalloc(512, 10, ctypes.c_void_p(a.data_ptr()), 1,
                                      ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _lib.GLG_ERR_UNSUPPORTED and "256" in _lib.last_error()
    rc = cuda_lib.glg_alm2map_noalloc(256, 1500, ctypes.c_void_p(a.data_ptr()), 8,
                                      ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _lib.GLG_ERR_UNSUPPORTED and "scratch" in _lib.last_error()
    # fits the scratch array at nside 1 but not the launch grid
    rc = cuda_lib.glg_alm2map_noalloc(1, 70000, ctypes.c_void_p(a.data_ptr()), 1,
                                      ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _lib.GLG_ERR_UNSUPPORTED and "65535" in _lib.last_error()
    rc = cuda_lib.glg_alm2map_noalloc(1, 0, ctypes.c_void_p(a.data_ptr()), 70000,
                                      ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _lib.GLG_ERR_UNSUPPORTED and "65535" in _lib.last_error()

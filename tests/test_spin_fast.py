"""Fast form of the spin-s synthesis (alm2map_spin, glass/healpix.py:81-108)
and of from_convergence (glass/lensing.py:185-371) against the oracle's FP64
spin synthesis and the plain FP64 GPU form.

The bar is the fast form's: relative RMS map error <= 1e-6 against FP64.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle.sht as osht
from tests.conftest import random_alm

pytestmark = pytest.mark.gpu
FAST_RMS = 1e-6


@pytest.fixture(scope="module")
def g(cuda_lib):
    import glass_gb300

    return glass_gb300


def rel_rms(a, b) -> float:
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.sqrt(np.mean(np.abs(a - b) ** 2)) / np.sqrt(np.mean(np.abs(b) ** 2)))


def _red_alm(lmax, seed, slope=-1.0):
    a = random_alm(lmax, seed=seed)
    ell = np.concatenate([np.arange(m, lmax + 1) for m in range(lmax + 1)])
    return a * (ell + 1.0) ** slope


@pytest.mark.parametrize("spin", [1, 2])
@pytest.mark.parametrize("with_b", [False, True])
def test_fast_spin_vs_oracle(g, spin, with_b):
    nside, lmax = 64, 128
    e = _red_alm(lmax, 31)
    b = _red_alm(lmax, 32) if with_b else None
    q, u = g.healpix.alm2map_spin([e, b if b is not None else np.zeros_like(e)], nside, spin, lmax, form="fast")
    assert q.dtype == np.float32 and u.dtype == np.float32
    rq, ru = osht.alm2map_spin([e, b], nside, spin, lmax)
    assert rel_rms(q + 1j * u, rq + 1j * ru) < FAST_RMS


def test_fast_spin_batch_matches_single(g):
    import torch

    from glass_gb300 import healpix as hp

    nside, lmax = 32, 64
    es = torch.as_tensor(np.stack([_red_alm(lmax, 40 + k) for k in range(3)]), device="cuda")
    bs = torch.as_tensor(np.stack([_red_alm(lmax, 50 + k) for k in range(3)]), device="cuda")
    q, u = hp._spin_synth_fast(es, bs, nside, 2, lmax)
    for k in range(3):
        q1, u1 = hp._spin_synth_fast(es[k], bs[k], nside, 2, lmax)
        ref = torch.complex(q1, u1).cpu().numpy()
        assert rel_rms(torch.complex(q[k], u[k]).cpu().numpy(), ref) < 1e-7


def test_fast_spin_table_budget(g):
    """The spin tables count against the P_lm table budget: with no budget
    left the fast spin synthesis refuses instead of allocating."""
    from glass_gb300 import _lib

    nside, lmax = 16, 40
    _lib.drop_plan(nside, lmax)
    _lib.lib().glg_set_plm_table_budget(0)
    try:
        e = _red_alm(lmax, 7)
        with pytest.raises(NotImplementedError, match="spin"):
            g.healpix.alm2map_spin([e, np.zeros_like(e)], nside, 2, lmax, form="fast")
    finally:
        _lib.lib().glg_set_plm_table_budget(160 << 30)
        _lib.drop_plan(nside, lmax)


@pytest.mark.parametrize("nside", [64, 512])
def test_from_convergence_fast_vs_plain(g, nside):
    """The 10-shell size at nside 512 (lmax 1535): potential, deflection and the
    discretized shear of a convergence map, fast vs FP64, <= 1e-6 RMS each."""
    lmax = 3 * nside - 1
    alm = _red_alm(lmax, 9, slope=-1.5) * 1e-2
    kappa = osht.alm2map(alm, nside, lmax) if nside <= 64 else g.healpix.alm2map(alm, nside, lmax=lmax)
    plain = g.from_convergence(kappa, potential=True, deflection=True, shear=True, form="plain")
    fast = g.from_convergence(kappa, potential=True, deflection=True, shear=True, form="fast")
    assert fast[0].dtype == np.float32 and fast[2].dtype == np.complex64
    for f, p in zip(fast, plain):
        assert rel_rms(f, p) < FAST_RMS

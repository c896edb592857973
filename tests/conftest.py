"""Test configuration: markers, fixtures and paths.

``-m "not gpu"`` runs the oracle, golden-fixture, host-logic and C-ABI load
tests on the CPU; ``-m gpu`` runs the parity tests of the CUDA library
against the oracle on a GB300.
"""

from __future__ import annotations

import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: larger parity cases")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(ROOT / "tests" / "golden" / "glass_fields.npz"))


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library, loaded on a GPU host (build() runs first)."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from glass_gb300 import _lib
    from glass_gb300.build import build

    build()
    return _lib.lib()


def spectra_powerlaw15(nshell: int, lmax: int):
    ell = np.arange(lmax + 1)
    auto = 1e-2 * (ell + 1.0) ** -1.5
    return [np.exp(-abs(i - j) / 2) * auto for i in range(nshell) for j in range(i, -1, -1)]


def spectra_damped12(nshell: int, lmax: int, seed: int = 0):
    rng = np.random.default_rng(seed)
    amp = 10 ** rng.uniform(-3, -1, nshell)
    lam = rng.uniform(0.5, 2.0, nshell)
    ell = np.arange(lmax + 1)
    auto = [a * (ell + 1.0) ** -1.2 * np.exp(-((ell / 800.0) ** 2)) for a in amp]
    gls = [np.exp(-abs(i - j) / 1.5) * np.sqrt(auto[i] * auto[j])
           for i in range(nshell) for j in range(i, -1, -1)]
    return gls, lam


def rel_err(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))


def random_alm(lmax: int, seed: int = 0, nmaps: int | None = None):
    rng = np.random.default_rng(seed)
    n = (lmax + 1) * (lmax + 2) // 2
    shape = (n,) if nmaps is None else (nmaps, n)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    a[..., : lmax + 1] = a[..., : lmax + 1].real  # m = 0 is real for a real field
    return a

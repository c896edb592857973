"""GPU tests of the continuous-batching request loop (glass_gb300.serving).

A request served in a mix of other requests -- batched into shared
transform launches, admitted while others run, on per-(nside, lmax) streams
-- must give the same maps as when it is served alone.  Tolerance: 1e-6
relative to the largest value (the fast form's own accuracy bound); in
practice every map is computed from its own alm column and is bit-identical.
"""

from __future__ import annotations

import numpy as np
import pytest

from tests.conftest import spectra_damped12

pytestmark = pytest.mark.gpu


def _request(serving, nside, nshell, seed):
    gls, lam = spectra_damped12(nshell, 2 * nside, seed=seed)
    return serving.Request(gls=gls, nside=nside, shifts=[float(x) for x in lam], seed=seed)


@pytest.mark.parametrize("graphs", [False, True])
def test_result_alone_equals_result_in_mix(cuda_lib, graphs):
    """Also through captured launch graphs with device epilogues (the mix
    replays each (nside, map count) graph with other requests' shells)."""
    from glass_gb300 import serving

    alone = serving.Server(hbm_budget=8 << 30)
    ra = alone.submit(_request(serving, 32, 5, seed=11))
    alone.drain()
    ref = np.stack([m.cpu().numpy() for m in ra.maps])

    mix = serving.Server(hbm_budget=8 << 30, max_maps_per_launch=16, graphs=graphs)
    others = [_request(serving, nside, n, seed=100 + k)
              for k, (nside, n) in enumerate([(32, 7), (64, 4), (32, 3), (16, 9), (64, 6)])]
    for r in others[:2]:
        mix.submit(r)
    mix.step()  # some requests already in flight when the target arrives
    rb = mix.submit(_request(serving, 32, 5, seed=11))
    for r in others[2:]:
        mix.submit(r)
    done = mix.drain()
    assert len(done) == 6
    got = np.stack([m.cpu().numpy() for m in rb.maps])
    assert np.max(np.abs(got - ref)) <= 1e-6 * np.max(np.abs(ref))
    for r in done:
        assert r.latency is not None and r.latency >= 0
        assert len(r.maps) == r.nshell


def test_admission_within_measured_budget(cuda_lib):
    """The budget bounds the device memory the server really uses: the
    allocator's peak over the run plus the plans' device tables."""
    import torch

    from glass_gb300 import _lib, serving

    nside, lmax, nshell = 64, 128, 6
    _lib.clear_plans()
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    fixed = serving.launch_bytes(nside, lmax, 40) + serving.plan_bytes(nside, lmax)
    need = serving.request_bytes(nside, lmax, nshell)
    budget = fixed + int(2.5 * need)  # room for two requests at a time
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    srv = serving.Server(hbm_budget=budget)
    reqs = [srv.submit(_request(serving, nside, nshell, seed=s)) for s in range(5)]
    while srv.queue or srv.active:
        srv.step()
        assert srv.used <= srv.budget
        for r in srv.finished:  # the client takes finished maps to the host
            r.maps = [m.cpu() for m in r.maps]
        srv.finished.clear()
    torch.cuda.synchronize()
    assert all(r.finished is not None for r in reqs)
    # two requests fit the budget with the plan's estimated bytes; once the
    # plan's measured (smaller) size replaces the estimate a third may fit,
    # never all five
    assert 2 <= srv.peak_active < 5
    plans = sum(int(_lib.lib().glg_plan_device_bytes(g.plan.handle)) for g in srv.groups.values())
    assert plans <= serving.plan_bytes(nside, lmax)
    measured = torch.cuda.max_memory_allocated() - base + plans
    assert measured <= budget, (measured, budget)
    with pytest.raises(MemoryError, match="over the HBM budget"):
        srv.submit(_request(serving, 1024, 20, seed=1))


def test_idle_group_evicted_for_new_request(cuda_lib):
    from glass_gb300 import serving

    a = serving.launch_bytes(32, 64, 40) + serving.plan_bytes(32, 64) + serving.request_bytes(32, 64, 3)
    b = serving.launch_bytes(64, 128, 40) + serving.plan_bytes(64, 128) + serving.request_bytes(64, 128, 3)
    srv = serving.Server(hbm_budget=max(a, b) + min(a, b) // 2)  # never both groups at once
    r1 = srv.submit(_request(serving, 32, 3, seed=1))
    srv.drain()
    assert list(srv.groups) == [(32, 64)]
    r2 = srv.submit(_request(serving, 64, 3, seed=2))
    srv.drain()
    assert list(srv.groups) == [(64, 128)]
    assert r1.finished is not None and r2.finished is not None

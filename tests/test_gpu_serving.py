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

from tests.conftest import spectra_cfg2

pytestmark = pytest.mark.gpu


def _request(serving, nside, nshell, seed):
    gls, lam = spectra_cfg2(nshell, 2 * nside, seed=seed)
    return serving.Request(gls=gls, nside=nside, shifts=[float(x) for x in lam], seed=seed)


def test_result_alone_equals_result_in_mix(cuda_lib):
    from glass_gb300 import serving

    alone = serving.Server(hbm_budget=8 << 30)
    ra = alone.submit(_request(serving, 32, 5, seed=11))
    alone.drain()
    ref = np.stack([m.cpu().numpy() for m in ra.maps])

    mix = serving.Server(hbm_budget=8 << 30, max_maps_per_launch=16)
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


def test_admission_within_budget(cuda_lib):
    from glass_gb300 import serving

    need = serving.request_bytes(64, 128, 6)
    srv = serving.Server(hbm_budget=int(2.5 * need))  # at most two requests resident
    reqs = [srv.submit(_request(serving, 64, 6, seed=s)) for s in range(5)]
    peak = 0
    while srv.queue or srv.active:
        srv.step()
        peak = max(peak, srv.used)
        assert srv.used <= srv.budget
    assert all(r.finished is not None for r in reqs)
    assert peak <= 2 * need
    assert serving.request_bytes(1024, 2048, 20) > srv.budget
    with pytest.raises(MemoryError, match="over the HBM budget"):
        srv.submit(_request(serving, 1024, 20, seed=1))

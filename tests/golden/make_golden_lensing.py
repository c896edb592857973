"""Golden fixtures of the map-level lensing steps, made by the reference.

Runs the reference's OWN glass.lensing.MultiPlaneConvergence
(glass/lensing.py:511-586) and glass.galaxies.galaxy_shear
(glass/galaxies.py:271-347), imported unmodified from a GLASS checkout
(``--reference``) with the stand-in modules of
``tests/golden/shims/``, the flat LambdaCDM of ``tests/golden/cosmo_stub.py``
as the cosmology, and healpy's ang2pix / npix2nside (healpy is not installed
offline) replaced by the oracle's RING restatement.  The fixtures pin the
convergence recurrence (float64 and float32 maps) and the reduced-shear
arithmetic; the pixelisation itself is pinned separately (round trips).

Writes ``tests/golden/glass_lensing.npz``; re-run with
``python tests/golden/make_golden_lensing.py`` from the repository root.
"""

from __future__ import annotations

import argparse
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent


def planes(dtype, nside: int = 16, n: int = 6, seed: int = 3):
    rng = np.random.default_rng(seed)
    npix = 12 * nside * nside
    zs = np.linspace(0.15, 1.2, n)
    ws = rng.uniform(0.5, 1.5, n)
    ds = [np.exp(rng.normal(0, 0.7, npix)).astype(dtype) - dtype(1) for _ in range(n)]
    return zs, ws, ds


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="path of a GLASS source checkout")
    ap.add_argument("--out", default=str(HERE / "glass_lensing.npz"))
    args = ap.parse_args()
    sys.path[:0] = [str(HERE / "shims"), args.reference, str(ROOT), str(HERE)]
    import glass.galaxies  # noqa: PLC0415
    import glass.lensing  # noqa: PLC0415

    import oracle.lensing as olens  # noqa: PLC0415
    from cosmo_stub import FlatLCDM  # noqa: PLC0415

    out = {}
    for tag, dtype in (("f64", np.float64), ("f32", np.float32)):
        zs, ws, ds = planes(dtype)
        mpc = glass.lensing.MultiPlaneConvergence(FlatLCDM())
        kap = []
        for z, w, d in zip(zs, ws, ds):
            mpc.add_plane(d, float(z), float(w))
            kap.append(np.array(mpc.kappa, copy=True))
        out[f"mpc_{tag}_z"] = zs
        out[f"mpc_{tag}_w"] = ws
        out[f"mpc_{tag}_delta"] = np.stack(ds)
        out[f"mpc_{tag}_kappa"] = np.stack(kap)

    ghp = glass.galaxies.hp
    ghp.ang2pix = lambda nside, lon, lat, lonlat=True, xp=None: olens.ang2pix_lonlat(nside, lon, lat)
    ghp.npix2nside = lambda npix: int(round((npix // 12) ** 0.5))
    rng = np.random.default_rng(7)
    nside = 16
    npix = 12 * nside * nside
    ngal = 5000
    lon = rng.uniform(-180, 360, ngal)
    lat = np.degrees(np.arcsin(rng.uniform(-1, 1, ngal)))
    eps = rng.normal(0, 0.2, ngal) + 1j * rng.normal(0, 0.2, ngal)
    kappa = rng.normal(0, 0.05, npix)
    g1 = rng.normal(0, 0.03, npix)
    g2 = rng.normal(0, 0.03, npix)
    for red in (True, False):
        out[f"shear_{int(red)}"] = glass.galaxies.galaxy_shear(lon, lat, eps, kappa, g1, g2, reduced_shear=red)
    out.update(shear_lon=lon, shear_lat=lat, shear_eps=eps, shear_kappa=kappa, shear_g1=g1, shear_g2=g2)
    np.savez_compressed(args.out, **out)
    print("wrote", args.out, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()

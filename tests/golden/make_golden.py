"""Generate the golden fixtures of the field-generation path from the reference.

Runs the reference's OWN Python (glass.fields, glass.harmonics, glass.grf)
unmodified, imported from a GLASS checkout given by ``--reference``, with
the small stand-in modules of ``tests/golden/shims/`` on ``sys.path`` for
dependencies that are not
installed offline (array_api_compat, array_api_extra, transformcl, healpy,
healpix, cosmology).  healpy's transform is replaced by ``oracle.sht`` while
capturing exactly the alm the reference hands to it, so the fixtures pin:

* iternorm against the reference's own implementation (glass/fields.py:101-188),
* cls2cov (glass/fields.py:191-236),
* the alm passed to alm2map by _generate_grf (glass/fields.py:334-429):
  numpy-rng draws, deque window, multalm sum, GLASS->HEALPix reorder, m=0 fix,
* generate / generate_lognormal output maps (glass/fields.py:839-894,
  glass/grf/_transformations.py:83-89) given that transform,
* multalm (glass/harmonics.py:17-47) and _glass_to_healpix_alm values.

Writes ``tests/golden/glass_fields.npz`` (a few hundred KB).  Re-run with
``python tests/golden/make_golden.py`` from the repository root.
"""

from __future__ import annotations

import argparse
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent


def spectra_powerlaw15(nshell: int, lmax: int) -> list[np.ndarray]:
    """Auto C_l = 1e-2 (l+1)^-1.5, cross exp(-|i-j|/2) sqrt(C^ii C^jj), GLASS order."""
    ell = np.arange(lmax + 1)
    auto = 1e-2 * (ell + 1.0) ** -1.5
    gls = []
    for i in range(nshell):
        for j in range(i, -1, -1):
            gls.append(np.exp(-abs(i - j) / 2) * auto)
    return gls


def spectra_damped12(nshell: int, lmax: int, seed: int = 0):
    """A_i log-uniform [1e-3, 1e-1]; C^ii = A_i (l+1)^-1.2 exp(-(l/800)^2); corr exp(-|i-j|/1.5)."""
    rng = np.random.default_rng(seed)
    amp = 10 ** rng.uniform(-3, -1, nshell)
    lam = rng.uniform(0.5, 2.0, nshell)
    ell = np.arange(lmax + 1)
    auto = [a * (ell + 1.0) ** -1.2 * np.exp(-((ell / 800.0) ** 2)) for a in amp]
    gls = []
    for i in range(nshell):
        for j in range(i, -1, -1):
            gls.append(np.exp(-abs(i - j) / 1.5) * np.sqrt(auto[i] * auto[j]))
    return gls, lam


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="path of a GLASS source checkout")
    ap.add_argument("--out", default=str(HERE / "glass_fields.npz"))
    args = ap.parse_args()

    sys.path[:0] = [str(HERE / "shims"), args.reference, str(ROOT)]
    import glass  # noqa: PLC0415
    import glass.fields  # noqa: PLC0415
    import glass.harmonics  # noqa: PLC0415
    import glass.healpix as ghp  # noqa: PLC0415

    import oracle.sht as osht  # noqa: PLC0415

    captured: list[np.ndarray] = []

    def alm2map_stub(alm, nside, *, inplace=False, lmax=None, pixwin=False, pol=True):
        assert not pixwin and not pol
        captured.append(np.array(alm, copy=True))
        return osht.alm2map(np.asarray(alm), nside)

    ghp.alm2map = alm2map_stub
    out: dict[str, np.ndarray] = {}

    # iternorm: the reference's own test matrices (k = 0, 1, 2; 0-d and n-d)
    cov3 = np.array([[1.0, 0.2, 0.1], [0.2, 0.5, 0.2], [0.1, 0.2, 0.3]])
    cov3b = np.array([[1.4, 0.4, 0.5], [0.4, 1.5, 0.8], [0.5, 0.8, 1.3]])
    for k in (0, 1, 2):
        for nd, cov in (("0d", cov3), ("nd", np.stack([cov3, cov3b]))):
            rows = [cov[..., i, i::-1][..., : min(i, k) + 1] for i in range(3)]
            ws = list(glass.iternorm(iter(rows)))
            for i, w in enumerate(ws):
                out[f"iternorm_k{k}_{nd}_row{i}"] = np.asarray(w)
                out[f"iternorm_k{k}_{nd}_in{i}"] = np.asarray(rows[i])

    # iternorm on cls2cov rows of a 6-shell / lmax-40 damped power-law spectrum set
    gls6, _ = spectra_damped12(6, 40, seed=3)
    for nc in (5, 2):
        covs = [np.array(c, copy=True) for c in glass.cls2cov(gls6, 41, 6, nc)]
        ws = list(glass.iternorm(iter(covs)))
        out[f"cls2cov_cfg2_nc{nc}"] = np.stack(covs)
        out[f"iternorm_cfg2_nc{nc}"] = np.stack(ws)
        for i, g in enumerate(gls6):
            out[f"gls6_{i}"] = g

    # _generate_grf alm and generate_lognormal maps, 3 shells cfg-1 spectra
    nside, lmax = 8, 16
    gls3 = spectra_powerlaw15(3, lmax)
    for i, g in enumerate(gls3):
        out[f"gls3_{i}"] = g
    for tag, ncorr in (("all", None), ("nc1", 1)):
        captured.clear()
        fields = [glass.grf.Lognormal(1.0), glass.grf.Lognormal(0.7), glass.grf.Normal()]
        maps = list(glass.generate(fields, gls3, nside, ncorr=ncorr, rng=np.random.default_rng(42)))
        out[f"generate_alm_{tag}"] = np.stack(captured)
        out[f"generate_maps_{tag}"] = np.stack(maps)

    # generate_lognormal (deprecated wrapper, shift 1.0) on 4 cfg-2 shells
    gls4, _ = spectra_damped12(4, 24, seed=5)
    for i, g in enumerate(gls4):
        out[f"gls4_{i}"] = g
    captured.clear()
    import warnings  # noqa: PLC0415

    with warnings.catch_warnings():
        warnings.simplefilter("ignore", DeprecationWarning)
        maps = list(glass.generate_lognormal(gls4, 4, rng=np.random.default_rng(7)))
    out["lognormal4_alm"] = np.stack(captured)
    out["lognormal4_maps"] = np.stack(maps)

    # multalm / reorder known answers
    rng = np.random.default_rng(11)
    alm = rng.standard_normal(55) + 1j * rng.standard_normal(55)
    bl = rng.standard_normal(10)
    out["multalm_alm"] = alm
    out["multalm_bl"] = bl
    out["multalm_out"] = np.asarray(glass.harmonics.multalm(alm, bl))
    out["reorder_in"] = alm
    out["reorder_out"] = np.asarray(glass.fields._glass_to_healpix_alm(alm))

    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out}: {len(out)} arrays")


if __name__ == "__main__":
    main()

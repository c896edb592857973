"""Golden C_l file written by the reference's own ``glass.user.save_cls``
(glass/user.py:42-64), imported unmodified from a GLASS checkout
(``--reference``) with the stand-in modules of
``tests/golden/shims/``.  The spectra are seeded (4 spectra of lengths 5, 7,
7, 3), so the file pins the reference's on-disk layout for
``glass_gb300.save_cls`` / ``load_cls``.

Writes ``tests/golden/glass_cls_ref.npz``; re-run with
``python tests/golden/make_golden_cls.py`` from the repository root.
"""

from __future__ import annotations

import argparse
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent


def spectra():
    rng = np.random.default_rng(0)
    return [rng.normal(size=n) for n in (5, 7, 7, 3)]


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="path of a GLASS source checkout")
    ap.add_argument("--out", default=str(HERE / "glass_cls_ref.npz"))
    args = ap.parse_args()
    sys.path[:0] = [str(HERE / "shims"), args.reference]
    import glass.user  # noqa: PLC0415

    glass.user.save_cls(args.out, spectra())
    print("wrote", args.out)


if __name__ == "__main__":
    main()

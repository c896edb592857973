"""Angular power spectra on disk (glass/user.py:42-86).

``save_cls`` / ``load_cls`` read and write the reference's ``.npz`` layout
(the spectra concatenated in GLASS order under ``values``, the cumulative
lengths of all but the last under ``split``), so files move between GLASS
and glass_gb300 unchanged; they are the request input of the serving loop
(``glass_gb300.serving.Request.from_cls_file``).
"""

from __future__ import annotations

import numpy as np

__all__ = ["load_cls", "save_cls"]


def save_cls(filename, cls) -> None:
    """Save spectra in GLASS order to ``filename`` (``.npz`` appended by numpy)."""
    arrs = [np.asarray(c.cpu() if hasattr(c, "cpu") else c) for c in cls]
    lengths = np.array([a.shape[0] for a in arrs[:-1]], dtype=np.int64)
    split = np.cumsum(lengths)
    np.savez(filename, values=np.concatenate(arrs), split=split)


def load_cls(filename) -> list[np.ndarray]:
    """Load the list of spectra saved by ``save_cls`` (or by GLASS)."""
    with np.load(filename) as npz:
        values = npz["values"]
        split = npz["split"]
    return np.split(values, split)

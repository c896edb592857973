"""Minimal stand-in for ``array_api_extra`` (numpy only, in-place ``at``).

Only used by ``tests/golden/make_golden.py``.  ``at(x)[idx].set(v)`` writes
into ``x`` in place and returns it, which is what the real package does for
writeable numpy arrays.
"""
import numpy as np


class _AtIndex:
    def __init__(self, x, idx):
        self.x, self.idx = x, idx

    def set(self, v, copy=None):
        self.x[self.idx] = v
        return self.x

    def add(self, v, copy=None):
        self.x[self.idx] += v
        return self.x

    def multiply(self, v, copy=None):
        self.x[self.idx] *= v
        return self.x


class at:  # noqa: N801
    def __init__(self, x, idx=None):
        self.x = x

    def __getitem__(self, idx):
        return _AtIndex(self.x, idx)


def pad(x, pad_width, mode="constant", constant_values=0, xp=None):
    return np.pad(x, pad_width, mode=mode, constant_values=constant_values)


def apply_where(cond, args, f1, f2=None, /, *, fill_value=None, xp=None):
    if not isinstance(args, tuple):
        args = (args,)
    cond = np.asarray(cond)
    out = np.empty(np.broadcast(cond, *args).shape, dtype=np.result_type(*args, np.float64))
    if fill_value is not None:
        out[...] = fill_value
    sel = [np.broadcast_to(a, out.shape)[cond] for a in args]
    out[cond] = f1(*sel)
    if f2 is not None:
        nsel = [np.broadcast_to(a, out.shape)[~cond] for a in args]
        out[~cond] = f2(*nsel)
    return out

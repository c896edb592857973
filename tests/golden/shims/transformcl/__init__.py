"""Minimal stand-in for ``transformcl`` (only ``cltovar`` is real).

``cltovar`` is the variance of a field with angular power spectrum ``cl``:
sum over l of (2l+1)/(4 pi) * cl[l].
"""
import numpy as np


def cltovar(cl):
    cl = np.asarray(cl)
    ell = np.arange(cl.shape[-1])
    return np.sum((2 * ell + 1) / (4 * np.pi) * cl, axis=-1)


def cltocorr(cl, closed=False):
    raise NotImplementedError("cltocorr is not available in this stand-in")


def corrtocl(corr, closed=False):
    raise NotImplementedError("corrtocl is not available in this stand-in")

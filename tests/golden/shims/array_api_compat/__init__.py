"""Minimal stand-in for ``array_api_compat``: every array is a numpy array.

Only used by ``tests/golden/make_golden.py`` to import the reference's own
field-generation code in a container without network access.
"""
import numpy as np


def array_namespace(*arrays, use_compat=None):
    return np


def is_numpy_namespace(xp):
    return xp is np


def is_jax_namespace(xp):
    return False


def is_array_api_strict_namespace(xp):
    return False


def is_torch_namespace(xp):
    return False

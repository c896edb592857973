"""Stand-in for ``cosmology.api``: subscriptable protocol placeholders."""
import typing


class _Proto(typing.Protocol):
    def __class_getitem__(cls, item):
        return cls


def __getattr__(name):
    return _Proto

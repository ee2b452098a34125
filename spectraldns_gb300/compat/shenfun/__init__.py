"""Subset of shenfun names imported by the spectralDNS demos (host arrays)."""
import numpy as np

from . import fourier  # noqa: F401
from .fourier import energy_fourier  # noqa: F401


def Function(space, buffer=None, val=0):
    """Spectral array of `space` (a solver Space), or `buffer` when given."""
    if buffer is not None:
        return buffer
    return np.full(space.shape(True), val, dtype=np.result_type(space.dtype, np.complex64))


def Array(space, buffer=None, val=0):
    """Physical array of `space`, or `buffer` when given."""
    if buffer is not None:
        return buffer
    return np.full(space.shape(False), val, dtype=space.dtype)


class CachedArrayDict(dict):
    def __getitem__(self, key):
        a, i = key[0], key[1]
        fill = key[2] if len(key) > 2 else True
        k = (a.shape, np.dtype(a.dtype).str, i)
        if k not in self:
            dict.__setitem__(self, k, np.zeros(a.shape, dtype=a.dtype))
        arr = dict.__getitem__(self, k)
        if fill:
            arr.fill(0)
        return arr

"""Minimal ``InfoArray``: a NumPy array carrying a ``.header``.

TomograPy passes geometry to its projector through a ``.header`` attribute on
the arrays (``fitsarray.InfoArray``/``FitsArray``, an external package that the
reference depends on but does not vendor; see ``tomograpy/siddon.py:66,297-305``
and ``tomograpy/C_siddon.c.template:472,486``).  Data stacks carry a *list* of
per-view dicts, cubes carry one dict.  This class is the smallest stand-in that
keeps that calling convention: an ``ndarray`` subclass whose ``header`` survives
slicing and ufuncs.
"""
import copy

import numpy as np

# FITS BITPIX codes <-> numpy dtype names (the subset TomograPy uses).
bitpix = {"8": "int8", "16": "int16", "32": "int32", "-32": "float32", "-64": "float64"}
bitpix_inv = {v: k for k, v in bitpix.items()}


def dtype_from_bitpix(code):
    return np.dtype(bitpix[str(int(code))])


def bitpix_from_dtype(dtype):
    return int(bitpix_inv[np.dtype(dtype).name])


class InfoArray(np.ndarray):
    """ndarray with a ``header`` attribute (dict for cubes, list of dicts for stacks)."""

    def __new__(cls, shape=None, data=None, header=None, dtype=None, order="C"):
        if data is not None:
            obj = np.asarray(data, dtype=dtype).view(cls)
        else:
            obj = np.zeros(shape, dtype=dtype if dtype is not None else np.float64, order=order).view(cls)
        obj.header = header if header is not None else {}
        return obj

    def __array_finalize__(self, obj):
        if obj is None:
            return
        self.header = getattr(obj, "header", {})

    def copy(self, order="C"):
        out = np.ndarray.copy(self, order=order).view(type(self))
        out.header = copy.deepcopy(self.header)
        return out


def asinfoarray(arr, header):
    out = np.asarray(arr).view(InfoArray)
    out.header = header
    return out


def zeros(shape, header=None, dtype=np.float64):
    return InfoArray(shape=shape, header=header if header is not None else {}, dtype=dtype)

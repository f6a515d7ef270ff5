"""Simulation helpers of the drop-in API.

Restates ``tomograpy/simu.py`` (Python 2 + ``fitsarray``) in Python 3 with the
same keywords: ``circular_trajectory_data`` places ``n_images`` viewpoints at
``radius`` on ``linspace(min_lon, max_lon, n_images)`` longitudes
(``tomograpy/simu.py:158-210``), with M = d (cos lat cos lon, cos lat sin lon,
sin lat) (``tomograpy/simu.py:122-128``) and R from LON/LAT/ROL.
"""
import copy

import numpy as np

from . import headers as _h
from .infoarray import InfoArray, dtype_from_bitpix

# Mandatory image keywords and their defaults (tomograpy/simu.py:82-86).
default_image_dict = {"NAXIS": 2, "NAXIS1": 1, "NAXIS2": 1, "BITPIX": -64, "SIMPLE": True,
                      "CRPIX1": 0.5, "CRPIX2": 0.5, "CDELT1": 1.0, "CDELT2": 1.0,
                      "LON": 0.0, "LAT": 0.0, "ROL": 0.0, "D": 1.0,
                      "M1": 1.0, "M2": 0.0, "M3": 0.0}

# Mandatory cube keywords and their defaults (tomograpy/simu.py:90-94).
default_object_dict = {"NAXIS": 3, "NAXIS1": 1, "NAXIS2": 1, "NAXIS3": 1, "BITPIX": -64,
                       "SIMPLE": True, "CRPIX1": 0.5, "CRPIX2": 0.5, "CRPIX3": 0.5,
                       "CRVAL1": 0.0, "CRVAL2": 0.0, "CRVAL3": 0.0,
                       "CDELT1": 1.0, "CDELT2": 1.0, "CDELT3": 1.0}


def update_observer(h):
    """Recompute M1..M3 from LON/LAT/D (tomograpy/simu.py:122-128)."""
    lon, lat, d = h["LON"], h["LAT"], h["D"]
    h["M1"] = d * np.cos(lat) * np.cos(lon)
    h["M2"] = d * np.cos(lat) * np.sin(lon)
    h["M3"] = d * np.sin(lat)


def image_header(**kw):
    h = copy.copy(default_image_dict)
    h.update(kw)
    return h


def circular_trajectory_data(**kargs):
    """Zero data stack ``(NAXIS1, NAXIS2, n_images)`` on a circular trajectory.

    Keywords ``radius`` (default 1), ``dtype`` (float64), ``n_images`` (1),
    ``min_lon`` (0), ``max_lon`` (2 pi) are consumed; every other keyword is
    copied into each view header.
    """
    radius = kargs.pop("radius", 1.0)
    dtype = kargs.pop("dtype", np.float64)
    n_images = int(kargs.pop("n_images", 1))
    min_lon = kargs.pop("min_lon", 0.0)
    max_lon = kargs.pop("max_lon", 2 * np.pi)
    longitudes = np.linspace(min_lon, max_lon, n_images)
    hdrs = []
    for lon in longitudes:
        h = copy.copy(kargs)
        for k, v in default_image_dict.items():
            h.setdefault(k, v)
        h["LON"] = float(lon)
        update_observer(h)
        h["D"] = radius
        update_observer(h)
        _h.header_rotation_matrix(h)
        hdrs.append(h)
    shape = (int(kargs["NAXIS1"]), int(kargs["NAXIS2"]), n_images)
    data = InfoArray(shape=shape, header=hdrs, dtype=dtype)
    return data


def object_from_header(header, **kwargs):
    """Cube filled with ``fill`` (default 0) of the shape/dtype a header gives."""
    header = dict(header)
    for k, v in default_object_dict.items():
        header.setdefault(k, v)
    shape = (int(header["NAXIS1"]), int(header["NAXIS2"]), int(header["NAXIS3"]))
    try:
        dtype = dtype_from_bitpix(header["BITPIX"])
    except KeyError:
        dtype = np.float64
    dtype = header.pop("dtype", dtype)
    dtype = kwargs.pop("dtype", dtype)
    fill = kwargs.pop("fill", 0.0)
    _h.map_borders(header)
    obj = InfoArray(shape=shape, header=header, dtype=dtype)
    obj[:] = fill
    return obj


def spherical_object(radius=1.0, **kargs):
    """Cube of ones inside a sphere of ``radius`` (solar radii), zeros outside."""
    obj = object_from_header(kargs)
    h = obj.header
    axes = [(np.arange(obj.shape[i]) - h["CRPIX%d" % (i + 1)] + 0.5) * h["CDELT%d" % (i + 1)]
            for i in range(3)]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    obj[np.sqrt(X ** 2 + Y ** 2 + Z ** 2) < radius] = 1.0
    return obj

"""Geometry / header helpers of the drop-in API (host side, NumPy float64).

A Python-3 restatement of TomograPy's header builders and of the NumPy twins of
its C setup stage, with the reference's names and argument meanings:

* cube / image / stack header builders -- ``tomograpy/siddon.py:297-453``;
* rotation matrix from LON/LAT/ROL -- ``tomograpy/siddon.py:457-529``;
* unit vectors and intersection parameters (NumPy twins used by the
  reference's own tests) -- ``tomograpy/siddon.py:531-617,652-699``;
* header array <-> dict conversions -- ``tomograpy/siddon.py:703-787``;
* map borders MMIN/MMAX/PSHAPE -- ``tomograpy/siddon.py:559-572``.

Units follow the reference: cube coordinates in solar radii, image CDELT/CRVAL
in radians, observer position M in solar radii.
"""
import re

import numpy as np

from .infoarray import InfoArray, bitpix_from_dtype, dtype_from_bitpix

# "Infinity" of the reference kernel (tomograpy/C_siddon.c.template:17,
# tomograpy/siddon.py:82): a finite stand-in used when a direction component is 0.
INF = 100000


# ---------------------------------------------------------------------------
# header <-> array conversions (tomograpy/siddon.py:703-787)

def array_to_dict(indict, name, arr, imin=1):
    """Store a 1-d / 2-d array as ``name<i>`` / ``name<i>_<j>`` keys (1-based)."""
    arr = np.asarray(arr)
    dtname = arr.dtype.name
    if "float" in dtname:
        convert = float
    elif "int" in dtname:
        convert = int
    else:
        def convert(x):
            return x
    if arr.ndim == 1:
        for i in range(arr.shape[0]):
            indict[name + str(i + imin)] = convert(arr[i])
    elif arr.ndim == 2:
        for i in range(arr.shape[0]):
            for j in range(arr.shape[1]):
                indict[name + "%i_%i" % (i + imin, j + imin)] = convert(arr[i, j])
    else:
        raise ValueError("Not implemented for arr.ndim > 2")


def _header_array_shape(h, name):
    n = len(name)
    imax = jmax = 0
    imin = jmin = 10
    is1d = is2d = False
    for k in h.keys():
        if not isinstance(k, str) or k[:n] != name:
            continue
        s = k[n:]
        if re.fullmatch(r"[0-9]+_[0-9]+", s):
            is2d = True
            i, j = (int(a) for a in s.split("_"))
            imax, imin = max(imax, i), min(imin, i)
            jmax, jmin = max(jmax, j), min(jmin, j)
        elif re.fullmatch(r"[0-9]+", s):
            is1d = True
            i = int(s)
            imax, imin = max(imax, i), min(imin, i)
    if is2d:
        return (imax + 1 - imin, jmax + 1 - jmin), imin, jmin
    if is1d:
        return (imax + 1 - imin,), imin, jmin
    raise ValueError("header does not contain this array.")


def dict_to_array(h, name):
    """Inverse of :func:`array_to_dict`."""
    shape, imin, jmin = _header_array_shape(h, name)
    arr = np.empty(shape)
    if len(shape) == 1:
        for i in range(shape[0]):
            arr[i] = h[name + str(i + imin)]
    else:
        for i in range(shape[0]):
            for j in range(shape[1]):
                arr[i, j] = h[name + "%i_%i" % (i + imin, j + jmin)]
    return arr


# ---------------------------------------------------------------------------
# rotation matrix (tomograpy/siddon.py:457-529)

def rotation_matrix(lon, lat, rol):
    """Rotation from the image frame to the cube frame for a viewpoint at
    longitude ``lon``, latitude ``lat`` and roll ``rol`` (radians)."""
    cosln, sinln = np.cos(lon), np.sin(lon)
    coslt, sinlt = np.cos(lat), np.sin(lat)
    cosrl, sinrl = np.cos(rol), np.sin(rol)
    R = np.empty((3, 3))
    R[0, 0] = -cosln * coslt
    R[0, 1] = -sinln * cosrl - cosln * sinlt * sinrl
    R[0, 2] = sinln * sinrl - cosln * sinlt * cosrl
    R[1, 0] = -sinln * coslt
    R[1, 1] = cosln * cosrl - sinln * sinlt * sinrl
    R[1, 2] = -cosln * sinrl - sinln * sinlt * cosrl
    R[2, 0] = -sinlt
    R[2, 1] = coslt * sinrl
    R[2, 2] = coslt * cosrl
    return R


def header_rotation_matrix(h):
    """Add ``R1_1 .. R3_3`` to a view header from its LON/LAT/ROL keys."""
    array_to_dict(h, "R", rotation_matrix(h["LON"], h["LAT"], h["ROL"]))


def full_rotation_matrix(data):
    for h in data.header:
        header_rotation_matrix(h)


# ---------------------------------------------------------------------------
# map borders (tomograpy/siddon.py:559-572)

def map_borders(h):
    """Add PSHAPE = CDELT*NAXIS, MMIN = -CRPIX*CDELT, MMAX = MMIN+PSHAPE."""
    cdelt = np.asarray(dict_to_array(h, "CDELT"))[:3]
    crpix = np.asarray(dict_to_array(h, "CRPIX"))[:3]
    naxis = np.asarray([h["NAXIS%d" % (i + 1)] for i in range(3)], dtype=np.float64)
    pshape = cdelt * naxis
    array_to_dict(h, "PSHAPE", pshape)
    mmin = -crpix * cdelt
    array_to_dict(h, "MMIN", mmin)
    array_to_dict(h, "MMAX", mmin + pshape)


# ---------------------------------------------------------------------------
# header builders (tomograpy/siddon.py:297-453)

def _triple(x, n, what):
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    if x.size == 1:
        return np.repeat(x, n)
    if x.size != n:
        raise ValueError("%s should be a 1 or %d tuple" % (what, n))
    return x


def centered_cubic_map_header(pshape, shape, dtype=np.float64):
    """Header of a cube of ``shape`` voxels spanning ``pshape`` solar radii, centred on 0."""
    shape = _triple(shape, 3, "shape").astype(int)
    pshape = _triple(pshape, 3, "physical shape")
    h = {"SIMPLE": True, "BITPIX": bitpix_from_dtype(dtype), "NAXIS": 3}
    for i in range(3):
        h["NAXIS%d" % (i + 1)] = int(shape[i])
        h["CRPIX%d" % (i + 1)] = shape[i] / 2.0
        h["CDELT%d" % (i + 1)] = pshape[i] / float(shape[i])
        h["CRVAL%d" % (i + 1)] = 0.0
    map_borders(h)
    return h


def centered_cubic_map(pshape, shape, fill=0.0, dtype=np.float64):
    h = centered_cubic_map_header(pshape, shape, dtype=dtype)
    cube = InfoArray(shape=(h["NAXIS1"], h["NAXIS2"], h["NAXIS3"]), header=dict(h), dtype=dtype)
    cube[:] = fill
    return cube


def centered_image_header(pshape, shape, dtype=np.float64):
    """Header of an image of ``shape`` pixels spanning ``pshape`` radians, centred on 0."""
    shape = _triple(shape, 2, "shape").astype(int)
    pshape = _triple(pshape, 2, "physical shape")
    h = {"SIMPLE": True, "BITPIX": bitpix_from_dtype(dtype), "NAXIS": 2}
    for i in range(2):
        h["NAXIS%d" % (i + 1)] = int(shape[i])
        h["CRPIX%d" % (i + 1)] = shape[i] / 2.0
        h["CDELT%d" % (i + 1)] = pshape[i] / float(shape[i])
        h["CRVAL%d" % (i + 1)] = 0.0
    return h


def centered_image(pshape, shape, fill=0.0, dtype=np.float64):
    h = centered_image_header(pshape, shape, dtype=dtype)
    im = InfoArray(shape=(h["NAXIS1"], h["NAXIS2"]), header=h, dtype=dtype)
    im[:] = fill
    return im


def centered_stack(pshape, shape, n_images=1, radius=1.0, min_lon=0.0, max_lon=np.pi,
                   fill=0.0, dtype=np.float64):
    """Stack of centred images on a circular trajectory (tomograpy/siddon.py:425-438)."""
    from .simu import circular_trajectory_data
    h = centered_image_header(pshape, shape, dtype=dtype)
    h.update({"n_images": n_images, "radius": radius, "min_lon": min_lon, "max_lon": max_lon})
    data = circular_trajectory_data(**h)
    data[:] = fill
    out = data.astype(dtype)
    out.header = data.header
    return out


def dataarray_from_header(header):
    """Zero data stack of the shape/dtype a list of view headers describes."""
    h0 = header[0]
    shape = [int(h0["NAXIS%d" % (i + 1)]) for i in range(int(h0["NAXIS"]))] + [len(header)]
    return InfoArray(shape=shape, header=header, dtype=dtype_from_bitpix(h0["BITPIX"]))


def fov(obj, radius):
    """Half field of view (radians) that encloses a cube seen from ``radius``."""
    h = obj.header if hasattr(obj, "header") else obj
    pshape = [h["NAXIS%d" % (i + 1)] * h["CDELT%d" % (i + 1)] for i in range(3)]
    pdiag = np.sqrt(np.sum(np.asarray(pshape) ** 2))
    return np.arctan2(pdiag, radius)


# ---------------------------------------------------------------------------
# NumPy twins of the C setup stage (tomograpy/siddon.py:531-617,652-699)

def apply_rotation(R, u2):
    u0 = np.empty(u2.shape)
    u0[..., 0] = R[0, 0] * u2[..., 0] + R[0, 1] * u2[..., 1] + R[0, 2] * u2[..., 2]
    u0[..., 1] = R[1, 0] * u2[..., 0] + R[1, 1] * u2[..., 1] + R[1, 2] * u2[..., 2]
    u0[..., 2] = R[2, 0] * u2[..., 0] + R[2, 1] * u2[..., 1] + R[2, 2] * u2[..., 2]
    return u0


def full_unit_vector(data):
    """Unit vector of every pixel ray, shape ``data.shape + (3,)`` (NumPy twin)."""
    u = np.empty(data.shape + (3,), dtype=data.dtype)
    u2 = np.empty(data.shape[:-1] + (3,))
    for i, h in enumerate(data.header):
        R = dict_to_array(h, "R")
        g = (np.arange(data.shape[0]) - h["CRPIX1"] + 1) * h["CDELT1"]
        lam = (np.arange(data.shape[1]) - h["CRPIX2"] + 1) * h["CDELT2"]
        L, G = np.meshgrid(lam, g)
        u2[..., 0] = np.cos(L) * np.cos(G)
        u2[..., 1] = np.cos(L) * np.sin(G)
        u2[..., 2] = np.sin(L)
        u[..., i, :] = apply_rotation(R, u2)
    return u


def full_intersection_parameters(data, obj, u):
    """a1/an: ray parameters of the MMIN/MMAX planes per axis (NumPy twin)."""
    mmin = dict_to_array(obj.header, "MMIN")
    mmax = dict_to_array(obj.header, "MMAX")
    a1 = np.empty(u.shape)
    an = np.empty(u.shape)
    with np.errstate(divide="ignore", invalid="ignore"):
        for t in range(data.shape[-1]):
            M = dict_to_array(data.header[t], "M")
            for i in range(3):
                a1[..., t, i] = (mmin[i] - M[i]) / u[..., t, i]
                an[..., t, i] = (mmax[i] - M[i]) / u[..., t, i]
    a1[np.isinf(a1)] = -INF
    an[np.isinf(an)] = INF
    return a1, an


def full_intersection_steps(obj, u):
    pshape = dict_to_array(obj.header, "PSHAPE")
    p = np.empty(u.shape)
    with np.errstate(divide="ignore"):
        for i in range(3):
            p[..., i] = pshape[i] / u[..., i]
    return p


def full_pabs(p):
    return np.abs(p)


def compare(a1, an):
    w = a1 < an
    imin = an.copy()
    imin[w] = a1[w]
    imax = a1.copy()
    imax[w] = an[w]
    return imin, imax


def max3(x, y, z):
    out = z.copy()
    w1 = (x > y) & (x > z)
    out[w1] = x[w1]
    w2 = (y >= x) & (y > z)
    out[w2] = y[w2]
    return out


def min3(x, y, z):
    out = z.copy()
    w1 = (x < y) & (x < z)
    out[w1] = x[w1]
    w2 = (y <= x) & (y < z)
    out[w2] = y[w2]
    return out


def full_intersect_cube(a1, an):
    imin, imax = compare(a1, an)
    amin = max3(imin[..., 0], imin[..., 1], imin[..., 2])
    amax = min3(imax[..., 0], imax[..., 1], imax[..., 2])
    return amin, amax


def intersect_cube(data, obj, u):
    """Flag the pixels whose ray intersects the cube (tomograpy/siddon.py:574-584)."""
    a1, an = full_intersection_parameters(data, obj, u)
    p = full_intersection_steps(obj, u)
    amin, amax = full_intersect_cube(a1, an)
    return amin < amax, p, a1, amin


def sign(arr):
    s = np.zeros(np.shape(arr), dtype=np.int64)
    s[np.asarray(arr) < 0] = -1
    s[np.asarray(arr) > 0] = 1
    return s


def define_unit_vector(lam, gam):
    c = np.cos(lam)
    return np.asarray([c * np.cos(gam), c * np.sin(gam), np.sin(lam)])

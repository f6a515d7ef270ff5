"""Solar tomography models on top of the GPU projector.

Restates the operator wiring of ``tomograpy/models.py`` (srt ``:19-54``,
stsrt ``:106-153``, thomson ``:190-235``) and the masks of
``tomograpy/solar.py`` (``define_data_mask`` ``:211-252``,
``distance_to_sun_center`` ``:253-292``, ``define_map_mask`` ``:295-312``)
for the GPU operators of this package.  Each model returns
``(P, D, obj_mask, data_mask)`` like the reference:

* ``P`` -- a :class:`ModelOperator`: the projector with the data mask applied
  inside the kernel (masked rays are not traced), the object mask applied as
  a restriction to the unmasked voxels (``P * Mo.T`` in the reference; here
  masked voxels are held at zero, which gives the same solution on the free
  voxels), and optional diagonal weights (Thomson: ``O * P * M``);
* ``D`` -- the smoothness priors as a list of axes for
  :class:`tomograpy_gb300.cg.NormalOperator` (``lo.diff`` along each cube
  axis, ``tomograpy/models.py:85-94``; 4-D adds the frame axis).

Time grouping for the 4-D model follows ``solar.temporal_groups_indexes``
(``tomograpy/solar.py:368-372``): a new group starts where consecutive
DATE_OBS are at least ``dt_min`` seconds apart.
"""
import datetime

import numpy as np

from . import headers as H
from . import lo_wrapper

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


# ---------------------------------------------------------------------------
# masks

def distance_to_sun_center(data):
    """Distance of every pixel to the image's Sun centre in solar radii of the
    image (tomograpy/solar.py:253-292: RSUN = atan(1/D) / CDELT pixels)."""
    n1, n2, T = data.shape
    R = np.zeros(data.shape)
    for t, h in enumerate(data.header):
        rsun1 = np.arctan(1.0 / h["D"]) / h["CDELT1"]
        rsun2 = np.arctan(1.0 / h["D"]) / h["CDELT2"]
        y = (np.arange(n1) - h["CRPIX1"]) / rsun1
        x = (np.arange(n2) - h["CRPIX2"]) / rsun2
        X, Y = np.meshgrid(x, y)
        R[..., t] = np.sqrt(X ** 2 + Y ** 2)
    return R


def define_data_mask(data, data_rmin=None, data_rmax=None, ring=None, mask_negative=False, mask_nan=True,
                     **kwargs):
    """Boolean mask of the data stack (True = pixel not traced)."""
    mask = np.zeros(data.shape, dtype=bool)
    if data_rmin is not None or data_rmax is not None or ring is not None:
        R = distance_to_sun_center(data)
        if data_rmin is not None:
            mask[R < data_rmin] = True
        if data_rmax is not None:
            mask[R > data_rmax] = True
        if ring is not None:
            mask[(ring[0] < R) & (R < ring[1])] = True
    arr = np.asarray(data)
    if mask_negative:
        mask[arr < 0.0] = True
    if mask_nan:
        mask[np.isnan(arr)] = True
    return mask


def voxel_axes(h, shape):
    """Voxel-centre coordinates of a cube header along each axis."""
    return [h["MMIN%d" % (k + 1)] + (np.arange(shape[k]) + 0.5) * h["CDELT%d" % (k + 1)] for k in range(3)]


def map_radius(h, shape):
    x, y, z = voxel_axes(h, shape)
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    return np.sqrt(X ** 2 + Y ** 2 + Z ** 2)


def define_map_mask(cube, obj_rmin=None, obj_rmax=None, obj_cylinder=None, remove_nan=False, **kwargs):
    """Boolean mask of the cube (True = voxel excluded from the unknowns)."""
    arr = np.asarray(cube)
    shape = arr.shape[:3]
    h = dict(cube.header)
    if "MMIN1" not in h:
        H.map_borders(h)
    mask = np.isnan(arr[..., 0] if arr.ndim == 4 else arr) if remove_nan else np.zeros(shape, dtype=bool)
    if obj_rmin is not None or obj_rmax is not None:
        R = map_radius(h, shape)
        if obj_rmin is not None:
            mask[R < obj_rmin] = True
        if obj_rmax is not None:
            mask[R > obj_rmax] = True
    if obj_cylinder is not None:
        x, y, _ = voxel_axes(h, shape)
        X, Y = np.meshgrid(x, y, indexing="ij")
        mask[(X ** 2 + Y ** 2 > obj_cylinder ** 2)[:, :, None].repeat(shape[2], axis=2)] = True
    return mask


# ---------------------------------------------------------------------------
# time grouping

def convert_time(s):
    s = s.rstrip("Z")
    for fmt in ("%Y-%m-%dT%H:%M:%S.%f", "%Y-%m-%dT%H:%M:%S"):
        try:
            return datetime.datetime.strptime(s, fmt).replace(tzinfo=datetime.timezone.utc).timestamp()
        except ValueError:
            pass
    raise ValueError("cannot parse DATE_OBS %r" % s)


def temporal_frames(headers, dt_min):
    """Frame index of every view: a new frame starts where consecutive
    DATE_OBS differ by at least ``dt_min`` seconds."""
    times = np.array([convert_time(h["DATE_OBS"]) for h in headers])
    new = np.concatenate([[0], (np.diff(times) >= dt_min).astype(int)])
    return np.cumsum(new)


# ---------------------------------------------------------------------------
# Thomson scattering weights (tomograpy/models.py:223-309)

def _pb_thomson_coef(omega):
    sino = np.sin(omega)
    sino2 = sino ** 2
    coso = np.cos(omega)
    coso2 = coso ** 2
    with np.errstate(divide="ignore", invalid="ignore"):
        lno = np.log((1.0 + sino) / coso) * (coso2 / sino)
    C1 = coso * sino2
    C2 = -(1.0 / 8.0) * (1.0 - 3.0 * sino2 - (1.0 + 3.0 * sino2) * lno)
    return C1, C2


def pb_data_coef(data):
    """Squared impact parameter of every pixel ray (floored at 1 radius)."""
    n1, n2, T = data.shape
    coefs = np.zeros(data.shape)
    for t, h in enumerate(data.header):
        a = (np.arange(n1) - h["CRPIX1"] + 1) * h["CDELT1"] + h.get("CRVAL1", 0.0)
        b = (np.arange(n2) - h["CRPIX2"] + 1) * h["CDELT2"] + h.get("CRVAL2", 0.0)
        A, B = np.meshgrid(a, b, indexing="ij")
        d = h.get("D", np.sqrt(h["M1"] ** 2 + h["M2"] ** 2 + h["M3"] ** 2))
        rho = d * np.sin(np.arccos(np.cos(A) * np.cos(B)))
        rho[rho < 1.0] = 1.0
        coefs[..., t] = rho ** 2
    return coefs


def pb_map_coef(h, shape, u=0.5, sigma=1.0):
    """Billings polarised-brightness weight of every voxel (0 where undefined)."""
    R = map_radius(h, shape)
    with np.errstate(divide="ignore", invalid="ignore"):
        omega = np.arcsin(1.0 / R)
        C1, C2 = _pb_thomson_coef(omega)
        coefs = ((1 - u) * C1 + u * C2) / (R ** 4)
    coefs[~np.isfinite(coefs)] = 0.0
    return coefs * np.pi * sigma / 2.0


# ---------------------------------------------------------------------------
# operators

class ModelOperator:
    """y = O . P . (M * keep) x with P the GPU projector (data mask inside),
    keep = 1 - object mask, M / O optional voxel / pixel weights."""

    def __init__(self, P, obj_mask=None, map_weights=None, data_weights=None):
        self.P = P
        dev = P.device
        dt = P.tdtype
        w = None
        if obj_mask is not None:
            keep = 1.0 - np.asarray(obj_mask, dtype=np.float64)
            if P.four_d and keep.ndim == 3:
                keep = np.repeat(keep[..., None], P.cube_shape[3], axis=3)
            w = keep
        if map_weights is not None:
            m = np.asarray(map_weights, dtype=np.float64)
            if P.four_d and m.ndim == 3:
                m = np.repeat(m[..., None], P.cube_shape[3], axis=3)
            w = m if w is None else w * m
        self.map_w = None if w is None else torch.from_numpy(w.astype(np.float32)).to(dev).to(dt)
        self.data_w = None if data_weights is None else torch.from_numpy(
            np.asarray(data_weights, dtype=np.float32)).to(dev).to(dt)
        self.cube_shape = P.cube_shape
        self.data_shape = P.data_shape
        self.four_d = P.four_d
        self.device = dev
        self.tdtype = dt

    def project(self, x, out=None):
        xd = self.P._dev(x, self.cube_shape)
        if self.map_w is not None:
            xd = xd * self.map_w
        y = self.P.project(xd)
        if self.data_w is not None:
            y = y * self.data_w
        return self.P._out(y, out)

    def backproject(self, y, out=None):
        yd = self.P._dev(y, self.data_shape)
        if self.data_w is not None:
            yd = yd * self.data_w
        x = self.P.backproject(yd)
        if self.map_w is not None:
            x = x * self.map_w
        return self.P._out(x, out)


def smoothness_prior(ndim):
    """Axes of the finite-difference priors (lo.diff along every axis)."""
    return list(range(ndim))


def srt(data, cube, **kwargs):
    """Solar rotational tomography: P with obstacle='sun' and the data mask,
    object mask by obj_rmin / obj_rmax, smoothness priors on the 3 axes."""
    data_mask = define_data_mask(data, **kwargs)
    P = lo_wrapper.siddon_lo(data.header, cube.header, mask=data_mask, obstacle="sun",
                             dtype=np.dtype(getattr(data, "dtype", np.float32)))
    obj_mask = _object_mask(cube, **kwargs)
    return ModelOperator(P, obj_mask=obj_mask), smoothness_prior(3), obj_mask, data_mask


def stsrt(data, cube, dt_min=None, frames=None, **kwargs):
    """Smooth temporal SRT: a 4-D cube with one frame per time group (views
    sorted by DATE_OBS), temporal smoothness on the frame axis."""
    data_mask = define_data_mask(data, **kwargs)
    if frames is None:
        if dt_min is None:
            times = [convert_time(h["DATE_OBS"]) for h in data.header]
            dt_min = (np.max(np.diff(times)) + 1) if len(times) > 1 else 1.0
        frames = temporal_frames(data.header, dt_min)
    frames = np.asarray(frames)
    n_frames = int(frames.max()) + 1
    ch = dict(cube.header)
    shape = tuple(int(v) for v in np.asarray(cube).shape[:3]) + (n_frames,)
    P = lo_wrapper.Siddon(data.header, ch, mask=data_mask, obstacle="sun", frames=frames, cube_shape=shape,
                          dtype=np.dtype(getattr(data, "dtype", np.float32)))
    obj_mask = _object_mask(cube, **kwargs)
    return ModelOperator(P, obj_mask=obj_mask), smoothness_prior(4), obj_mask, data_mask


def thomson(data, cube, u=0.5, **kwargs):
    """Thomson-scattering (polarised brightness) model O . P . M."""
    data_mask = define_data_mask(data, **kwargs)
    P = lo_wrapper.siddon_lo(data.header, cube.header, mask=data_mask, obstacle="sun",
                             dtype=np.dtype(getattr(data, "dtype", np.float32)))
    h = dict(cube.header)
    if "MMIN1" not in h:
        H.map_borders(h)
    shape = np.asarray(cube).shape[:3]
    M = pb_map_coef(h, shape, u)
    O = pb_data_coef(data)
    kwargs["remove_nan"] = True
    obj_mask = _object_mask(cube, **kwargs)
    return ModelOperator(P, obj_mask=obj_mask, map_weights=M, data_weights=O), smoothness_prior(3), obj_mask, \
        data_mask


def _object_mask(cube, obj_rmin=None, obj_rmax=None, obj_cylinder=None, remove_nan=False, **kwargs):
    if obj_rmin is None and obj_rmax is None and obj_cylinder is None and not remove_nan:
        return None
    return define_map_mask(cube, obj_rmin=obj_rmin, obj_rmax=obj_rmax, obj_cylinder=obj_cylinder,
                           remove_nan=remove_nan)

"""Shared helpers of the test-suite: golden fixtures, header rebuilding, error
metrics and the degenerate-ray classification used by the parity tests.

Tolerances (float32 GPU path against the float64 reference / oracle):

* images: per-pixel max relative error <= 1e-5 over pixels whose reference
  value is >= 1e-3 of the image maximum and whose ray is not degenerate, and
  normwise error max|dy| / max|y| <= 1e-5 over all non-degenerate pixels;
* backprojected cubes: per-voxel max relative error <= 1e-4 over voxels >= 1e-2
  of the cube maximum, normwise <= 1e-4 (degenerate rays masked out of both
  sides).  A voxel below 1% of the maximum is made of a few short corner
  segments; a float32 segment length carries an absolute error of about one
  float32 ulp of the ray parameter (~5e-7 radii at the far side of a 3-radii
  cube), which is not small relative to such a voxel.  Sparse backprojections
  (a few views) are checked per voxel only where a voxel holds at least a
  quarter of one full-weight voxel chord (``cube_errors``);
* adjoint: |<Px, y> - <x, P^T y>| / |<Px, y>| <= 1e-5.

A ray is *degenerate* when a component of its direction is non-zero but
smaller than 1e-12: it runs within 1e-12 rad of a plane family, so which side
of a voxel plane it is traced on depends on the last bits of the set-up
arithmetic (in the reference too).
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "reference_siddon.npz")

VIEW_KEYS = ["CRPIX1", "CRPIX2", "CDELT1", "CDELT2", "CRVAL1", "CRVAL2", "M1", "M2", "M3"] + \
    ["R%d_%d" % (i, j) for i in (1, 2, 3) for j in (1, 2, 3)]
CUBE_KEYS = ["CDELT1", "CDELT2", "CDELT3", "PSHAPE1", "PSHAPE2", "PSHAPE3",
             "MMIN1", "MMIN2", "MMIN3", "MMAX1", "MMAX2", "MMAX3"]

IMG_TOL = 1e-5
CUBE_TOL = 1e-4
CUBE_SIG = 1e-2
ADJ_TOL = 1e-5

_golden = None


def golden():
    global _golden
    if _golden is None:
        _golden = dict(np.load(GOLDEN))
    return _golden


def views_from_array(a, n1, n2):
    hdrs = []
    for row in a:
        h = {k: float(v) for k, v in zip(VIEW_KEYS, row)}
        h.update({"NAXIS": 2, "NAXIS1": n1, "NAXIS2": n2, "BITPIX": -64})
        hdrs.append(h)
    return hdrs


def cube_from_array(a, shape):
    h = {k: float(v) for k, v in zip(CUBE_KEYS, a)}
    h.update({"NAXIS": len(shape), "BITPIX": -64})
    for i, n in enumerate(shape):
        h["NAXIS%d" % (i + 1)] = int(n)
    return h


def golden_case(prefix, n1, n2, cube_shape):
    g = golden()
    return views_from_array(g[prefix + "_views"], n1, n2), cube_from_array(g[prefix + "_cube_hdr"], cube_shape)


def unit_vectors(views, n1, n2):
    """float64 ray directions (N1, N2, T, 3), reference formula in NumPy."""
    T = len(views)
    u = np.empty((n1, n2, T, 3))
    for t, h in enumerate(views):
        R = np.array([[h["R%d_%d" % (a, b)] for b in (1, 2, 3)] for a in (1, 2, 3)])
        g = (np.arange(n1) - h["CRPIX1"] + 1) * h["CDELT1"] + h["CRVAL1"]
        lam = (np.arange(n2) - h["CRPIX2"] + 1) * h["CDELT2"] + h["CRVAL2"]
        L, G = np.meshgrid(lam, g)
        u2 = np.stack([np.cos(L) * np.cos(G), np.cos(L) * np.sin(G), np.sin(L)], axis=-1)
        u[:, :, t, :] = u2 @ R.T
    return u


def degenerate_rays(views, n1, n2):
    u = unit_vectors(views, n1, n2)
    a = np.abs(u)
    return np.any((a > 0) & (a < 1e-12), axis=-1)


def image_errors(y, ref, exclude=None, sig=1e-3):
    """(per-element max relative error over elements >= sig * max|ref|,
    normwise max|y - ref| / max|ref|).  Images use sig = 1e-3, cubes
    CUBE_SIG."""
    y = np.asarray(y, np.float64)
    ref = np.asarray(ref, np.float64)
    keep = np.ones(ref.shape, bool) if exclude is None else ~exclude
    scale = np.abs(ref[keep]).max() if keep.any() else 0.0
    if scale == 0:
        return 0.0, float(np.abs(y[keep]).max()) if keep.any() else 0.0
    d = np.abs(y - ref)
    norm = d[keep].max() / scale
    big = keep & (np.abs(ref) >= sig * scale)
    rel = (d[big] / np.abs(ref[big])).max() if big.any() else 0.0
    return float(rel), float(norm)


def cube_errors(c, ref, y_max, cdelt):
    """(per-voxel max relative error, normwise error) of a backprojected cube.

    The per-voxel error is taken over voxels whose reference value is at
    least CUBE_SIG of the cube's maximum AND at least a quarter of one voxel
    chord at full weight (cdelt * y_max / 4).  The second floor matters only
    for sparse backprojections (a few views): a voxel below it holds only
    short corner segments, whose float32 lengths carry an absolute error of
    a few 1e-7 radii (the rounding of the crossing parameters), which no
    float32 walk can make small relative to such a voxel.  With many views
    (the workloads) the first floor is the larger one."""
    c = np.asarray(c, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = np.abs(ref).max()
    if scale == 0:
        return 0.0, float(np.abs(c).max())
    d = np.abs(c - ref)
    norm = d.max() / scale
    big = np.abs(ref) >= max(CUBE_SIG * scale, 0.25 * cdelt * y_max)
    rel = (d[big] / np.abs(ref[big])).max() if big.any() else 0.0
    return float(rel), float(norm)


def worst_element(y, ref, exclude=None, sig=1e-3):
    """Where the per-element relative error of image_errors is largest:
    (index, reference value / max |ref|, absolute error)."""
    y = np.asarray(y, np.float64)
    ref = np.asarray(ref, np.float64)
    keep = np.ones(ref.shape, bool) if exclude is None else ~exclude
    scale = np.abs(ref[keep]).max()
    big = keep & (np.abs(ref) >= sig * scale)
    r = np.where(big, np.abs(y - ref) / np.maximum(np.abs(ref), 1e-300), 0.0)
    k = np.unravel_index(np.argmax(r), r.shape)
    return [int(v) for v in k], float(ref[k] / scale), float(abs(y[k] - ref[k]))


def rel_dot(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


def record(name, **values):
    """Append one measured-error record (JSON line) to the file named by the
    TG_PARITY_REPORT environment variable, when it is set; the parity tests
    call it so that a run can collect the errors it measured."""
    path = os.environ.get("TG_PARITY_REPORT")
    if not path:
        return
    import json
    with open(path, "a") as f:
        f.write(json.dumps(dict(test=name, **values)) + "\n")

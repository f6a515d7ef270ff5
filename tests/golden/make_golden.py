"""Generate golden fixtures by running the reference's own compiled Siddon kernel.

Run in a checkout that has the reference available (``oracle/build_ref.py``
compiles ``tomograpy/C_siddon.c.template`` into ``oracle/_ref/``)::

    python tests/golden/make_golden.py

It writes ``tests/golden/*.npz``: seeded inputs (headers packed as arrays,
cubes, data, masks) and the reference's outputs for them.  The tests use these
files to pin the oracle (``tests/test_oracle_golden.py``) and the CUDA path
(``tests/test_gpu_parity.py``) without needing the reference at run time.

Cases (all float64 unless stated):

* ``small24``  -- the plain-method geometry at reduced size: 24^3 cube spanning
  [-1.5, 1.5], 13 views of 40^2 over 0..pi (so lon = 0 and lon = pi, the
  degenerate views, are included), d = 215, shell + blob phantom; pj / bpj
  with obstacle sun and none, with and without a data mask, plus the
  reference's float32 path for pj (to record its own float32 error);
* ``frames12`` -- pjt / bpjt on a 12^3 x 7-frame cube, 7 views of 24^2;
* ``cases`` -- the reference test-suite geometry (``tests/test_cases.py``): a
  16^3 and a 1^3 cube spanning 3 radii, 32^2 images whose field of view is
  ``fov(obj, 200)``, 17 views over 0..2 pi at radius 200; projection of ones,
  backprojection of ones;
* ``diag``  -- the reference's unit vectors and intersection parameters
  (``full_unit_vector`` / ``full_intersection_parameters``) for 5 views.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402
from tomograpy_gb300 import headers as H  # noqa: E402
from tomograpy_gb300 import simu, synthetic  # noqa: E402
from tomograpy_gb300.infoarray import InfoArray  # noqa: E402

VIEW_KEYS = ["CRPIX1", "CRPIX2", "CDELT1", "CDELT2", "CRVAL1", "CRVAL2", "M1", "M2", "M3"] + \
    ["R%d_%d" % (i, j) for i in (1, 2, 3) for j in (1, 2, 3)]
CUBE_KEYS = ["CDELT1", "CDELT2", "CDELT3", "PSHAPE1", "PSHAPE2", "PSHAPE3",
             "MMIN1", "MMIN2", "MMIN3", "MMAX1", "MMAX2", "MMAX3"]


def pack_views(hdrs):
    return np.array([[float(h[k]) for k in VIEW_KEYS] for h in hdrs])


def pack_cube(h):
    return np.array([float(h[k]) for k in CUBE_KEYS])


def ref_run(data, cube, mask, obstacle, mode, ctype="double"):
    mod = build_ref.load(ctype, obstacle if obstacle else "none", mode)
    # single thread: the reference's atomic backprojection sums in a fixed order
    mod.conic_full_projector(data, cube, mask, 1)


def small24(out):
    n, T, N, d = 24, 13, 40, 215.0
    ch = synthetic.cube_header(n, dtype=np.float64)
    vh = synthetic.view_headers(T, N, d=d, lon_range=(0.0, np.pi), dtype=np.float64)
    x = synthetic.phantom(ch, seed=3, dtype=np.float64)
    rng = np.random.default_rng(11)
    y = rng.random((N, N, T))
    mask = (rng.random((N, N, T)) < 0.1).astype(np.float64)
    out["small24_views"] = pack_views(vh)
    out["small24_cube_hdr"] = pack_cube(ch)
    out["small24_x"] = x
    out["small24_y"] = y
    out["small24_mask"] = mask
    for obstacle in ("sun", "none"):
        for use_mask in (False, True):
            m = mask if use_mask else np.zeros((N, N, T))
            tag = "%s_%s" % (obstacle, "mask" if use_mask else "nomask")
            data = InfoArray(data=np.zeros((N, N, T)), header=[dict(h) for h in vh])
            cube = InfoArray(data=x.copy(), header=dict(ch))
            ref_run(data, cube, m, obstacle, "pj")
            out["small24_pj_" + tag] = np.asarray(data)
            data = InfoArray(data=y.copy(), header=[dict(h) for h in vh])
            cube = InfoArray(data=np.zeros((n, n, n)), header=dict(ch))
            ref_run(data, cube, m, obstacle, "bpj")
            out["small24_bpj_" + tag] = np.asarray(cube)
    # the reference's own float32 path on the same inputs
    data = InfoArray(data=np.zeros((N, N, T), np.float32), header=[dict(h) for h in vh])
    cube = InfoArray(data=x.astype(np.float32), header=dict(ch))
    ref_run(data, cube, np.zeros((N, N, T), np.float32), "sun", "pj", ctype="float")
    out["small24_pj_sun_nomask_float32ref"] = np.asarray(data)


def frames12(out):
    """4-D variants on a smaller geometry: 12^3 x 7 frames, 7 views of 24^2."""
    n, T, N, d = 12, 7, 24, 215.0
    ch = synthetic.cube_header(n, dtype=np.float64)
    vh = synthetic.view_headers(T, N, d=d, lon_range=(0.0, np.pi), dtype=np.float64)
    x = synthetic.phantom(ch, seed=5, dtype=np.float64)
    x4 = np.stack([x * (1.0 + 0.1 * t) for t in range(T)], axis=-1)
    y = np.random.default_rng(12).random((N, N, T))
    out["frames12_views"] = pack_views(vh)
    out["frames12_cube_hdr"] = pack_cube(ch)
    out["frames12_x4"] = x4
    out["frames12_y"] = y
    for obstacle in ("sun", "none"):
        data = InfoArray(data=np.zeros((N, N, T)), header=[dict(h) for h in vh])
        cube = InfoArray(data=x4.copy(), header=dict(ch))
        ref_run(data, cube, np.zeros((N, N, T)), obstacle, "pjt")
        out["frames12_pjt_" + obstacle] = np.asarray(data)
        data = InfoArray(data=y.copy(), header=[dict(h) for h in vh])
        cube = InfoArray(data=np.zeros((n, n, n, T)), header=dict(ch))
        ref_run(data, cube, np.zeros((N, N, T)), obstacle, "bpjt")
        out["frames12_bpjt_" + obstacle] = np.asarray(cube)


def test_case_geometry(n_cube, n_images, n_pix=32):
    obj_h = H.centered_cubic_map_header(3.0, 16)
    im_ps = H.fov(obj_h, 200.0)
    ch = H.centered_cubic_map_header(3.0, n_cube)
    ih = H.centered_image_header(im_ps, n_pix)
    ih.update({"radius": 200.0, "max_lon": 2 * np.pi, "n_images": n_images})
    data = simu.circular_trajectory_data(**ih)
    return ch, data


def cases(out):
    for n_cube in (16, 1):
        ch, data = test_case_geometry(n_cube, 17)
        key = "cases%d" % n_cube
        out[key + "_views"] = pack_views(data.header)
        out[key + "_cube_hdr"] = pack_cube(ch)
        cube = InfoArray(data=np.ones((n_cube,) * 3), header=dict(ch))
        d = data.copy()
        d[:] = 0
        ref_run(d, cube, np.zeros(d.shape), None, "pj")
        out[key + "_pj_ones"] = np.asarray(d)
        d = data.copy()
        d[:] = 1
        cube = InfoArray(data=np.zeros((n_cube,) * 3), header=dict(ch))
        ref_run(d, cube, np.zeros(d.shape), None, "bpj")
        out[key + "_bpj_ones"] = np.asarray(cube)


def diag(out):
    ch, data = test_case_geometry(16, 5)
    out["diag_views"] = pack_views(data.header)
    out["diag_cube_hdr"] = pack_cube(ch)
    mod = build_ref.load("double", "none", "pj")
    u = np.zeros(data.shape + (3,))
    mod.full_unit_vector(data, u)
    a1 = np.zeros(u.shape)
    an = np.zeros(u.shape)
    cube = InfoArray(data=np.zeros((16, 16, 16)), header=dict(ch))
    mod.full_intersection_parameters(data, cube, u, a1, an)
    out["diag_u"] = u
    out["diag_a1"] = a1
    out["diag_an"] = an


def main():
    build_ref.build(quiet=True)
    out = {}
    small24(out)
    frames12(out)
    cases(out)
    diag(out)
    path = os.path.join(HERE, "reference_siddon.npz")
    np.savez_compressed(path, **out)
    print("wrote %s (%d arrays, %.0f KB)" % (path, len(out), os.path.getsize(path) / 1024))


if __name__ == "__main__":
    main()

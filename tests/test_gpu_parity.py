"""GPU parity: the CUDA path (through the C ABI) against the reference's golden
vectors and the oracle.  Tolerances are defined in tests/helpers.py:
float32 images <= 1e-5 (per-pixel relative on significant pixels, and
normwise), float32 cubes <= 1e-4, adjoint <= 1e-5, float64 path <= 1e-12
(normwise) against the reference's own double-precision output."""
import numpy as np
import pytest

import oracle
import tomograpy_gb300 as tg
from helpers import (ADJ_TOL, CUBE_SIG, CUBE_TOL, IMG_TOL, degenerate_rays, golden, golden_case, image_errors, record,
                     rel_dot)
from tomograpy_gb300 import synthetic
from tomograpy_gb300.infoarray import InfoArray

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def _hdrs(vh):
    return [dict(h) for h in vh]


# --------------------------------------------------------------------------
# against the reference's golden outputs

@pytest.mark.parametrize("obstacle", ["sun", "none"])
@pytest.mark.parametrize("use_mask", [False, True])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_golden_projection(obstacle, use_mask, dtype):
    g = golden()
    vh, ch = golden_case("small24", 40, 40, (24, 24, 24))
    degen = degenerate_rays(vh, 40, 40)
    assert degen.any()  # the lon = pi view is in this geometry
    data = InfoArray(shape=(40, 40, 13), header=_hdrs(vh), dtype=dtype)
    cube = InfoArray(data=g["small24_x"].astype(dtype), header=dict(ch))
    mask = g["small24_mask"] if use_mask else None
    tg.projector(data, cube, mask=mask, obstacle=obstacle)
    ref = g["small24_pj_%s_%s" % (obstacle, "mask" if use_mask else "nomask")]
    if dtype == np.float32:
        # the reference's float64 output on the float32-rounded cube is the target
        r = InfoArray(shape=(40, 40, 13), header=_hdrs(vh))
        oracle.projector(r, InfoArray(data=g["small24_x"].astype(np.float32).astype(np.float64), header=dict(ch)),
                         mask=mask, obstacle=obstacle)
        rel, norm = image_errors(data, r, exclude=degen)
        assert rel <= IMG_TOL and norm <= IMG_TOL, (rel, norm)
        rel0, norm0 = image_errors(data, ref, exclude=degen)
        assert norm0 <= IMG_TOL  # includes the float32 rounding of the phantom itself
    else:
        rel, norm = image_errors(data, ref, exclude=degen)
        assert norm <= 1e-12 and rel <= 1e-11, (rel, norm)


@pytest.mark.parametrize("obstacle", ["sun", "none"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_golden_backprojection(obstacle, dtype):
    g = golden()
    vh, ch = golden_case("small24", 40, 40, (24, 24, 24))
    degen = degenerate_rays(vh, 40, 40)
    y = g["small24_y"].copy()
    y[degen] = 0.0  # degenerate rays are compared separately
    cube = InfoArray(shape=(24, 24, 24), header=dict(ch), dtype=dtype)
    tg.backprojector(InfoArray(data=y.astype(dtype), header=_hdrs(vh)), cube, obstacle=obstacle)
    ref = InfoArray(shape=(24, 24, 24), header=dict(ch))
    oracle.backprojector(InfoArray(data=y.astype(dtype).astype(np.float64), header=_hdrs(vh)), ref,
                         obstacle=obstacle)
    rel, norm = image_errors(cube, ref, sig=CUBE_SIG)
    tol = CUBE_TOL if dtype == np.float32 else 1e-12
    assert rel <= tol and norm <= tol, (rel, norm)


def _analytic_chords(views, ch, n1, n2):
    """Exact chord length of every ray through the cube (no obstacle), with
    direction components below 1e-14 taken as zero."""
    from helpers import unit_vectors
    u = unit_vectors(views, n1, n2)
    u[np.abs(u) < 1e-14] = 0.0
    lo = np.full(u.shape[:3], -np.inf)
    hi = np.full(u.shape[:3], np.inf)
    for t, h in enumerate(views):
        M = [h["M1"], h["M2"], h["M3"]]
        for k in range(3):
            uk = u[:, :, t, k]
            mn, mx = ch["MMIN%d" % (k + 1)], ch["MMAX%d" % (k + 1)]
            with np.errstate(divide="ignore", invalid="ignore"):
                a = (mn - M[k]) / uk
                b = (mx - M[k]) / uk
            inside = (M[k] > mn) & (M[k] < mx)
            a = np.where(uk == 0, -np.inf if inside else np.inf, a)
            b = np.where(uk == 0, np.inf if inside else -np.inf, b)
            lo[:, :, t] = np.maximum(lo[:, :, t], np.minimum(a, b))
            hi[:, :, t] = np.minimum(hi[:, :, t], np.maximum(a, b))
    return np.clip(hi - lo, 0, None)


def test_degenerate_rays_trace_their_chord():
    """Rays within 1e-12 rad of a voxel-plane family (the central rows of the
    lon = pi/2 and lon = pi views) are traced as lying in the plane.  The
    reference's double path returns rounding noise there (its plane distance
    next*p + a1 - amin cancels catastrophically, giving 0 or negative segment
    lengths), so those rays are checked against the exact chord instead."""
    vh, ch = golden_case("small24", 40, 40, (24, 24, 24))
    degen = degenerate_rays(vh, 40, 40)
    data = InfoArray(shape=(40, 40, 13), header=_hdrs(vh), dtype=np.float32)
    tg.projector(data, InfoArray(data=np.ones((24, 24, 24), np.float32), header=dict(ch)))
    chord = _analytic_chords(vh, ch, 40, 40)
    d = np.asarray(data, np.float64)
    np.testing.assert_allclose(d[degen], chord[degen], rtol=IMG_TOL)
    np.testing.assert_allclose(d[~degen], chord[~degen], rtol=IMG_TOL, atol=1e-6)


@pytest.mark.parametrize("obstacle", ["sun", "none"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_golden_time_dependent(obstacle, dtype):
    g = golden()
    vh, ch = golden_case("frames12", 24, 24, (12, 12, 12, 7))
    degen = degenerate_rays(vh, 24, 24)
    data = InfoArray(shape=(24, 24, 7), header=_hdrs(vh), dtype=dtype)
    cube = InfoArray(data=g["frames12_x4"].astype(dtype), header=dict(ch))
    tg.projector4d(data, cube, obstacle=obstacle)
    rel, norm = image_errors(data, g["frames12_pjt_" + obstacle], exclude=degen)
    tol = 2e-6 if dtype == np.float32 else 1e-12  # includes the float32 rounding of the cube
    assert norm <= tol, (rel, norm)
    y = g["frames12_y"].copy()
    y[degen] = 0
    cube = InfoArray(shape=(12, 12, 12, 7), header=dict(ch), dtype=dtype)
    tg.backprojector4d(InfoArray(data=y.astype(dtype), header=_hdrs(vh)), cube, obstacle=obstacle)
    ref = InfoArray(shape=(12, 12, 12, 7), header=dict(ch))
    oracle.backprojector4d(InfoArray(data=y.astype(dtype).astype(np.float64), header=_hdrs(vh)), ref,
                           obstacle=obstacle)
    rel, norm = image_errors(cube, ref, sig=CUBE_SIG)
    assert norm <= (CUBE_TOL if dtype == np.float32 else 1e-12), (rel, norm)


@pytest.mark.parametrize("n_cube", [16, 1])
def test_golden_reference_test_geometry(n_cube):
    """Projection of ones / backprojection of ones on the reference test
    geometry (17 views over 2 pi: axis-aligned and diagonal rays)."""
    g = golden()
    key = "cases%d" % n_cube
    vh, ch = golden_case(key, 32, 32, (n_cube,) * 3)
    degen = degenerate_rays(vh, 32, 32)
    for dtype in (np.float32, np.float64):
        data = InfoArray(shape=(32, 32, 17), header=_hdrs(vh), dtype=dtype)
        tg.projector(data, InfoArray(data=np.ones((n_cube,) * 3, dtype), header=dict(ch)))
        ref = g[key + "_pj_ones"]
        # test_special_cases: non-zero <=> the ray meets the cube
        np.testing.assert_array_equal((np.asarray(data) != 0)[~degen], (ref != 0)[~degen])
        rel, norm = image_errors(data, ref, exclude=degen)
        assert norm <= (IMG_TOL if dtype == np.float32 else 1e-12)


# --------------------------------------------------------------------------
# the reference's own property tests (tests/test_siddon.py), on the GPU

def _test_case_data(n_images=17, n_pix=32, dtype=np.float64):
    obj_h = tg.centered_cubic_map_header(3.0, 16)
    ih = tg.centered_image_header(tg.fov(obj_h, 200.0), n_pix)
    ih.update({"radius": 200.0, "max_lon": 2 * np.pi, "n_images": n_images, "dtype": dtype})
    return tg.simu.circular_trajectory_data(**ih)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_full_versus_image(dtype):
    obj = tg.simu.object_from_header(tg.centered_cubic_map_header(3.0, 16), dtype=dtype)
    obj[:] = np.random.default_rng(0).random(obj.shape)
    d1 = _test_case_data(dtype=dtype)
    d2 = _test_case_data(dtype=dtype)
    tg.projector(d1, obj)
    for t in range(d2.shape[-1]):
        tg.conic_image_projector(d2, obj, t)
    np.testing.assert_array_equal(np.asarray(d1), np.asarray(d2))


def test_parallel_ray():
    for n in (1, 16):
        data = tg.simu.circular_trajectory_data(**dict(tg.centered_image_header(0.01, 1), n_images=1,
                                                       radius=200.0))
        data.header[0]["CRPIX1"] = 1.0
        data.header[0]["CRPIX2"] = 1.0
        obj = tg.InfoArray(shape=(n, n, n), header=tg.centered_cubic_map_header(3.0, n))
        data[:] = 1.0
        tg.backprojector(data, obj)
        assert np.sum(obj) == obj.header["PSHAPE1"]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_sum_bpj(dtype):
    data = _test_case_data(n_images=9, dtype=dtype)
    data[:] = 1.0
    obj16 = tg.InfoArray(shape=(16, 16, 16), header=tg.centered_cubic_map_header(3.0, 16), dtype=dtype)
    obj1 = tg.InfoArray(shape=(1, 1, 1), header=tg.centered_cubic_map_header(3.0, 1), dtype=dtype)
    tg.backprojector(data, obj16)
    tg.backprojector(data, obj1)
    # float32: the single voxel sums 9216 chords by float32 atomics
    tol = CUBE_TOL if dtype == np.float32 else 1e-13
    np.testing.assert_allclose(np.sum(obj16, dtype=np.float64), float(obj1[0, 0, 0]), rtol=tol)
    if dtype == np.float32:
        # exact (fixed-point) accumulation: partition of unity to float32 segment precision
        d16 = tg.InfoArray(shape=(16, 16, 16), header=tg.centered_cubic_map_header(3.0, 16), dtype=dtype)
        d1 = tg.InfoArray(shape=(1, 1, 1), header=tg.centered_cubic_map_header(3.0, 1), dtype=dtype)
        tg.backprojector(data, d16, deterministic=True)
        tg.backprojector(data, d1, deterministic=True)
        np.testing.assert_allclose(np.sum(d16, dtype=np.float64), float(d1[0, 0, 0]), rtol=1e-6)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_scale_factor(dtype):
    obj = tg.simu.object_from_header(tg.centered_cubic_map_header(3.0, 16), dtype=dtype, fill=1.0)
    obj10 = tg.simu.object_from_header(tg.centered_cubic_map_header(3.0, 16), dtype=dtype, fill=10.0)
    d1 = _test_case_data(dtype=dtype)
    d10 = _test_case_data(dtype=dtype)
    tg.projector(d1, obj)
    tg.projector(d10, obj10)
    np.testing.assert_allclose(10 * np.asarray(d1), np.asarray(d10), rtol=1e-6 if dtype == np.float32 else 1e-14)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_unit_vectors_and_intersections(dtype):
    g = golden()
    vh, ch = golden_case("diag", 32, 32, (16, 16, 16))
    data = InfoArray(shape=(32, 32, 5), header=_hdrs(vh), dtype=dtype)
    u = tg.C_full_unit_vector(data)
    if dtype == np.float64:
        np.testing.assert_allclose(u, g["diag_u"], rtol=0, atol=1e-15)
        a1, an = tg.C_full_intersection_parameters(data, InfoArray(shape=(16, 16, 16), header=dict(ch)), g["diag_u"])
        np.testing.assert_allclose(a1, g["diag_a1"], rtol=1e-15)
        np.testing.assert_allclose(an, g["diag_an"], rtol=1e-15)
    else:
        np.testing.assert_allclose(u, g["diag_u"], rtol=0, atol=3e-7)


# --------------------------------------------------------------------------
# oracle comparisons on larger / generic geometries

def _geometry(n, T, N, lons, d=215.0, lat=0.0, rol=0.0, crval=(0.0, 0.0), dtype=np.float32, shape=None, pshape=3.0):
    cdelt = 2.0 * np.arctan(1.6 / d) / N
    hdrs = []
    for k, lon in enumerate(lons):
        h = tg.centered_image_header(cdelt * N, N, dtype=dtype)
        la = lat[k] if np.ndim(lat) else lat
        ro = rol[k] if np.ndim(rol) else rol
        h.update({"LON": float(lon), "LAT": float(la), "ROL": float(ro), "CRVAL1": crval[0], "CRVAL2": crval[1]})
        h["M1"] = d * np.cos(la) * np.cos(lon)
        h["M2"] = d * np.cos(la) * np.sin(lon)
        h["M3"] = d * np.sin(la)
        tg.header_rotation_matrix(h)
        hdrs.append(h)
    ch = tg.centered_cubic_map_header(pshape, n if shape is None else shape)
    return ch, hdrs


def _compare_pj_bpj(ch, vh, x, y, obstacle, shape_img, name="case"):
    n1, n2, T = shape_img
    degen = degenerate_rays(vh, n1, n2)
    data = InfoArray(shape=shape_img, header=_hdrs(vh), dtype=np.float32)
    tg.projector(data, InfoArray(data=x.astype(np.float32), header=dict(ch)), obstacle=obstacle)
    ref = InfoArray(shape=shape_img, header=_hdrs(vh))
    oracle.projector(ref, InfoArray(data=x.astype(np.float32).astype(np.float64), header=dict(ch)),
                     obstacle=obstacle)
    rel, norm = image_errors(data, ref, exclude=degen)
    record(name + "_pj", rel=rel, norm=norm)
    assert rel <= IMG_TOL and norm <= IMG_TOL, ("pj", rel, norm)
    yy = y.astype(np.float32).copy()
    yy[degen] = 0
    cube = InfoArray(shape=x.shape, header=dict(ch), dtype=np.float32)
    tg.backprojector(InfoArray(data=yy, header=_hdrs(vh)), cube, obstacle=obstacle)
    cref = InfoArray(shape=x.shape, header=dict(ch))
    oracle.backprojector(InfoArray(data=yy.astype(np.float64), header=_hdrs(vh)), cref, obstacle=obstacle)
    rel, norm = image_errors(cube, cref, sig=CUBE_SIG)
    record(name + "_bpj", rel=rel, norm=norm)
    assert rel <= CUBE_TOL and norm <= CUBE_TOL, ("bpj", rel, norm)


@pytest.mark.parametrize("obstacle", ["sun", None])
def test_plain64_full_size_phantom(obstacle):
    ch, vh = synthetic.make_geometry("plain64")
    x = synthetic.phantom(ch, seed=0)
    y = np.random.default_rng(1).random((128, 128, 60))
    _compare_pj_bpj(ch, vh, x, y, obstacle, (128, 128, 60), name="plain64_%s" % obstacle)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_geometry_random_cube(seed):
    rng = np.random.default_rng(seed)
    T = 7
    lons = rng.uniform(0, 2 * np.pi, T)
    lat = rng.uniform(-0.5, 0.5, T)
    rol = rng.uniform(-np.pi, np.pi, T)
    shape = (int(rng.integers(8, 40)), int(rng.integers(8, 40)), int(rng.integers(8, 40)))
    ch, vh = _geometry(None, T, 48, lons, d=float(rng.uniform(3, 230)), lat=lat, rol=rol,
                       crval=(float(rng.uniform(-1e-3, 1e-3)), float(rng.uniform(-1e-3, 1e-3))), shape=shape,
                       pshape=(3.0, 2.4, 3.3))
    for h in vh:
        h["NAXIS2"] = 40
    x = rng.random(shape)
    y = rng.random((48, 40, T))
    # non-square image: 48 x 40
    for h in vh:
        h["CRPIX2"] = 20.0
    _compare_pj_bpj(ch, vh, x, y, "sun" if seed % 2 == 0 else None, (48, 40, T), name="random%d" % seed)


def test_observer_inside_cube_and_small_cube_inside_sun():
    # observer inside the cube: the reference traces from amin < 0 (behind the observer)
    ch, vh = _geometry(None, 3, 24, [0.2, 1.5, 4.0], d=1.2, shape=(12, 12, 12))
    x = np.random.default_rng(3).random((12, 12, 12))
    _compare_pj_bpj(ch, vh, x, np.ones((24, 24, 3)), None, (24, 24, 3))
    # a cube smaller than the sun: every ray stops at its entry voxel check
    ch2, vh2 = _geometry(None, 3, 24, [0.2, 1.5, 4.0], d=10.0, shape=(8, 8, 8), pshape=1.0)
    data = InfoArray(shape=(24, 24, 3), header=_hdrs(vh2), dtype=np.float32)
    tg.projector(data, InfoArray(data=np.ones((8, 8, 8), np.float32), header=dict(ch2)), obstacle="sun")
    ref = InfoArray(shape=(24, 24, 3), header=_hdrs(vh2))
    oracle.projector(ref, InfoArray(data=np.ones((8, 8, 8)), header=dict(ch2)), obstacle="sun")
    np.testing.assert_allclose(np.asarray(data), ref, rtol=IMG_TOL, atol=1e-7)


def test_adjoint_dot_product():
    ch, vh = synthetic.make_geometry("plain64")
    rng = np.random.default_rng(5)
    x = rng.random((64, 64, 64)).astype(np.float32)
    y = rng.random((128, 128, 60)).astype(np.float32)
    px = InfoArray(shape=y.shape, header=_hdrs(vh), dtype=np.float32)
    tg.projector(px, InfoArray(data=x, header=dict(ch)), obstacle="sun")
    pty = InfoArray(shape=x.shape, header=dict(ch), dtype=np.float32)
    tg.backprojector(InfoArray(data=y, header=_hdrs(vh)), pty, obstacle="sun")
    a = float(np.dot(np.asarray(px, np.float64).ravel(), y.astype(np.float64).ravel()))
    b = float(np.dot(x.astype(np.float64).ravel(), np.asarray(pty, np.float64).ravel()))
    assert rel_dot(a, b) <= ADJ_TOL, rel_dot(a, b)


# --------------------------------------------------------------------------
# layouts, masks, determinism, errors

def test_torch_tensors_any_strides():
    import torch
    ch, vh = synthetic.make_geometry({"n": 32, "T": 6, "N": 48, "d": 215.0, "lon_range": (0.1, 2.0)})
    x = synthetic.phantom(ch, seed=2)
    dev = torch.device("cuda")
    xt = torch.from_numpy(x).to(dev)
    y_c = torch.zeros((48, 48, 6), device=dev)
    tg.projector(y_c, xt, obstacle="sun", data_header=_hdrs(vh), cube_header=dict(ch))
    # view-major storage presented as (N1, N2, T) through strides
    y_v = torch.zeros((6, 48, 48), device=dev).permute(1, 2, 0)
    tg.projector(y_v, xt, obstacle="sun", data_header=_hdrs(vh), cube_header=dict(ch))
    torch.testing.assert_close(y_c, y_v, rtol=0, atol=0)
    # frame-major cube through strides
    xf = torch.from_numpy(np.ascontiguousarray(x.transpose(2, 1, 0))).to(dev).permute(2, 1, 0)
    y_f = torch.zeros((48, 48, 6), device=dev)
    tg.projector(y_f, xf, obstacle="sun", data_header=_hdrs(vh), cube_header=dict(ch))
    torch.testing.assert_close(y_c, y_f, rtol=0, atol=0)


def test_mask_dtypes_are_read_elementwise():
    ch, vh = synthetic.make_geometry({"n": 16, "T": 4, "N": 32, "d": 215.0, "lon_range": (0.1, 2.0)})
    x = synthetic.phantom(ch, seed=4)
    m = np.random.default_rng(0).random((32, 32, 4)) < 0.3
    outs = []
    for mask in (m, m.astype(np.float64), m.astype(np.float32), m.astype(np.uint8)):
        data = InfoArray(shape=(32, 32, 4), header=_hdrs(vh), dtype=np.float32)
        tg.projector(data, InfoArray(data=x, header=dict(ch)), mask=mask, obstacle="sun")
        outs.append(np.asarray(data))
    for o in outs[1:]:
        np.testing.assert_array_equal(outs[0], o)
    assert np.all(outs[0][m] == 0) and np.any(outs[0][~m] != 0)


def test_deterministic_backprojection():
    import torch
    ch, vh = synthetic.make_geometry({"n": 48, "T": 20, "N": 96, "d": 215.0, "lon_range": (0.0, 3.0)})
    degen = degenerate_rays(vh, 96, 96)
    y = np.random.default_rng(7).random((96, 96, 20)).astype(np.float32)
    y[degen] = 0
    dev = torch.device("cuda")
    yt = torch.from_numpy(y).to(dev)
    outs = []
    for _ in range(2):
        c = torch.zeros((48, 48, 48), device=dev)
        tg.backprojector(yt, c, obstacle="sun", data_header=_hdrs(vh), cube_header=dict(ch), deterministic=True)
        outs.append(c.cpu().numpy())
    np.testing.assert_array_equal(outs[0], outs[1])
    ref = InfoArray(shape=(48, 48, 48), header=dict(ch))
    oracle.backprojector(InfoArray(data=y.astype(np.float64), header=_hdrs(vh)), ref, obstacle="sun")
    rel, norm = image_errors(outs[0], ref, sig=CUBE_SIG)
    assert rel <= CUBE_TOL and norm <= CUBE_TOL, (rel, norm)


def test_errors_like_the_reference():
    ch, vh = synthetic.make_geometry({"n": 8, "T": 2, "N": 8, "d": 215.0, "lon_range": (0.1, 2.0)})
    data = InfoArray(shape=(8, 8, 2), header=_hdrs(vh), dtype=np.float32)
    with pytest.raises(ValueError):
        tg.projector(data, InfoArray(shape=(8, 8, 8), header=dict(ch), dtype=np.float64))
    bad = InfoArray(shape=(8, 8, 2), header=tuple(_hdrs(vh)), dtype=np.float32)
    with pytest.raises(ValueError):
        tg.projector(bad, InfoArray(shape=(8, 8, 8), header=dict(ch), dtype=np.float32))
    with pytest.raises(ValueError):
        tg.projector4d(data, InfoArray(shape=(8, 8, 8, 1), header=dict(ch), dtype=np.float32))
    # headers completed in place like check_projector_inputs
    h = [dict(v) for v in vh]
    for v in h:
        for k in list(v):
            if k.startswith("R") and "_" in k:
                del v[k]
    c = dict(ch)
    for k in list(c):
        if k.startswith(("MMIN", "MMAX", "PSHAPE")):
            del c[k]
    d2 = InfoArray(shape=(8, 8, 2), header=h, dtype=np.float32)
    tg.projector(d2, InfoArray(data=np.ones((8, 8, 8), np.float32), header=c))
    assert "R1_1" in d2.header[0]


def test_empty_and_tiny_inputs():
    ch, vh = synthetic.make_geometry({"n": 4, "T": 1, "N": 1, "d": 215.0, "lon_range": (0.3, 0.3)})
    data = InfoArray(shape=(1, 1, 1), header=_hdrs(vh), dtype=np.float32)
    tg.projector(data, InfoArray(data=np.ones((4, 4, 4), np.float32), header=dict(ch)))
    ref = InfoArray(shape=(1, 1, 1), header=_hdrs(vh))
    oracle.projector(ref, InfoArray(data=np.ones((4, 4, 4)), header=dict(ch)))
    np.testing.assert_allclose(np.asarray(data), ref, rtol=IMG_TOL)
    empty = InfoArray(shape=(1, 1, 0), header=[], dtype=np.float32)
    tg.projector(empty, InfoArray(data=np.ones((4, 4, 4), np.float32), header=dict(ch)))


def test_cube_offsets_beyond_32_bits():
    """A cube whose element offsets exceed 2^31 (a strided view into an 8.6 GB
    buffer) takes the 64-bit offset kernels; results match the oracle on the
    compact cube."""
    import torch
    n, T, N = 24, 5, 40
    ch, vh = _geometry(n, T, N, np.linspace(0.3, 5.0, T))
    x = np.random.default_rng(7).random((n, n, n)).astype(np.float32)
    s0 = (1 << 31) // (n - 1) + n * n
    big = torch.zeros(s0 * (n - 1) + n * n, dtype=torch.float32, device="cuda")
    cube = big.as_strided((n, n, n), (s0, n, 1))
    cube.copy_(torch.from_numpy(x))
    views = tg.siddon.upload_views(vh, None, cube.device)
    mh = tg.siddon.pack_map_header(ch)
    y = torch.zeros((N, N, T), device="cuda")
    tg.siddon.run_device("pj", y, cube, views, mh, T, obstacle="sun")
    ref = InfoArray(shape=(N, N, T), header=_hdrs(vh))
    oracle.projector(ref, InfoArray(data=x.astype(np.float64), header=dict(ch)), obstacle="sun")
    degen = degenerate_rays(vh, N, N)
    rel, norm = image_errors(y.cpu().numpy(), ref, exclude=degen)
    assert rel <= IMG_TOL and norm <= IMG_TOL, (rel, norm)
    yy = np.random.default_rng(8).random((N, N, T)).astype(np.float32)
    yy[degen] = 0
    cube.zero_()
    tg.siddon.run_device("bpj", torch.from_numpy(yy).cuda(), cube, views, mh, T, obstacle="sun")
    cref = InfoArray(shape=(n, n, n), header=dict(ch))
    oracle.backprojector(InfoArray(data=yy.astype(np.float64), header=_hdrs(vh)), cref, obstacle="sun")
    rel, norm = image_errors(cube.cpu().numpy(), cref, sig=CUBE_SIG)
    assert rel <= CUBE_TOL and norm <= CUBE_TOL, (rel, norm)
    del big
    torch.cuda.empty_cache()


def _exact_segment_count(M, u, ch, n):
    """Voxel segments of one ray through an n^3 cube (float64 plane crossings;
    crossings closer than 1e-9 count as one, like the reference's ties)."""
    mmin = np.array([ch["MMIN%d" % (k + 1)] for k in range(3)])
    cd = np.array([ch["CDELT%d" % (k + 1)] for k in range(3)])
    lo, hi = [], []
    for k in range(3):
        if u[k] == 0:
            if not (mmin[k] <= M[k] <= mmin[k] + n * cd[k]):
                return 0
            continue
        a = (mmin[k] - M[k]) / u[k], (mmin[k] + n * cd[k] - M[k]) / u[k]
        lo.append(min(a))
        hi.append(max(a))
    amin, amax = max(lo), min(hi)
    if amax <= amin:
        return 0
    pts = []
    for k in range(3):
        if u[k] != 0:
            a = (mmin[k] + np.arange(n + 1) * cd[k] - M[k]) / u[k]
            pts.extend(a[(a > amin + 1e-9) & (a < amax - 1e-9)].tolist())
    pts = np.sort(np.array(pts))
    merged = 0 if len(pts) == 0 else 1 + int(np.sum(np.diff(pts) > 1e-9))
    return merged + 1


def test_segment_counts_are_exact_integers():
    """tg_segment_counts (the intersection count behind the throughput and
    roofline figures) against an exact float64 count, ray by ray."""
    import torch
    n, T, N = 16, 6, 24
    lons = np.linspace(0.4, 5.5, T)
    ch, vh = _geometry(n, T, N, lons, lat=np.linspace(-0.3, 0.3, T), rol=0.2)
    views = tg.siddon.upload_views(vh, None, torch.device("cuda"))
    counts = tg.siddon.segment_counts(views, tg.siddon.pack_map_header(ch), (n, n, n), N, N, T).cpu().numpy()
    assert np.all(counts == np.round(counts))
    from helpers import unit_vectors
    U = unit_vectors(vh, N, N)
    exact = np.zeros_like(counts)
    for t in range(T):
        M = np.array([vh[t]["M%d" % (k + 1)] for k in range(3)])
        for i in range(N):
            for j in range(N):
                exact[i, j, t] = _exact_segment_count(M, U[i, j, t], ch, n)
    # rays through a cube edge or corner take zero-length steps where two or
    # three planes meet the entry / exit point, which the float64 count
    # merges: at most two segments apart there, equal elsewhere
    assert np.abs(counts - exact).max() <= 2
    assert np.mean(counts == exact) >= 0.99
    assert abs(counts.sum() - exact.sum()) <= 1e-3 * exact.sum() and counts.sum() > 0


# --------------------------------------------------------------------------
# per-ray and per-view diagnostics (tomograpy/siddon.py:221-243,341-350)

def _diag_geometry():
    ch, vh = _geometry(None, 4, 40, [0.3, 1.2, 2.6, 4.4], lat=[0.0, 0.2, -0.3, 0.1], rol=[0.0, 0.5, -1.0, 2.0],
                       shape=(24, 20, 28), pshape=(3.0, 2.5, 3.5))
    x = np.random.default_rng(17).random((24, 20, 28))
    return ch, vh, x


@pytest.mark.parametrize("obstacle", ["sun", None])
def test_ray_projector_matches_oracle(obstacle):
    """ray_projector traces one pixel's ray: that pixel gets the oracle's
    value, every other pixel stays as it was; backprojecting one ray equals
    the oracle's backprojection of a stack with only that pixel set; a mask
    element equal to 1 skips the ray (the reference's test at
    tomograpy/C_siddon.c.template:269-271)."""
    ch, vh, x = _diag_geometry()
    ref = InfoArray(shape=(40, 40, 4), header=_hdrs(vh))
    oracle.projector(ref, InfoArray(data=x.astype(np.float32).astype(np.float64), header=dict(ch)),
                     obstacle=obstacle)
    degen = degenerate_rays(vh, 40, 40)
    pixels = [(20, 20, 0), (3, 31, 1), (27, 8, 2), (39, 39, 3), (11, 19, 3)]
    cube = InfoArray(data=x.astype(np.float32), header=dict(ch))
    for (i, j, t) in pixels:
        assert not degen[i, j, t]
        data = InfoArray(shape=(40, 40, 4), header=_hdrs(vh), dtype=np.float32)
        data[...] = -1.0
        tg.ray_projector(data, cube, (i, j, t), obstacle=obstacle)
        d = np.asarray(data, np.float64)
        others = np.ones(d.shape, bool)
        others[i, j, t] = False
        assert np.all(d[others] == -1.0)
        np.testing.assert_allclose(d[i, j, t] + 1.0, ref[i, j, t], rtol=IMG_TOL, atol=1e-6 * np.abs(ref).max())
        # one ray backprojected
        y = np.zeros((40, 40, 4), np.float32)
        y[i, j, t] = 0.75
        bc = InfoArray(shape=x.shape, header=dict(ch), dtype=np.float32)
        tg.ray_projector(InfoArray(data=y, header=_hdrs(vh)), bc, (i, j, t), obstacle=obstacle, mode="bpj")
        bref = InfoArray(shape=x.shape, header=dict(ch))
        oracle.backprojector(InfoArray(data=y.astype(np.float64), header=_hdrs(vh)), bref, obstacle=obstacle)
        rel, norm = image_errors(bc, bref, sig=CUBE_SIG)
        assert norm <= CUBE_TOL, ((i, j, t), rel, norm)
    # mask == 1 skips the ray
    mask = np.zeros((40, 40, 4))
    mask[20, 20, 0] = 1.0
    data = InfoArray(shape=(40, 40, 4), header=_hdrs(vh), dtype=np.float32)
    tg.ray_projector(data, cube, (20, 20, 0), mask=mask, obstacle=obstacle)
    assert not np.asarray(data).any()


def test_conic_image_backprojector_matches_oracle():
    """Backprojecting view t alone equals the oracle's backprojection of the
    stack with every other view zeroed, and the per-view cubes sum to the
    full backprojection."""
    ch, vh, x = _diag_geometry()
    degen = degenerate_rays(vh, 40, 40)
    y = np.random.default_rng(18).random((40, 40, 4)).astype(np.float32)
    y[degen] = 0
    total = np.zeros(x.shape)
    for t in range(4):
        cube = InfoArray(shape=x.shape, header=dict(ch), dtype=np.float32)
        out = tg.conic_image_backprojector(InfoArray(data=y, header=_hdrs(vh)), cube, t, obstacle="sun")
        assert out is cube
        yt = np.zeros_like(y, dtype=np.float64)
        yt[:, :, t] = y[:, :, t]
        ref = InfoArray(shape=x.shape, header=dict(ch))
        oracle.backprojector(InfoArray(data=yt, header=_hdrs(vh)), ref, obstacle="sun")
        rel, norm = image_errors(cube, ref, sig=CUBE_SIG)
        assert rel <= CUBE_TOL and norm <= CUBE_TOL, (t, rel, norm)
        total += np.asarray(cube, np.float64)
    full = InfoArray(shape=x.shape, header=dict(ch), dtype=np.float32)
    tg.backprojector(InfoArray(data=y, header=_hdrs(vh)), full, obstacle="sun")
    np.testing.assert_allclose(total, np.asarray(full, np.float64), rtol=1e-5, atol=1e-6 * np.abs(total).max())

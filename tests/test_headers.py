"""Host-side header / geometry helpers (tomograpy/siddon.py:297-787,
tomograpy/simu.py) against their definitions and the reference's golden
unit vectors.  CPU only."""
import numpy as np
import pytest

import tomograpy_gb300 as tg
from helpers import golden, golden_case
from tomograpy_gb300 import headers as H
from tomograpy_gb300 import simu, synthetic


@pytest.mark.parametrize("lon,lat,rol", [(0, 0, 0), (0.3, 0.2, 0.1), (np.pi, -0.4, 2.0)])
def test_rotation_matrix_orthonormal(lon, lat, rol):
    R = tg.rotation_matrix(lon, lat, rol)
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-15)
    # the reference's image frame is mirrored: det(R) = -1 (tomograpy/siddon.py:486-494)
    assert np.isclose(abs(np.linalg.det(R)), 1.0)


def test_rotation_points_at_cube_centre():
    # The reference pixel (gamma = lambda = 0) looks from M towards the origin.
    lon = 0.7
    R = tg.rotation_matrix(lon, 0.0, 0.0)
    M = 200 * np.array([np.cos(lon), np.sin(lon), 0.0])
    np.testing.assert_allclose(R @ np.array([1.0, 0, 0]), -M / np.linalg.norm(M), atol=1e-15)


def test_map_borders_and_centered_header():
    h = tg.centered_cubic_map_header(3.0, 16)
    assert h["CRPIX1"] == 8.0 and h["CDELT1"] == 3.0 / 16
    assert h["MMIN1"] == -1.5 and h["MMAX1"] == 1.5 and h["PSHAPE3"] == 3.0
    h2 = tg.centered_cubic_map_header((3.0, 2.0, 1.0), (4, 8, 2))
    assert (h2["PSHAPE1"], h2["PSHAPE2"], h2["PSHAPE3"]) == (3.0, 2.0, 1.0)
    with pytest.raises(ValueError):
        tg.centered_cubic_map_header(3.0, (4, 4))


def test_array_dict_round_trip():
    h = {}
    R = np.arange(9.0).reshape(3, 3)
    H.array_to_dict(h, "R", R)
    assert h["R2_3"] == 5.0
    np.testing.assert_array_equal(H.dict_to_array(h, "R"), R)
    H.array_to_dict(h, "M", np.array([1.0, 2.0, 3.0]))
    np.testing.assert_array_equal(H.dict_to_array(h, "M"), [1, 2, 3])


def test_circular_trajectory():
    ih = tg.centered_image_header(0.02, 8)
    data = simu.circular_trajectory_data(**dict(ih, n_images=5, radius=200.0, max_lon=np.pi))
    assert data.shape == (8, 8, 5) and len(data.header) == 5
    lons = [h["LON"] for h in data.header]
    np.testing.assert_allclose(lons, np.linspace(0, np.pi, 5))
    for h in data.header:
        M = np.array([h["M1"], h["M2"], h["M3"]])
        assert np.isclose(np.linalg.norm(M), 200.0)
        assert "R3_3" in h


def test_numpy_twin_unit_vectors_match_reference():
    g = golden()
    vh, _ = golden_case("diag", 32, 32, (16, 16, 16))
    data = tg.InfoArray(shape=(32, 32, 5), header=vh)
    u = tg.full_unit_vector(data)
    np.testing.assert_allclose(u, g["diag_u"], rtol=0, atol=4e-16)


def test_numpy_twin_intersection_parameters_match_reference():
    g = golden()
    vh, ch = golden_case("diag", 32, 32, (16, 16, 16))
    data = tg.InfoArray(shape=(32, 32, 5), header=vh)
    obj = tg.InfoArray(shape=(16, 16, 16), header=ch)
    a1, an = tg.full_intersection_parameters(data, obj, g["diag_u"])
    np.testing.assert_allclose(a1, g["diag_a1"], rtol=1e-14)
    np.testing.assert_allclose(an, g["diag_an"], rtol=1e-14)


def test_intersect_cube_matches_reference_nonzero_pattern():
    # test_special_cases of the reference: data != 0 <=> the ray meets the cube
    g = golden()
    vh, ch = golden_case("cases16", 32, 32, (16, 16, 16))
    data = tg.InfoArray(shape=(32, 32, 17), header=vh)
    obj = tg.InfoArray(shape=(16, 16, 16), header=ch)
    u = tg.full_unit_vector(data)
    flag, _, _, _ = tg.intersect_cube(data, obj, u)
    np.testing.assert_array_equal(g["cases16_pj_ones"] != 0, flag)


def test_synthetic_geometry():
    ch, vh = synthetic.make_geometry("plain64")
    assert ch["NAXIS1"] == 64 and len(vh) == 60 and vh[0]["NAXIS1"] == 128
    fov = vh[0]["CDELT1"] * 128 / 2
    assert np.isclose(np.tan(fov) * 215.0, 1.6)
    x = synthetic.phantom(ch, seed=0)
    assert x.shape == (64, 64, 64) and x.dtype == np.float32
    assert x.max() > 1e7 and x[32, 32, 32] == 0.0

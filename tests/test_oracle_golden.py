"""Pin the oracle (oracle/siddon_oracle.c) against outputs of the reference's
own compiled kernel (tests/golden/reference_siddon.npz, made by
tests/golden/make_golden.py).  CPU only."""
import platform

import numpy as np
import pytest

import oracle
from helpers import golden, golden_case
from tomograpy_gb300.infoarray import InfoArray

X86 = platform.machine() in ("x86_64", "AMD64")


def _same(a, b, exact):
    a = np.asarray(a)
    b = np.asarray(b)
    if exact:
        assert np.array_equal(a, b)
    else:
        scale = max(np.abs(b).max(), 1e-300)
        assert np.abs(a - b).max() / scale <= 1e-12


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


@pytest.mark.parametrize("obstacle", ["sun", "none"])
@pytest.mark.parametrize("use_mask", [False, True])
def test_small24_projection(obstacle, use_mask):
    g = golden()
    vh, ch = golden_case("small24", 40, 40, (24, 24, 24))
    data = InfoArray(shape=(40, 40, 13), header=vh)
    cube = InfoArray(data=g["small24_x"].copy(), header=ch)
    oracle.projector(data, cube, mask=g["small24_mask"] if use_mask else None, obstacle=obstacle)
    tag = "%s_%s" % (obstacle, "mask" if use_mask else "nomask")
    _same(data, g["small24_pj_" + tag], exact=X86)


@pytest.mark.parametrize("obstacle", ["sun", "none"])
@pytest.mark.parametrize("use_mask", [False, True])
def test_small24_backprojection(obstacle, use_mask):
    g = golden()
    vh, ch = golden_case("small24", 40, 40, (24, 24, 24))
    data = InfoArray(data=g["small24_y"].copy(), header=vh)
    cube = InfoArray(shape=(24, 24, 24), header=ch)
    oracle.backprojector(data, cube, mask=g["small24_mask"] if use_mask else None, obstacle=obstacle, nthread=1)
    tag = "%s_%s" % (obstacle, "mask" if use_mask else "nomask")
    _same(cube, g["small24_bpj_" + tag], exact=X86)


@pytest.mark.parametrize("obstacle", ["sun", "none"])
def test_frames12_time_dependent(obstacle):
    g = golden()
    vh, ch = golden_case("frames12", 24, 24, (12, 12, 12, 7))
    data = InfoArray(shape=(24, 24, 7), header=vh)
    cube = InfoArray(data=g["frames12_x4"].copy(), header=ch)
    oracle.projector4d(data, cube, obstacle=obstacle)
    _same(data, g["frames12_pjt_" + obstacle], exact=X86)
    data = InfoArray(data=g["frames12_y"].copy(), header=vh)
    cube = InfoArray(shape=(12, 12, 12, 7), header=ch)
    oracle.backprojector4d(data, cube, obstacle=obstacle, nthread=1)
    _same(cube, g["frames12_bpjt_" + obstacle], exact=X86)


def test_float32_path_matches_reference_float32():
    g = golden()
    vh, ch = golden_case("small24", 40, 40, (24, 24, 24))
    data = InfoArray(shape=(40, 40, 13), header=vh, dtype=np.float32)
    cube = InfoArray(data=g["small24_x"].astype(np.float32), header=ch)
    oracle.projector(data, cube, obstacle="sun")
    _same(data, g["small24_pj_sun_nomask_float32ref"], exact=X86)


@pytest.mark.parametrize("n_cube", [16, 1])
def test_reference_test_geometry(n_cube):
    g = golden()
    key = "cases%d" % n_cube
    vh, ch = golden_case(key, 32, 32, (n_cube,) * 3)
    data = InfoArray(shape=(32, 32, 17), header=vh)
    cube = InfoArray(data=np.ones((n_cube,) * 3), header=ch)
    oracle.projector(data, cube)
    _same(data, g[key + "_pj_ones"], exact=X86)
    data = InfoArray(data=np.ones((32, 32, 17)), header=vh)
    cube = InfoArray(shape=(n_cube,) * 3, header=ch)
    oracle.backprojector(data, cube, nthread=1)
    _same(cube, g[key + "_bpj_ones"], exact=X86)


def test_diagnostics():
    g = golden()
    vh, ch = golden_case("diag", 32, 32, (16, 16, 16))
    data = InfoArray(shape=(32, 32, 5), header=vh)
    u = oracle.full_unit_vector(data)
    _same(u, g["diag_u"], exact=X86)
    a1, an = oracle.full_intersection_parameters(data, ch, g["diag_u"])
    _same(a1, g["diag_a1"], exact=X86)
    _same(an, g["diag_an"], exact=X86)


def test_golden_planted_error_is_caught():
    """A mistake planted in the oracle's output must fail the comparison."""
    g = golden()
    vh, ch = golden_case("small24", 40, 40, (24, 24, 24))
    data = InfoArray(shape=(40, 40, 13), header=vh)
    oracle.projector(data, InfoArray(data=g["small24_x"].copy(), header=ch), obstacle="sun")
    bad = np.asarray(data).copy()
    bad[20, 20, 3] *= 1.0 + 1e-9
    with pytest.raises(AssertionError):
        _same(bad, g["small24_pj_sun_nomask"], exact=True)

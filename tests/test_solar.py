"""FITS / WCS header ingestion (tomograpy/solar.py:16-209), on hand-built
SOHO- and STEREO-style headers and FITS files written here.  CPU only."""
import numpy as np
import pytest

from tomograpy_gb300 import siddon, solar
from tomograpy_gb300.models import convert_time

RSUN = 695000000.0


def soho_header(**kw):
    h = {"CRLN_OBS": 123.5, "CRLT_OBS": -6.25, "PC1_1": 0.999, "PC2_1": 0.0447, "CDELT1": 11.4,
         "CDELT2": 11.6, "CRVAL1": 2.5, "CRVAL2": -1.5, "CUNIT1": "arcsec", "CUNIT2": "arcsec",
         "DSUN_OBS": 1.4706e11, "DATE_OBS": "2008-03-01T12:34:56.250Z", "CRPIX1": 512.5, "CRPIX2": 512.5,
         "NAXIS1": 1024, "NAXIS2": 1024, "INSTRUME": "EIT", "TELESCOP": "SOHO"}
    h.update(kw)
    return h


def test_update_header_soho_style():
    h = soho_header()
    solar.update_header(h)
    lon, lat = np.radians(123.5), np.radians(-6.25)
    assert h["LON"] == pytest.approx(lon, rel=1e-15)
    assert h["LAT"] == pytest.approx(lat, rel=1e-15)
    assert h["ROL"] == pytest.approx(np.arctan2(0.0447 * 11.6, 0.999 * 11.4), rel=1e-15)
    d = 1.4706e11 / RSUN
    assert h["D"] == pytest.approx(d, rel=1e-15)
    np.testing.assert_allclose([h["M1"], h["M2"], h["M3"]],
                               [d * np.cos(lat) * np.cos(lon), d * np.cos(lat) * np.sin(lon), d * np.sin(lat)],
                               rtol=1e-15)
    arcsec = np.pi / 648000
    assert h["CDELT1"] == pytest.approx(11.4 * arcsec, rel=1e-15)
    assert h["CDELT2"] == pytest.approx(11.6 * arcsec, rel=1e-15)
    assert h["CRVAL1"] == pytest.approx(2.5 * arcsec, rel=1e-15)
    assert h["CRVAL2"] == pytest.approx(-1.5 * arcsec, rel=1e-15)
    assert h["TIME"] == pytest.approx(convert_time("2008-03-01T12:34:56") + 0.25, abs=1e-6)


def test_update_header_stereo_style_fallbacks():
    """No PC matrix: roll from CROTA2; no DSUN_OBS: distance from the
    heliocentric-aries-ecliptic position (HAE*_OBS, else HAE*); degree units."""
    h = soho_header(CUNIT1="degree", CUNIT2="degree", CDELT1=0.004, CDELT2=0.004, CROTA2=7.0)
    for k in ("PC1_1", "PC2_1", "DSUN_OBS"):
        del h[k]
    h.update({"HAEX_OBS": 1.2e11, "HAEY_OBS": -8.0e10, "HAEZ": 3.0e9})
    solar.update_header(h)
    assert h["ROL"] == pytest.approx(np.radians(7.0))
    assert h["D"] == pytest.approx(np.sqrt(1.2e11 ** 2 + 8.0e10 ** 2 + 3.0e9 ** 2) / RSUN)
    assert h["CDELT1"] == pytest.approx(np.radians(0.004))
    # an unknown unit is left as it is (as in the reference)
    h2 = soho_header(CUNIT1="mas")
    solar.update_header(h2)
    assert h2["CDELT1"] == 11.4


def test_updated_header_drives_the_geometry():
    """The updated header gives the projector's rotation matrix and observer."""
    h = soho_header()
    solar.update_header(h)
    R = siddon.H.rotation_matrix(h["LON"], h["LAT"], h["ROL"])
    siddon.H.header_rotation_matrix(h)
    np.testing.assert_allclose([[h["R%d_%d" % (a, b)] for b in (1, 2, 3)] for a in (1, 2, 3)], R, rtol=0, atol=0)
    M = np.array([h["M1"], h["M2"], h["M3"]])
    assert np.linalg.norm(M) == pytest.approx(h["D"], rel=1e-14)


@pytest.mark.parametrize("dtype", [np.uint8, np.int16, np.int32, np.int64, np.float32, np.float64])
def test_fits_round_trip(tmp_path, dtype):
    rng = np.random.default_rng(0)
    data = (rng.random((7, 5)) * 100).astype(dtype)
    h = soho_header(NAXIS1=7, NAXIS2=5, OBJECT="it's the sun", FLAG=True)
    p = tmp_path / "img.fits"
    solar.write_fits(str(p), h, data)
    assert p.stat().st_size % 2880 == 0
    h2, d2 = solar.read_fits(str(p))
    assert d2.shape == (7, 5) and d2.dtype == np.dtype(dtype)
    np.testing.assert_array_equal(d2, data)
    assert h2["OBJECT"] == "it's the sun" and h2["FLAG"] is True
    assert h2["DATE_OBS"] == h["DATE_OBS"] and h2["CDELT1"] == h["CDELT1"] and h2["NAXIS"] == 2


def test_fits_reader_scales_integers(tmp_path):
    """BITPIX 16 with BZERO / BSCALE, big-endian, written card by card."""
    raw = np.array([[0, 1, -2], [300, -32768, 32767]], dtype=">i2")   # FITS order (NAXIS2, NAXIS1)
    cards = ["SIMPLE  =                    T", "BITPIX  =                   16", "NAXIS   =                    2",
             "NAXIS1  =                    3", "NAXIS2  =                    2", "BSCALE  =                  0.5",
             "BZERO   =              32768.0", "COMMENT no value here", "EXPTIME =               1.5D+0 / s",
             "END"]
    text = "".join(c.ljust(80) for c in cards)
    text += " " * (-len(text) % 2880)
    body = raw.tobytes()
    body += b"\0" * (-len(body) % 2880)
    p = tmp_path / "int16.fits"
    p.write_bytes(text.encode() + body)
    h, d = solar.read_fits(str(p))
    assert h["EXPTIME"] == 1.5
    np.testing.assert_array_equal(d, raw.astype(np.float64).T * 0.5 + 32768.0)
    with pytest.raises(IOError):
        (tmp_path / "bad.fits").write_bytes(b"not a fits file")
        solar.read_fits(str(tmp_path / "bad.fits"))


def test_read_data_stacks_filters_and_sorts(tmp_path):
    times = ["2008-03-01T12:00:00", "2008-03-01T10:00:00", "2008-03-01T11:00:00.5", "2008-03-01T11:00:30"]
    rng = np.random.default_rng(1)
    imgs = []
    for k, t in enumerate(times):
        img = rng.random((8, 6)).astype(np.float32)
        imgs.append(img)
        h = soho_header(NAXIS1=8, NAXIS2=6, CRPIX1=4.5, CRPIX2=3.5, DATE_OBS=t, CRLN_OBS=10.0 * k,
                        INSTRUME="EIT" if k != 3 else "LASCO")
        solar.write_fits(str(tmp_path / ("f%d.fits" % k)), h, img)
    (tmp_path / "notes.txt").write_text("not an image")
    data = solar.read_data(str(tmp_path), dtype=np.float32)
    assert data.shape == (8, 6, 4) and data.dtype == np.float32
    order = [1, 2, 3, 0]                                  # sorted by DATE_OBS
    for i, k in enumerate(order):
        np.testing.assert_array_equal(data[..., i], imgs[k])
        assert data.header[i]["LON"] == pytest.approx(np.radians(10.0 * k))
        assert data.header[i]["BITPIX"] == -32
    # instrument and time-window filters, time step
    d2 = solar.read_data(str(tmp_path), instrume=["EIT"], time_window=("2008-03-01T12:30:00", "2008-03-01T10:30:00"))
    assert d2.shape[-1] == 2 and [h["LON"] for h in d2.header] == pytest.approx([np.radians(20.0), 0.0])
    d3 = solar.read_data(str(tmp_path), time_step=3600.0)
    assert d3.shape[-1] == 2                              # 11:00:00.5 and 11:00:30 fall within the step
    assert solar.read_data(str(tmp_path), telescop=["STEREO"]) is None
    # binning keeps the sky positions of the pixel grid
    d4 = solar.read_data(str(tmp_path), bin_factor=2)
    assert d4.shape == (4, 3, 4)
    np.testing.assert_allclose(d4[..., 0], imgs[1].reshape(4, 2, 3, 2).mean(axis=(1, 3)), rtol=1e-6)
    h0, hb = data.header[0], d4.header[0]
    x_orig = (0.5 - h0["CRPIX1"] + 1) * h0["CDELT1"]      # between pixels 0 and 1 (0-based)
    x_bin = (0 - hb["CRPIX1"] + 1) * hb["CDELT1"]         # binned pixel 0
    assert x_bin == pytest.approx(x_orig, rel=1e-12)
    with pytest.raises(ValueError):
        solar.read_data(str(tmp_path / "missing"))

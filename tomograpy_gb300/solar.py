"""Solar data ingestion: FITS files -> projector-ready data stacks.

Restates the header handling of ``tomograpy/solar.py:16-209``:

* :func:`update_header` turns the WCS / observer keywords of a SOHO or
  STEREO image into the keys the projector reads (``tomograpy/solar.py:59-115``):
  Carrington longitude / latitude of the observer (CRLN_OBS / CRLT_OBS,
  degrees -> LON / LAT radians), the roll angle (from the PC matrix and the
  pixel sizes when present, else CROTA2), the observer distance in solar radii
  (DSUN_OBS in metres, else the norm of HAEX/Y/Z[_OBS]), the observer position
  M1-3, pixel sizes and reference values converted to radians according to
  CUNIT1/2, and TIME (seconds) from DATE_OBS;
* :func:`filter_files` keeps the images of given instruments / telescopes,
  inside a time window and at least ``time_step`` apart, sorted by time
  (``tomograpy/solar.py:145-209``);
* :func:`read_data` reads a directory of FITS files into an
  :class:`~tomograpy_gb300.infoarray.InfoArray` stack ``(N1, N2, T)`` with one
  header dict per image (``tomograpy/solar.py:16-57``).

The reference reads files with ``pyfits`` and ``fitsarray``, neither of which
is installed here; :func:`read_fits` / :func:`write_fits` are a small
self-contained reader / writer of a FITS primary HDU (header cards and a
big-endian image with BITPIX 8, 16, 32, 64, -32 or -64, BSCALE / BZERO),
which is all the reference uses of those packages.

Deliberate differences, all documented at the function: times are read as
UTC (the reference converts with ``time.mktime``, i.e. in the machine's local
time zone), the ``deg`` unit and the ``DATE-OBS`` spelling are accepted
besides the reference's ``degree`` / ``DATE_OBS``, and ``bin_factor``
averages ``b x b`` pixel blocks (the reference delegates binning to
``fitsarray``, whose source is not available).
"""
import os

import numpy as np

from .infoarray import InfoArray, bitpix_from_dtype
from .models import convert_time

solar_radius = 695000000.0                   # metres (tomograpy/solar.py:11)
arcsecond_to_radian = np.pi / 648000.0       # pi / (60 * 60 * 180)


def arcsec2radians(val):
    return val * arcsecond_to_radian


def no_conversion(val):
    return val


cunit_to_conversion = {"arcsec": arcsec2radians, "degree": np.radians, "deg": np.radians,
                       None: no_conversion, "": no_conversion}


def _header(obj):
    return obj.header if hasattr(obj, "header") else obj


def _date_obs(h):
    return h["DATE_OBS"] if "DATE_OBS" in h else h["DATE-OBS"]


def update_header(array):
    """Add LON, LAT, ROL, D, M1-3 and TIME to the header of ``array`` (an
    array with a ``.header`` dict, or the dict itself) and convert CDELT1-2 /
    CRVAL1-2 to radians, in place (tomograpy/solar.py:59-115).  Returns the
    header."""
    h = _header(array)
    lon = np.radians(h["CRLN_OBS"])
    lat = np.radians(h["CRLT_OBS"])
    # roll: from the PC matrix and the pixel sizes when present, else CROTA2
    if all(k in h for k in ("PC2_1", "PC1_1", "CDELT1", "CDELT2")):
        rol = np.arctan2(h["PC2_1"] * h["CDELT2"], h["PC1_1"] * h["CDELT1"])
    else:
        rol = np.radians(h["CROTA2"])
    # observer distance in solar radii
    if "DSUN_OBS" in h:
        d = h["DSUN_OBS"] / solar_radius
    else:
        x = h["HAEX_OBS"] if "HAEX_OBS" in h else h["HAEX"]
        y = h["HAEY_OBS"] if "HAEY_OBS" in h else h["HAEY"]
        z = h["HAEZ_OBS"] if "HAEZ_OBS" in h else h["HAEZ"]
        d = np.sqrt(x ** 2 + y ** 2 + z ** 2) / solar_radius
    h["LON"] = float(lon)
    h["LAT"] = float(lat)
    h["ROL"] = float(rol)
    h["D"] = float(d)
    h["M1"] = float(d * np.cos(lat) * np.cos(lon))
    h["M2"] = float(d * np.cos(lat) * np.sin(lon))
    h["M3"] = float(d * np.sin(lat))
    for k in ("1", "2"):
        conv = cunit_to_conversion.get(h.get("CUNIT" + k), no_conversion)
        h["CDELT" + k] = float(conv(h["CDELT" + k]))
        h["CRVAL" + k] = float(conv(h["CRVAL" + k]))
    h["TIME"] = convert_time(_date_obs(h))
    return h


def filter_files(files, instrume=None, telescop=None, time_window=None, time_step=None, tmin=None, tmax=None):
    """Images (objects with a ``.header``) sorted by DATE_OBS and kept when
    their INSTRUME / TELESCOP is in the given collections, their time is
    inside [time_window] (``tmin`` / ``tmax`` take precedence) and, with
    ``time_step`` (seconds, or a date string as in the reference), at least
    that far from the previously kept image (tomograpy/solar.py:145-199)."""
    files = sorted(files, key=lambda f: convert_time(_date_obs(_header(f))))
    time_min = time_max = None
    if time_window is not None:
        time_min, time_max = sorted((convert_time(time_window[0]), convert_time(time_window[1])))
    if tmin is not None:
        time_min = convert_time(tmin)
    if tmax is not None:
        time_max = convert_time(tmax)
    step = None
    if time_step is not None:
        step = convert_time(time_step) if isinstance(time_step, str) else float(time_step)
    out = []
    for f in files:
        h = _header(f)
        if instrume is not None and h.get("INSTRUME") not in instrume:
            continue
        if telescop is not None and h.get("TELESCOP") not in telescop:
            continue
        t = convert_time(_date_obs(h))
        if time_min is not None and t < time_min:
            continue
        if time_max is not None and t > time_max:
            continue
        if step is not None and out and abs(convert_time(_date_obs(_header(out[-1]))) - t) < step:
            continue
        out.append(f)
    return out


# ---------------------------------------------------------------------------
# FITS primary HDU

_BLOCK = 2880
_BITPIX = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}


def _parse_value(text):
    text = text.strip()
    if text.startswith("'"):
        # quoted string ('' is an escaped quote); a comment may follow
        out, k = [], 1
        while k < len(text):
            if text[k] == "'":
                if k + 1 < len(text) and text[k + 1] == "'":
                    out.append("'")
                    k += 2
                    continue
                break
            out.append(text[k])
            k += 1
        return "".join(out).rstrip()
    v = text.split("/", 1)[0].strip()
    if v == "T":
        return True
    if v == "F":
        return False
    if v == "":
        return None
    try:
        return int(v)
    except ValueError:
        pass
    try:
        return float(v.replace("D", "E").replace("d", "e"))
    except ValueError:
        return v


def read_fits(path):
    """(header dict, image) of the primary HDU of a FITS file.  The image is
    returned in FITS axis order transposed to NumPy order, i.e. with shape
    (NAXIS1, NAXIS2[, ...]), scaled by BSCALE / BZERO when present."""
    with open(path, "rb") as f:
        raw = f.read()
    if raw[:9] != b"SIMPLE  =":
        raise IOError("%s is not a FITS file" % path)
    header = {}
    pos = 0
    end = False
    while not end:
        if pos + _BLOCK > len(raw):
            raise IOError("%s: truncated FITS header" % path)
        block = raw[pos:pos + _BLOCK].decode("ascii", errors="replace")
        pos += _BLOCK
        for c in range(0, _BLOCK, 80):
            card = block[c:c + 80]
            key = card[:8].strip()
            if key == "END":
                end = True
                break
            if card[8:10] == "= " and key:
                header[key] = _parse_value(card[10:])
    bitpix = int(header["BITPIX"])
    naxis = int(header.get("NAXIS", 0))
    shape = tuple(int(header["NAXIS%d" % (k + 1)]) for k in range(naxis))
    if bitpix not in _BITPIX:
        raise IOError("%s: unsupported BITPIX %d" % (path, bitpix))
    count = int(np.prod(shape)) if naxis else 0
    dt = np.dtype(_BITPIX[bitpix])
    if pos + count * dt.itemsize > len(raw):
        raise IOError("%s: truncated FITS data" % path)
    data = np.frombuffer(raw, dtype=dt, count=count, offset=pos)
    # FITS stores NAXIS1 fastest: C order (NAXISn, ..., NAXIS1), transposed
    data = data.reshape(shape[::-1]).T if naxis else data
    data = data.astype(dt.newbyteorder("="))
    if "BSCALE" in header or "BZERO" in header:
        data = data * float(header.get("BSCALE", 1.0)) + float(header.get("BZERO", 0.0))
    return header, data


def _card(key, value):
    if isinstance(value, bool):
        v = "%20s" % ("T" if value else "F")
    elif isinstance(value, (int, np.integer)):
        v = "%20d" % value
    elif isinstance(value, (float, np.floating)):
        v = "%20s" % repr(float(value)).upper()
    else:
        v = "'%-8s'" % str(value).replace("'", "''")
    return ("%-8s= %s" % (key[:8], v)).ljust(80)[:80]


def write_fits(path, header, data):
    """Write ``data`` (shape (NAXIS1, NAXIS2, ...), NumPy order as returned by
    :func:`read_fits`) and the scalar entries of ``header`` as a FITS primary
    HDU; BITPIX follows the array's dtype."""
    data = np.asarray(data)
    bitpix = {np.dtype(v).newbyteorder("="): k for k, v in _BITPIX.items()}[data.dtype.newbyteorder("=")]
    cards = [_card("SIMPLE", True), _card("BITPIX", bitpix), _card("NAXIS", data.ndim)]
    cards += [_card("NAXIS%d" % (k + 1), n) for k, n in enumerate(data.shape)]
    skip = {"SIMPLE", "BITPIX", "NAXIS", "END", "BSCALE", "BZERO"}
    for k, v in header.items():
        key = str(k).upper()
        if key in skip or key.startswith("NAXIS") or not isinstance(v, (bool, int, float, str, np.number)):
            continue
        cards.append(_card(key, v))
    cards.append("END".ljust(80))
    text = "".join(cards)
    text += " " * (-len(text) % _BLOCK)
    body = np.ascontiguousarray(data.T).astype(_BITPIX[bitpix]).tobytes()
    body += b"\0" * (-len(body) % _BLOCK)
    with open(path, "wb") as f:
        f.write(text.encode("ascii") + body)


class _Image:
    def __init__(self, header, data):
        self.header = header
        self.data = data


def bin_image(header, data, b):
    """Average ``b x b`` pixel blocks (trailing rows / columns that do not
    fill a block are dropped) and update NAXIS, CDELT and CRPIX so that the
    binned pixels map to the same sky positions."""
    b = int(b)
    n1, n2 = data.shape[0] // b, data.shape[1] // b
    out = data[:n1 * b, :n2 * b].reshape(n1, b, n2, b).mean(axis=(1, 3))
    h = dict(header)
    for k, n in (("1", n1), ("2", n2)):
        h["NAXIS" + k] = n
        h["CDELT" + k] = h["CDELT" + k] * b
        h["CRPIX" + k] = (h["CRPIX" + k] - 0.5) / b + 0.5
    return h, out


def read_data(path, dtype=np.float64, bin_factor=None, **kargs):
    """Read the SOHO / STEREO FITS images of directory ``path`` into an
    (N1, N2, T) stack whose ``.header`` is the list of updated image headers
    (tomograpy/solar.py:16-57).  ``kargs`` go to :func:`filter_files`.
    Files that are not FITS are skipped; returns None when no file matches."""
    if not os.path.isdir(path):
        raise ValueError("Directory does not exist")
    files = []
    for fname in sorted(os.listdir(path)):
        try:
            files.append(_Image(*read_fits(os.path.join(path, fname))))
        except (IOError, OSError, KeyError, ValueError):
            pass
    files = filter_files(files, **kargs)
    if not files:
        return None
    imgs, hdrs = [], []
    for f in files:
        h, d = dict(f.header), f.data
        if bin_factor is not None:
            h, d = bin_image(h, d, bin_factor)
        update_header(h)
        h["BITPIX"] = bitpix_from_dtype(dtype)
        imgs.append(np.asarray(d, dtype=dtype))
        hdrs.append(h)
    shape = imgs[0].shape
    if any(im.shape != shape for im in imgs):
        raise ValueError("images of different sizes cannot be stacked")
    data = InfoArray(shape=shape + (len(imgs),), header=hdrs, dtype=dtype)
    for i, im in enumerate(imgs):
        data[..., i] = im
    return data

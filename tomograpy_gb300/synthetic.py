"""Seeded synthetic solar-tomography workloads.

Geometry follows TomograPy's simulation conventions
(``tomograpy/simu.py:158-210``, ``tomograpy/siddon.py:307-405``): a centred
cube of ``n`` voxels per side spanning [-1.5, 1.5] solar radii
(CRPIX = n/2, CDELT = 3/n), observers at distance ``d`` in the solar
equatorial plane (LAT = ROL = 0) at longitudes ``linspace(lon0, lon1, T)``,
images of ``N x N`` pixels with CRPIX = N/2, CRVAL = 0 and
CDELT = 2 atan(1.6/d)/N radians (field of view +-1.6 solar radii).

The phantom is a radial electron-density shell
n(r) = 1e8 exp(-(r-1)/0.1) for 1.05 < r < 1.5 (zero elsewhere) plus 8 seeded
Gaussian blobs (sigma 0.05, amplitude 0.5 n(r_blob)) inside the shell,
sampled at voxel centres.  These stand in for real SOHO/STEREO data, which the
reference reads with pyfits (out of scope).
"""
import numpy as np

from . import headers as H
from .infoarray import InfoArray

RSUN_SHELL = (1.05, 1.5)


def view_headers(T, N, d=215.0, lon_range=(0.0, np.pi), fov_rsun=1.6, dtype=np.float32, lons=None):
    """List of ``T`` view header dicts on a circular equatorial trajectory."""
    cdelt = 2.0 * np.arctan(fov_rsun / d) / N
    if lons is None:
        lons = np.linspace(lon_range[0], lon_range[1], T)
    hdrs = []
    for lon in lons:
        h = H.centered_image_header(cdelt * N, N, dtype=dtype)
        h.update({"LON": float(lon), "LAT": 0.0, "ROL": 0.0, "D": float(d)})
        h["M1"] = d * np.cos(0.0) * np.cos(lon)
        h["M2"] = d * np.cos(0.0) * np.sin(lon)
        h["M3"] = d * np.sin(0.0)
        H.header_rotation_matrix(h)
        hdrs.append(h)
    return hdrs


def cube_header(n, dtype=np.float32, n_frames=None):
    h = H.centered_cubic_map_header(3.0, n, dtype=dtype)
    if n_frames is not None:
        h["NAXIS"] = 4
        h["NAXIS4"] = int(n_frames)
        h["CRVAL4"] = 0.0
    return h


def voxel_centres(h):
    axes = [h["MMIN%d" % (k + 1)] + (np.arange(int(h["NAXIS%d" % (k + 1)])) + 0.5) * h["CDELT%d" % (k + 1)]
            for k in range(3)]
    return np.meshgrid(*axes, indexing="ij")


def radial_density(r):
    out = 1e8 * np.exp(-(r - 1.0) / 0.1)
    out[(r <= RSUN_SHELL[0]) | (r >= RSUN_SHELL[1])] = 0.0
    return out


def blob_centres(seed, n_blobs=8):
    rng = np.random.default_rng(seed)
    r = rng.uniform(1.1, 1.4, n_blobs)
    v = rng.normal(size=(n_blobs, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v * r[:, None]


def phantom(h, seed=0, amplitudes=None, dtype=np.float32, sigma=0.05):
    """Shell + 8 Gaussian blobs at the voxel centres of cube header ``h``."""
    X, Y, Z = voxel_centres(h)
    r = np.sqrt(X * X + Y * Y + Z * Z)
    out = radial_density(r)
    c = blob_centres(seed)
    if amplitudes is None:
        amplitudes = np.ones(len(c))
    shell = (r > RSUN_SHELL[0]) & (r < RSUN_SHELL[1])
    for k in range(len(c)):
        rc = np.linalg.norm(c[k])
        amp = 0.5 * 1e8 * np.exp(-(rc - 1.0) / 0.1) * amplitudes[k]
        g = amp * np.exp(-((X - c[k, 0]) ** 2 + (Y - c[k, 1]) ** 2 + (Z - c[k, 2]) ** 2) / (2 * sigma ** 2))
        out = out + np.where(shell, g, 0.0)
    return out.astype(dtype)


def phantom4d(h, n_frames, seed=0, period=14.0, dtype=np.float32):
    """Per-frame phantoms whose blob amplitudes vary sinusoidally in time."""
    rng = np.random.default_rng(seed + 1000)
    phases = rng.uniform(0, 2 * np.pi, 8)
    frames = []
    for f in range(n_frames):
        amps = 1.0 + 0.5 * np.sin(2 * np.pi * f / period + phases)
        frames.append(phantom(h, seed, amplitudes=amps, dtype=dtype))
    return np.stack(frames, axis=-1)


def poisson_noise(y, peak_counts=1e4, seed=0):
    rng = np.random.default_rng(seed + 7)
    y = np.asarray(y, dtype=np.float64)
    peak = max(float(y.max()), 1e-30)
    counts = rng.poisson(np.clip(y, 0, None) / peak * peak_counts)
    return (counts * (peak / peak_counts)).astype(np.float32)


# Config sizes of the benchmark workloads.
CONFIGS = {
    # plain method, CPU-runnable
    "plain64": dict(n=64, T=60, N=128, d=215.0, lon_range=(0.0, np.pi)),
    # differentiable reconstruction (the throughput headline)
    "recon256": dict(n=256, T=360, N=512, d=215.0, lon_range=(0.0, 2 * np.pi)),
    # time-dependent: 28 frames x 28 views
    "frames128": dict(n=128, T=784, N=256, d=215.0, lon_range=(0.0, 2 * np.pi), n_frames=28),
}


def make_geometry(name_or_cfg, dtype=np.float32):
    cfg = CONFIGS[name_or_cfg] if isinstance(name_or_cfg, str) else name_or_cfg
    ch = cube_header(cfg["n"], dtype=dtype, n_frames=cfg.get("n_frames"))
    vh = view_headers(cfg["T"], cfg["N"], d=cfg["d"], lon_range=cfg["lon_range"], dtype=dtype)
    return ch, vh


def empty_data(view_hdrs, dtype=np.float32):
    h0 = view_hdrs[0]
    return InfoArray(shape=(int(h0["NAXIS1"]), int(h0["NAXIS2"]), len(view_hdrs)), header=view_hdrs,
                     dtype=dtype)


# Uneven multi-instance batch: seeded cube edges, view counts, image sides and
# observer distances (the configuration of the packed-launch benchmark).
UNEVEN_EDGES = (32, 48, 64, 96, 128, 160, 192)
UNEVEN_SIDES = (64, 128, 256, 512)


def uneven_specs(n_jobs=32, seed=0, edges=UNEVEN_EDGES, sides=UNEVEN_SIDES, views=(16, 256), dist=(150.0, 230.0)):
    """List of dicts {n, T, N, d, lon_range} for ``n_jobs`` seeded jobs."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_jobs):
        out.append(dict(n=int(rng.choice(edges)), T=int(rng.integers(views[0], views[1] + 1)),
                        N=int(rng.choice(sides)), d=float(rng.uniform(*dist)),
                        lon_range=(0.0, float(rng.uniform(np.pi, 2 * np.pi)))))
    return out


def make_job(spec, seed=0, with_data=True):
    """(cube header, view headers, phantom, noisy data) for one job spec."""
    from .batch import Job
    ch, vh = make_geometry(spec)
    job = Job(ch, vh)
    if with_data:
        job.phantom = phantom(ch, seed=seed) / np.float32(1e8)
    return job

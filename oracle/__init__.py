"""ORACLE -- test infrastructure only.

CPU restatement of TomograPy's Siddon projector (``oracle/siddon_oracle.c``)
and its ctypes binding.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may use this package, and only as the checker
or the timed CPU baseline; the product (``tomograpy_gb300``) never imports it.

Parity of the restatement is pinned against the reference's own compiled
C kernel through the golden fixtures in ``tests/golden/`` (see
``tests/test_oracle_golden.py``).

The Python entry points mirror ``tomograpy.siddon.projector`` & co.
(``tomograpy/siddon.py:85-219``): they take arrays with a ``.header`` (list of
per-view dicts for the data stack, a dict for the cube), accumulate in place
and return the updated array.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle_siddon.so")
SOURCES = [os.path.join(HERE, f) for f in ("siddon_oracle.c", "siddon_oracle_body.h", "siddon_oracle.h")]

PJ, BPJ, PJT, BPJT = 0, 1, 2, 3
MODES = {"pj": PJ, "bpj": BPJ, "pjt": PJT, "bpjt": BPJT}
OBSTACLES = {None: 0, "none": 0, "sun": 1}


class MapHeader(ctypes.Structure):
    _fields_ = [("cdelt", ctypes.c_double * 3), ("pshape", ctypes.c_double * 3),
                ("mmin", ctypes.c_double * 3), ("mmax", ctypes.c_double * 3)]


class ImageHeader(ctypes.Structure):
    _fields_ = [("crpix", ctypes.c_double * 2), ("cdelt", ctypes.c_double * 2),
                ("crval", ctypes.c_double * 2), ("M", ctypes.c_double * 3),
                ("R", ctypes.c_double * 9)]


def build(force=False):
    """Compile oracle/siddon_oracle.c into oracle/liboracle_siddon.so (gcc, OpenMP)."""
    if not force and os.path.exists(LIB_PATH):
        newest = max(os.path.getmtime(s) for s in SOURCES)
        if os.path.getmtime(LIB_PATH) >= newest:
            return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=gnu99", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", tmp, os.path.join(HERE, "siddon_oracle.c"), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        I = ctypes.c_int
        LL = ctypes.c_longlong
        for name in ("oracle_conic_full_projector_f64", "oracle_conic_full_projector_f32"):
            f = getattr(L, name)
            f.restype = I
            f.argtypes = [P, P, I, P, LL, LL, P, P, P, P, P, P, I, I, I]
        L.oracle_full_unit_vector_f64.restype = I
        L.oracle_full_unit_vector_f64.argtypes = [P, I, P, LL, LL, P, P, P]
        L.oracle_full_intersection_parameters_f64.restype = I
        L.oracle_full_intersection_parameters_f64.argtypes = [P, P, I, LL, LL, P, P, P, P]
        _lib = L
    return _lib


def pack_map_header(h):
    m = MapHeader()
    for k in range(3):
        s = str(k + 1)
        m.cdelt[k] = float(h["CDELT" + s])
        m.pshape[k] = float(h["PSHAPE" + s])
        m.mmin[k] = float(h["MMIN" + s])
        m.mmax[k] = float(h["MMAX" + s])
    return m


def pack_image_headers(hdrs):
    arr = (ImageHeader * len(hdrs))()
    for t, h in enumerate(hdrs):
        g = arr[t]
        for k in range(2):
            s = str(k + 1)
            g.crpix[k] = float(h["CRPIX" + s])
            g.cdelt[k] = float(h["CDELT" + s])
            g.crval[k] = float(h["CRVAL" + s])
        for k in range(3):
            g.M[k] = float(h["M%d" % (k + 1)])
            for l in range(3):
                g.R[3 * k + l] = float(h["R%d_%d" % (k + 1, l + 1)])
    return arr


def _strides(a):
    return (ctypes.c_longlong * len(a.strides))(*[s // a.itemsize for s in a.strides])


def conic_full_projector(data, cube, mask=None, obstacle=None, mode="pj", nthread=0,
                         data_header=None, cube_header=None):
    """Run the oracle on NumPy arrays in place (data (N1,N2,T); cube (n0,n1,n2[,F]))."""
    dh = data.header if data_header is None else data_header
    ch = cube.header if cube_header is None else cube_header
    if data.dtype != cube.dtype:
        raise ValueError("data and cube map should have the same data-type")
    dt = data.dtype
    if dt == np.float64:
        fn = lib().oracle_conic_full_projector_f64
    elif dt == np.float32:
        fn = lib().oracle_conic_full_projector_f32
    else:
        raise TypeError("oracle supports float32/float64 only")
    mode_i = MODES[mode]
    if data.ndim != 3 or cube.ndim not in (3, 4) or len(dh) != data.shape[2]:
        raise ValueError("bad shapes")
    mh = pack_map_header(ch)
    views = pack_image_headers(dh)
    ds = _strides(data)
    if cube.ndim == 3:
        ms = (ctypes.c_longlong * 4)(*([s // cube.itemsize for s in cube.strides] + [0]))
    else:
        ms = _strides(cube)
    if mode_i in (PJT, BPJT) and (cube.ndim != 4 or cube.shape[3] < data.shape[2]):
        raise ValueError("4-D modes need a cube with at least one frame per view")
    mshape = (ctypes.c_longlong * 3)(*cube.shape[:3])
    if mask is not None:
        mask = np.asarray(mask)
        if mask.dtype != dt:
            mask = mask.astype(dt)
        if mask.shape != data.shape:
            raise ValueError("mask shape")
        mptr = mask.ctypes.data
        ks = _strides(mask)
    else:
        mptr = None
        ks = (ctypes.c_longlong * 3)(0, 0, 0)
    st = fn(ctypes.byref(mh), views, len(dh), data.ctypes.data, data.shape[0], data.shape[1], ds,
            cube.ctypes.data, mshape, ms, mptr, ks, OBSTACLES[obstacle], mode_i, int(nthread))
    if st != 0:
        raise ValueError("oracle rejected its arguments (%d)" % st)
    return data if mode_i in (PJ, PJT) else cube


def projector(data, cube, mask=None, obstacle=None, nthread=0):
    return conic_full_projector(data, cube, mask, obstacle, "pj", nthread)


def backprojector(data, cube, mask=None, obstacle=None, nthread=0):
    return conic_full_projector(data, cube, mask, obstacle, "bpj", nthread)


def projector4d(data, cube, mask=None, obstacle=None, nthread=0):
    return conic_full_projector(data, cube, mask, obstacle, "pjt", nthread)


def backprojector4d(data, cube, mask=None, obstacle=None, nthread=0):
    return conic_full_projector(data, cube, mask, obstacle, "bpjt", nthread)


def full_unit_vector(data):
    """u[i,j,t,:] of every non-NaN pixel (float64), like C_full_unit_vector."""
    u = np.zeros(data.shape + (3,))
    d = np.ascontiguousarray(data, dtype=np.float64)
    views = pack_image_headers(data.header)
    lib().oracle_full_unit_vector_f64(views, len(data.header), d.ctypes.data, d.shape[0], d.shape[1],
                                      _strides(d), u.ctypes.data, _strides(u))
    return u


def full_intersection_parameters(data, cube_header, u):
    a1 = np.zeros(u.shape)
    an = np.zeros(u.shape)
    u = np.ascontiguousarray(u, dtype=np.float64)
    mh = pack_map_header(cube_header)
    views = pack_image_headers(data.header)
    lib().oracle_full_intersection_parameters_f64(ctypes.byref(mh), views, len(data.header),
                                                  u.shape[0], u.shape[1], u.ctypes.data,
                                                  _strides(u), a1.ctypes.data, an.ctypes.data)
    return a1, an

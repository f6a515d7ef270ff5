"""The C-ABI library loads and exports every function include/*.h declares;
argument validation returns TG_EINVAL before any CUDA call.  CPU only."""
import ctypes
import glob
import os
import re

import pytest

from tomograpy_gb300 import _build, _lib

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_functions():
    names = set()
    for path in glob.glob(os.path.join(INCLUDE, "*.h")):
        text = open(path).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(tg_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib(built):
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "tg_conic_full_projector" in names and len(names) >= 9


@pytest.mark.parametrize("name", declared_functions())
def test_symbol_exported(lib, name):
    assert hasattr(lib, name), "missing symbol %s" % name


def test_abi_version(lib):
    assert lib.tg_abi_version() == 2


def test_workspace_size(lib):
    n = lib.tg_deterministic_workspace_bytes(_lib.i64([4, 5, 6, 1]))
    assert n >= 256 + 4 * 5 * 6 * 8 and n % 256 == 0


def test_validation_without_gpu(lib):
    # NULL cube header: rejected before any CUDA call
    st = lib.tg_conic_full_projector(None, None, 0, 0, None, 1, 1, _lib.i64([1, 1, 1]), None,
                                     _lib.i64([1, 1, 1, 1]), _lib.i64([1, 1, 1, 0]), None, 2,
                                     _lib.i64([0, 0, 0]), 0, 0, None)
    assert st == _lib.TG_EINVAL
    assert b"NULL" in lib.tg_last_error()
    mh = _lib.MapHeader()
    for k in range(3):
        mh.cdelt[k] = 0.0
        mh.pshape[k] = 1.0
    buf = ctypes.create_string_buffer(64)
    st = lib.tg_conic_full_projector(ctypes.byref(mh), buf, 1, 0, buf, 1, 1, _lib.i64([1, 1, 1]), buf,
                                     _lib.i64([1, 1, 1, 1]), _lib.i64([1, 1, 1, 0]), None, 2,
                                     _lib.i64([0, 0, 0]), 0, 0, None)
    assert st == _lib.TG_EINVAL and b"positive" in lib.tg_last_error()
    st = lib.tg_conic_full_projector(ctypes.byref(mh), buf, 1, 0, buf, 1, 1, _lib.i64([1, 1, 1]), buf,
                                     _lib.i64([1, 1, 1, 1]), _lib.i64([1, 1, 1, 0]), None, 2,
                                     _lib.i64([0, 0, 0]), 0, 7, None)
    assert st == _lib.TG_EINVAL and b"mode" in lib.tg_last_error()


def test_library_built_for_sm103a():
    assert "arch=compute_103a,code=sm_103a" in " ".join(_build.ARCH)
    assert os.path.exists(_build.LIB)


def test_workspace_size_saturates_on_overflow(lib):
    # 2^20 x 2^20 x 2^20 x 16 voxels of 8 bytes do not fit in size_t: the
    # size saturates instead of wrapping to a small number
    size_max = ctypes.c_size_t(-1).value
    assert lib.tg_deterministic_workspace_bytes(_lib.i64([1 << 20, 1 << 20, 1 << 20, 16])) == size_max
    assert lib.tg_deterministic_workspace_bytes(_lib.i64([1 << 20, 1 << 20, 1 << 20, 1])) == \
        256 + 8 * (1 << 60)


def _overflow_args():
    mh = _lib.MapHeader()
    for k in range(3):
        mh.cdelt[k] = 1.0
        mh.pshape[k] = float(1 << 20)
        mh.mmin[k] = -0.5 * (1 << 20)
        mh.mmax[k] = 0.5 * (1 << 20)
    buf = ctypes.create_string_buffer(256)
    shape = _lib.i64([1 << 20, 1 << 20, 1 << 20, 16])
    strides = _lib.i64([1 << 40, 1 << 20, 1, 1 << 60])
    return mh, buf, shape, strides


def test_deterministic_entry_points_reject_overflowing_cubes(lib):
    """A cube whose accumulator size overflows is rejected on the host by both
    deterministic entry points (no device access happens)."""
    mh, buf, shape, strides = _overflow_args()
    common = (ctypes.byref(mh), buf, 1, buf, 1, 1, _lib.i64([1, 1, 1]), buf, shape, strides, None, 2,
              _lib.i64([0, 0, 0]), 0, _lib.TG_BPJT)
    # a 256-byte aligned address that is never dereferenced (rejected first)
    st = lib.tg_conic_full_backprojector_deterministic(*common, ctypes.c_void_p(1 << 20),
                                                       ctypes.c_size_t(-1).value // 2, None)
    assert st == _lib.TG_EINVAL and b"too large" in lib.tg_last_error()
    st = lib.tg_conic_full_backprojector_deterministic_noalloc(*common, None)
    assert st == _lib.TG_ENOMEM and b"scratch" in lib.tg_last_error()
    # more frames than an int holds: rejected by the shared validation
    shape4 = _lib.i64([8, 8, 8, 1 << 31])
    st = lib.tg_conic_full_projector(ctypes.byref(mh), buf, 1, 0, buf, 1, 1, _lib.i64([1, 1, 1]), buf, shape4,
                                     _lib.i64([64, 8, 1, 512]), None, 2, _lib.i64([0, 0, 0]), 0, _lib.TG_PJT, None)
    assert st == _lib.TG_EINVAL and b"frames" in lib.tg_last_error()

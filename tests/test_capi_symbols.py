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


def _host_job(n=16, N=32, T=4):
    """A tg_job whose pointers are never dereferenced by the host-side plan."""
    from tomograpy_gb300 import batch
    J = batch.TgJob()
    for k in range(3):
        J.map_header.cdelt[k] = 3.0 / n
        J.map_header.pshape[k] = 3.0
        J.map_header.mmin[k] = -1.5
        J.map_header.mmax[k] = 1.5
        J.map_shape[k] = n
    J.map_shape[3] = 1
    J.map_strides[0], J.map_strides[1], J.map_strides[2] = n * n, n, 1
    J.views = 1 << 20                      # placeholders: a host plan only records them
    J.n_views = T
    J.n1 = J.n2 = N
    J.data_strides[0], J.data_strides[1], J.data_strides[2] = N, 1, N * N
    J.mask_dtype = _lib.TG_U8
    J.data = 1 << 21
    J.map = 1 << 22
    return J


def test_host_plan_schedules_and_workspace(lib):
    """tg_packed_plan_scheduled_host: tile counts follow the schedule, the
    deterministic workspace covers every job, bad schedules are rejected --
    all on the host."""
    from tomograpy_gb300 import batch
    batch._bind(lib)
    jobs = (batch.TgJob * 2)(_host_job(16, 32, 4), _host_job(24, 64, 3))
    nbytes = lib.tg_packed_plan_bytes(2)
    buf = ctypes.create_string_buffer(nbytes)
    tiles = {}
    for sched in ((4, 1, 0), (1, 1, 16), (2, 0, 0)):
        info = batch.TgPackedInfo()
        sc = batch.TgSchedule(*sched, 0)
        st = lib.tg_packed_plan_scheduled_host(jobs, 2, ctypes.byref(sc), 0, buf, nbytes, ctypes.byref(info))
        assert st == _lib.TG_OK, lib.tg_last_error()
        assert (info.rows_per_warp, info.lane_axis, info.batch_steps) == sched
        rows = 8 * sched[0]
        tc, tr = (32, rows) if sched[1] else (rows, 32)
        want = sum(-(-N // tc) * -(-N // tr) * T for (N, T) in ((32, 4), (64, 3)))
        assert info.tiles == want
        ws = lib.tg_deterministic_workspace_bytes(_lib.i64([16, 16, 16, 1])) + \
            lib.tg_deterministic_workspace_bytes(_lib.i64([24, 24, 24, 1]))
        assert info.det_workspace_bytes == ws
        tiles[sched] = info.tiles
    for bad in ((3, 1, 0), (4, 2, 0), (4, 1, 8)):
        info = batch.TgPackedInfo()
        st = lib.tg_packed_plan_scheduled_host(jobs, 2, ctypes.byref(batch.TgSchedule(*bad, 0)), 0, buf, nbytes,
                                               ctypes.byref(info))
        assert st == _lib.TG_EINVAL


def test_host_alias_rejects_plain_memory(lib):
    """Pageable host memory has no device alias (and without a GPU the query
    itself fails cleanly)."""
    buf = ctypes.create_string_buffer(64)
    out = ctypes.c_void_p()
    assert lib.tg_host_alias(buf, ctypes.byref(out)) != _lib.TG_OK
    assert out.value is None
    assert lib.tg_host_alias(None, ctypes.byref(out)) == _lib.TG_EINVAL


def test_packed_launch_rejects_inconsistent_info(lib):
    # a plan description with no jobs, or more CTAs than a launch takes, is
    # refused on the host before any launch
    from tomograpy_gb300.batch import TgPackedInfo
    P = ctypes.c_void_p
    lib.tg_packed_projector.argtypes = [P, P, ctypes.c_int32, ctypes.c_int32, P]
    lib.tg_packed_projector.restype = ctypes.c_int
    buf = ctypes.create_string_buffer(4096)
    info = TgPackedInfo(n_jobs=0, rows_per_warp=4, tiles=10, lane_axis=1)
    st = lib.tg_packed_projector(ctypes.addressof(buf), ctypes.byref(info), _lib.TG_PJ, 0, None)
    assert st == _lib.TG_EINVAL and b"jobs" in lib.tg_last_error()
    info = TgPackedInfo(n_jobs=1, rows_per_warp=4, tiles=1 << 31, lane_axis=1)
    st = lib.tg_packed_projector(ctypes.addressof(buf), ctypes.byref(info), _lib.TG_PJ, 0, None)
    assert st == _lib.TG_EUNSUPPORTED and b"too large" in lib.tg_last_error()

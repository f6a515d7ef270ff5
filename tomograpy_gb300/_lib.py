"""ctypes binding of libtomograpy_gb300.so (the C ABI in include/tomograpy_gb300.h).

The library is built in-tree (``tomograpy_gb300/_build.py``).  Loading fails
loudly when it is missing: there is no CPU fallback for the projector.
"""
import ctypes
import os

from . import _build

TG_OK, TG_EINVAL, TG_ENOMEM, TG_ELAUNCH, TG_EUNSUPPORTED = 0, 1, 2, 3, 4
TG_PJ, TG_BPJ, TG_PJT, TG_BPJT = 0, 1, 2, 3
TG_OVERWRITE = 16
TG_OBSTACLE_NONE, TG_OBSTACLE_SUN = 0, 1
TG_F32, TG_F64, TG_U8 = 0, 1, 2

MODES = {"pj": TG_PJ, "bpj": TG_BPJ, "pjt": TG_PJT, "bpjt": TG_BPJT}
OBSTACLES = {None: TG_OBSTACLE_NONE, "none": TG_OBSTACLE_NONE, "sun": TG_OBSTACLE_SUN}


class MapHeader(ctypes.Structure):
    """tg_map_header: CDELT1-3, PSHAPE1-3, MMIN1-3, MMAX1-3."""
    _fields_ = [("cdelt", ctypes.c_double * 3), ("pshape", ctypes.c_double * 3),
                ("mmin", ctypes.c_double * 3), ("mmax", ctypes.c_double * 3)]


class ImageHeader(ctypes.Structure):
    """tg_image_header: CRPIX1-2, CDELT1-2, CRVAL1-2, M1-3, R (row-major), frame."""
    _fields_ = [("crpix", ctypes.c_double * 2), ("cdelt", ctypes.c_double * 2),
                ("crval", ctypes.c_double * 2), ("M", ctypes.c_double * 3),
                ("R", ctypes.c_double * 9), ("frame", ctypes.c_int32), ("reserved", ctypes.c_int32)]


assert ctypes.sizeof(ImageHeader) == 152

_lib = None


class TomograpyError(RuntimeError):
    pass


def load(build_if_missing=True):
    """Load (building first if needed) the C-ABI library."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB) or not _build.up_to_date():
        if not build_if_missing:
            raise TomograpyError("libtomograpy_gb300.so is not built (run __graft_entry__.build())")
        _build.build()
    L = ctypes.CDLL(_build.LIB)
    P, I32, I64, SZ = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_size_t
    proj_args = [P, P, I32, I32, P, I64, I64, P, P, P, P, P, I32, P, I32, I32, P]
    L.tg_conic_full_projector.argtypes = proj_args
    L.tg_conic_image_projector.argtypes = [P, P, I32, I32] + proj_args[3:]
    L.tg_ray_projector.argtypes = [P, P, I32, I32, I32, I32] + proj_args[3:]
    L.tg_unit_vector.argtypes = [P, I32, I32, I32, P, I64, I64, P, P, P, P]
    L.tg_intersection_parameters.argtypes = [P, P, I32, I32, I32, I64, I64, P, P, P, P, P]
    L.tg_deterministic_workspace_bytes.argtypes = [P]
    L.tg_deterministic_workspace_bytes.restype = SZ
    L.tg_conic_full_backprojector_deterministic.argtypes = proj_args[:3] + [P, I64, I64, P, P, P, P, P, I32, P,
                                                                            I32, I32, P, SZ, P]
    L.tg_segment_counts.argtypes = [P, P, I32, P, I64, I64, P, P, P, I32, P, I32, P]
    L.tg_noalloc_scratch_bytes.argtypes = []
    L.tg_noalloc_scratch_bytes.restype = SZ
    L.tg_conic_full_backprojector_deterministic_noalloc.argtypes = proj_args[:3] + [P, I64, I64, P, P, P, P, P,
                                                                                    I32, P, I32, I32, P]
    L.tg_conic_full_backprojector_deterministic_noalloc.restype = ctypes.c_int
    L.tg_dot_workspace_bytes.argtypes = []
    L.tg_dot_workspace_bytes.restype = SZ
    L.tg_dot_f32.argtypes = [P, P, I64, P, P, SZ, P]
    for name in ("tg_dot_f32", "tg_segment_counts", "tg_conic_full_projector", "tg_conic_image_projector", "tg_ray_projector", "tg_unit_vector",
                 "tg_intersection_parameters", "tg_conic_full_backprojector_deterministic"):
        getattr(L, name).restype = ctypes.c_int
    L.tg_host_alias.argtypes = [P, ctypes.POINTER(P)]
    L.tg_host_alias.restype = ctypes.c_int
    L.tg_last_error.restype = ctypes.c_char_p
    L.tg_last_error.argtypes = []
    L.tg_abi_version.restype = ctypes.c_int32
    _lib = L
    return L


def check(status):
    if status == TG_OK:
        return
    msg = load().tg_last_error().decode(errors="replace")
    if status == TG_EINVAL:
        raise ValueError(msg)
    raise TomograpyError("libtomograpy_gb300 status %d: %s" % (status, msg))


def i64(values):
    vals = list(values)
    return (ctypes.c_int64 * len(vals))(*vals)


def host_alias(t):
    """Device address of a pinned (page-locked) host tensor that kernels can
    read and write directly over the host link, or None when ``t`` is not
    such memory (pageable host memory, device memory)."""
    if t is None or t.is_cuda or not t.is_pinned():
        return None
    out = ctypes.c_void_p()
    if load().tg_host_alias(ctypes.c_void_p(t.data_ptr()), ctypes.byref(out)) != TG_OK:
        return None
    return out.value

"""Drop-in projector API: ``projector``, ``backprojector``, ``projector4d``,
``backprojector4d`` and friends, over the GB300 C ABI.

Names, arguments, in-place accumulation and errors follow
``tomograpy/siddon.py:85-294``:

* ``projector(data, cube, mask=None, obstacle=None, nthread=0)`` adds the
  projection of ``cube`` into ``data`` and returns ``data``;
  ``backprojector`` adds the backprojection of ``data`` into ``cube`` and
  returns ``cube``; the ``4d`` variants read / write the cube frame of each
  view (the view index, as in the reference, unless ``frames`` says
  otherwise).
* ``data.header`` must be a list of per-view dicts, ``cube.header`` a dict;
  missing rotation matrices (R1_1..R3_3) are computed from LON/LAT/ROL and
  missing MMIN/MMAX/PSHAPE from the cube header, in place
  (``check_projector_inputs``, ``tomograpy/siddon.py:245-270``).
* ``data`` and ``cube`` must share their dtype (float32 or float64);
  ``ValueError`` otherwise.
* ``nthread`` is accepted and ignored (the work runs on the GPU).

Inputs may be NumPy arrays (``InfoArray`` or any ndarray with a ``.header``;
they are staged to the GPU and the result is written back in place) or CUDA
``torch.Tensor``s (updated in place on the GPU; headers from a ``.header``
attribute or the ``data_header`` / ``cube_header`` keywords).

Mask semantics: a pixel is skipped when its mask element is non-zero, whatever
the mask's dtype.  (The reference reads the mask with the data's C type,
``tomograpy/C_siddon.c.template:29-31,520``, so a bool mask or a float64 mask
on float32 data is misread there; reading each element by its own dtype is a
deliberate fix.)
"""
import ctypes

import numpy as np

from . import _lib
from . import headers as H

try:
    import torch
except ImportError:  # pragma: no cover - torch is a hard requirement on the GPU path
    torch = None

VIEW_KEYS = ("CRPIX1", "CRPIX2", "CDELT1", "CDELT2", "CRVAL1", "CRVAL2", "M1", "M2", "M3",
             "R1_1", "R1_2", "R1_3", "R2_1", "R2_2", "R2_3", "R3_1", "R3_2", "R3_3")

VIEW_DTYPE = np.dtype([("crpix", "<f8", 2), ("cdelt", "<f8", 2), ("crval", "<f8", 2), ("M", "<f8", 3),
                       ("R", "<f8", 9), ("frame", "<i4"), ("reserved", "<i4")])
assert VIEW_DTYPE.itemsize == 152


# ---------------------------------------------------------------------------
# header handling

def check_projector_inputs(data, cube, data_header=None, cube_header=None):
    """Validate and complete headers in place (tomograpy/siddon.py:245-270)."""
    dh = data.header if data_header is None else data_header
    ch = cube.header if cube_header is None else cube_header
    if not isinstance(ch, dict):
        ch = dict(ch)
        if cube_header is None:
            cube.header = ch
    if not isinstance(dh, list):
        raise ValueError("data.header should be a list.")
    for i in range(len(dh)):
        if not isinstance(dh[i], dict):
            dh[i] = dict(dh[i])
        if "R1_1" not in dh[i]:
            H.header_rotation_matrix(dh[i])
    if _dtype_name(data) != _dtype_name(cube):
        raise ValueError("data and cube map should have the same data-type")
    if "MMAX1" not in ch:
        H.map_borders(ch)
    return dh, ch


def _dtype_name(a):
    if torch is not None and isinstance(a, torch.Tensor):
        return str(a.dtype).replace("torch.", "")
    return np.dtype(a.dtype).name


def pack_map_header(h):
    m = _lib.MapHeader()
    for k in range(3):
        s = str(k + 1)
        m.cdelt[k] = float(h["CDELT" + s])
        m.pshape[k] = float(h["PSHAPE" + s])
        m.mmin[k] = float(h["MMIN" + s])
        m.mmax[k] = float(h["MMAX" + s])
    return m


def pack_views(hdrs, frames=None):
    """Per-view header table (tg_image_header records) as a structured array."""
    T = len(hdrs)
    out = np.zeros(T, dtype=VIEW_DTYPE)
    try:
        cols = {k: np.array([float(h[k]) for h in hdrs], dtype=np.float64) for k in VIEW_KEYS}
    except KeyError as e:
        raise ValueError("view header is missing %s" % e)
    out["crpix"][:, 0], out["crpix"][:, 1] = cols["CRPIX1"], cols["CRPIX2"]
    out["cdelt"][:, 0], out["cdelt"][:, 1] = cols["CDELT1"], cols["CDELT2"]
    out["crval"][:, 0], out["crval"][:, 1] = cols["CRVAL1"], cols["CRVAL2"]
    for k in range(3):
        out["M"][:, k] = cols["M%d" % (k + 1)]
    for a in range(3):
        for b in range(3):
            out["R"][:, 3 * a + b] = cols["R%d_%d" % (a + 1, b + 1)]
    out["frame"] = np.arange(T, dtype=np.int32) if frames is None else np.asarray(frames, dtype=np.int32)
    return out


def _device():
    if torch is None or not torch.cuda.is_available():
        raise _lib.TomograpyError("tomograpy_gb300 needs a CUDA GPU (no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def upload_views(hdrs, frames=None, device=None):
    """Device copy (uint8 tensor) of the packed view table."""
    table = pack_views(hdrs, frames)
    dev = device or _device()
    return torch.from_numpy(table.view(np.uint8).reshape(-1).copy()).to(dev)


def _stream_ptr():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _strides(t):
    return _lib.i64(t.stride())


def _dtype_code(t):
    if t.dtype == torch.float32:
        return _lib.TG_F32
    if t.dtype == torch.float64:
        return _lib.TG_F64
    if t.dtype in (torch.uint8, torch.bool):
        return _lib.TG_U8
    raise TypeError("unsupported dtype %s" % t.dtype)


# ---------------------------------------------------------------------------
# device-level core (torch tensors on the GPU)

def run_device(mode, data, cube, views_dev, map_header, n_views, mask=None, obstacle=None, view=None,
               ray=None, deterministic=False, workspace=None, overwrite=False, data_ptr=None):
    """Launch one projector call on CUDA tensors (in place, on the current stream).

    data: (N1, N2, T) tensor; cube: (n0, n1, n2) or (n0, n1, n2, F) tensor;
    views_dev: uint8 device tensor from :func:`upload_views`; map_header: a
    dict or a packed ``MapHeader``.  ``overwrite`` (projections): every pixel
    is written instead of added.  ``data_ptr``: the device address to use for
    ``data`` -- a pinned host tensor's :func:`_lib.host_alias`, so that the
    kernel reads / writes the stack in host memory directly.
    """
    L = _lib.load()
    mode_i = _lib.MODES[mode] if isinstance(mode, str) else int(mode)
    if obstacle not in _lib.OBSTACLES:
        raise ValueError("obstacle must be None or 'sun'")
    obst = _lib.OBSTACLES[obstacle]
    if not (cube.is_cuda and (data.is_cuda or data_ptr is not None)):
        raise ValueError("data and cube must be CUDA tensors (or data a pinned host tensor with its alias)")
    if data.dtype != cube.dtype:
        raise ValueError("data and cube map should have the same data-type")
    dt = _dtype_code(data)
    if dt == _lib.TG_U8:
        raise ValueError("data must be float32 or float64")
    if data.dim() != 3:
        raise ValueError("data must be (N1, N2, T)")
    four_d = mode_i in (_lib.TG_PJT, _lib.TG_BPJT)
    if four_d and cube.dim() != 4:
        raise ValueError("4-D projectors need a 4-D cube (n0, n1, n2, F)")
    if not four_d and cube.dim() != 3:
        raise ValueError("cube must be 3-D (n0, n1, n2)")
    mh = map_header if isinstance(map_header, _lib.MapHeader) else pack_map_header(map_header)
    cshape = list(cube.shape) + ([1] if cube.dim() == 3 else [])
    cstr = list(cube.stride()) + ([0] if cube.dim() == 3 else [])
    if mask is not None:
        if mask.dtype == torch.bool:
            mask = mask.view(torch.uint8)
        if tuple(mask.shape) != tuple(data.shape):
            raise ValueError("mask shape %s differs from data shape %s" % (tuple(mask.shape), tuple(data.shape)))
        mptr, mdt, mstr = ctypes.c_void_p(mask.data_ptr()), _dtype_code(mask), _strides(mask)
    else:
        mptr, mdt, mstr = None, _lib.TG_U8, _lib.i64([0, 0, 0])
    n1, n2 = int(data.shape[0]), int(data.shape[1])
    dptr = data.data_ptr() if data_ptr is None else int(data_ptr)
    if overwrite and mode_i not in (_lib.TG_PJ, _lib.TG_PJT):
        raise ValueError("overwrite is for projections")
    common = (dt, ctypes.c_void_p(dptr), n1, n2, _strides(data), ctypes.c_void_p(cube.data_ptr()),
              _lib.i64(cshape), _lib.i64(cstr), mptr, mdt, mstr, obst,
              mode_i | (_lib.TG_OVERWRITE if overwrite else 0), _stream_ptr())
    vptr = ctypes.c_void_p(views_dev.data_ptr())
    if deterministic:
        if dt != _lib.TG_F32 or mode_i not in (_lib.TG_BPJ, _lib.TG_BPJT) or view is not None or ray is not None:
            raise ValueError("deterministic mode is for float32 full backprojection")
        need = L.tg_deterministic_workspace_bytes(_lib.i64(cshape if four_d else cshape[:3] + [1]))
        if workspace is None or workspace.numel() * workspace.element_size() < need:
            workspace = torch.empty(need, dtype=torch.uint8, device=cube.device)
        st = L.tg_conic_full_backprojector_deterministic(
            ctypes.byref(mh), vptr, n_views, ctypes.c_void_p(dptr), n1, n2, _strides(data),
            ctypes.c_void_p(cube.data_ptr()), _lib.i64(cshape), _lib.i64(cstr), mptr, mdt, mstr, obst, mode_i,
            ctypes.c_void_p(workspace.data_ptr()), workspace.numel() * workspace.element_size(), _stream_ptr())
    elif ray is not None:
        i, j, t = (int(v) for v in ray)
        st = L.tg_ray_projector(ctypes.byref(mh), vptr, n_views, i, j, t, *common)
    elif view is not None:
        st = L.tg_conic_image_projector(ctypes.byref(mh), vptr, n_views, int(view), *common)
    else:
        st = L.tg_conic_full_projector(ctypes.byref(mh), vptr, n_views, *common)
    _lib.check(st)
    return data if mode_i in (_lib.TG_PJ, _lib.TG_PJT) else cube


def segment_counts(views_dev, map_header, cube_shape, n1, n2, n_views, mask=None, obstacle=None, counts=None):
    """Number of voxel segments the float32 kernel accumulates along each ray,
    as a float32 (n1, n2, n_views) CUDA tensor (diagnostic; gives the exact
    intersection count behind throughput and roofline figures)."""
    L = _lib.load()
    mh = map_header if isinstance(map_header, _lib.MapHeader) else pack_map_header(map_header)
    if counts is None:
        counts = torch.zeros((n1, n2, n_views), dtype=torch.float32, device=views_dev.device)
    if mask is not None:
        if mask.dtype == torch.bool:
            mask = mask.view(torch.uint8)
        mptr, mdt, mstr = ctypes.c_void_p(mask.data_ptr()), _dtype_code(mask), _strides(mask)
    else:
        mptr, mdt, mstr = None, _lib.TG_U8, _lib.i64([0, 0, 0])
    st = L.tg_segment_counts(ctypes.byref(mh), ctypes.c_void_p(views_dev.data_ptr()), n_views,
                             ctypes.c_void_p(counts.data_ptr()), n1, n2, _strides(counts),
                             _lib.i64(list(cube_shape)[:3]), mptr, mdt, mstr, _lib.OBSTACLES[obstacle], _stream_ptr())
    _lib.check(st)
    return counts


# ---------------------------------------------------------------------------
# host-facing drop-in entry points

def _is_torch(a):
    return torch is not None and isinstance(a, torch.Tensor)


def _mask_to_device(mask, dev):
    if mask is None:
        return None
    if _is_torch(mask):
        return mask.to(dev)
    m = np.asarray(mask)
    return torch.from_numpy(np.ascontiguousarray(m != 0).view(np.uint8)).to(dev)


def _run(mode, data, cube, mask, obstacle, view=None, ray=None, frames=None, deterministic=False,
         data_header=None, cube_header=None):
    dh, ch = check_projector_inputs(data, cube, data_header, cube_header)
    four_d = mode in ("pjt", "bpjt")
    T = data.shape[2] if len(data.shape) == 3 else None
    if len(data.shape) != 3 or len(dh) != T:
        raise ValueError("data must be (N1, N2, T) with one header per view")
    if four_d:
        if len(cube.shape) != 4:
            raise ValueError("4-D projectors need a 4-D cube")
        fr = np.arange(T) if frames is None else np.asarray(frames)
        if fr.shape != (T,):
            raise ValueError("frames must give one frame index per view")
        if T and (fr.min() < 0 or fr.max() >= cube.shape[3]):
            raise ValueError("view frame index outside the cube's %d frames" % cube.shape[3])
    else:
        fr = None
    dev = _device()
    views_dev = upload_views(dh, fr, dev)
    mh = pack_map_header(ch)
    if _is_torch(data) and data.is_cuda:
        out = run_device(mode, data, cube, views_dev, mh, T, _mask_to_device(mask, data.device), obstacle,
                         view, ray, deterministic)
        return out
    if _is_torch(data):
        # host tensors (pinned for asynchronous copies): stage through the GPU
        d_t = data.to(dev, non_blocking=True)
        c_t = cube.to(dev, non_blocking=True)
        run_device(mode, d_t, c_t, views_dev, mh, T, _mask_to_device(mask, dev), obstacle, view, ray,
                   deterministic)
        if mode in ("pj", "pjt"):
            data.copy_(d_t, non_blocking=True)
            torch.cuda.current_stream().synchronize()
            return data
        cube.copy_(c_t, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return cube
    # NumPy inputs: stage through the GPU and write the accumulated result back.
    d_np = np.asarray(data)
    c_np = np.asarray(cube)
    if d_np.dtype not in (np.float32, np.float64):
        raise ValueError("data must be float32 or float64")
    d_t = torch.from_numpy(np.ascontiguousarray(d_np)).to(dev)
    c_t = torch.from_numpy(np.ascontiguousarray(c_np)).to(dev)
    run_device(mode, d_t, c_t, views_dev, mh, T, _mask_to_device(mask, dev), obstacle, view, ray, deterministic)
    _write_back(d_np if mode in ("pj", "pjt") else c_np, d_t if mode in ("pj", "pjt") else c_t)
    return data if mode in ("pj", "pjt") else cube


def _write_back(dst, src):
    """Device result -> the caller's NumPy array, in place (one copy when the
    array is C-contiguous in the result's dtype)."""
    if dst.flags.c_contiguous and dst.dtype == np.dtype(str(src.dtype).replace("torch.", "")):
        torch.from_numpy(dst).copy_(src.reshape(dst.shape))
    else:
        dst[...] = src.cpu().numpy()


def projector(data, cube, mask=None, obstacle=None, nthread=0, **kw):
    """Add the conic projection of ``cube`` into ``data``; returns ``data``."""
    return _run("pj", data, cube, mask, obstacle, **kw)


def backprojector(data, cube, mask=None, obstacle=None, nthread=0, **kw):
    """Add the backprojection of ``data`` into ``cube``; returns ``cube``."""
    return _run("bpj", data, cube, mask, obstacle, **kw)


def projector4d(data, cube, mask=None, obstacle=None, nthread=0, frames=None, **kw):
    """Project a 4-D cube; view t reads frame ``frames[t]`` (default t)."""
    return _run("pjt", data, cube, mask, obstacle, frames=frames, **kw)


def backprojector4d(data, cube, mask=None, obstacle=None, nthread=0, frames=None, **kw):
    """Backproject into a 4-D cube; view t writes frame ``frames[t]`` (default t)."""
    return _run("bpjt", data, cube, mask, obstacle, frames=frames, **kw)


def conic_image_projector(data, cube, t, mask=None, obstacle=None, **kw):
    """Project into view ``t`` only (tomograpy/siddon.py:221-231)."""
    if not 0 <= int(t) < data.shape[2]:
        raise ValueError("view index out of range")
    return _run("pj", data, cube, mask, obstacle, view=int(t), **kw)


def conic_image_backprojector(data, cube, t, mask=None, obstacle=None, **kw):
    """Backproject view ``t`` only.  Returns ``cube`` (the reference returns
    ``data`` here, tomograpy/siddon.py:243, which is a slip)."""
    if not 0 <= int(t) < data.shape[2]:
        raise ValueError("view index out of range")
    return _run("bpj", data, cube, mask, obstacle, view=int(t), **kw)


def ray_projector(data, cube, index, mask=None, obstacle=None, mode="pj", **kw):
    """Trace the single ray of pixel ``index = (i, j, t)``.  As in the
    reference's ``ray_projector`` (tomograpy/C_siddon.c.template:250-307) the
    ray is skipped when its mask element equals 1."""
    i, j, t = (int(v) for v in index)
    if not (0 <= i < data.shape[0] and 0 <= j < data.shape[1] and 0 <= t < data.shape[2]):
        raise ValueError("pixel index out of range")
    if mask is not None:
        m = np.asarray(mask.cpu() if _is_torch(mask) else mask)
        if m[i, j, t] == 1:
            return data if mode in ("pj", "pjt") else cube
    return _run(mode, data, cube, None, obstacle, ray=(i, j, t), **kw)


def C_full_unit_vector(data, data_header=None):
    """Unit vector of every non-NaN pixel ray, (N1, N2, T, 3) float64
    (tomograpy/siddon.py:272-280), computed on the GPU."""
    L = _lib.load()
    dh = data.header if data_header is None else data_header
    dev = _device()
    views_dev = upload_views(dh, None, dev)
    d_t = data if _is_torch(data) else torch.from_numpy(np.ascontiguousarray(np.asarray(data))).to(dev)
    if d_t.dtype not in (torch.float32, torch.float64):
        d_t = d_t.double()
    u = torch.zeros(tuple(d_t.shape) + (3,), dtype=torch.float64, device=dev)
    st = L.tg_unit_vector(views_dev.data_ptr(), len(dh), -1, _dtype_code(d_t), d_t.data_ptr(),
                          int(d_t.shape[0]), int(d_t.shape[1]), _strides(d_t), u.data_ptr(), _strides(u),
                          _stream_ptr())
    _lib.check(st)
    return u if _is_torch(data) else u.cpu().numpy()


def C_full_intersection_parameters(data, cube, u, data_header=None, cube_header=None):
    """a1 / an of every pixel ray for unit vectors ``u`` (tomograpy/siddon.py:282-294)."""
    L = _lib.load()
    dh = data.header if data_header is None else data_header
    ch = dict(cube.header if cube_header is None else cube_header)
    if "MMAX1" not in ch:
        H.map_borders(ch)
    dev = _device()
    views_dev = upload_views(dh, None, dev)
    u_t = u if _is_torch(u) else torch.from_numpy(np.ascontiguousarray(np.asarray(u, dtype=np.float64))).to(dev)
    a1 = torch.zeros_like(u_t)
    an = torch.zeros_like(u_t)
    dt = _lib.TG_F32 if _dtype_name(data) == "float32" else _lib.TG_F64
    mh = pack_map_header(ch)
    st = L.tg_intersection_parameters(ctypes.byref(mh), views_dev.data_ptr(), len(dh), -1, dt, int(u_t.shape[0]),
                                      int(u_t.shape[1]), u_t.data_ptr(), _strides(u_t), a1.data_ptr(),
                                      an.data_ptr(), _stream_ptr())
    _lib.check(st)
    if _is_torch(u):
        return a1, an
    return a1.cpu().numpy(), an.cpu().numpy()

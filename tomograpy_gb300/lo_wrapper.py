"""Linear-operator wrappers of the projector: ``siddon_lo`` / ``siddon4d_lo``.

TomograPy wraps its projector for the ``lo`` package (``tomograpy/lo_wrapper.py:10-73``):
``matvec`` = zero the output, project; ``rmatvec`` = zero the output,
backproject; the 4-D operator loops over ``ng`` interleaved sub-stacks, view
``j`` of sub-stack ``i`` (global view ``i + j*ng``) reading cube frame ``j``.
``lo`` is not available here, so :class:`Siddon` is a
``scipy.sparse.linalg.LinearOperator`` with the same behaviour on flattened
NumPy vectors, plus a device-resident interface (:meth:`Siddon.project`,
:meth:`Siddon.backproject`) on torch tensors that CG loops use without any
host round trip.

Differences from the reference, on purpose:

* the geometry (view table, cube header) is uploaded to the GPU once, at
  construction, instead of being re-marshalled at every call;
* ``matvec`` / ``rmatvec`` return a fresh array (the reference returns the
  same buffer at every call, ``tomograpy/lo_wrapper.py:25,31``, so its callers
  must copy);
* the 4-D operator maps every view to its frame in one launch (frame =
  view // ng) instead of ``ng`` launches over strided sub-stacks, and its
  ``rmatvec`` uses the data headers of the sub-stack (the reference assigns
  ``xi.header = xi.header[i::ng]``, ``tomograpy/lo_wrapper.py:63``).
"""
import numpy as np

from . import _lib
from . import siddon as S

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None

from scipy.sparse.linalg import LinearOperator


class Siddon(LinearOperator):
    """Projector ``P`` (cube -> data) as a linear operator.

    Parameters mirror ``tomograpy.lo_wrapper.Siddon(data_header, cube_header,
    **kwargs)``; ``kwargs`` may hold ``mask`` and ``obstacle`` as for
    ``projector``.  ``frames`` (4-D only) gives the cube frame of each view.
    """

    def __init__(self, data_header, cube_header, mask=None, obstacle=None, dtype=np.float32, frames=None,
                 cube_shape=None, deterministic=False, device=None, nthread=0):
        self.data_header = [dict(h) for h in data_header]
        self.map_header = dict(cube_header)
        if "MMAX1" not in self.map_header:
            S.H.map_borders(self.map_header)
        for h in self.data_header:
            if "R1_1" not in h:
                S.H.header_rotation_matrix(h)
        h0 = self.data_header[0]
        self.n1, self.n2, self.n_views = int(h0["NAXIS1"]), int(h0["NAXIS2"]), len(self.data_header)
        if cube_shape is None:
            cube_shape = tuple(int(self.map_header["NAXIS%d" % (k + 1)]) for k in range(3))
        self.cube_shape = tuple(int(v) for v in cube_shape)
        self.four_d = len(self.cube_shape) == 4
        self.frames = None
        if self.four_d:
            fr = np.arange(self.n_views) if frames is None else np.asarray(frames)
            if fr.min() < 0 or fr.max() >= self.cube_shape[3]:
                raise ValueError("view frame index outside the cube's frames")
            self.frames = fr
        self.device = device or S._device()
        self.tdtype = torch.float32 if np.dtype(dtype) == np.float32 else torch.float64
        self.views_dev = S.upload_views(self.data_header, self.frames, self.device)
        self.mh = S.pack_map_header(self.map_header)
        self.mask = S._mask_to_device(mask, self.device) if mask is not None else None
        self.obstacle = obstacle
        self.deterministic = deterministic
        self._workspace = None
        self._blocks = None
        self._stream = None
        self.data_shape = (self.n1, self.n2, self.n_views)
        n_in = int(np.prod(self.cube_shape))
        n_out = int(np.prod(self.data_shape))
        super().__init__(dtype=np.dtype(dtype), shape=(n_out, n_in))

    # -- device interface ------------------------------------------------
    def _dev(self, a, shape):
        if torch.is_tensor(a):
            # a host tensor is copied before the call returns, so its owner may
            # reuse it at once (an asynchronous copy from pinned memory could
            # still be reading it)
            t = a if a.is_cuda else a.to(self.device)
        else:
            t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=self.dtype))).to(self.device)
        return t.reshape(shape)

    def new_cube(self):
        """A zeroed cube of the operator's shape.  4-D cubes are stored
        frame-major (each frame contiguous, presented as (n0, n1, n2, F)
        through strides): a frame's views then gather from one contiguous,
        L2-resident block instead of frames interleaved in every sector."""
        if self.four_d:
            n0, n1, n2, F = self.cube_shape
            return torch.zeros((F, n0, n1, n2), dtype=self.tdtype, device=self.device).permute(1, 2, 3, 0)
        return torch.zeros(self.cube_shape, dtype=self.tdtype, device=self.device)

    # -- host <-> device pipelining ------------------------------------------
    PIPE_BLOCKS = 8

    def _row_blocks(self):
        """Blocks of image rows (multiples of 32, the kernels' tile height) and
        their view tables: a block of rows [a, b) is the image of views whose
        CRPIX1 is shifted by a, so it is traced with exactly the same ray
        directions, and its slice of the (N1, N2, T) stack is contiguous."""
        if self._blocks is None:
            step = -(-self.n1 // self.PIPE_BLOCKS)
            step = max(32, -(-step // 32) * 32)
            blocks = []
            for a in range(0, self.n1, step):
                hdrs = [dict(h, CRPIX1=float(h["CRPIX1"]) - a) for h in self.data_header]
                blocks.append((a, min(self.n1, a + step), S.upload_views(hdrs, self.frames, self.device)))
            self._blocks = blocks
        return self._blocks

    def _pipelined(self, host):
        return (torch.is_tensor(host) and not host.is_cuda and host.is_pinned() and self.n1 >= 64
                and self.tdtype == torch.float32 and host.dtype == torch.float32)

    # pinned host stacks: traced in place over the host link when the GPU can
    # address them (True), else staged in row blocks
    HOST_DIRECT = True

    def _host_stack(self, host):
        """(stack view, device alias) of a pinned float32 host stack the kernels
        can read / write in place over the host link, or None.  Taken when the
        stack's image axis 1 is contiguous (e.g. view-major (T, N1, N2)
        storage presented as (N1, N2, T))."""
        if not (self.HOST_DIRECT and torch.is_tensor(host) and not host.is_cuda and host.is_pinned()
                and host.dtype == torch.float32 and self.tdtype == torch.float32):
            return None
        stack = host if tuple(host.shape) == self.data_shape else None
        if stack is None:
            if not host.is_contiguous() or host.numel() != int(np.prod(self.data_shape)):
                return None
            stack = host.view(self.data_shape)
        if stack.stride(1) != 1:
            # a warp's lanes hold neighbouring pixels along image axis 1: with
            # that axis strided (e.g. the reference's (N1, N2, T) order, T
            # fastest) the lanes' host accesses do not coalesce and the link
            # carries a transaction per pixel (measured 2x slower than the
            # row-block staging), so such stacks are staged
            return None
        alias = _lib.host_alias(host)
        if alias is None:
            return None
        return stack, alias + (stack.data_ptr() - host.data_ptr())

    def _copy_stream(self):
        if self._stream is None:
            self._stream = torch.cuda.Stream(device=self.device)
        return self._stream

    def _project_to_host(self, xd, out):
        """P x into pinned host memory: each block of image rows is copied out
        on a second stream while the next block is traced."""
        y = torch.zeros(self.data_shape, dtype=self.tdtype, device=self.device)
        o = out.view(self.data_shape)
        main, copy = torch.cuda.current_stream(self.device), self._copy_stream()
        mode = "pjt" if self.four_d else "pj"
        for a, b, views in self._row_blocks():
            S.run_device(mode, y[a:b], xd, views, self.mh, self.n_views,
                         None if self.mask is None else self.mask[a:b], self.obstacle)
            copy.wait_stream(main)
            with torch.cuda.stream(copy):
                o[a:b].copy_(y[a:b], non_blocking=True)
        main.wait_stream(copy)
        copy.synchronize()
        return out

    def _backproject_from_host(self, yh, out):
        """P^T y from pinned host memory: each block of image rows is sent on a
        second stream while the previous block is backprojected."""
        yh = yh.view(self.data_shape)
        yd = torch.empty(self.data_shape, dtype=self.tdtype, device=self.device)
        x = self.new_cube()
        main, copy = torch.cuda.current_stream(self.device), self._copy_stream()
        copy.wait_stream(main)
        mode = "bpjt" if self.four_d else "bpj"
        for a, b, views in self._row_blocks():
            with torch.cuda.stream(copy):
                yd[a:b].copy_(yh[a:b], non_blocking=True)
            main.wait_stream(copy)
            S.run_device(mode, yd[a:b], x, views, self.mh, self.n_views,
                         None if self.mask is None else self.mask[a:b], self.obstacle)
        yd.record_stream(copy)
        copy.synchronize()   # every block has left the caller's host stack
        return self._out(x, out)

    def project(self, x, out=None):
        """y = P x.  ``x``: cube (CUDA or host tensor / array).  Returns a CUDA
        tensor, or fills ``out`` (device or host tensor) and returns it.  A
        pinned float32 host ``out`` whose image axis 1 is contiguous is written
        by the kernel itself over the host link -- every pixel, so it needs no
        zeroing and no staging copy; other pinned stacks are filled block by
        block while the GPU traces."""
        xd = self._dev(x, self.cube_shape)
        hs = self._host_stack(out) if out is not None else None
        if hs is not None:
            # the kernel writes every pixel of the pinned host stack directly
            # (overwrite mode: no zeroing pass, no staging copy)
            stack, alias = hs
            S.run_device("pjt" if self.four_d else "pj", stack, xd, self.views_dev, self.mh, self.n_views, self.mask,
                         self.obstacle, overwrite=True, data_ptr=alias)
            torch.cuda.current_stream().synchronize()
            return out
        if out is not None and self._pipelined(out):
            return self._project_to_host(xd, out)
        y = torch.zeros(self.data_shape, dtype=self.tdtype, device=self.device)
        S.run_device("pjt" if self.four_d else "pj", y, xd, self.views_dev, self.mh, self.n_views, self.mask,
                     self.obstacle)
        return self._out(y, out)

    def backproject(self, y, out=None):
        """x = P^T y.  ``y``: data stack (CUDA or host tensor / array).  A
        pinned float32 host stack whose image axis 1 is contiguous is read by
        the kernel itself over the host link; other pinned stacks are sent
        block by block while the GPU traces."""
        hs = self._host_stack(y)
        if hs is not None:
            # the kernel reads the pinned host stack directly
            yd, alias = hs
        elif self._pipelined(y) and not self.deterministic:
            return self._backproject_from_host(y, out)
        else:
            yd, alias = self._dev(y, self.data_shape), None
        x = self.new_cube()
        if self.deterministic and self.tdtype == torch.float32:
            need = _lib.load().tg_deterministic_workspace_bytes(
                _lib.i64(list(self.cube_shape) + ([] if self.four_d else [1])))
            if self._workspace is None or self._workspace.numel() < need:
                self._workspace = torch.empty(need, dtype=torch.uint8, device=self.device)
            S.run_device("bpjt" if self.four_d else "bpj", yd, x, self.views_dev, self.mh, self.n_views, self.mask,
                         self.obstacle, deterministic=True, workspace=self._workspace, data_ptr=alias)
        else:
            S.run_device("bpjt" if self.four_d else "bpj", yd, x, self.views_dev, self.mh, self.n_views, self.mask,
                         self.obstacle, data_ptr=alias)
        if alias is not None:
            torch.cuda.current_stream().synchronize()   # the caller may reuse its host stack at once
        return self._out(x, out)

    def _out(self, r, out):
        if out is None:
            return r
        out.view(r.shape).copy_(r, non_blocking=True)
        if not out.is_cuda:
            torch.cuda.current_stream().synchronize()
        return out

    # -- scipy LinearOperator interface (flattened NumPy vectors) ----------
    def _matvec(self, x):
        return self.project(np.asarray(x).reshape(self.cube_shape)).reshape(-1).cpu().numpy()

    def _rmatvec(self, y):
        return self.backproject(np.asarray(y).reshape(self.data_shape)).reshape(-1).cpu().numpy()

    def _adjoint(self):
        return _Adjoint(self)


class _Adjoint(LinearOperator):
    def __init__(self, op):
        self.op = op
        super().__init__(dtype=op.dtype, shape=(op.shape[1], op.shape[0]))

    def _matvec(self, y):
        return self.op._rmatvec(y)

    def _rmatvec(self, x):
        return self.op._matvec(x)


def siddon_lo(data_header, cube_header, **kwargs):
    """3-D projector operator (tomograpy/lo_wrapper.py:69-70)."""
    return Siddon(data_header, cube_header, **kwargs)


def siddon4d_lo(data_header, cube_header, ng=1, **kwargs):
    """4-D projector operator: the stack is split into ``ng`` interleaved
    sub-stacks and view ``i + j*ng`` uses cube frame ``j``
    (tomograpy/lo_wrapper.py:38-67,72-73)."""
    T = len(data_header)
    frames = np.arange(T) // int(ng)
    ch = dict(cube_header)
    cube_shape = kwargs.pop("cube_shape", None)
    if cube_shape is None:
        cube_shape = tuple(int(ch["NAXIS%d" % (k + 1)]) for k in range(3)) + (int(frames.max()) + 1,)
    return Siddon(data_header, cube_header, frames=frames, cube_shape=cube_shape, **kwargs)

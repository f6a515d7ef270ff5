"""Many reconstructions at once: packed launches and batched CG.

The plain drop-in path launches one projector per stack, which leaves most of
a GB300 idle when the stacks are small (a 32^3 cube seen in 16 views of 64^2
is ~130 CTAs for 152 SMs) and pays one launch per job per operation.  Here:

* :class:`PackedJobs` keeps every job's cube, data stack and CG vectors in
  flat device buffers and builds device plans (``tg_packed_plan``) so that one
  ``tg_packed_projector`` launch traces all jobs' rays; CTAs of different jobs
  share the GPU, largest jobs first;
* :func:`batched_cg` runs CG on every job's (P^T P + lam I) x = P^T y at once:
  per-job float64 inner products (``tg_segmented_dot_f32``) and per-job
  scalars stay on the device (``tg_cg_update_x`` / ``_p``), so an iteration
  is a fixed sequence of launches, captured once in a CUDA graph and replayed;
* :meth:`PackedJobs.autotune` picks the CTA tile height (rows per warp) by timing the
  packed projector + backprojector on the actual job set, cached per job-set
  signature;
* :func:`sequential_cg` is the plain per-job loop the batched form is
  measured against.
"""
import ctypes
import time

import numpy as np

from . import _lib
from . import siddon as S

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


class TgJob(ctypes.Structure):
    _fields_ = [("map_header", _lib.MapHeader), ("views", ctypes.c_void_p), ("n_views", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("n1", ctypes.c_int64), ("n2", ctypes.c_int64),
                ("data_strides", ctypes.c_int64 * 3), ("map_shape", ctypes.c_int64 * 4),
                ("map_strides", ctypes.c_int64 * 4), ("mask", ctypes.c_void_p), ("mask_strides", ctypes.c_int64 * 3),
                ("mask_dtype", ctypes.c_int32), ("reserved2", ctypes.c_int32), ("data", ctypes.c_void_p),
                ("map", ctypes.c_void_p)]


class TgPackedInfo(ctypes.Structure):
    _fields_ = [("n_jobs", ctypes.c_int32), ("rows_per_warp", ctypes.c_int32), ("four_d", ctypes.c_int32),
                ("idx64", ctypes.c_int32), ("tiles", ctypes.c_int64), ("det_workspace_bytes", ctypes.c_int64),
                ("det_idx64", ctypes.c_int32), ("lane_axis", ctypes.c_int32), ("batch_steps", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class TgSchedule(ctypes.Structure):
    """Tile schedule of a packed plan: rows per warp (1, 2, 4), the image axis
    a warp's lanes run along (1: lambda, 0: gamma) and the walk's batch
    length (0: default, 16)."""
    _fields_ = [("rows_per_warp", ctypes.c_int32), ("lane_axis", ctypes.c_int32),
                ("batch_steps", ctypes.c_int32), ("reserved", ctypes.c_int32)]


DEFAULT_SCHEDULE = (4, 1, 0)


def _bind(L):
    if getattr(L, "_tg_packed_bound", False):
        return L
    P, I32, SZ = ctypes.c_void_p, ctypes.c_int32, ctypes.c_size_t
    L.tg_packed_plan_bytes.argtypes = [I32]
    L.tg_packed_plan_bytes.restype = SZ
    L.tg_packed_plan.argtypes = [P, I32, I32, I32, P, SZ, P]
    L.tg_packed_plan.restype = ctypes.c_int
    L.tg_packed_plan_host.argtypes = [P, I32, I32, I32, P, SZ, P]
    L.tg_packed_plan_host.restype = ctypes.c_int
    L.tg_packed_plan_scheduled.argtypes = [P, I32, P, I32, P, SZ, P]
    L.tg_packed_plan_scheduled.restype = ctypes.c_int
    L.tg_packed_plan_scheduled_host.argtypes = [P, I32, P, I32, P, SZ, P]
    L.tg_packed_plan_scheduled_host.restype = ctypes.c_int
    L.tg_packed_projector.argtypes = [P, P, I32, I32, P]
    L.tg_packed_projector.restype = ctypes.c_int
    L.tg_packed_backprojector_deterministic.argtypes = [P, P, I32, P, SZ, P]
    L.tg_packed_backprojector_deterministic.restype = ctypes.c_int
    L.tg_segmented_workspace_bytes.argtypes = [I32]
    L.tg_segmented_workspace_bytes.restype = SZ
    L.tg_segmented_dot_f32.argtypes = [P, P, P, I32, P, P, SZ, P]
    L.tg_segmented_dot_f32.restype = ctypes.c_int
    L.tg_cg_update_x.argtypes = [P, P, P, P, P, P, P, I32, P]
    L.tg_cg_update_x.restype = ctypes.c_int
    L.tg_cg_update_p.argtypes = [P, P, P, P, P, I32, P]
    L.tg_cg_update_p.restype = ctypes.c_int
    L.tg_segmented_axpby.argtypes = [P, P, ctypes.c_float, ctypes.c_float, P, I32, P]
    L.tg_segmented_axpby.restype = ctypes.c_int
    L._tg_packed_bound = True
    return L


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class Job:
    """One reconstruction: cube header, view headers, optional data (N1, N2, T).

    ``frames`` (one cube frame index per view) makes it a time-dependent job
    with a (n0, n1, n2, F) cube, F = max(frames) + 1."""

    def __init__(self, cube_header, view_headers, data=None, obstacle="sun", frames=None):
        self.cube_header = dict(cube_header)
        if "MMAX1" not in self.cube_header:
            S.H.map_borders(self.cube_header)
        self.view_headers = [dict(h) for h in view_headers]
        for h in self.view_headers:
            if "R1_1" not in h:
                S.H.header_rotation_matrix(h)
        self.cube_shape = tuple(int(self.cube_header["NAXIS%d" % (k + 1)]) for k in range(3))
        self.frames = None
        if frames is not None:
            self.frames = np.asarray(frames, dtype=np.int64)
            if self.frames.shape != (len(self.view_headers),) or self.frames.min() < 0:
                raise ValueError("frames must give one non-negative frame index per view")
            self.cube_shape = self.cube_shape + (int(self.frames.max()) + 1,)
        h0 = self.view_headers[0]
        self.data_shape = (int(h0["NAXIS1"]), int(h0["NAXIS2"]), len(self.view_headers))
        self.data = data
        self.obstacle = obstacle


class PackedJobs:
    """Flat device buffers and packed plans for a list of :class:`Job`s.

    ``schedule`` = (rows per warp, lane axis, batch steps) of the packed
    tiles (see :class:`TgSchedule`); ``rows_per_warp`` alone means the
    lambda-major default batches; with neither, :meth:`autotune` picks one."""

    _tune_cache = {}

    def __init__(self, jobs, obstacle="sun", rows_per_warp=None, device=None, schedule=None):
        self.L = _bind(_lib.load())
        self.jobs = list(jobs)
        self.n = len(self.jobs)
        self.device = device or S._device()
        self.obstacle = obstacle
        cube_sizes = [int(np.prod(j.cube_shape)) for j in self.jobs]
        data_sizes = [int(np.prod(j.data_shape)) for j in self.jobs]
        self.cube_off = np.concatenate([[0], np.cumsum(cube_sizes)]).astype(np.int64)
        self.data_off = np.concatenate([[0], np.cumsum(data_sizes)]).astype(np.int64)
        dev = self.device
        # per-job element ranges [start, end) of the flat cube buffers
        self.cube_seg_dev = torch.from_numpy(np.stack([self.cube_off[:-1], self.cube_off[1:]], 1).reshape(-1).copy()).to(dev)
        self.four_d = any(j.frames is not None for j in self.jobs)
        if self.four_d and not all(j.frames is not None for j in self.jobs):
            raise ValueError("a pack holds either 3-D or time-dependent (4-D) jobs, not both")
        self.views = [S.upload_views(j.view_headers, j.frames, dev) for j in self.jobs]
        self.mhs = [S.pack_map_header(j.cube_header) for j in self.jobs]
        self.data = torch.zeros(int(self.data_off[-1]), dtype=torch.float32, device=dev)
        self._plans = {}
        self._det_ws = None
        self.tune_table = None
        if schedule is not None:
            self.schedule = tuple(int(v) for v in schedule)
        elif rows_per_warp is not None:
            self.schedule = (int(rows_per_warp), 1, 0)
        else:
            self.schedule = self.autotune()

    @property
    def rows_per_warp(self):
        return self.schedule[0]

    # views of the flat buffers -------------------------------------------------
    def data_view(self, flat, k):
        """(N1, N2, T) view of job k's stack in a flat data buffer (view-major storage)."""
        n1, n2, T = self.jobs[k].data_shape
        seg = flat[int(self.data_off[k]):int(self.data_off[k + 1])]
        return seg.view(T, n1, n2).permute(1, 2, 0)

    def cube_view(self, flat, k):
        """Job k's cube in a flat cube buffer; 4-D cubes are stored frame-major
        (F, n0, n1, n2) and viewed as (n0, n1, n2, F)."""
        seg = flat[int(self.cube_off[k]):int(self.cube_off[k + 1])]
        shape = self.jobs[k].cube_shape
        if len(shape) == 4:
            return seg.view(shape[3], *shape[:3]).permute(1, 2, 3, 0)
        return seg.view(*shape)

    def new_cube(self):
        return torch.zeros(int(self.cube_off[-1]), dtype=torch.float32, device=self.device)

    # plans ------------------------------------------------------------------------
    def plan(self, cube_flat, schedule=None):
        """Device plan tracing all jobs between ``cube_flat`` and ``self.data``."""
        sched = tuple(schedule or self.schedule)
        key = (cube_flat.data_ptr(), sched)
        if key in self._plans:
            return self._plans[key]
        arr = (TgJob * self.n)()
        for k, j in enumerate(self.jobs):
            d = self.data_view(self.data, k)
            c = self.cube_view(cube_flat, k)
            J = arr[k]
            J.map_header = self.mhs[k]
            J.views = self.views[k].data_ptr()
            J.n_views = j.data_shape[2]
            J.n1, J.n2 = j.data_shape[0], j.data_shape[1]
            for a in range(3):
                J.data_strides[a] = d.stride()[a]
                J.map_shape[a] = c.shape[a]
                J.map_strides[a] = c.stride()[a]
            J.map_shape[3] = c.shape[3] if c.dim() == 4 else 1
            J.map_strides[3] = c.stride()[3] if c.dim() == 4 else 0
            J.mask = None
            J.mask_dtype = _lib.TG_U8
            J.data = d.data_ptr()
            J.map = c.data_ptr()
        nbytes = self.L.tg_packed_plan_bytes(self.n)
        buf = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        info = TgPackedInfo()
        sc = TgSchedule(sched[0], sched[1], sched[2], 0)
        _lib.check(self.L.tg_packed_plan_scheduled(arr, self.n, ctypes.byref(sc), int(self.four_d), _ptr(buf), nbytes,
                                                   ctypes.byref(info)))
        self._plans[key] = (buf, info, arr)
        return self._plans[key]

    def project(self, cube_flat, schedule=None):
        """self.data = P cube (all jobs, one launch; data zeroed first)."""
        buf, info, _ = self.plan(cube_flat, schedule)
        self.data.zero_()
        _lib.check(self.L.tg_packed_projector(_ptr(buf), ctypes.byref(info), _lib.TG_PJT if self.four_d else _lib.TG_PJ,
                                              _lib.OBSTACLES[self.obstacle], _stream()))
        return self.data

    def backproject(self, cube_flat, schedule=None, deterministic=False):
        """cube_flat = P^T self.data (all jobs, one launch; cube zeroed first).
        ``deterministic``: every job's cube is bitwise the single-job
        deterministic backprojection of that job alone
        (``tg_packed_backprojector_deterministic``, on lambda-major tiles),
        whatever the other jobs."""
        sched = tuple(schedule or self.schedule)
        if deterministic and sched[1] != 1:
            sched = (sched[0], 1, sched[2])
        buf, info, _ = self.plan(cube_flat, sched)
        cube_flat.zero_()
        if deterministic:
            need = int(info.det_workspace_bytes)
            if self._det_ws is None or self._det_ws.numel() < need:
                self._det_ws = torch.empty(need, dtype=torch.uint8, device=self.device)
            _lib.check(self.L.tg_packed_backprojector_deterministic(
                _ptr(buf), ctypes.byref(info), _lib.OBSTACLES[self.obstacle], _ptr(self._det_ws),
                self._det_ws.numel(), _stream()))
            return cube_flat
        _lib.check(self.L.tg_packed_projector(_ptr(buf), ctypes.byref(info),
                                              _lib.TG_BPJT if self.four_d else _lib.TG_BPJ,
                                              _lib.OBSTACLES[self.obstacle], _stream()))
        return cube_flat

    # autotuning --------------------------------------------------------------------
    def signature(self):
        return tuple((j.cube_shape, j.data_shape) for j in self.jobs) + (self.obstacle,)

    def _time(self, sched, x, z, repeats):
        self.project(x, sched)
        self.backproject(z, sched)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(repeats):
            self.project(x, sched)
            self.backproject(z, sched)
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / repeats

    def autotune(self, repeats=2):
        """Tile schedule with the fastest packed pj + bpj on this job set,
        by coordinate descent: rows per warp (1, 2, 4) on lambda-major
        tiles, then the lane axis (lambda / gamma), then the batch length
        (default / 16).  Cached per job-size signature; the timings are kept
        in ``tune_table`` ({schedule: seconds per pj + bpj})."""
        sig = self.signature()
        if sig in PackedJobs._tune_cache:
            self.tune_table = PackedJobs._tune_cache[sig][1]
            return PackedJobs._tune_cache[sig][0]
        x = self.new_cube().fill_(1.0)
        z = self.new_cube()
        table = {}

        def t(sched):
            if sched not in table:
                table[sched] = self._time(sched, x, z, repeats)
            return table[sched]
        best = min(((rpw, 1, 0) for rpw in (1, 2, 4)), key=t)
        best = min((best, (best[0], 0, best[2])), key=t)
        best = min((best, (best[0], best[1], 16)), key=t)
        self._plans = {k: v for k, v in self._plans.items() if k[0] not in (x.data_ptr(), z.data_ptr())}
        self.tune_table = table
        PackedJobs._tune_cache[sig] = (best, table)
        return best


def batched_cg(pack, b, lam=1e-2, iters=20, graph=True, deterministic=False):
    """CG on every job's (P^T P + lam I) x = b at once (b, x: flat cube buffers).
    Returns (x, residual history (iters + 1, n_jobs) of ||r|| / ||b||).
    With ``deterministic`` the backprojections are the fixed-point ones, so
    every job's iterates are bitwise those of the same job solved alone (here
    or with :func:`sequential_cg` and a deterministic operator)."""
    from .cg import SegmentOps
    dev = pack.device
    n = pack.n
    ops = SegmentOps(pack.cube_seg_dev, dev)
    x = torch.zeros_like(b)
    r = b.clone()
    p = b.clone()
    Ap = torch.zeros_like(b)
    rr = torch.zeros(n, dtype=torch.float64, device=dev)
    rr_new = torch.zeros_like(rr)
    pAp = torch.zeros_like(rr)
    bb = torch.zeros_like(rr)
    ops.dot(r, r, rr)
    ops.dot(b, b, bb)
    hist = torch.zeros(iters + 1, n, dtype=torch.float64, device=dev)
    hist[0] = torch.sqrt(rr / bb)
    k_dev = torch.zeros((), dtype=torch.int64, device=dev)
    # deterministic mode keeps the default walk batches, so that the
    # projection is bitwise the single-job one as well
    sched = (pack.schedule[0], 1, 0) if deterministic else pack.schedule
    pack.plan(p, sched)
    pack.plan(Ap, sched)

    def step():
        pack.project(p, sched)
        pack.backproject(Ap, sched, deterministic=deterministic)
        if lam:
            ops.axpby(Ap, p, lam, 1.0)          # Ap = lam p + Ap, one fmaf per element
        ops.dot(p, Ap, pAp)
        ops.update_x(x, r, p, Ap, rr, pAp)
        ops.dot(r, r, rr_new)
        ops.update_p(p, r, rr, rr_new)
        k_dev.add_(1)
        hist.index_copy_(0, k_dev.view(1), torch.sqrt(rr / bb).view(1, n))

    if graph:
        saved = [t.clone() for t in (x, r, p, rr, hist, k_dev)]
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            step()
        torch.cuda.current_stream().wait_stream(s)
        for t, v in zip((x, r, p, rr, hist, k_dev), saved):
            t.copy_(v)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            step()
        for _ in range(iters):
            g.replay()
    else:
        for _ in range(iters):
            step()
    return x, hist


def sequential_cg(jobs, rhs, lam=1e-2, iters=20, device=None, deterministic=False):
    """The plain per-job loop: one job after another, each with its own
    operator and CG (tomograpy_gb300.cg), single-job kernel launches."""
    from . import cg, lo_wrapper
    out = []
    for j, b in zip(jobs, rhs):
        op = lo_wrapper.siddon_lo(j.view_headers, j.cube_header, obstacle=j.obstacle, dtype=np.float32,
                                  device=device, deterministic=deterministic)
        res = cg.cg(cg.NormalOperator(op, lam=lam), b, maxiter=iters)
        out.append(res.x)
    return out

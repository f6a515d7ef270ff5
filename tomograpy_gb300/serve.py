"""Continuous-batching reconstruction server.

Requests (a job's geometry and its data stack) arrive over time.  The server
keeps every admitted job's data stack and CG vectors resident on the GPU and,
at each scheduler step, advances *all* in-flight jobs by one CG iteration on
(P^T P + lam I) x = P^T y with packed launches (``tg_packed_projector``, one
launch per direction for all jobs, plus segmented vector kernels).  Jobs join
as soon as device memory allows (first-fit arenas; admission is by bytes and
in-flight rays, not by a slot count; shortest job first with aging) and leave
when they converge (relative residual <= tol) or reach their iteration
budget, so requests that arrive while others are on the GPU overlap with
them.

Reported per run: p50 / p99 time-to-solution (arrival to result on the host),
jobs/s and CG-iterations/s.  :func:`fifo_plain` is the baseline: the same
requests served one at a time in arrival order with the plain single-job path.
"""
import ctypes
import time

import numpy as np

from . import _lib
from . import batch as B
from . import siddon as S

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


class Arena:
    """First-fit allocator of element ranges in [0, size) (64-element aligned)."""

    ALIGN = 64

    def __init__(self, size):
        self.size = int(size)
        self.free = [(0, self.size)]  # sorted (start, length)

    def alloc(self, n):
        n = (int(n) + self.ALIGN - 1) // self.ALIGN * self.ALIGN
        for k, (st, ln) in enumerate(self.free):
            if ln >= n:
                if ln == n:
                    self.free.pop(k)
                else:
                    self.free[k] = (st + n, ln - n)
                return st, n
        return None

    def release(self, st, n):
        self.free.append((st, n))
        self.free.sort()
        merged = []
        for a, ln in self.free:
            if merged and merged[-1][0] + merged[-1][1] == a:
                merged[-1] = (merged[-1][0], merged[-1][1] + ln)
            else:
                merged.append((a, ln))
        self.free = merged


class Request:
    def __init__(self, rid, job, data, arrival, max_iters=20, tol=1e-4):
        self.id = rid
        self.job = job          # batch.Job (geometry)
        self.data = data        # host (N1, N2, T) float32 data stack (pinned torch tensor or NumPy)
        self.arrival = arrival  # seconds (relative to the run start)
        self.max_iters = max_iters
        self.tol = tol
        self.iters = 0
        self.t_admit = None
        self.t_done = None
        self.result = None      # host cube
        self.residual = None


class PinnedStaging:
    """Host -> device uploads that never stall the stream: arrays are copied
    into one preallocated pinned buffer (bump allocation) and sent with an
    asynchronous copy; when the buffer wraps, the host waits for the copies
    staged since the previous wrap (rare with a buffer of a few MB)."""

    def __init__(self, nbytes=8 << 20):
        self.buf = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        self.host = self.buf.numpy()
        self.head = 0
        self.events = []

    def upload(self, array, dev):
        a = np.ascontiguousarray(array)
        nb = a.nbytes
        if nb > self.buf.numel():
            return torch.from_numpy(a).to(dev)
        if self.head + nb > self.buf.numel():
            for ev in self.events:
                ev.synchronize()
            self.events.clear()
            self.head = 0
        self.host[self.head:self.head + nb] = a.reshape(-1).view(np.uint8)
        out = torch.empty(nb, dtype=torch.uint8, device=dev)
        out.copy_(self.buf[self.head:self.head + nb], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record()
        self.events.append(ev)
        self.head += (nb + 255) & ~255
        return out.view(_TORCH_DTYPES[a.dtype.str]).view(a.shape)


_TORCH_DTYPES = {}


def _torch_dtypes():
    if not _TORCH_DTYPES and torch is not None:
        _TORCH_DTYPES.update({np.dtype(np.int64).str: torch.int64, np.dtype(np.uint8).str: torch.uint8,
                              np.dtype(np.float32).str: torch.float32, np.dtype(np.float64).str: torch.float64})


class _Slot:
    """Device residency of one admitted request."""

    def __init__(self, req, c, d, views, slot, nc, nd):
        self.req, self.c, self.d, self.views, self.slot, self.nc, self.nd = req, c, d, views, slot, nc, nd
        self.rec = {}       # packed job records (bytes) per direction
        self.converged = False


class Server:
    """Continuous-batching CG server on one GPU.

    ``budget_bytes`` bounds the device memory of resident jobs (cube vectors
    x, r, p, Ap and the data stack of every in-flight job; default: half of
    the free device memory).  The host never waits for the GPU inside the
    loop except to keep at most two steps queued: plans and segment tables
    go up from pinned memory, residual norms and results come back through
    pinned memory and CUDA events.  A job retires after ``max_iters``
    iterations, or once the host sees its relative residual at or below
    ``tol`` (read one or two steps late, so such a job may run one or two
    iterations past its tolerance)."""

    def __init__(self, budget_bytes=None, lam=1e-2, obstacle="sun", rows_per_warp=4, device=None,
                 cube_fraction=0.4, max_rays=1 << 23, max_wait=1.0, max_slots=4096, deterministic=False,
                 on_done=None):
        self.L = B._bind(_lib.load())
        self.dev = device or S._device()
        self.lam = float(lam)
        # fixed-point backprojections: a request's result is then bitwise the
        # same alone, in any mix, and in the plain loop with a deterministic
        # operator (see batch.batched_cg)
        self.deterministic = bool(deterministic)
        self._ws = None
        self.on_done = on_done   # called with each request once its result is on the host
        self.obstacle = obstacle
        self.rpw = rows_per_warp
        self.max_rays = int(max_rays)
        self.max_wait = float(max_wait)
        if budget_bytes is None:  # half of the free device memory
            budget_bytes = torch.cuda.mem_get_info(self.dev)[0] // 2
        # the budget is split once into two arenas: the four cube vectors of
        # every job (cube_fraction of it) and the data stacks (the rest); a
        # job is admitted when both have room
        n_floats = int(budget_bytes) // 4
        self.cube_elems = int(n_floats * cube_fraction) // 4
        self.data_elems = n_floats - 4 * self.cube_elems
        self.vec = {k: torch.zeros(self.cube_elems, dtype=torch.float32, device=self.dev) for k in "xrpa"}
        self.data = torch.zeros(self.data_elems, dtype=torch.float32, device=self.dev)
        self.cube_arena = Arena(self.cube_elems)
        self.data_arena = Arena(self.data_elems)
        # ||b||^2 per slot, written by the device at admission (read by the
        # host only after a later step's event, so always complete)
        self.bb_host = torch.ones(max_slots, dtype=torch.float64, pin_memory=True)
        self.free_slots = list(range(max_slots))[::-1]
        self.inflight = []       # _Slot list, in plan order
        self.dirty = True
        self.iterations = 0
        self.completed = []
        self.max_inflight = 0
        _torch_dtypes()
        self.staging = PinnedStaging()
        self._rel_ring = torch.empty((8, max_slots), dtype=torch.float64, pin_memory=True)
        self._nsteps = 0
        self._limbo = []         # (steps launched at retirement, slot)
        self._steps = []         # queued steps: (event, pinned r.r, slots, step number)
        self._results = []       # (request, pinned cube, event)
        # host seconds per activity; "wait" is time blocked on the GPU (the
        # events of queued steps), "retire" the retirement work around it
        self.host_s = {"admit": 0.0, "rebuild": 0.0, "step": 0.0, "retire": 0.0, "wait": 0.0, "collect": 0.0}
        self.rebuilds = 0

    def _workspace(self, nbytes):
        """Deterministic-backprojection workspace (grown, never shrunk)."""
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = torch.empty(max(int(nbytes), 2 * (0 if self._ws is None else self._ws.numel())),
                                   dtype=torch.uint8, device=self.dev)
        return self._ws

    def _bpj_single(self, dv, cube, views, mh, T):
        if self.deterministic:
            need = self.L.tg_deterministic_workspace_bytes(_lib.i64(list(cube.shape) + [1]))
            S.run_device("bpj", dv, cube, views, mh, T, obstacle=self.obstacle, deterministic=True,
                         workspace=self._workspace(need))
        else:
            S.run_device("bpj", dv, cube, views, mh, T, obstacle=self.obstacle)

    # admission -------------------------------------------------------------
    def try_admit(self, req):
        nc = int(np.prod(req.job.cube_shape))
        nd = int(np.prod(req.job.data_shape))
        if not self.free_slots:
            return False
        c = self.cube_arena.alloc(nc)
        if c is None:
            return False
        d = self.data_arena.alloc(nd)
        if d is None:
            self.cube_arena.release(*c)
            return False
        views = self.staging.upload(S.pack_views(req.job.view_headers).view(np.uint8).reshape(-1), self.dev)
        job = _Slot(req, c, d, views, self.free_slots.pop(), nc, nd)
        n1, n2, T = req.job.data_shape
        dv = self.data[d[0]:d[0] + nd].view(T, n1, n2).permute(1, 2, 0)
        host = req.data if torch.is_tensor(req.data) else torch.from_numpy(np.ascontiguousarray(req.data))
        dv.copy_(host, non_blocking=True)
        # r = p = b = P^T y (single-job backprojection), x = 0; after this the
        # data slot is the job's scratch for P p
        r = self.vec["r"][c[0]:c[0] + nc]
        r.zero_()
        mh = S.pack_map_header(req.job.cube_header)
        job.mh = mh
        self._bpj_single(dv, r.view(*req.job.cube_shape), views, mh, T)
        self.vec["p"][c[0]:c[0] + nc].copy_(r)
        self.vec["x"][c[0]:c[0] + nc].zero_()
        rd = r.double()
        self.bb_host[job.slot:job.slot + 1].copy_(torch.dot(rd, rd).clamp_min(1e-300).view(1), non_blocking=True)
        for key, vecname in (("pj", "p"), ("bpj", "a")):
            cv = self.vec[vecname][c[0]:c[0] + nc].view(*req.job.cube_shape)
            J = B.TgJob()
            J.map_header = mh
            J.views = views.data_ptr()
            J.n_views = T
            J.n1, J.n2 = n1, n2
            for k in range(3):
                J.data_strides[k] = dv.stride()[k]
                J.map_shape[k] = cv.shape[k]
                J.map_strides[k] = cv.stride()[k]
            J.map_shape[3] = 1
            J.map_strides[3] = 0
            J.mask = None
            J.mask_dtype = _lib.TG_U8
            J.data = dv.data_ptr()
            J.map = cv.data_ptr()
            job.rec[key] = bytes(J)
        req.t_admit = time.perf_counter() - self.t_start
        self.inflight.append(job)
        self.max_inflight = max(self.max_inflight, len(self.inflight))
        self.dirty = True
        return True

    # packed structures for the current in-flight set ---------------------------
    def _rebuild(self):
        from .cg import SegmentOps
        n = len(self.inflight)
        seg = np.zeros(2 * n, dtype=np.int64)
        dseg = np.zeros(2 * n, dtype=np.int64)
        for k, job in enumerate(self.inflight):
            seg[2 * k], seg[2 * k + 1] = job.c[0], job.c[0] + job.nc
            dseg[2 * k], dseg[2 * k + 1] = job.d[0], job.d[0] + job.nd
        self.cube_ops = SegmentOps(self.staging.upload(seg, self.dev), self.dev)
        self.data_ops = SegmentOps(self.staging.upload(dseg, self.dev), self.dev)
        self.n = n
        self.plans = {}
        for key in ("pj", "bpj"):
            arr = (B.TgJob * n).from_buffer_copy(b"".join(job.rec[key] for job in self.inflight))
            nbytes = self.L.tg_packed_plan_bytes(n)
            host = np.empty(nbytes, dtype=np.uint8)
            info = B.TgPackedInfo()
            _lib.check(self.L.tg_packed_plan_host(arr, n, self.rpw, 0, ctypes.c_void_p(host.ctypes.data), nbytes,
                                                  ctypes.byref(info)))
            self.plans[key] = (self.staging.upload(host, self.dev), info)
        # per-job scalars: rr = r.r recomputed from the resident vectors (the
        # segmented dot of a range does not depend on the other ranges)
        self.rr = torch.zeros(n, dtype=torch.float64, device=self.dev)
        self.rr_new = torch.zeros_like(self.rr)
        self.pAp = torch.zeros_like(self.rr)
        self.cube_ops.dot(self.vec["r"], self.vec["r"], self.rr)
        self.dirty = False

    # one CG iteration for every in-flight job ----------------------------------
    def step(self):
        if self.dirty:
            t0 = time.perf_counter()
            self._rebuild()
            self.rebuilds += 1
            self.host_s["rebuild"] += time.perf_counter() - t0
        t0 = time.perf_counter()
        L, st, ops, v = self.L, B._stream(), self.cube_ops, self.vec
        ob = _lib.OBSTACLES[self.obstacle]
        self.data_ops.axpby(self.data, None, 0.0, 0.0)            # scratch = 0
        if self.n == 1:
            # a job alone (a large one, given max_rays) takes the single-job
            # kernels, whose geometry is a kernel parameter (a few % faster)
            job = self.inflight[0]
            n1, n2, T = job.req.job.data_shape
            shape = job.req.job.cube_shape
            dv = self.data[job.d[0]:job.d[0] + job.nd].view(T, n1, n2).permute(1, 2, 0)
            S.run_device("pj", dv, v["p"][job.c[0]:job.c[0] + job.nc].view(*shape), job.views, job.mh, T,
                         obstacle=self.obstacle)
            ops.axpby(v["a"], None, 0.0, 0.0)
            self._bpj_single(dv, v["a"][job.c[0]:job.c[0] + job.nc].view(*shape), job.views, job.mh, T)
        else:
            buf, info = self.plans["pj"]
            _lib.check(L.tg_packed_projector(B._ptr(buf), ctypes.byref(info), _lib.TG_PJ, ob, st))   # P p
            ops.axpby(v["a"], None, 0.0, 0.0)
            buf, info = self.plans["bpj"]
            if self.deterministic:                                                                    # P^T P p
                ws = self._workspace(info.det_workspace_bytes)
                _lib.check(L.tg_packed_backprojector_deterministic(B._ptr(buf), ctypes.byref(info), ob, B._ptr(ws),
                                                                   ws.numel(), st))
            else:
                _lib.check(L.tg_packed_projector(B._ptr(buf), ctypes.byref(info), _lib.TG_BPJ, ob, st))
        if self.lam:
            ops.axpby(v["a"], v["p"], self.lam, 1.0)
        ops.dot(v["p"], v["a"], self.pAp)
        ops.update_x(v["x"], v["r"], v["p"], v["a"], self.rr, self.pAp)
        ops.dot(v["r"], v["r"], self.rr_new)
        ops.update_p(v["p"], v["r"], self.rr, self.rr_new)
        rel = self._rel_ring[self._nsteps % self._rel_ring.shape[0], :self.n]   # <= 3 steps outstanding
        self._nsteps += 1
        rel.copy_(self.rr, non_blocking=True)                      # r.r after the update
        ev = torch.cuda.Event()
        ev.record()
        self._steps.append((ev, rel, list(self.inflight), self._nsteps))
        self.iterations += self.n
        for job in self.inflight:
            job.req.iters += 1
        self.host_s["step"] += time.perf_counter() - t0

    def _read_residuals(self, keep_queued=2):
        """Consume the residuals of finished steps, waiting only while more
        than `keep_queued` steps are queued."""
        while self._steps and (len(self._steps) > keep_queued or self._steps[0][0].query()):
            ev, rel, jobs, step_no = self._steps.pop(0)
            t0 = time.perf_counter()
            ev.synchronize()
            self.host_s["wait"] += time.perf_counter() - t0
            bb = self.bb_host.numpy()[[job.slot for job in jobs]]
            vals = np.sqrt(rel.numpy() / bb)
            for job, r in zip(jobs, vals):
                job.req.residual = float(r)
                if r <= job.req.tol:
                    job.converged = True
            # slots of retired jobs whose last step has now been read
            while self._limbo and self._limbo[0][0] <= step_no:
                self.free_slots.append(self._limbo.pop(0)[1])

    def retire(self):
        """Move converged / exhausted jobs out (results copied back
        asynchronously); returns how many left."""
        self._read_residuals()
        keep, done = [], []
        for job in self.inflight:
            (done if job.converged or job.req.iters >= job.req.max_iters else keep).append(job)
        for job in done:
            req = job.req
            out = torch.empty(job.nc, dtype=torch.float32, pin_memory=True)
            out.copy_(self.vec["x"][job.c[0]:job.c[0] + job.nc], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record()
            self._results.append((req, out.view(*req.job.cube_shape), ev))
            self.cube_arena.release(*job.c)   # stream order protects the copy
            self.data_arena.release(*job.d)
            # the slot (its ||b||^2 entry) is reused only after the residuals
            # of every step this job took part in have been read
            self._limbo.append((self._nsteps, job.slot))
        if done:
            self.inflight = keep
            self.dirty = True
        return len(done)

    def _collect(self, wait=False):
        while self._results and (wait or self._results[0][2].query()):
            req, out, ev = self._results.pop(0)
            ev.synchronize()
            req.result = out
            req.t_done = time.perf_counter() - self.t_start
            if req.residual is None:
                req.residual = float("nan")
            self.completed.append(req)
            if self.on_done is not None:
                self.on_done(req)

    def _rays_inflight(self):
        return sum(job.nd for job in self.inflight)

    def _admit(self, queue, now):
        """Admit queued requests while the in-flight rays stay under
        ``max_rays`` (one step is then a few tens of waves of the GPU) and
        memory allows.  Requests that have waited at least ``max_wait``
        seconds go first, oldest first, and the first of them that does not
        fit stops further admissions until the server has drained enough for
        it (so no request waits behind a stream of later ones); the others
        follow shortest job first (fewest rays: a small request is not held
        behind a large one).  An empty server always admits its first
        candidate."""
        if not queue:
            return
        rays = self._rays_inflight()

        def key(k):
            q = queue[k]
            if now - q.arrival >= self.max_wait:
                return (0, q.arrival, 0)
            return (1, int(np.prod(q.job.data_shape)), q.arrival)
        order = sorted(range(len(queue)), key=key)
        admitted = set()
        for k in order:
            req = queue[k]
            need = int(np.prod(req.job.data_shape))
            if (not self.inflight or rays + need <= self.max_rays) and self.try_admit(req):
                admitted.add(k)
                rays += need
                continue
            if now - req.arrival >= self.max_wait:
                break  # an old request is waiting: let the server drain for it
        if admitted:
            queue[:] = [r for k, r in enumerate(queue) if k not in admitted]

    def run(self, requests):
        """Serve ``requests`` (sorted by arrival time, seconds from now)."""
        pending = list(requests)
        queue = []
        self.t_start = time.perf_counter()
        while pending or queue or self.inflight:
            now = time.perf_counter() - self.t_start
            while pending and pending[0].arrival <= now:
                queue.append(pending.pop(0))
            t0 = time.perf_counter()
            self._admit(queue, now)
            t1 = time.perf_counter()
            self._collect()
            t2 = time.perf_counter()
            self.host_s["admit"] += t1 - t0
            self.host_s["collect"] += t2 - t1
            if not self.inflight and queue and self._limbo:
                self._read_residuals(keep_queued=0)  # release the slots of retired jobs
                self._admit(queue, now)
            if not self.inflight:
                if queue:
                    raise RuntimeError("request %d does not fit the memory budget" % queue[0].id)
                if pending:
                    time.sleep(max(0.0, pending[0].arrival - (time.perf_counter() - self.t_start)))
                continue
            self.step()
            t0 = time.perf_counter()
            w0 = self.host_s["wait"]
            self.retire()
            self.host_s["retire"] += (time.perf_counter() - t0) - (self.host_s["wait"] - w0)
        self._read_residuals(keep_queued=0)
        self._collect(wait=True)
        torch.cuda.synchronize()
        return summarize(self.completed, time.perf_counter() - self.t_start, self.iterations)


def summarize(done, wall, iterations):
    tts = np.array([r.t_done - r.arrival for r in done])
    return {"jobs": len(done), "wall_s": wall, "jobs_per_s": len(done) / wall, "cg_it_per_s": iterations / wall,
            "p50_s": float(np.percentile(tts, 50)), "p99_s": float(np.percentile(tts, 99)),
            "max_residual": float(max(r.residual for r in done))}


def fifo_plain(requests, lam=1e-2, obstacle="sun", device=None, deterministic=False, on_done=None):
    """Baseline: requests served one at a time in arrival order with the plain
    single-job operator and CG (stopping at the same tolerance / budget).
    ``on_done`` is called with each request once its result is on the host."""
    from . import cg, lo_wrapper
    dev = device or S._device()
    t_start = time.perf_counter()
    iterations = 0
    for req in requests:
        now = time.perf_counter() - t_start
        if req.arrival > now:
            time.sleep(req.arrival - now)
        op = lo_wrapper.siddon_lo(req.job.view_headers, req.job.cube_header, obstacle=obstacle, dtype=np.float32,
                                  device=dev, deterministic=deterministic)
        host = req.data if torch.is_tensor(req.data) else torch.from_numpy(np.ascontiguousarray(req.data))
        b = op.backproject(host.to(dev))
        res = cg.cg(cg.NormalOperator(op, lam=lam), b, maxiter=req.max_iters, tol=req.tol)
        req.result = res.x.cpu()
        req.residual = res.residuals[-1]
        req.iters = res.iterations
        iterations += res.iterations
        req.t_done = time.perf_counter() - t_start
        if on_done is not None:
            on_done(req)
    torch.cuda.synchronize()
    return summarize(list(requests), time.perf_counter() - t_start, iterations)


def poisson_requests(specs, rate, seed=0, max_iters=20, tol=1e-4, device=None):
    """Requests for job specs arriving as a Poisson process of ``rate`` jobs/s;
    each carries P(phantom) computed on the GPU (float32, pinned host)."""
    from . import lo_wrapper, synthetic
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k, spec in enumerate(specs):
        t += rng.exponential(1.0 / rate)
        job = synthetic.make_job(spec, seed=k)
        op = lo_wrapper.siddon_lo(job.view_headers, job.cube_header, obstacle="sun", dtype=np.float32, device=device)
        y = op.project(torch.from_numpy(job.phantom).to(op.device)).cpu().pin_memory()
        out.append(Request(k, job, y, t, max_iters=max_iters, tol=tol))
    return out

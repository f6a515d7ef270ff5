"""Continuous-batching reconstruction server.

Requests (a job's geometry and its data stack) arrive over time.  The server
keeps every admitted job's data stack and CG vectors resident on the GPU and,
at each scheduler step, advances *all* in-flight jobs by one CG iteration on
(P^T P + lam I) x = P^T y with packed launches (``tg_packed_projector``, one
launch per direction for all jobs, plus segmented vector kernels).  Jobs join
as soon as device memory allows (first-fit arenas; admission is by bytes,
not by a slot count) and leave when they converge (relative residual <= tol)
or reach their iteration budget, so requests that arrive while others are on
the GPU overlap with them.

Reported per run: p50 / p99 time-to-solution (arrival to result on the host),
jobs/s and CG-iterations/s.  :func:`fifo_plain` is the baseline: the same
requests served one at a time in arrival order with the plain single-job path.
"""
import ctypes
import heapq
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


class Server:
    """Continuous-batching CG server on one GPU.

    ``budget_bytes`` bounds the device memory of resident jobs (cube vectors
    x, r, p, Ap and the data stack of every in-flight job)."""

    def __init__(self, budget_bytes=None, lam=1e-2, obstacle="sun", rows_per_warp=4, device=None,
                 cube_fraction=0.4, max_rays=1 << 23, max_wait=1.0):
        self.L = B._bind(_lib.load())
        self.dev = device or S._device()
        self.lam = float(lam)
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
        self.inflight = []       # list of (request, cube range, data range, views_dev)
        self.dirty = True
        self.iterations = 0
        self.completed = []
        self.max_inflight = 0

    # admission -------------------------------------------------------------
    def try_admit(self, req):
        nc = int(np.prod(req.job.cube_shape))
        nd = int(np.prod(req.job.data_shape))
        c = self.cube_arena.alloc(nc)
        if c is None:
            return False
        d = self.data_arena.alloc(nd)
        if d is None:
            self.cube_arena.release(*c)
            return False
        views = S.upload_views(req.job.view_headers, None, self.dev)
        n1, n2, T = req.job.data_shape
        dv = self.data[d[0]:d[0] + nd].view(T, n1, n2).permute(1, 2, 0)
        host = req.data if torch.is_tensor(req.data) else torch.from_numpy(np.ascontiguousarray(req.data))
        dv.copy_(host, non_blocking=True)
        # r = p = b = P^T y (single-job backprojection), x = 0; after this the
        # data slot is the job's scratch for P p
        r = self.vec["r"][c[0]:c[0] + nc]
        r.zero_()
        S.run_device("bpj", dv, r.view(*req.job.cube_shape), views, S.pack_map_header(req.job.cube_header), T,
                     obstacle=self.obstacle)
        self.vec["p"][c[0]:c[0] + nc].copy_(r)
        self.vec["x"][c[0]:c[0] + nc].zero_()
        req.bb = float(torch.dot(r.double(), r.double()))
        req.t_admit = time.perf_counter() - self.t_start
        self.inflight.append((req, c, d, views))
        self.max_inflight = max(self.max_inflight, len(self.inflight))
        self.dirty = True
        return True

    # packed structures for the current in-flight set ---------------------------
    def _rebuild(self):
        from .cg import SegmentOps
        n = len(self.inflight)
        seg = np.zeros(2 * n, dtype=np.int64)
        dseg = np.zeros(2 * n, dtype=np.int64)
        for k, (req, c, d, views) in enumerate(self.inflight):
            seg[2 * k], seg[2 * k + 1] = c[0], c[0] + int(np.prod(req.job.cube_shape))
            dseg[2 * k], dseg[2 * k + 1] = d[0], d[0] + int(np.prod(req.job.data_shape))
        self.cube_ops = SegmentOps(torch.from_numpy(seg).to(self.dev), self.dev)
        self.data_ops = SegmentOps(torch.from_numpy(dseg).to(self.dev), self.dev)
        self.n = n
        self.plans = {}
        for key, vecname in (("pj", "p"), ("bpj", "a")):
            arr = (B.TgJob * n)()
            for k, (req, c, d, views) in enumerate(self.inflight):
                n1, n2, T = req.job.data_shape
                nd = n1 * n2 * T
                dv = self.data[d[0]:d[0] + nd].view(T, n1, n2).permute(1, 2, 0)
                cv = self.vec[vecname][c[0]:c[0] + int(np.prod(req.job.cube_shape))].view(*req.job.cube_shape)
                J = arr[k]
                J.map_header = S.pack_map_header(req.job.cube_header)
                J.views = views.data_ptr()
                J.n_views = T
                J.n1, J.n2 = n1, n2
                for a in range(3):
                    J.data_strides[a] = dv.stride()[a]
                    J.map_shape[a] = cv.shape[a]
                    J.map_strides[a] = cv.stride()[a]
                J.map_shape[3] = 1
                J.map_strides[3] = 0
                J.mask = None
                J.mask_dtype = _lib.TG_U8
                J.data = dv.data_ptr()
                J.map = cv.data_ptr()
            nbytes = self.L.tg_packed_plan_bytes(n)
            buf = torch.empty(nbytes, dtype=torch.uint8, device=self.dev)
            info = B.TgPackedInfo()
            _lib.check(self.L.tg_packed_plan(arr, n, self.rpw, 0, B._ptr(buf), nbytes, ctypes.byref(info)))
            self.plans[key] = (buf, info, arr)
        # per-job scalars: rr = r.r recomputed from the resident vectors (the
        # segmented dot of a segment does not depend on the other segments)
        self.rr = torch.zeros(n, dtype=torch.float64, device=self.dev)
        self.rr_new = torch.zeros_like(self.rr)
        self.pAp = torch.zeros_like(self.rr)
        self.cube_ops.dot(self.vec["r"], self.vec["r"], self.rr)
        self.bb = torch.tensor([max(req.bb, 1e-300) for req, *_ in self.inflight], dtype=torch.float64,
                               device=self.dev)
        self.dirty = False

    # one CG iteration for every in-flight job ----------------------------------
    def step(self):
        if self.dirty:
            self._rebuild()
        L, st, ops, v = self.L, B._stream(), self.cube_ops, self.vec
        ob = _lib.OBSTACLES[self.obstacle]
        self.data_ops.axpby(self.data, None, 0.0, 0.0)            # scratch = 0
        buf, info, _ = self.plans["pj"]
        _lib.check(L.tg_packed_projector(B._ptr(buf), ctypes.byref(info), _lib.TG_PJ, ob, st))   # P p
        ops.axpby(v["a"], None, 0.0, 0.0)
        buf, info, _ = self.plans["bpj"]
        _lib.check(L.tg_packed_projector(B._ptr(buf), ctypes.byref(info), _lib.TG_BPJ, ob, st))  # P^T P p
        if self.lam:
            ops.axpby(v["a"], v["p"], self.lam, 1.0)
        ops.dot(v["p"], v["a"], self.pAp)
        ops.update_x(v["x"], v["r"], v["p"], v["a"], self.rr, self.pAp)
        ops.dot(v["r"], v["r"], self.rr_new)
        ops.update_p(v["p"], v["r"], self.rr, self.rr_new)
        self.iterations += self.n
        for req, *_ in self.inflight:
            req.iters += 1

    def retire(self):
        """Move converged / exhausted jobs out; returns how many left."""
        rel = torch.sqrt(self.rr / self.bb).cpu().numpy()
        keep, done = [], []
        for k, item in enumerate(self.inflight):
            req = item[0]
            if rel[k] <= req.tol or req.iters >= req.max_iters:
                done.append((item, float(rel[k])))
            else:
                keep.append(item)
        for (req, c, d, views), res in done:
            nc = int(np.prod(req.job.cube_shape))
            req.result = self.vec["x"][c[0]:c[0] + nc].view(*req.job.cube_shape).cpu()
            req.residual = res
            req.t_done = time.perf_counter() - self.t_start
            self.cube_arena.release(*c)
            self.data_arena.release(*d)
            self.completed.append(req)
        if done:
            self.inflight = keep
            self.dirty = True
        return len(done)

    def _rays_inflight(self):
        return sum(int(np.prod(r.job.data_shape)) for r, *_ in self.inflight)

    def _admit(self, queue, now):
        """Admit queued requests: in arrival order while the in-flight rays stay
        under ``max_rays`` (one step is then a few tens of waves of the GPU, so
        a newcomer waits at most one such step) and memory allows; a request
        that does not fit is skipped by later, smaller ones (backfill) unless
        it has waited ``max_wait`` seconds, and it is always admitted into an
        empty server."""
        rays = self._rays_inflight()
        k = 0
        while k < len(queue):
            req = queue[k]
            need = int(np.prod(req.job.data_shape))
            if (not self.inflight or rays + need <= self.max_rays) and self.try_admit(req):
                queue.pop(k)
                rays += need
                continue
            if k == 0 and now - req.arrival >= self.max_wait:
                break  # the head has waited long enough: let the server drain for it
            k += 1

    def run(self, requests):
        """Serve ``requests`` (sorted by arrival time, seconds from now)."""
        pending = list(requests)
        queue = []
        self.t_start = time.perf_counter()
        while pending or queue or self.inflight:
            now = time.perf_counter() - self.t_start
            while pending and pending[0].arrival <= now:
                queue.append(pending.pop(0))
            self._admit(queue, now)
            if not self.inflight:
                if queue:
                    raise RuntimeError("request %d does not fit the memory budget" % queue[0].id)
                if pending:
                    time.sleep(max(0.0, pending[0].arrival - (time.perf_counter() - self.t_start)))
                continue
            self.step()
            self.retire()
        torch.cuda.synchronize()
        return summarize(self.completed, time.perf_counter() - self.t_start, self.iterations)


def summarize(done, wall, iterations):
    tts = np.array([r.t_done - r.arrival for r in done])
    return {"jobs": len(done), "wall_s": wall, "jobs_per_s": len(done) / wall, "cg_it_per_s": iterations / wall,
            "p50_s": float(np.percentile(tts, 50)), "p99_s": float(np.percentile(tts, 99)),
            "max_residual": float(max(r.residual for r in done))}


def fifo_plain(requests, lam=1e-2, obstacle="sun", device=None):
    """Baseline: requests served one at a time in arrival order with the plain
    single-job operator and CG (stopping at the same tolerance / budget)."""
    from . import cg, lo_wrapper
    dev = device or S._device()
    t_start = time.perf_counter()
    iterations = 0
    for req in requests:
        now = time.perf_counter() - t_start
        if req.arrival > now:
            time.sleep(req.arrival - now)
        op = lo_wrapper.siddon_lo(req.job.view_headers, req.job.cube_header, obstacle=obstacle, dtype=np.float32,
                                  device=dev)
        host = req.data if torch.is_tensor(req.data) else torch.from_numpy(np.ascontiguousarray(req.data))
        b = op.backproject(host.to(dev))
        res = cg.cg(cg.NormalOperator(op, lam=lam), b, maxiter=req.max_iters, tol=req.tol)
        req.result = res.x.cpu()
        req.residual = res.residuals[-1]
        req.iters = res.iterations
        iterations += res.iterations
        req.t_done = time.perf_counter() - t_start
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

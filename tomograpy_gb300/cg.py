"""Conjugate gradients on the GPU around the projector.

TomograPy solves its models with ``lo.acg`` (``tomograpy/srt.py:225``,
``tests/test_models.py:31``): CG on the regularised normal equations
(P^T P + sum_i h_i D_i^T D_i) x = P^T y, written out at
``exemples/test_siddon_cgs_secchi.py:32-33``, with D_i the finite differences
of ``lo.diff`` along each cube axis (``tomograpy/models.py:85-94``).  ``lo`` is
a third-party package absent from the reference tree; this module restates
textbook CG (Hestenes-Stiefel) for that system:

* vectors in float32 on the device; inner products and residual norms
  accumulated in float64 (``tg_segmented_dot_f32``, a fixed-order
  reduction), with the same kernels as the batched multi-job CG;
* scalars (alpha, beta, residual norms) stay on the device as 0-d tensors, so
  an iteration needs no host synchronisation and can be captured once in a
  CUDA graph and replayed (``graph=True``).
"""
import ctypes

import torch

from . import _lib


class Dot:
    """float64-accumulated inner products of float32 device vectors."""

    def __init__(self, device, n_slots=8):
        L = _lib.load()
        self.ws = torch.empty(L.tg_dot_workspace_bytes() // 8, dtype=torch.float64, device=device)
        self.out = torch.zeros(n_slots, dtype=torch.float64, device=device)

    def __call__(self, a, b, slot=0):
        L = _lib.load()
        a = a.reshape(-1)
        b = b.reshape(-1)
        if a.dtype != torch.float32 or b.dtype != torch.float32 or not (a.is_contiguous() and b.is_contiguous()):
            raise ValueError("dot takes contiguous float32 vectors")
        st = L.tg_dot_f32(ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()), a.numel(),
                          ctypes.c_void_p(self.out.data_ptr() + 8 * slot), ctypes.c_void_p(self.ws.data_ptr()),
                          self.ws.numel() * 8, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        _lib.check(st)
        return self.out[slot]


def diff_normal(x, axis):
    """D^T D x for the forward difference D along ``axis`` (lo.diff's operator)."""
    d = torch.diff(x, dim=axis)
    out = torch.zeros_like(x)
    n = x.shape[axis]
    out.narrow(axis, 0, n - 1).sub_(d)
    out.narrow(axis, 1, n - 1).add_(d)
    return out


class NormalOperator:
    """A x = P^T P x + lam x + sum_i h_i D_i^T D_i x (+ mu D_t^T D_t x for 4-D).

    ``P`` is a :class:`tomograpy_gb300.lo_wrapper.Siddon`; ``hypers`` are the
    h_i of the spatial finite-difference priors (axes 0..2), ``temporal`` the
    weight of the frame-difference prior of a 4-D cube (axis 3).
    """

    def __init__(self, P, lam=0.0, hypers=(), temporal=0.0):
        self.P = P
        self._ops, self._ops_n = None, 0
        self.lam = float(lam)
        self.hypers = tuple(float(h) for h in hypers)
        self.temporal = float(temporal)

    def __call__(self, x):
        y = self.P.project(x)
        out = self.P.backproject(y)
        if self.lam:
            if out.stride() == x.stride() and out.dtype == torch.float32 and dense(x):
                # out = lam x + out as one fmaf per element, the arithmetic of
                # the batched and served solvers (tg_segmented_axpby)
                if self._ops is None or self._ops_n != x.numel():
                    self._ops, self._ops_n = SegmentOps([0, x.numel()], x.device), x.numel()
                self._ops.axpby(out, x, self.lam, 1.0)
            else:
                out.add_(x, alpha=self.lam)
        for axis, h in enumerate(self.hypers):
            if h:
                out.add_(diff_normal(x, axis), alpha=h)
        if self.temporal and x.dim() == 4 and x.shape[3] > 1:
            out.add_(diff_normal(x, 3), alpha=self.temporal)
        return out


class CGResult:
    def __init__(self, x, iterations, residuals):
        self.x = x
        self.iterations = iterations
        self.residuals = residuals  # ||r_k|| / ||b||, float64 host list


class SegmentOps:
    """Inner products and CG vector updates over element ranges of flat
    float32 buffers (``tg_segmented_dot_f32``, ``tg_cg_update_x``,
    ``tg_cg_update_p``): one range for a single solve, one per job for the
    batched solves, so both run the same arithmetic."""

    def __init__(self, seg, device):
        from .batch import _bind
        self.L = _bind(_lib.load())
        self.seg = seg if torch.is_tensor(seg) else torch.tensor(seg, dtype=torch.int64, device=device)
        self.n = self.seg.numel() // 2
        nb = max(8, self.L.tg_segmented_workspace_bytes(self.n))
        self.ws = torch.empty(nb // 8, dtype=torch.float64, device=device)

    @staticmethod
    def _p(t):
        return ctypes.c_void_p(t.data_ptr())

    @staticmethod
    def _st():
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def dot(self, a, b, out):
        _lib.check(self.L.tg_segmented_dot_f32(self._p(a), self._p(b), self._p(self.seg), self.n, self._p(out),
                                               self._p(self.ws), self.ws.numel() * 8, self._st()))
        return out

    def update_x(self, x, r, p, Ap, rr, pAp):
        _lib.check(self.L.tg_cg_update_x(self._p(x), self._p(r), self._p(p), self._p(Ap), self._p(rr),
                                         self._p(pAp), self._p(self.seg), self.n, self._st()))

    def update_p(self, p, r, rr, rr_new):
        _lib.check(self.L.tg_cg_update_p(self._p(p), self._p(r), self._p(rr), self._p(rr_new), self._p(self.seg),
                                         self.n, self._st()))

    def axpby(self, y, x, alpha, beta):
        _lib.check(self.L.tg_segmented_axpby(self._p(y), None if x is None else self._p(x), alpha, beta,
                                             self._p(self.seg), self.n, self._st()))


def dense(t):
    """True when ``t`` covers its storage without gaps: contiguous after a
    permutation of its axes (e.g. a frame-major 4-D cube)."""
    order = sorted(range(t.dim()), key=lambda d: -t.stride(d))
    return t.permute(*order).is_contiguous()


def cg(A, b, x0=None, maxiter=10, tol=0.0, graph=False):
    """Solve A x = b (A symmetric positive definite, callable on device tensors).

    Runs ``maxiter`` iterations (stopping early on the host only when
    ``tol`` > 0 and ``graph`` is False).  Returns a :class:`CGResult`.
    Per iteration: alpha = rr / pAp, x += alpha p, r -= alpha Ap,
    beta = rr_new / rr, p = r + beta p (scalars in float64 on the device,
    vector updates as single float32 FMAs).
    """
    dev = b.device
    if b.dtype != torch.float32 or not dense(b):
        raise ValueError("cg takes a dense float32 right-hand side (contiguous up to a permutation of axes)")
    ops = SegmentOps([0, b.numel()], dev)
    # every vector shares b's layout (the vector kernels run on flat storage)
    x = torch.zeros_like(b) if x0 is None else torch.empty_like(b).copy_(x0)
    r = torch.empty_like(b).copy_(b - A(x)) if x0 is not None else b.clone()
    p = r.clone()
    rr = torch.zeros(1, dtype=torch.float64, device=dev)
    rr_new = torch.zeros_like(rr)
    pAp = torch.zeros_like(rr)
    bb = torch.zeros_like(rr)
    ops.dot(r, r, rr)
    ops.dot(b, b, bb)
    hist = torch.zeros(maxiter + 1, dtype=torch.float64, device=dev)
    hist[0] = torch.sqrt(rr / bb)[0]
    k_dev = torch.zeros((), dtype=torch.int64, device=dev)

    def step():
        Ap = A(p)
        if Ap.stride() != p.stride():  # the vector kernels run on flat storage
            Ap = torch.empty_like(p).copy_(Ap)
        ops.dot(p, Ap, pAp)
        ops.update_x(x, r, p, Ap, rr, pAp)
        ops.dot(r, r, rr_new)
        ops.update_p(p, r, rr, rr_new)
        k_dev.add_(1)
        hist.index_copy_(0, k_dev.view(1), torch.sqrt(rr / bb))

    if graph:
        # capture one iteration (after a warm-up on a side stream) and replay it
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        saved = (x.clone(), r.clone(), p.clone(), rr.clone(), hist.clone(), k_dev.clone())
        with torch.cuda.stream(s):
            step()
        torch.cuda.current_stream().wait_stream(s)
        x.copy_(saved[0]); r.copy_(saved[1]); p.copy_(saved[2]); rr.copy_(saved[3])
        hist.copy_(saved[4]); k_dev.copy_(saved[5])
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            step()
        for _ in range(maxiter):
            g.replay()
        its = maxiter
    else:
        its = 0
        for _ in range(maxiter):
            step()
            its += 1
            if tol > 0 and float(hist[its]) <= tol:
                break
    return CGResult(x, its, hist[: its + 1].cpu().tolist())

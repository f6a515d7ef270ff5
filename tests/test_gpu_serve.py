"""Continuous-batching server: overlap, memory admission and isolation.

Each request is CG on (P^T P + lam I) x = P^T y for its own geometry; the
server runs all in-flight requests' iterations together in packed launches.
A request's result must not depend on what else is in flight: it is compared
with the same request served alone and with the plain one-job-at-a-time loop
(the arithmetic is the same; float atomics in the backprojection differ in
order, whose effect after 10 CG iterations is ~1e-6, see test_gpu_batch)."""
import numpy as np
import pytest

from helpers import CUBE_TOL
from tomograpy_gb300 import serve, synthetic

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SPECS = [dict(n=24, T=7, N=40, d=200.0, lon_range=(0.1, 3.0)),
         dict(n=32, T=16, N=64, d=150.0, lon_range=(0.2, 5.0)),
         dict(n=16, T=5, N=32, d=230.0, lon_range=(0.3, 2.0)),
         dict(n=40, T=12, N=96, d=180.0, lon_range=(0.0, 6.0)),
         dict(n=20, T=9, N=48, d=210.0, lon_range=(0.5, 4.0))]
ITERS = 10


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def _requests(arrivals):
    reqs = serve.poisson_requests(SPECS, rate=1.0, seed=0, max_iters=ITERS, tol=1e-6)
    for r, t in zip(reqs, arrivals):
        r.arrival = t
    return reqs


def _alone(req, budget):
    r = serve.Request(req.id, req.job, req.data, 0.0, req.max_iters, req.tol)
    serve.Server(budget_bytes=budget).run([r])
    return r


def _close(a, b):
    a = a.numpy().astype(np.float64)
    b = b.numpy().astype(np.float64)
    return np.abs(a - b).max() <= CUBE_TOL * np.abs(b).max()


def test_requests_overlap_and_match_alone_and_plain():
    budget = 256 << 20
    reqs = _requests([0.0, 0.0, 0.001, 0.002, 0.003])
    srv = serve.Server(budget_bytes=budget)
    summ = srv.run(reqs)
    assert summ["jobs"] == len(SPECS)
    assert srv.max_inflight >= 2
    # work overlapped: some request was admitted before another one finished
    assert any(b.t_admit < a.t_done and a is not b for a in reqs for b in reqs)
    for r in reqs:
        assert r.iters == ITERS and np.isfinite(r.result.numpy()).all()
        assert _close(r.result, _alone(r, budget).result), r.id
    plain = _requests([0.0] * len(SPECS))
    serve.fifo_plain(plain)
    for r, p in zip(reqs, plain):
        assert p.iters == ITERS
        assert _close(r.result, p.result), r.id
    assert summ["p99_s"] >= summ["p50_s"] > 0


def test_admission_waits_for_device_memory():
    reqs = _requests([0.0] * len(SPECS))
    need = max(max(4 * np.prod(r.job.cube_shape) / 0.4, np.prod(r.job.data_shape) / 0.6) for r in reqs)
    budget = int(4 * need * 1.3)         # the largest job fits, not all of them at once
    srv = serve.Server(budget_bytes=budget)
    srv.run(reqs)
    assert len(srv.completed) == len(SPECS)
    assert 1 <= srv.max_inflight < len(SPECS)
    for r in reqs:
        assert _close(r.result, _alone(r, budget).result), r.id


def test_request_larger_than_budget_is_refused():
    reqs = _requests([0.0])[:1]
    srv = serve.Server(budget_bytes=4096)
    with pytest.raises(RuntimeError, match="does not fit"):
        srv.run(reqs)


def test_deterministic_serving_is_bitwise_isolated():
    """With fixed-point backprojections a served request's 20-iteration result
    is bitwise the same in the mix, served alone and in the FIFO plain loop."""
    budget = 256 << 20
    reqs = serve.poisson_requests(SPECS, rate=1.0, seed=0, max_iters=20, tol=0.0)
    for r, t in zip(reqs, [0.0, 0.0, 0.001, 0.002, 0.003]):
        r.arrival = t
    srv = serve.Server(budget_bytes=budget, deterministic=True)
    srv.run(reqs)
    assert srv.max_inflight >= 2
    plain = serve.poisson_requests(SPECS, rate=1.0, seed=0, max_iters=20, tol=0.0)
    for r in plain:
        r.arrival = 0.0
    serve.fifo_plain(plain, deterministic=True)
    for r, p in zip(reqs, plain):
        assert r.iters == 20 and p.iters == 20
        a = serve.Request(r.id, r.job, r.data, 0.0, 20, 0.0)
        serve.Server(budget_bytes=budget, deterministic=True).run([a])
        assert torch.equal(r.result, a.result), r.id
        assert torch.equal(r.result, p.result), r.id

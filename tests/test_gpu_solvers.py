"""GPU CG (float32 vectors, float64 reductions, CUDA-graph replay) and the
autograd projector, against float64 restatements driven by the oracle."""
import numpy as np
import pytest

import oracle
from helpers import CUBE_TOL, degenerate_rays
from tomograpy_gb300 import synthetic
from tomograpy_gb300.infoarray import InfoArray

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def small_geometry(n=24, T=12, N=40, lon=(0.1, 3.0)):
    return synthetic.make_geometry({"n": n, "T": T, "N": N, "d": 215.0, "lon_range": lon})


def oracle_P(vh, ch, shape_img, shape_cube):
    def P(x):
        d = InfoArray(shape=shape_img, header=[dict(h) for h in vh])
        oracle.projector(d, InfoArray(data=x.reshape(shape_cube), header=dict(ch)), obstacle="sun")
        return np.asarray(d)

    def PT(y):
        c = InfoArray(shape=shape_cube, header=dict(ch))
        oracle.backprojector(InfoArray(data=y.reshape(shape_img), header=[dict(h) for h in vh]), c, obstacle="sun")
        return np.asarray(c)
    return P, PT


def numpy_cg(A, b, iters):
    x = np.zeros_like(b)
    r = b.copy()
    p = r.copy()
    rr = float(np.vdot(r, r))
    for _ in range(iters):
        Ap = A(p)
        alpha = rr / float(np.vdot(p, Ap))
        x += alpha * p
        r -= alpha * Ap
        rr_new = float(np.vdot(r, r))
        p = r + (rr_new / rr) * p
        rr = rr_new
    return x


def test_dot_float64_accumulation():
    from tomograpy_gb300.cg import Dot
    dev = torch.device("cuda")
    rng = np.random.default_rng(0)
    for n in (1, 7, 1000, 1 << 20, (1 << 20) + 3):
        a = rng.standard_normal(n).astype(np.float32)
        b = rng.standard_normal(n).astype(np.float32)
        dot = Dot(dev)
        got = float(dot(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)))
        ref = float(np.dot(a.astype(np.float64), b.astype(np.float64)))
        assert abs(got - ref) <= 1e-12 * max(1.0, np.abs(a.astype(np.float64) * b).sum())
    # fixed reduction order: bitwise reproducible
    x = torch.from_numpy(rng.standard_normal(1 << 22).astype(np.float32)).to(dev)
    v1 = float(Dot(dev)(x, x))
    v2 = float(Dot(dev)(x, x))
    assert v1 == v2


def _problem():
    from tomograpy_gb300 import lo_wrapper
    ch, vh = small_geometry()
    degen = degenerate_rays(vh, 40, 40)
    assert not degen.any()
    x_true = synthetic.phantom(ch, seed=1).astype(np.float64) / 1e8
    P, PT = oracle_P(vh, ch, (40, 40, 12), (24, 24, 24))
    y = P(x_true)
    op = lo_wrapper.siddon_lo(vh, ch, obstacle="sun", dtype=np.float32)
    return ch, vh, x_true, y, P, PT, op


@pytest.mark.parametrize("graph", [False, True])
def test_cg_normal_equations_match_float64(graph):
    from tomograpy_gb300 import cg
    ch, vh, x_true, y, P, PT, op = _problem()
    lam = 1e-2
    b = PT(y)
    x_ref = numpy_cg(lambda v: PT(P(v)) + lam * v, b, 10)
    dev = torch.device("cuda")
    bt = torch.from_numpy(b.astype(np.float32)).to(dev)
    res = cg.cg(cg.NormalOperator(op, lam=lam), bt, maxiter=10, graph=graph)
    x = res.x.cpu().numpy().astype(np.float64)
    err = np.abs(x - x_ref).max() / np.abs(x_ref).max()
    assert err <= 1e-3, err
    assert res.residuals[-1] < res.residuals[0]


def test_cg_graph_equals_eager():
    from tomograpy_gb300 import cg, lo_wrapper
    ch, vh, x_true, y, P, PT, _ = _problem()
    op = lo_wrapper.siddon_lo(vh, ch, obstacle="sun", dtype=np.float32, deterministic=True)
    dev = torch.device("cuda")
    bt = torch.from_numpy(PT(y).astype(np.float32)).to(dev)
    A = cg.NormalOperator(op, lam=1e-2, hypers=(1e-3, 1e-3, 1e-3))
    r1 = cg.cg(A, bt, maxiter=6, graph=False)
    r2 = cg.cg(A, bt, maxiter=6, graph=True)
    np.testing.assert_array_equal(r1.x.cpu().numpy(), r2.x.cpu().numpy())
    np.testing.assert_allclose(r1.residuals, r2.residuals, rtol=0, atol=0)


def test_autograd_gradient_is_backprojected_residual():
    from tomograpy_gb300 import autograd
    ch, vh, x_true, y, P, PT, op = _problem()
    dev = torch.device("cuda")
    x0 = (0.5 * x_true).astype(np.float32)
    x = torch.from_numpy(x0).to(dev).requires_grad_(True)
    yt = torch.from_numpy(y.astype(np.float32)).to(dev)
    loss = 0.5 * ((autograd.project(x, op) - yt) ** 2).sum()
    loss.backward()
    g_ref = PT(P(x0.astype(np.float64)) - y)
    err = np.abs(x.grad.cpu().numpy() - g_ref).max() / np.abs(g_ref).max()
    assert err <= CUBE_TOL, err


def test_autograd_finite_differences_float64():
    from tomograpy_gb300 import autograd, lo_wrapper
    ch, vh = small_geometry(n=16, T=6, N=24)
    op = lo_wrapper.siddon_lo(vh, ch, obstacle="sun", dtype=np.float64)
    dev = torch.device("cuda")
    rng = np.random.default_rng(3)
    x = torch.from_numpy(rng.random((16, 16, 16))).to(dev).requires_grad_(True)
    y = torch.from_numpy(rng.random((24, 24, 6))).to(dev)

    def loss_of(v):
        return 0.5 * ((autograd.project(v, op) - y) ** 2).sum()

    loss = loss_of(x)
    loss.backward()
    g = x.grad.detach()
    idx = rng.integers(0, 16, size=(32, 3))
    h = 1e-3
    for i, j, k in idx:
        e = torch.zeros_like(x)
        e[i, j, k] = h
        with torch.no_grad():
            fd = (loss_of(x + e) - loss_of(x - e)) / (2 * h)
        assert abs(float(fd) - float(g[i, j, k])) <= 1e-6 * max(1.0, abs(float(fd)))


def test_backproject_autograd_is_projection():
    from tomograpy_gb300 import autograd
    ch, vh, x_true, y, P, PT, op = _problem()
    dev = torch.device("cuda")
    yt = torch.from_numpy(np.random.default_rng(2).random((40, 40, 12)).astype(np.float32)).to(dev)
    yt.requires_grad_(True)
    w = torch.from_numpy(np.random.default_rng(4).random((24, 24, 24)).astype(np.float32)).to(dev)
    (autograd.backproject(yt, op) * w).sum().backward()
    ref = P(w.cpu().numpy().astype(np.float64))
    err = np.abs(yt.grad.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err <= 1e-5, err


def test_lbfgs_reconstruction_decreases_loss():
    from tomograpy_gb300 import autograd
    ch, vh, x_true, y, P, PT, op = _problem()
    dev = torch.device("cuda")
    yt = torch.from_numpy(y.astype(np.float32)).to(dev)
    x, losses = autograd.reconstruct_lbfgs(op, yt, iters=15)
    assert losses[-1] < 0.05 * losses[0]
    assert float(x.min()) >= 0.0

"""Time-dependent (4-D) operator: view -> frame grouping, frame-major cube
storage and CG with the temporal smoothness term, against the oracle's
projector4d / backprojector4d (tomograpy/C_siddon.c.template:915-944, where
frame = view index) and a float64 CG on the same normal equations."""
import numpy as np
import pytest

import oracle
from helpers import CUBE_SIG, CUBE_TOL, IMG_TOL, image_errors
from tomograpy_gb300 import lo_wrapper, synthetic
from tomograpy_gb300.infoarray import InfoArray

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

NG = 3          # consecutive views per frame
F = 4           # frames
T = NG * F
N = 24
n = 12


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def _geometry():
    ch, vh = synthetic.make_geometry({"n": n, "T": T, "N": N, "d": 215.0, "lon_range": (0.2, 5.5),
                                      "n_frames": F})
    x = synthetic.phantom4d(ch, F, seed=3).astype(np.float64) / 1e8
    return ch, vh, x


def _expand(x):
    """Cube with one frame per view (the reference's 4-D convention)."""
    return np.repeat(x, NG, axis=3)


def _oracle_pj(ch, vh, x):
    d = InfoArray(shape=(N, N, T), header=[dict(h) for h in vh])
    oracle.projector4d(d, InfoArray(data=_expand(x), header=dict(ch)), obstacle="sun")
    return np.asarray(d)


def _oracle_bpj(ch, vh, y):
    c = InfoArray(shape=(n, n, n, T), header=dict(ch))
    oracle.backprojector4d(InfoArray(data=y, header=[dict(h) for h in vh]), c, obstacle="sun")
    return np.asarray(c).reshape(n, n, n, F, NG).sum(axis=4)


def test_grouped_frames_match_oracle():
    ch, vh, x = _geometry()
    op = lo_wrapper.siddon4d_lo(vh, ch, ng=NG, obstacle="sun", dtype=np.float32)
    y = op.project(torch.from_numpy(x.astype(np.float32)).cuda()).cpu().numpy()
    rel, norm = image_errors(y, _oracle_pj(ch, vh, x.astype(np.float32).astype(np.float64)))
    assert rel <= IMG_TOL and norm <= IMG_TOL, (rel, norm)
    yr = np.random.default_rng(0).random((N, N, T))
    c = op.backproject(torch.from_numpy(yr.astype(np.float32)).cuda()).cpu().numpy()
    rel, norm = image_errors(c, _oracle_bpj(ch, vh, yr.astype(np.float32).astype(np.float64)), sig=CUBE_SIG)
    assert rel <= CUBE_TOL and norm <= CUBE_TOL, (rel, norm)


def test_frame_major_storage():
    ch, vh, x = _geometry()
    op = lo_wrapper.siddon4d_lo(vh, ch, ng=NG, obstacle="sun", dtype=np.float32)
    c = op.new_cube()
    assert c.shape == (n, n, n, F) and c.stride(3) == n * n * n and c.stride(2) == 1
    # a C-ordered (reference layout) cube and its frame-major copy project alike
    xc = torch.from_numpy(x.astype(np.float32)).cuda()
    xf = op.new_cube().copy_(xc)
    torch.testing.assert_close(op.project(xc), op.project(xf), rtol=0, atol=0)
    assert op.backproject(op.project(xf)).stride() == c.stride()


def test_temporal_cg_matches_float64():
    from tomograpy_gb300 import cg
    ch, vh, x = _geometry()
    lam, mu, iters = 1e-2, 1e-2, 10
    y = _oracle_pj(ch, vh, x)

    def dtd(v):  # D_t^T D_t along the frame axis
        d = np.diff(v, axis=3)
        out = np.zeros_like(v)
        out[..., :-1] -= d
        out[..., 1:] += d
        return out

    def A(v):
        return _oracle_bpj(ch, vh, _oracle_pj(ch, vh, v)) + lam * v + mu * dtd(v)

    b = _oracle_bpj(ch, vh, y)
    xr = np.zeros_like(b)
    r = b.copy()
    p = r.copy()
    rr = float(np.vdot(r, r))
    for _ in range(iters):
        Ap = A(p)
        alpha = rr / float(np.vdot(p, Ap))
        xr += alpha * p
        r -= alpha * Ap
        rr_new = float(np.vdot(r, r))
        p = r + (rr_new / rr) * p
        rr = rr_new

    op = lo_wrapper.siddon4d_lo(vh, ch, ng=NG, obstacle="sun", dtype=np.float32)
    bt = op.backproject(torch.from_numpy(y.astype(np.float32)).cuda())
    for graph in (False, True):
        res = cg.cg(cg.NormalOperator(op, lam=lam, temporal=mu), bt, maxiter=iters, graph=graph)
        assert res.x.stride() == bt.stride()
        xg = res.x.cpu().numpy().astype(np.float64)
        err = np.abs(xg - xr).max() / np.abs(xr).max()
        assert err <= 1e-3, (graph, err)
        assert res.residuals[-1] < res.residuals[0]

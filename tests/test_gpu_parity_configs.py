"""GPU parity at the sizes the benchmark runs, against the float64 oracle.

* recon256: the 256^3 cube with the shell + blob phantom and 512 x 512 views
  of the 360-view circle at d = 215 (five of its views, spread over 0-360 deg,
  plus views at exactly lon = pi/2 and pi, whose central rows are degenerate
  and excluded as everywhere else; and the whole 360-view orbit): 214 voxel
  segments per ray on average, four times the chord of the 64^3 case;
* frames128: the 128^3 x 28-frame time-dependent geometry with 784 views of
  256 x 256 (view v in frame v // 28): the views of three frames, with their
  real frame numbers, traced into / out of a 28-frame cube;
* the 32-job uneven mix (cube edges 32-192, 64-512 px, d in [150, 230]),
  three views of each job traced in ONE packed launch, every job's slice
  compared with the oracle on that job alone;
* a request served in the continuous-batching server next to others, its CG
  iterate compared with float64 CG on the oracle's operator.

Tolerances as in tests/helpers.py (images 1e-5, cubes 1e-4; the packed
jobs' three-view backprojections are sparse and use the sampling-aware
per-voxel floor of helpers.cube_errors); the measured errors are appended to
$TG_PARITY_REPORT when that variable is set.
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle
import tomograpy_gb300 as tg
from helpers import (ADJ_TOL, CUBE_SIG, CUBE_TOL, IMG_TOL, cube_errors, degenerate_rays, image_errors, record,
                     rel_dot, worst_element)
from tomograpy_gb300 import batch, synthetic
from tomograpy_gb300.infoarray import InfoArray

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

THREADS = os.cpu_count() or 4


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def _hdrs(vh):
    return [dict(h) for h in vh]


def _oracle_pj(vh, ch, x, n1, n2, nthread=THREADS):
    ref = InfoArray(shape=(n1, n2, len(vh)), header=_hdrs(vh))
    oracle.projector(ref, InfoArray(data=np.asarray(x, np.float32).astype(np.float64), header=dict(ch)),
                     obstacle="sun", nthread=nthread)
    return np.asarray(ref)


def _oracle_bpj(vh, ch, y, shape, nthread=THREADS):
    ref = InfoArray(shape=shape, header=dict(ch))
    oracle.backprojector(InfoArray(data=np.asarray(y, np.float32).astype(np.float64), header=_hdrs(vh)), ref,
                         obstacle="sun", nthread=nthread)
    return np.asarray(ref)


# --------------------------------------------------------------------------
# 256^3 cube, 512 x 512 views

def test_recon256_views_against_oracle():
    cfg = synthetic.CONFIGS["recon256"]
    n, N = cfg["n"], cfg["N"]
    ch, vh_all = synthetic.make_geometry("recon256")
    pick = [0, 97, 180, 263, 359]
    vh = [vh_all[k] for k in pick] + synthetic.view_headers(2, N, d=cfg["d"], lons=[np.pi / 2, np.pi])
    T = len(vh)
    degen = degenerate_rays(vh, N, N)
    assert degen[:, :, 0].sum() == 0 and degen[:, :, -1].any() and degen[:, :, -2].any()
    x = synthetic.phantom(ch, seed=0)
    dev = torch.device("cuda")
    views = tg.siddon.upload_views(vh, None, dev)
    mh = tg.siddon.pack_map_header(ch)
    xt = torch.from_numpy(x).to(dev)
    y = torch.zeros((T, N, N), device=dev).permute(1, 2, 0)   # the benchmark's view-major layout
    tg.siddon.run_device("pj", y, xt, views, mh, T, obstacle="sun")
    ref = _oracle_pj(vh, ch, x, N, N)
    y = y.cpu().numpy()
    rel, norm = image_errors(y, ref, exclude=degen)
    record("recon256_pj", rel=rel, norm=norm, views=T, rays=N * N * T, worst=worst_element(y, ref, degen))
    assert rel <= IMG_TOL and norm <= IMG_TOL, (rel, norm)
    # backprojection of a random stack (degenerate rays zeroed on both sides)
    yy = np.random.default_rng(11).random((N, N, T)).astype(np.float32)
    yy[degen] = 0
    c = torch.zeros((n, n, n), device=dev)
    yt = torch.from_numpy(np.ascontiguousarray(yy.transpose(2, 0, 1))).to(dev).permute(1, 2, 0)
    tg.siddon.run_device("bpj", yt, c, views, mh, T, obstacle="sun")
    cref = _oracle_bpj(vh, ch, yy, (n, n, n))
    c = c.cpu().numpy()
    rel, norm = image_errors(c, cref, sig=CUBE_SIG)
    big = np.abs(cref) >= CUBE_SIG * np.abs(cref).max()
    worst = np.unravel_index(np.argmax(np.where(big, np.abs(c - cref) / np.maximum(np.abs(cref), 1e-300), 0)),
                             cref.shape)
    record("recon256_bpj", rel=rel, norm=norm, views=T, worst_voxel=[int(v) for v in worst],
           worst_value_frac=float(cref[worst] / np.abs(cref).max()),
           worst_abs_err=float(abs(c[worst] - cref[worst])))
    assert rel <= CUBE_TOL and norm <= CUBE_TOL, (rel, norm)


def test_recon256_full_orbit_against_oracle():
    """The benchmark's own configuration, every one of its 360 views: the
    phantom's projection and the backprojection of a random stack against the
    float64 oracle (~25 s of oracle time on 16 host cores)."""
    cfg = synthetic.CONFIGS["recon256"]
    n, N, T = cfg["n"], cfg["N"], cfg["T"]
    ch, vh = synthetic.make_geometry("recon256")
    degen = degenerate_rays(vh, N, N)
    x = synthetic.phantom(ch, seed=0)
    dev = torch.device("cuda")
    views = tg.siddon.upload_views(vh, None, dev)
    mh = tg.siddon.pack_map_header(ch)
    y = torch.zeros((T, N, N), device=dev).permute(1, 2, 0)
    tg.siddon.run_device("pj", y, torch.from_numpy(x).to(dev), views, mh, T, obstacle="sun")
    y = y.cpu().numpy()
    ref = _oracle_pj(vh, ch, x, N, N)
    rel, norm = image_errors(y, ref, exclude=degen)
    record("recon256_full_pj", rel=rel, norm=norm, views=T, worst=worst_element(y, ref, degen))
    assert rel <= IMG_TOL and norm <= IMG_TOL, (rel, norm)
    del ref
    yy = np.random.default_rng(14).random((N, N, T)).astype(np.float32)
    yy[degen] = 0
    c = torch.zeros((n, n, n), device=dev)
    yt = torch.from_numpy(np.ascontiguousarray(yy.transpose(2, 0, 1))).to(dev).permute(1, 2, 0)
    tg.siddon.run_device("bpj", yt, c, views, mh, T, obstacle="sun")
    c = c.cpu().numpy()
    # adjoint at the benchmark size: <P x, y> = <x, P^T y> (float64 dots of the
    # float32 GPU results)
    a = float(np.dot(y.astype(np.float64).ravel(), yy.astype(np.float64).ravel()))
    b = float(np.dot(x.astype(np.float64).ravel(), c.astype(np.float64).ravel()))
    record("recon256_full_adjoint", rel=rel_dot(a, b))
    assert rel_dot(a, b) <= ADJ_TOL, rel_dot(a, b)
    cref = _oracle_bpj(vh, ch, yy, (n, n, n))
    rel, norm = image_errors(c, cref, sig=CUBE_SIG)
    record("recon256_full_bpj", rel=rel, norm=norm, views=T)
    assert rel <= CUBE_TOL and norm <= CUBE_TOL, (rel, norm)


# --------------------------------------------------------------------------
# 128^3 x 28 frames, 256 x 256 views

def test_frames128_views_against_oracle():
    cfg = synthetic.CONFIGS["frames128"]
    n, N, F, T_all = cfg["n"], cfg["N"], cfg["n_frames"], cfg["T"]
    ch, vh_all = synthetic.make_geometry("frames128")
    per = T_all // F
    sel = [0, 13, 27]
    idx = [v for f in sel for v in range(f * per, (f + 1) * per)]
    vh = [vh_all[v] for v in idx]
    frames = np.array([v // per for v in idx])
    T = len(vh)
    degen = degenerate_rays(vh, N, N)
    # per-frame phantoms with the time-varying blob amplitudes of the workload
    rng = np.random.default_rng(1000)
    phases = rng.uniform(0, 2 * np.pi, 8)
    x4 = np.zeros((n, n, n, F), np.float32)
    for f in sel:
        x4[..., f] = synthetic.phantom(ch, 0, amplitudes=1.0 + 0.5 * np.sin(2 * np.pi * f / 14.0 + phases))
    dev = torch.device("cuda")
    views = tg.siddon.upload_views(vh, frames, dev)
    mh = tg.siddon.pack_map_header(ch)
    xt = torch.empty((F, n, n, n), device=dev).permute(1, 2, 3, 0)   # frame-major storage
    xt.copy_(torch.from_numpy(x4))
    y = torch.zeros((T, N, N), device=dev).permute(1, 2, 0)
    tg.siddon.run_device("pjt", y, xt, views, mh, T, obstacle="sun")
    y = y.cpu().numpy()
    yy = np.random.default_rng(12).random((N, N, T)).astype(np.float32)
    yy[degen] = 0
    c = torch.zeros((F, n, n, n), device=dev).permute(1, 2, 3, 0)
    tg.siddon.run_device("bpjt", torch.from_numpy(yy).to(dev), c, views, mh, T, obstacle="sun")
    c = c.cpu().numpy()
    ch3 = dict(ch)
    ch3["NAXIS"] = 3
    for k, f in enumerate(sel):
        s = slice(k * per, (k + 1) * per)
        ref = _oracle_pj(vh[s], ch3, x4[..., f], N, N)
        rel, norm = image_errors(y[:, :, s], ref, exclude=degen[:, :, s])
        record("frames128_pjt", frame=f, rel=rel, norm=norm, worst=worst_element(y[:, :, s], ref, degen[:, :, s]))
        assert rel <= IMG_TOL and norm <= IMG_TOL, (f, rel, norm)
        cref = _oracle_bpj(vh[s], ch3, yy[:, :, s], (n, n, n))
        rel, norm = image_errors(c[..., f], cref, sig=CUBE_SIG)
        record("frames128_bpjt", frame=f, rel=rel, norm=norm)
        assert rel <= CUBE_TOL and norm <= CUBE_TOL, (f, rel, norm)
    # frames that no selected view touches stay zero
    assert not c[..., 5].any()


# --------------------------------------------------------------------------
# the uneven 32-job mix in one packed launch

def _uneven_jobs(views_per_job=3):
    jobs = []
    for k, spec in enumerate(synthetic.uneven_specs(32, seed=0)):
        ch, vh = synthetic.make_geometry(spec)
        T = len(vh)
        keep = sorted({0, T // 2, T - 1})[:views_per_job]
        j = batch.Job(ch, [vh[v] for v in keep])
        j.phantom = synthetic.phantom(ch, seed=k) / np.float32(1e8)
        jobs.append(j)
    return jobs


def test_packed_uneven_mix_against_oracle():
    jobs = _uneven_jobs()
    pack = batch.PackedJobs(jobs, obstacle="sun", rows_per_warp=4)
    x = pack.new_cube()
    for k, j in enumerate(jobs):
        pack.cube_view(x, k).copy_(torch.from_numpy(j.phantom))
    pack.project(x)
    rng = np.random.default_rng(13)
    ys = []
    for j in jobs:
        yy = rng.random(j.data_shape).astype(np.float32)
        yy[degenerate_rays(j.view_headers, j.data_shape[0], j.data_shape[1])] = 0
        ys.append(yy)
    got_pj = [pack.data_view(pack.data, k).cpu().numpy() for k in range(len(jobs))]
    for k in range(len(jobs)):
        pack.data_view(pack.data, k).copy_(torch.from_numpy(ys[k]))
    z = pack.backproject(pack.new_cube())
    got_bpj = [pack.cube_view(z, k).cpu().numpy() for k in range(len(jobs))]

    def check(k):
        j = jobs[k]
        n1, n2, T = j.data_shape
        degen = degenerate_rays(j.view_headers, n1, n2)
        ref = _oracle_pj(j.view_headers, j.cube_header, j.phantom, n1, n2, nthread=T)
        r1 = image_errors(got_pj[k], ref, exclude=degen)
        cref = _oracle_bpj(j.view_headers, j.cube_header, ys[k], j.cube_shape, nthread=T)
        # three views per job: a sparse backprojection (see cube_errors)
        r2 = cube_errors(got_bpj[k], cref, float(ys[k].max()), float(j.cube_header["CDELT1"]))
        return r1, r2

    with ThreadPoolExecutor(max_workers=max(1, THREADS // 3)) as ex:
        results = list(ex.map(check, range(len(jobs))))
    for k, ((rel, norm), (crel, cnorm)) in enumerate(results):
        j = jobs[k]
        record("packed_uneven", job=k, n=j.cube_shape[0], N=j.data_shape[0], rel=rel, norm=norm, cube_rel=crel,
               cube_norm=cnorm)
        assert rel <= IMG_TOL and norm <= IMG_TOL, (k, rel, norm)
        assert crel <= CUBE_TOL and cnorm <= CUBE_TOL, (k, crel, cnorm)


# --------------------------------------------------------------------------
# a served request against float64 CG on the oracle's operator

SERVE_SPECS = [dict(n=24, T=7, N=40, d=200.0, lon_range=(0.1, 3.0)),
               dict(n=32, T=16, N=64, d=150.0, lon_range=(0.2, 5.0)),
               dict(n=16, T=5, N=32, d=230.0, lon_range=(0.3, 2.0)),
               dict(n=40, T=12, N=96, d=180.0, lon_range=(0.0, 6.0))]


def test_served_request_against_oracle_cg():
    from tomograpy_gb300 import serve
    iters, lam = 10, 1e-2
    reqs = serve.poisson_requests(SERVE_SPECS, rate=1e6, seed=0, max_iters=iters, tol=0.0)
    srv = serve.Server(budget_bytes=256 << 20)
    srv.run(reqs)
    assert srv.max_inflight >= 2
    for r in reqs[:2]:
        assert r.iters == iters
        j = r.job
        n1, n2, T = j.data_shape
        y = r.data.numpy().astype(np.float64)

        def A(v):
            ref = InfoArray(shape=(n1, n2, T), header=_hdrs(j.view_headers))
            oracle.projector(ref, InfoArray(data=v.reshape(j.cube_shape), header=dict(j.cube_header)),
                             obstacle="sun")
            c = InfoArray(shape=j.cube_shape, header=dict(j.cube_header))
            oracle.backprojector(InfoArray(data=np.asarray(ref), header=_hdrs(j.view_headers)), c, obstacle="sun")
            return np.asarray(c) + lam * v

        b = _oracle_bpj(j.view_headers, j.cube_header, y, j.cube_shape)
        x = np.zeros_like(b)
        res = b.copy()
        p = res.copy()
        rr = float(np.vdot(res, res))
        for _ in range(iters):
            Ap = A(p)
            alpha = rr / float(np.vdot(p, Ap))
            x += alpha * p
            res -= alpha * Ap
            rr_new = float(np.vdot(res, res))
            p = res + (rr_new / rr) * p
            rr = rr_new
        got = r.result.numpy().astype(np.float64)
        err = np.abs(got - x).max() / np.abs(x).max()
        record("served_cg", request=r.id, iters=iters, rel=err)
        assert err <= 1e-3, (r.id, err)

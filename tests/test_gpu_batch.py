"""Packed multi-job launches and batched CG against the single-job path."""
import numpy as np
import pytest

from helpers import CUBE_SIG, CUBE_TOL, image_errors
from tomograpy_gb300 import batch, lo_wrapper, synthetic

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SPECS = [dict(n=24, T=7, N=40, d=200.0, lon_range=(0.1, 3.0)),
         dict(n=32, T=16, N=64, d=150.0, lon_range=(0.2, 5.0)),
         dict(n=16, T=5, N=32, d=230.0, lon_range=(0.3, 2.0)),
         dict(n=40, T=12, N=96, d=180.0, lon_range=(0.0, 6.0))]


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def _pack(rpw=None):
    jobs = [synthetic.make_job(s, seed=k) for k, s in enumerate(SPECS)]
    return jobs, batch.PackedJobs(jobs, obstacle="sun", rows_per_warp=rpw)


@pytest.mark.parametrize("rpw", [1, 2, 4])
def test_packed_projection_equals_single_job(rpw):
    jobs, pack = _pack(rpw)
    x = pack.new_cube()
    for k, j in enumerate(jobs):
        pack.cube_view(x, k).copy_(torch.from_numpy(j.phantom))
    pack.project(x)
    for k, j in enumerate(jobs):
        op = lo_wrapper.siddon_lo(j.view_headers, j.cube_header, obstacle="sun", dtype=np.float32)
        ref = op.project(torch.from_numpy(j.phantom).cuda())
        # same rays, same arithmetic: bitwise equal whatever the tile shape
        torch.testing.assert_close(pack.data_view(pack.data, k), ref, rtol=0, atol=0)


def test_packed_backprojection_matches_single_job():
    jobs, pack = _pack()
    rng = np.random.default_rng(3)
    for k, j in enumerate(jobs):
        pack.data_view(pack.data, k).copy_(torch.from_numpy(rng.random(j.data_shape).astype(np.float32)))
    z = pack.backproject(pack.new_cube())
    for k, j in enumerate(jobs):
        op = lo_wrapper.siddon_lo(j.view_headers, j.cube_header, obstacle="sun", dtype=np.float32)
        ref = op.backproject(pack.data_view(pack.data, k).contiguous())
        rel, norm = image_errors(pack.cube_view(z, k).cpu().numpy(), ref.cpu().numpy(), sig=CUBE_SIG)
        assert rel <= CUBE_TOL and norm <= CUBE_TOL, (k, rel, norm)


# Float32 CG on these small sun-occulted systems amplifies rounding with the
# iteration count, and the backprojection's float atomics make two plain runs
# of the same job differ by ~3e-6 after 10 iterations and ~1e-3 after 20.
# The batched solver runs the same per-job arithmetic (same kernels, same
# dots and updates), so its iterates are compared with the plain loop's at 10
# iterations against the cube tolerance.
CG_ITERS = 10


def test_batched_cg_matches_sequential_and_is_isolated():
    jobs, pack = _pack()
    x_true = pack.new_cube()
    for k, j in enumerate(jobs):
        pack.cube_view(x_true, k).copy_(torch.from_numpy(j.phantom))
    pack.project(x_true)
    b = pack.backproject(pack.new_cube())
    x, hist = batched_cg(pack, b)
    seq = batch.sequential_cg(jobs, [pack.cube_view(b, k).clone() for k in range(len(jobs))], iters=CG_ITERS)
    for k in range(len(jobs)):
        xk = pack.cube_view(x, k).cpu().numpy().astype(np.float64)
        sk = seq[k].cpu().numpy().astype(np.float64)
        assert np.abs(xk - sk).max() <= CUBE_TOL * np.abs(sk).max(), k
    h = hist.cpu().numpy()
    assert np.all(h[-1] < h[0])
    # isolation: job 1 alone in a pack of one gives the same iterates
    alone = batch.PackedJobs([jobs[1]], obstacle="sun", rows_per_warp=pack.rows_per_warp)
    ba = alone.new_cube()
    ba.copy_(pack.cube_view(b, 1).reshape(-1))
    xa, _ = batched_cg(alone, ba)
    d = np.abs(xa.cpu().numpy() - pack.cube_view(x, 1).reshape(-1).cpu().numpy()).max()
    assert d <= CUBE_TOL * np.abs(xa.cpu().numpy()).max()


def batched_cg(pack, b):
    return batch.batched_cg(pack, b, lam=1e-2, iters=CG_ITERS, graph=True)


def test_packed_time_dependent_jobs_match_single_job():
    """Time-dependent jobs of different sizes and frame groupings in one pack:
    the packed 4-D projection equals each job's own 4-D operator bitwise, the
    backprojection within the cube tolerance."""
    specs = [(dict(n=16, T=6, N=32, d=200.0, lon_range=(0.1, 3.0), n_frames=3), 2),
             (dict(n=24, T=8, N=48, d=180.0, lon_range=(0.4, 5.0), n_frames=2), 4)]
    jobs, ops = [], []
    for k, (sp, ng) in enumerate(specs):
        ch, vh = synthetic.make_geometry(sp)
        frames = np.arange(sp["T"]) // ng
        j = batch.Job(ch, vh, frames=frames)
        j.phantom = synthetic.phantom4d(ch, sp["n_frames"], seed=k) / np.float32(1e8)
        jobs.append(j)
        ops.append(lo_wrapper.siddon4d_lo(vh, ch, ng=ng, obstacle="sun", dtype=np.float32))
    pack = batch.PackedJobs(jobs, obstacle="sun", rows_per_warp=2)
    assert pack.four_d
    x = pack.new_cube()
    for k, j in enumerate(jobs):
        assert pack.cube_view(x, k).shape == j.cube_shape
        pack.cube_view(x, k).copy_(torch.from_numpy(j.phantom))
    pack.project(x)
    for k, j in enumerate(jobs):
        ref = ops[k].project(torch.from_numpy(j.phantom).cuda())
        torch.testing.assert_close(pack.data_view(pack.data, k), ref, rtol=0, atol=0)
    z = pack.backproject(pack.new_cube())
    for k, j in enumerate(jobs):
        ref = ops[k].backproject(pack.data_view(pack.data, k).contiguous())
        rel, norm = image_errors(pack.cube_view(z, k).cpu().numpy(), ref.cpu().numpy(), sig=CUBE_SIG)
        assert rel <= CUBE_TOL and norm <= CUBE_TOL, (k, rel, norm)


# --------------------------------------------------------------------------
# deterministic (fixed-point) backprojection: bitwise isolation

def test_packed_deterministic_backprojection_equals_single_job_bitwise():
    """tg_packed_backprojector_deterministic gives every job exactly the
    single-job deterministic backprojection (3-D and time-dependent packs)."""
    jobs, pack = _pack(2)
    rng = np.random.default_rng(4)
    for k, j in enumerate(jobs):
        pack.data_view(pack.data, k).copy_(torch.from_numpy(rng.random(j.data_shape).astype(np.float32)))
    z = pack.backproject(pack.new_cube(), deterministic=True)
    for k, j in enumerate(jobs):
        op = lo_wrapper.siddon_lo(j.view_headers, j.cube_header, obstacle="sun", dtype=np.float32, deterministic=True)
        ref = op.backproject(pack.data_view(pack.data, k).contiguous())
        assert torch.equal(pack.cube_view(z, k), ref), k
    # time-dependent jobs: frame-major 4-D accumulators
    specs = [(dict(n=16, T=6, N=32, d=200.0, lon_range=(0.1, 3.0), n_frames=3), 2),
             (dict(n=24, T=8, N=48, d=180.0, lon_range=(0.4, 5.0), n_frames=2), 4)]
    jobs4, ops4 = [], []
    for sp, ng in specs:
        ch, vh = synthetic.make_geometry(sp)
        jobs4.append(batch.Job(ch, vh, frames=np.arange(sp["T"]) // ng))
        ops4.append(lo_wrapper.siddon4d_lo(vh, ch, ng=ng, obstacle="sun", dtype=np.float32, deterministic=True))
    pack4 = batch.PackedJobs(jobs4, obstacle="sun", rows_per_warp=1)
    for k, j in enumerate(jobs4):
        pack4.data_view(pack4.data, k).copy_(torch.from_numpy(rng.random(j.data_shape).astype(np.float32)))
    z4 = pack4.backproject(pack4.new_cube(), deterministic=True)
    for k in range(len(jobs4)):
        ref = ops4[k].backproject(pack4.data_view(pack4.data, k).contiguous())
        assert torch.equal(pack4.cube_view(z4, k), ref), k


def test_deterministic_cg_is_bitwise_isolated():
    """With fixed-point backprojections, a job's 20th CG iterate is bitwise
    the same in a batch of four, alone in a batch and in the plain per-job
    loop (the float-atomic path differs by up to ~1e-2 at 20 iterations)."""
    jobs, pack = _pack()
    x_true = pack.new_cube()
    for k, j in enumerate(jobs):
        pack.cube_view(x_true, k).copy_(torch.from_numpy(j.phantom))
    pack.project(x_true)
    b = pack.backproject(pack.new_cube(), deterministic=True)
    x, _ = batch.batched_cg(pack, b, lam=1e-2, iters=20, graph=True, deterministic=True)
    seq = batch.sequential_cg(jobs, [pack.cube_view(b, k).clone() for k in range(len(jobs))], iters=20,
                              deterministic=True)
    for k in range(len(jobs)):
        assert torch.equal(pack.cube_view(x, k), seq[k]), k
    alone = batch.PackedJobs([jobs[3]], obstacle="sun", rows_per_warp=pack.rows_per_warp)
    ba = alone.new_cube()
    ba.copy_(pack.cube_view(b, 3).reshape(-1))
    xa, _ = batch.batched_cg(alone, ba, lam=1e-2, iters=20, graph=False, deterministic=True)
    assert torch.equal(xa, pack.cube_view(x, 3).reshape(-1))


# --------------------------------------------------------------------------
# tile schedules of the autotuner

@pytest.mark.parametrize("sched", [(2, 0, 0), (4, 0, 0), (1, 1, 16), (4, 0, 16)])
def test_packed_schedules_match_single_job(sched):
    """Lanes along gamma trace the same rays with the same arithmetic
    (bitwise-equal projections); 16-step batches regroup the walk's
    roundings (projection within the image tolerance, backprojection within
    the cube tolerance).  One job of the pack has views rolled by 90 degrees,
    the case gamma-major lanes are for."""
    from helpers import IMG_TOL
    specs = SPECS[:3]
    jobs = [synthetic.make_job(s, seed=k) for k, s in enumerate(specs)]
    ch, vh = synthetic.make_geometry(dict(n=24, T=5, N=48, d=190.0, lon_range=(0.2, 2.5)))
    for h in vh:
        h["ROL"] = np.pi / 2
        for key in [k for k in h if k.startswith("R") and "_" in k]:
            del h[key]
    rolled = batch.Job(ch, vh)
    rolled.phantom = synthetic.phantom(ch, seed=9) / np.float32(1e8)
    jobs.append(rolled)
    pack = batch.PackedJobs(jobs, obstacle="sun", schedule=sched)
    x = pack.new_cube()
    for k, j in enumerate(jobs):
        pack.cube_view(x, k).copy_(torch.from_numpy(j.phantom))
    pack.project(x)
    rng = np.random.default_rng(6)
    ys = []
    for k, j in enumerate(jobs):
        op = lo_wrapper.siddon_lo(j.view_headers, j.cube_header, obstacle="sun", dtype=np.float32)
        ref = op.project(torch.from_numpy(j.phantom).cuda())
        got = pack.data_view(pack.data, k)
        if sched[2] == 0:
            torch.testing.assert_close(got, ref, rtol=0, atol=0)
        else:
            rel, norm = image_errors(got.cpu().numpy(), ref.cpu().numpy())
            assert rel <= IMG_TOL and norm <= IMG_TOL, (k, rel, norm)
        ys.append(rng.random(j.data_shape).astype(np.float32))
    for k in range(len(jobs)):
        pack.data_view(pack.data, k).copy_(torch.from_numpy(ys[k]))
    z = pack.backproject(pack.new_cube())
    for k, j in enumerate(jobs):
        op = lo_wrapper.siddon_lo(j.view_headers, j.cube_header, obstacle="sun", dtype=np.float32)
        ref = op.backproject(torch.from_numpy(ys[k]).cuda())
        rel, norm = image_errors(pack.cube_view(z, k).cpu().numpy(), ref.cpu().numpy(), sig=CUBE_SIG)
        assert rel <= CUBE_TOL and norm <= CUBE_TOL, (k, rel, norm)


def test_autotune_searches_schedules():
    jobs, _ = _pack(4)
    batch.PackedJobs._tune_cache.clear()
    pack = batch.PackedJobs(jobs, obstacle="sun")
    table = pack.tune_table
    assert batch.DEFAULT_SCHEDULE in table and pack.schedule in table
    assert {(1, 1, 0), (2, 1, 0), (4, 1, 0)} <= set(table)
    assert any(k[1] == 0 for k in table) and any(k[2] == 16 for k in table)
    assert table[pack.schedule] == min(table.values())

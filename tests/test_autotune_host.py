"""Host logic of the packed-launch autotuner (``batch.PackedJobs.autotune``)
with the timing replaced by a cost table: the coordinate-descent order
(rows per warp on lambda lanes, then the lane axis, then the batch length),
the choice of the fastest schedule, and the cache per job-size signature.
CPU only."""
import pytest

torch = pytest.importorskip("torch")

from tomograpy_gb300 import batch  # noqa: E402


class _Job:
    def __init__(self, cube_shape, data_shape):
        self.cube_shape, self.data_shape = cube_shape, data_shape


def _pack(costs, shapes=((16, 16, 16), (32, 32, 4))):
    """A PackedJobs whose schedule timings come from ``costs`` (no GPU)."""
    p = batch.PackedJobs.__new__(batch.PackedJobs)
    p.jobs = [_Job(shapes[0], shapes[1])]
    p.obstacle = "sun"
    p._plans = {}
    p.timed = []
    p.new_cube = lambda: torch.zeros(8)

    def fake_time(sched, x, z, repeats):
        p.timed.append(sched)
        return costs[sched]
    p._time = fake_time
    return p


ALL = [(1, 1, 0), (2, 1, 0), (4, 1, 0), (1, 0, 0), (2, 0, 0), (4, 0, 0), (1, 1, 16), (2, 1, 16), (4, 1, 16),
       (1, 0, 16), (2, 0, 16), (4, 0, 16)]


@pytest.fixture(autouse=True)
def _clear_cache():
    batch.PackedJobs._tune_cache.clear()
    yield
    batch.PackedJobs._tune_cache.clear()


def test_coordinate_descent_order_and_choice():
    costs = {s: 10.0 for s in ALL}
    costs[(2, 1, 0)] = 5.0      # best rows per warp on lambda lanes
    costs[(2, 0, 0)] = 4.0      # gamma lanes better still
    costs[(2, 0, 16)] = 3.0     # and 16-step batches on top
    p = _pack(costs)
    assert p.autotune() == (2, 0, 16)
    assert p.timed == [(1, 1, 0), (2, 1, 0), (4, 1, 0), (2, 0, 0), (2, 0, 16)]
    assert p.tune_table == {s: costs[s] for s in p.timed}


def test_keeps_the_default_when_nothing_is_faster():
    costs = {s: 10.0 for s in ALL}
    costs[(4, 1, 0)] = 1.0
    p = _pack(costs)
    assert p.autotune() == (4, 1, 0)
    # each later coordinate tried once, from the best so far
    assert p.timed == [(1, 1, 0), (2, 1, 0), (4, 1, 0), (4, 0, 0), (4, 1, 16)]


def test_cached_per_signature():
    costs = {s: 10.0 for s in ALL}
    costs[(1, 1, 0)] = 1.0
    p = _pack(costs)
    assert p.autotune() == (1, 1, 0)
    q = _pack({s: 0.0 for s in ALL})           # same job sizes: no timing at all
    assert q.autotune() == (1, 1, 0) and q.timed == [] and q.tune_table == p.tune_table
    r = _pack({s: 0.0 for s in ALL}, shapes=((16, 16, 16), (32, 32, 5)))   # another signature
    r.autotune()
    assert r.timed

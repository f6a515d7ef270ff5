"""Host logic of the serving loop: first-fit arena and request bookkeeping."""
import numpy as np

from tomograpy_gb300.serve import Arena, summarize


def test_first_fit_alloc_release_merge():
    a = Arena(1024)
    r1 = a.alloc(100)      # rounded up to 128
    r2 = a.alloc(200)      # 256
    r3 = a.alloc(64)
    assert r1 == (0, 128) and r2 == (128, 256) and r3 == (384, 64)
    assert a.alloc(1024) is None
    a.release(*r2)
    assert a.alloc(300) == (448, 320)      # the 256 hole is too small: first fit after r3
    r4 = a.alloc(256)
    assert r4 == (128, 256)                # reuses the hole
    a.release(*r1)
    a.release(*r4)
    a.release(*r3)
    assert a.free[0] == (0, 448)           # neighbours merged
    a.release(448, 320)
    assert a.free == [(0, 1024)]


def test_arena_random_sequence_never_overlaps():
    rng = np.random.default_rng(0)
    a = Arena(1 << 16)
    live = []
    for _ in range(2000):
        if live and rng.random() < 0.45:
            a.release(*live.pop(int(rng.integers(len(live)))))
        else:
            r = a.alloc(int(rng.integers(1, 4000)))
            if r is not None:
                live.append(r)
        spans = sorted(live + a.free)
        pos = 0
        for st, ln in spans:
            assert st == pos and ln > 0
            pos = st + ln
        assert pos == 1 << 16


class _R:
    def __init__(self, arrival, done, residual):
        self.arrival, self.t_done, self.residual = arrival, done, residual


def test_summary_percentiles():
    done = [_R(0.0, 1.0 + k, 1e-3) for k in range(100)]
    s = summarize(done, wall=10.0, iterations=2000)
    assert s["jobs"] == 100 and s["jobs_per_s"] == 10.0 and s["cg_it_per_s"] == 200.0
    assert abs(s["p50_s"] - 50.5) < 1e-9 and s["p99_s"] > 99.0

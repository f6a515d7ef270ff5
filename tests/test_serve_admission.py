"""Admission policy of the serving loop (``serve.Server._admit``) on the host,
with memory admission replaced by a byte budget: shortest job first among
young requests, oldest first once a request has waited ``max_wait``, no
admission past an old request that does not fit, the in-flight ray bound,
and an empty server always taking its first candidate.  CPU only."""
import pytest

pytest.importorskip("torch")

from tomograpy_gb300 import serve  # noqa: E402


class _Job:
    def __init__(self, rays):
        self.data_shape = (rays, 1, 1)


class _Req:
    def __init__(self, rid, rays, arrival):
        self.id, self.job, self.arrival = rid, _Job(rays), arrival


class _Slot:
    def __init__(self, req):
        self.req, self.nd = req, req.job.data_shape[0]


def _server(max_rays=100, max_wait=1.0, memory=10**9):
    s = serve.Server.__new__(serve.Server)
    s.inflight = []
    s.max_rays = max_rays
    s.max_wait = max_wait
    s.admitted = []

    def try_admit(req):            # memory admission: a byte budget
        used = sum(j.nd for j in s.inflight)
        if used + req.job.data_shape[0] > memory:
            return False
        s.inflight.append(_Slot(req))
        s.admitted.append(req.id)
        return True
    s.try_admit = try_admit
    return s


def test_young_requests_shortest_first_within_the_ray_bound():
    s = _server(max_rays=100)
    queue = [_Req(0, 60, 0.0), _Req(1, 10, 0.1), _Req(2, 30, 0.2), _Req(3, 50, 0.3)]
    s._admit(queue, now=0.5)
    assert s.admitted == [1, 2, 3]          # 10 + 30 + 50 <= 100; 60 would pass the bound
    assert [r.id for r in queue] == [0]


def test_old_request_goes_first_and_is_not_bypassed():
    s = _server(max_rays=100, memory=100)
    s.inflight.append(_Slot(_Req(9, 50, 0.0)))             # 50 rays already in flight
    queue = [_Req(0, 80, 0.0), _Req(1, 10, 1.5), _Req(2, 20, 1.6)]
    s._admit(queue, now=2.0)                               # request 0 has waited 2 s
    assert s.admitted == []                                # it does not fit: nothing passes it
    assert [r.id for r in queue] == [0, 1, 2]
    s.inflight.clear()                                     # the server drains
    s._admit(queue, now=2.1)
    assert s.admitted == [0, 1]                            # the old one first, then the shortest young


def test_old_requests_oldest_first():
    s = _server(max_rays=1000)
    queue = [_Req(0, 300, 0.5), _Req(1, 100, 0.2), _Req(2, 5, 1.9)]
    s._admit(queue, now=2.0)
    assert s.admitted == [1, 0, 2]          # 1 and 0 are old (by arrival), then 2 (young)


def test_empty_server_takes_a_large_first_request():
    s = _server(max_rays=100)
    queue = [_Req(0, 500, 0.0), _Req(1, 20, 0.1)]
    s._admit(queue, now=0.2)
    assert s.admitted == [1]                # shortest first: the small one
    s.inflight.clear()
    s._admit(queue, now=0.3)
    assert s.admitted == [1, 0]             # alone, a request above the ray bound is admitted

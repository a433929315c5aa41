"""Scheduling logic of the serving loop, on the CPU with a fake executor:
admission by memory budget, rejection, chunking of large transmission
spectroscopy requests, round-robin work items, completion and statistics."""
import threading
import time

import numpy as np
import pytest

from pytransit_gb300.serving import RRServer, request_bytes, shape_request, work_items, Request


class FakeExecutor:
    """Completes a request one step after its last items were issued."""

    def __init__(self, setup_delay=0.0):
        self.log = []
        self.lock = threading.Lock()
        self.max_inflight_bytes = 0
        self.setup_delay = setup_delay

    def setup(self, req, ts_chunk_bytes):
        if self.setup_delay:
            time.sleep(self.setup_delay)     # the other requests are queued meanwhile
        self.log.append(('setup', req.rid))

    def step(self, batch, ts):
        self.log.append(('step', [(r.rid, tuple(w)) for r, ws in batch for w in ws], [r.rid for r in ts]))

    def start_copy(self, req):
        req.state['copy_at'] = len(self.log)

    def poll_copy(self, req):
        shape = (req.npv, req.npb_out, req.npt) if req.kind == 'ts' else (req.npv, req.npt)
        return np.full(shape, float(req.rid))

    def release(self, req):
        self.log.append(('release', req.rid))

    def shutdown(self):
        pass


def rr_req(npv, npt):
    return dict(time=np.linspace(0, 1, npt)), dict(k=np.full((npv, 1), 0.1), ldc=[0.3, 0.1], t0=np.zeros(npv),
                                                   p=np.full(npv, 2.0), a=5.0, i=1.5, e=0.0, w=0.0)


def test_work_items_cover_everything_once():
    for npv, npt in [(1, 10), (3, 128 * 300 + 5), (100, 1000), (4096, 500)]:
        items = work_items(npv, npt)
        ntiles = (npt + 127) // 128
        cover = np.zeros((npv, ntiles), int)
        for pv0, pv1, t0, t1 in items:
            cover[pv0:pv1, t0:t1] += 1
        assert (cover == 1).all()


def test_request_bytes_grow_with_size():
    a = Request('rr', 'quadratic', *rr_req(10, 1000))
    b = Request('rr', 'quadratic', *rr_req(100, 1000))
    shape_request(a), shape_request(b)
    assert request_bytes(b) > request_bytes(a) > 10 * 1000 * 4


def test_admission_by_budget_and_completion():
    ex = FakeExecutor()
    one = Request('rr', 'quadratic', *rr_req(64, 5000))
    shape_request(one)
    budget = int(request_bytes(one) * 2.5)        # room for two at a time
    srv = RRServer(executor=ex, hbm_budget=budget, step_items=8)
    futs = [srv.submit('rr', 'quadratic', *rr_req(64, 5000)) for _ in range(6)]
    res = [f.result(timeout=10) for f in futs]
    srv.close()
    for i, r in enumerate(res):
        assert r.shape == (64, 5000) and r[0, 0] == i
    st = srv.stats.summary()
    assert st['completed'] == 6 and st['rejected'] == 0
    assert st['peak_hbm_bytes'] <= budget
    assert st['p99_s'] >= st['p50_s'] >= 0


def test_requests_share_steps_round_robin():
    ex = FakeExecutor(setup_delay=0.05)
    srv = RRServer(executor=ex, hbm_budget=1e12, step_items=6)
    futs = [srv.submit('rr', 'quadratic', *rr_req(40, 128 * 10)) for _ in range(3)]
    [f.result(timeout=10) for f in futs]
    srv.close()
    steps = [e for e in ex.log if e[0] == 'step']
    mixed = [s for s in steps if len({rid for rid, _ in s[1]}) > 1]
    assert mixed, "items of several requests should share a step"
    for s in steps:
        assert len(s[1]) <= 6


def test_rejects_what_can_never_fit():
    ex = FakeExecutor()
    srv = RRServer(executor=ex, hbm_budget=1e6)
    f = srv.submit('rr', 'quadratic', *rr_req(1000, 100000))
    with pytest.raises(MemoryError):
        f.result(timeout=5)
    srv.close()
    assert srv.stats.rejected == 1


def test_large_ts_request_is_admitted_in_chunks():
    ex = FakeExecutor()
    data = dict(time=np.linspace(-0.1, 0.1, 20000))
    params = dict(k=np.full((400, 200), 0.1), ldc=np.tile([0.3, 0.1], (400, 200, 1)), t0=np.zeros(400),
                  p=np.full(400, 2.0), a=np.full(400, 5.0), i=np.full(400, 1.5), e=np.zeros(400), w=np.zeros(400))
    srv = RRServer(executor=ex, hbm_budget=2e9, ts_chunk_bytes=1e9)
    f = srv.submit('ts', 'quadratic', data, params)
    out = f.result(timeout=10)
    srv.close()
    assert out.shape == (400, 200, 20000)
    assert srv.stats.peak_bytes <= 2e9


def test_unknown_law_and_kind():
    srv = RRServer(executor=FakeExecutor())
    with pytest.raises(ValueError):
        srv.submit('rr', 'no-such-law', *rr_req(1, 10))
    with pytest.raises(ValueError):
        srv.submit('xx', 'quadratic', *rr_req(1, 10))
    srv.close()

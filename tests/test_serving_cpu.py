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
        return np.broadcast_to(np.float64(req.rid), shape)    # a view: no memory for large shapes

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


class FailingExecutor(FakeExecutor):
    """Raises in set-up, step or poll for the requests whose npv is in the
    matching set; everything else completes normally."""

    def __init__(self, fail_setup=(), fail_step=(), fail_poll=()):
        super().__init__()
        self.fail_setup, self.fail_step, self.fail_poll = set(fail_setup), set(fail_step), set(fail_poll)
        self.released = []

    def setup(self, req, ts_chunk_bytes):
        if req.npv in self.fail_setup:
            raise RuntimeError(f"set-up of {req.rid} failed")
        super().setup(req, ts_chunk_bytes)

    def step(self, batch, ts):
        if any(r.npv in self.fail_step for r, _ in batch) or any(r.npv in self.fail_step for r in ts):
            raise RuntimeError("launch failed")
        super().step(batch, ts)

    def poll_copy(self, req):
        if req.npv in self.fail_poll:
            raise RuntimeError(f"copy of {req.rid} failed")
        return super().poll_copy(req)

    def release(self, req):
        self.released.append(req.rid)
        super().release(req)


@pytest.mark.parametrize("where", ["setup", "poll"])
def test_executor_failure_fails_only_its_request(where):
    ex = FailingExecutor(**{f"fail_{where}": {7}})
    srv = RRServer(executor=ex, hbm_budget=1e12, step_items=4)
    good = [srv.submit('rr', 'quadratic', *rr_req(5, 1000)) for _ in range(3)]
    bad = srv.submit('rr', 'quadratic', *rr_req(7, 1000))
    later = srv.submit('rr', 'quadratic', *rr_req(5, 1000))
    with pytest.raises(RuntimeError):
        bad.result(timeout=10)
    for f in good + [later]:
        assert f.result(timeout=10).shape == (5, 1000)
    srv.close()
    st = srv.stats.summary()
    assert st['failed'] >= 1 and st['rejected'] == 0
    assert st['completed'] + st['failed'] == 5
    assert srv._used == 0                         # every admitted byte was given back
    if where == "poll":
        assert 3 in ex.released                   # the failed request (the fourth, rid 3) was released


def test_step_failure_fails_the_whole_step_and_the_loop_goes_on():
    """A launch that raises fails every request with items in that step (their
    device state is unknown); requests admitted later are served."""
    gate = threading.Event()

    class Held(FailingExecutor):
        def setup(self, req, ts_chunk_bytes):
            gate.wait(10)                          # both requests queue up, then join one step
            super().setup(req, ts_chunk_bytes)

    ex = Held(fail_step={9})
    srv = RRServer(executor=ex, hbm_budget=1e12, step_items=64)
    fs = [srv.submit('rr', 'quadratic', *rr_req(9, 500)), srv.submit('rr', 'quadratic', *rr_req(4, 500))]
    gate.set()
    for f in fs:
        with pytest.raises(RuntimeError):
            f.result(timeout=10)
    ok = srv.submit('rr', 'quadratic', *rr_req(3, 500))
    assert ok.result(timeout=10).shape == (3, 500)
    srv.close()
    assert srv.stats.failed == 2 and srv.stats.completed == 1
    assert sorted(ex.released) == [0, 1, 2]
    assert srv._used == 0


def test_cancelled_while_queued_is_dropped():
    gate = threading.Event()

    class Slow(FakeExecutor):
        def setup(self, req, ts_chunk_bytes):
            gate.wait(10)
            super().setup(req, ts_chunk_bytes)

    ex = Slow()
    srv = RRServer(executor=ex, hbm_budget=1e12)
    first = srv.submit('rr', 'quadratic', *rr_req(2, 300))
    time.sleep(0.05)                               # the loop is inside first's set-up
    second = srv.submit('rr', 'quadratic', *rr_req(2, 300))
    assert second.cancel()
    gate.set()
    assert first.result(timeout=10).shape == (2, 300)
    assert second.cancelled()
    srv.close()
    st = srv.stats.summary()
    assert st['cancelled'] == 1 and st['completed'] == 1 and st['failed'] == 0
    assert ('setup', 1) not in ex.log
    # a running request can no longer be cancelled
    assert not first.cancel()


def test_small_requests_pass_a_blocked_head_until_it_has_waited():
    """A big request that does not fit yet must not hold back small ones that
    do; once it has waited hol_max_wait_s nothing passes it any more."""
    gate = threading.Event()

    class Gate(FakeExecutor):
        def poll_copy(self, req):
            if req.npv == 50 and not gate.is_set():
                return None                        # the first big request runs until the gate opens
            return super().poll_copy(req)

    big = Request('rr', 'quadratic', *rr_req(50, 20000))
    shape_request(big)
    budget = int(request_bytes(big) * 1.5)         # one big request at a time
    ex = Gate()
    srv = RRServer(executor=ex, hbm_budget=budget, hol_max_wait_s=0.3)
    f_big1 = srv.submit('rr', 'quadratic', *rr_req(50, 20000))
    time.sleep(0.05)
    f_big2 = srv.submit('rr', 'quadratic', *rr_req(50, 20000))     # blocked behind big1
    small = [srv.submit('rr', 'quadratic', *rr_req(1, 500)) for _ in range(3)]
    for f in small:
        assert f.result(timeout=5).shape == (1, 500)               # passed the blocked head
    assert not f_big2.done()
    assert srv.stats.bypassed >= 3
    time.sleep(0.35)                               # big2 has now waited longer than hol_max_wait_s
    late = srv.submit('rr', 'quadratic', *rr_req(1, 500))
    time.sleep(0.1)
    assert not late.done()                         # memory is kept for the head
    gate.set()
    assert f_big1.result(timeout=5).shape == (50, 20000)
    assert f_big2.result(timeout=5).shape == (50, 20000)
    assert late.result(timeout=5).shape == (1, 500)
    srv.close()
    assert srv.stats.peak_bytes <= budget


def test_step_items_is_checked_at_construction():
    with pytest.raises(ValueError):
        RRServer(executor=FakeExecutor(), step_items=10 ** 6)
    with pytest.raises(ValueError):
        RRServer(executor=FakeExecutor(), step_items=0)


def test_submit_after_close_raises():
    srv = RRServer(executor=FakeExecutor())
    srv.close()
    with pytest.raises(RuntimeError):
        srv.submit('rr', 'quadratic', *rr_req(1, 10))


def test_served_future_carries_the_error_bound():
    class Bounded(FakeExecutor):
        def poll_copy(self, req):
            req.state['error_bound'] = 1e-7 * req.npv
            return super().poll_copy(req)

    srv = RRServer(executor=Bounded())
    f = srv.submit('rr', 'quadratic', *rr_req(3, 100))
    f.result(timeout=5)
    srv.close()
    assert f.error_bound == pytest.approx(3e-7)


def test_ts_work_items_slices_match_the_whole():
    from pytransit_gb300.serving import ts_work_items
    for npv, npt in [(1, 10), (5, 128 * 33 + 1), (37, 100000)]:
        items = ts_work_items(npv, npt)
        whole = items[:]
        assert whole.shape == (len(items), 4) and whole.dtype == np.int32
        ntiles = (npt + 127) // 128
        cover = np.zeros((npv, ntiles), int)
        for pv0, pv1, t0, t1 in whole:
            assert pv1 == pv0 + 1 and 0 < t1 - t0 <= 16
            cover[pv0:pv1, t0:t1] += 1
        assert (cover == 1).all()
        c = len(items) // 3
        np.testing.assert_array_equal(np.concatenate([items[:c], items[c:2 * c], items[2 * c:]]), whole)

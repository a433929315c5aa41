"""Serving loop: continuous batching of RoadRunner evaluations on one GB300.

Requests (a light curve set, a population of parameter vectors, an LD law;
plain RoadRunner or transmission spectroscopy) arrive from any thread via
``submit`` and get a ``concurrent.futures.Future`` for their flux.  One
scheduler thread owns the GPU:

* admission: a request enters when its device memory (data, tables,
  workspace, output) fits the HBM budget; requests that can never fit are
  rejected, transmission-spectroscopy requests too large as a whole are run in
  parameter-vector chunks;
* set-up per admitted request on the GPU: FP32-pair times and tile summaries,
  LD tables, and the prologue (LD means, orbit, bounding boxes), kept on the
  device until the request finishes;
* steps: every step takes up to ``step_items`` work items (request, pv range,
  tile range) from all admitted requests, round-robin, and runs them in one
  persistent kernel launch (rr_serve_flux_split) replayed from a captured CUDA
  graph; requests admitted while a step runs join the next one, so work from
  many requests overlaps on the device;
* completion: a request whose last items ran is copied to pinned host memory
  on a copy stream and its future resolved; latency = resolve - submit;
* failures: an exception in a request's set-up, in a step or in a copy fails
  the futures of the requests concerned (``stats.failed``; memory refusals
  count as ``stats.rejected``) and the loop goes on serving the others; a
  future cancelled while queued is dropped at admission.

The GPU work is behind ``GpuExecutor`` so that the scheduling logic can be
exercised on the CPU with a fake executor (tests/test_serving_cpu.py).
"""
import bisect
import collections
import concurrent.futures as cf
import gc
import ctypes as C
import itertools
import threading
import time
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import ldmodels as _ldm

__all__ = ['Request', 'RRServer', 'GpuExecutor', 'ServerStats', 'ServedFuture']

TILE = 128
TS_ITEM_TILES = 16     # tiles per work item of a transmission-spectroscopy request (<= 32)

# rr_serve_request (include/pytransit_gb300.h), field by field
SERVE_REQUEST_DTYPE = np.dtype([('times_ff', 'u8'), ('lcids', 'u8'), ('orb32', 'u8'), ('lc32', 'u8'), ('ldm', 'u8'),
                                ('flux', 'u8'), ('ldflux', 'i8'), ('npt', 'i4'), ('npv', 'i4'), ('nlc', 'i4'),
                                ('npb', 'i4'), ('ng', 'i4'), ('kind', 'i4'), ('inv_dg', 'f4'), ('exptime0', 'f4'),
                                ('dg', 'f8'), ('nsamples0', 'i4'), ('pad', 'i4')])


# rr_serve_setup_args (include/pytransit_gb300.h), field by field, all 8 bytes
SETUP_ARGS_DTYPE = np.dtype(
    [(n, 'u8') for n in ('stage', 'dst')] + [('n_in', 'i8')] +
    [(n, 'u8') for n in ('time', 'lcids', 'pbids', 'epids', 'nsamples', 'exptimes', 'k', 't0', 'p', 'a', 'inc', 'e',
                         'w', 'ldc', 'times_ff', 'ldp', 'istar', 'ws', 'bnd', 'bmax', 'flux', 'mu', 'basis',
                         'weights', 'z_edges')] +
    [(n, 'i8') for n in ('npt', 'npv', 'nlc', 'npb', 'nep', 'nkc', 'npar', 'law', 'nb', 'nk', 'nz', 'ng', 'ldflux',
                         'wsb', 'nsamples0')] +
    [(n, 'f8') for n in ('t_ref', 't_abs', 'dk', 'kmin', 'kmax', 'dg', 'exptime0')] +
    [(n, 'u8') for n in ('bound_host', 'desc')])


@dataclass
class Request:
    """One evaluation.  kind 'rr' (flux[npv, npt]) or 'ts' (flux[npv, npb, npt]).
    data: time, lcids, pbids, nsamples, exptimes, epids (as set_data);
    params: k, ldc, t0, p, a, i, e, w (as evaluate)."""
    kind: str
    ld: str
    data: dict
    params: dict
    rid: int = -1
    t_submit: float = 0.0
    t_admit: float = 0.0
    t_done: float = 0.0
    future: Optional[cf.Future] = None
    # filled at admission
    npv: int = 0
    npt: int = 0
    npb_out: int = 1
    nbytes: int = 0
    state: dict = field(default_factory=dict)

    @property
    def points(self) -> int:
        return self.npv * self.npt * self.npb_out


@dataclass
class ServerStats:
    """Counters of a server.  ``rejected``: requests refused for memory (larger
    than the budget or the arena); ``failed``: requests whose set-up, launch or
    copy raised; ``cancelled``: futures the caller cancelled while queued;
    ``bypassed``: admissions that passed a blocked request at the head of the
    queue.  Time of the scheduler thread (seconds): ``admit_s`` in admission
    and per-request set-up, ``step_s`` in issuing steps, ``poll_s`` in
    completions; ``gpu_step_s``: device time of the finished batched steps
    (CUDA events around each step's kernel)."""
    submitted: int = 0
    admitted: int = 0
    completed: int = 0
    rejected: int = 0
    failed: int = 0
    cancelled: int = 0
    bypassed: int = 0
    steps: int = 0
    points: int = 0
    peak_bytes: int = 0
    max_queue: int = 0
    admit_s: float = 0.0
    step_s: float = 0.0
    poll_s: float = 0.0
    gpu_step_s: float = 0.0
    latencies: list = field(default_factory=list)
    done_times: list = field(default_factory=list)

    def summary(self):
        lat = np.array(self.latencies) if self.latencies else np.zeros(1)
        return dict(submitted=self.submitted, admitted=self.admitted, completed=self.completed,
                    rejected=self.rejected, failed=self.failed, cancelled=self.cancelled, bypassed=self.bypassed,
                    steps=self.steps, points=self.points, peak_hbm_bytes=self.peak_bytes,
                    max_queue=self.max_queue, admit_s=self.admit_s, step_s=self.step_s, poll_s=self.poll_s,
                    gpu_step_s=self.gpu_step_s, p50_s=float(np.percentile(lat, 50)),
                    p99_s=float(np.percentile(lat, 99)), mean_s=float(lat.mean()))


class ServedFuture(cf.Future):
    """The future of one request.  Besides the result it carries
    ``error_bound``: the request's maximum absolute flux error against the
    FP64 model, set before the result (None where the executor states none)."""

    def __init__(self):
        super().__init__()
        self.error_bound = None


def shape_request(req: Request):
    """Normalise the arrays of a request (host side, no GPU)."""
    d, p = req.data, req.params
    time_ = np.asarray(d['time'], np.float64)
    npt = time_.size
    lcids = np.asarray(d.get('lcids', np.zeros(npt, int)), np.int32)
    nlc = int(lcids.max()) + 1 if npt else 1
    pbids = np.asarray(d.get('pbids', np.zeros(nlc, int)), np.int32)
    epids = np.asarray(d.get('epids', np.zeros(nlc, int)), np.int32)
    ns = np.broadcast_to(np.asarray(d.get('nsamples', 1), np.int32), (nlc,)).copy()
    ex = np.broadcast_to(np.asarray(d.get('exptimes', 0.0), np.float64), (nlc,)).copy()
    pv = np.atleast_1d(np.asarray(p['p'], np.float64))
    npv = pv.size
    k = np.asarray(p['k'], np.float64)
    k = k.reshape(npv, -1)
    ldc = np.asarray(p['ldc'], np.float64)
    npb = int(pbids.max()) + 1 if req.kind == 'rr' else k.shape[1]
    ldc = np.ascontiguousarray(np.broadcast_to(ldc.reshape(-1, npb, ldc.shape[-1]) if ldc.ndim > 1 else
                                               ldc.reshape(1, 1, -1), (npv, npb, ldc.shape[-1])))
    t0 = np.asarray(p['t0'], np.float64).reshape(npv, -1)
    vec = {n: np.ascontiguousarray(np.broadcast_to(np.atleast_1d(np.asarray(p[n], np.float64)), (npv,)))
           for n in ('a', 'i', 'e', 'w')}
    req.npv, req.npt = npv, npt
    req.npb_out = k.shape[1] if req.kind == 'ts' else 1
    # the time range for the split path's reference time, on the caller's
    # thread rather than the scheduler's
    tmin, tmax = (float(time_.min()), float(time_.max())) if npt else (0.0, 0.0)
    req.state['host'] = dict(time=time_, lcids=lcids, pbids=pbids, epids=epids, nsamples=ns, exptimes=ex,
                             k=np.ascontiguousarray(k), ldc=ldc, t0=np.ascontiguousarray(t0), p=pv, nlc=nlc,
                             npb=npb, tmin=tmin, tmax=tmax, **vec)
    return req


def request_bytes(req: Request, ng: int = 100, nz: int = 40) -> int:
    """Device bytes a request holds while admitted (data, tables, output)."""
    h = req.state['host']
    npv, npt, npb, nlc = req.npv, req.npt, h['npb'], h['nlc']
    data = npt * (8 + 4 + 8) + (npt // TILE + 1) * 16 + nlc * 24
    params = npv * (8 * (h['k'].shape[1] + h['t0'].shape[1] + 5) + 8 * npb * h['ldc'].shape[2])
    tables = npv * npb * (nz + 1) * 4 + npv * (64 + nlc * 64 + npb * ng * 4) + 4096
    if req.kind == 'ts':
        tables += npv * npb * (16 + ng * 4) + npv * 160
    out = npv * req.npb_out * ((npt + 3) // 4 * 4) * 4
    return int(data + params + tables + out)


def _layout(parts):
    """Byte offsets (256-byte aligned) of named parts in one buffer, and its size."""
    off, cur = {}, 0
    for name, nbytes in parts:
        cur = (cur + 255) & ~255
        off[name] = cur
        cur += int(nbytes)
    return off, max(cur, 256)


class _DeviceArena:
    """The serving loop's device memory: one allocation made when the server
    starts, sized to the HBM budget plus headroom, from which every admitted
    request takes one contiguous block (first fit, 256-byte aligned, freed
    blocks merged with their neighbours).  No cudaMalloc/cudaFree while
    serving."""

    def __init__(self, torch, device, nbytes):
        self.size = int(nbytes) & ~255
        self.buf = torch.empty(self.size, dtype=torch.uint8, device=device)
        self.base = self.buf.data_ptr()
        self.free_list = [(0, self.size)]     # (offset, size), sorted by offset
        self.used = 0

    def alloc(self, n):
        n = (int(n) + 255) & ~255
        for j, (o, sz) in enumerate(self.free_list):
            if sz >= n:
                if sz == n:
                    del self.free_list[j]
                else:
                    self.free_list[j] = (o + n, sz - n)
                self.used += n
                return o
        return None

    def free(self, o, n):
        n = (int(n) + 255) & ~255
        self.used -= n
        fl = self.free_list
        j = bisect.bisect_left(fl, (o, 0))
        fl.insert(j, (o, n))
        if j + 1 < len(fl) and fl[j][0] + fl[j][1] == fl[j + 1][0]:
            fl[j] = (fl[j][0], fl[j][1] + fl[j + 1][1])
            del fl[j + 1]
        if j > 0 and fl[j - 1][0] + fl[j - 1][1] == fl[j][0]:
            fl[j - 1] = (fl[j - 1][0], fl[j - 1][1] + fl[j][1])
            del fl[j]


class _PinnedRing:
    """Pinned host staging for request uploads, used as a ring: a region is
    handed out again once the event recorded after its copy has completed."""

    def __init__(self, torch, nbytes):
        self.buf = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        self.np = self.buf.numpy()
        self.size = nbytes
        self.head = 0
        self.live = collections.deque()       # (start, end, event) in allocation order

    def alloc(self, n):
        """Offset of n free bytes, or None if n does not fit the ring."""
        n = (n + 255) & ~255
        if n > self.size:
            return None
        if self.head + n > self.size:
            self.head = 0
        lo, hi = self.head, self.head + n
        last = None
        for a, b, ev in self.live:
            if a < hi and lo < b:
                last = ev
        if last is not None:
            last.synchronize()
        while self.live and self.live[0][2].query():
            self.live.popleft()
        self.head = hi
        return lo

    def commit(self, lo, n, event):
        self.live.append((lo, lo + ((n + 255) & ~255), event))


class WorkItems:
    """The work items of one request, rows (pv0, pv1, tile0, tile1) (int32),
    computed for the slice a step takes rather than kept per request: a large
    request has hundreds of thousands of items.  Either every item is one pv
    and a range of `per` tiles (`by_tiles`), or a range of `per` pvs over all
    tiles."""

    def __init__(self, npv: int, ntiles: int, per: int, by_tiles: bool):
        self.npv, self.ntiles, self.per, self.by_tiles = npv, ntiles, per, by_tiles
        self.nt = -(-ntiles // per) if by_tiles else 1           # items per pv
        self.n = npv * self.nt if by_tiles else -(-npv // per)
        # a short list is cheaper kept whole than computed slice by slice
        self._rows = self._make(slice(None)) if self.n <= 4096 else None

    def __len__(self):
        return self.n

    def __getitem__(self, sl):
        return self._rows[sl] if self._rows is not None else self._make(sl)

    def _make(self, sl):
        i = np.arange(*sl.indices(self.n), dtype=np.int64)
        out = np.empty((i.size, 4), np.int32)
        if self.by_tiles:
            pv, t = np.divmod(i, self.nt)
            t *= self.per
            out[:, 0] = pv
            out[:, 1] = pv + 1
            out[:, 2] = t
            np.minimum(t + self.per, self.ntiles, out=t)
            out[:, 3] = t
        else:
            pv0 = i * self.per
            out[:, 0] = pv0
            np.minimum(pv0 + self.per, self.npv, out=pv0)
            out[:, 1] = pv0
            out[:, 2] = 0
            out[:, 3] = self.ntiles
        return out

    def __iter__(self):
        return iter(self[:])


def ts_work_items(npv: int, npt: int, tiles: int = TS_ITEM_TILES) -> WorkItems:
    """Items (pv, pv + 1, tile0, tile1) of at most `tiles` tiles each, for a
    transmission-spectroscopy request: every tile writes all its channel
    rows, so an item is one pv and a short tile range."""
    return WorkItems(npv, max(1, (npt + TILE - 1) // TILE), tiles, True)


def work_items(npv: int, npt: int, target_tiles: int = 256) -> WorkItems:
    """Items (pv0, pv1, tile0, tile1) of about target_tiles pv-tiles each."""
    ntiles = max(1, (npt + TILE - 1) // TILE)
    if ntiles >= target_tiles:
        return WorkItems(npv, ntiles, target_tiles, True)
    return WorkItems(npv, ntiles, max(1, target_tiles // ntiles), False)


class RRServer:
    """Continuous-batching server (see the module docstring)."""

    def __init__(self, executor=None, hbm_budget: float = 120e9, step_items: int = 4096,
                 ts_chunk_bytes: float = 4e9, device=None, result: str = 'host', freeze_gc: bool = True,
                 hol_max_wait_s: float = 0.1, admit_scan: int = 64):
        """freeze_gc: move every object that exists when the server starts (the
        imported modules of torch, numpy, ...) out of the cyclic garbage
        collector's generations (gc.freeze), so that a full collection during
        serving scans only the objects made since, not pausing every thread
        for tens of milliseconds.

        Admission is in arrival order, except that a request at the head of the
        queue that does not fit yet lets later requests that fit pass it (up to
        ``admit_scan`` requests deep) until it has waited ``hol_max_wait_s``;
        from then on nothing passes it, so the memory that running requests
        give back goes to it."""
        step_items = int(step_items)
        max_items = getattr(executor, 'MAX_ITEMS', GpuExecutor.MAX_ITEMS)
        if not 1 <= step_items <= max_items:
            raise ValueError(f"step_items must be in [1, {max_items}], got {step_items}")
        self.ex = executor if executor is not None else GpuExecutor(
            device, result=result, arena_bytes=int(hbm_budget * 1.1) + (1 << 30))
        if freeze_gc:
            gc.collect()
            gc.freeze()
        self.budget = int(hbm_budget)
        self.step_items = step_items
        self.ts_chunk_bytes = ts_chunk_bytes
        self.hol_max_wait_s = float(hol_max_wait_s)
        self.admit_scan = max(1, int(admit_scan))
        self.stats = ServerStats()
        self._ids = itertools.count()
        self._queue = collections.deque()
        self._active = collections.OrderedDict()
        self._issued = collections.OrderedDict()     # all GPU work enqueued, result pending
        self._ts_new = []
        self._used = 0
        self._cv = threading.Condition()
        self._stop = False
        self._thread = threading.Thread(target=self._loop, name="rr-server", daemon=True)
        self._thread.start()

    # -- client side ------------------------------------------------------
    def submit(self, kind: str, ld: str, data: dict, params: dict, keep_result: bool = True) -> cf.Future:
        """Queue one evaluation.  The future resolves to the flux (numpy in
        pinned host memory, or a CUDA tensor with result='device'); with
        keep_result=False to the number of model points, the flux being
        dropped as soon as it is complete (for consumers that only time or
        count)."""
        if kind not in ('rr', 'ts'):
            raise ValueError("kind must be 'rr' or 'ts'")
        if ld not in _ldm.LAW_IDS:
            raise ValueError(f"unknown limb darkening law {ld}")
        req = Request(kind=kind, ld=ld, data=data, params=params)
        req.state['keep'] = keep_result
        req.future = ServedFuture()
        req.rid = next(self._ids)
        req.t_submit = time.perf_counter()
        shape_request(req)
        req.nbytes = request_bytes(req)
        with self._cv:
            if self._stop:
                raise RuntimeError("the server is closed")
            self.stats.submitted += 1
            if self._min_bytes(req) > self.budget:
                self.stats.rejected += 1
                req.future.set_exception(MemoryError(
                    f"request {req.rid} needs {self._min_bytes(req) / 1e9:.1f} GB of device memory, "
                    f"more than the {self.budget / 1e9:.1f} GB budget"))
                return req.future
            self._queue.append(req)
            self.stats.max_queue = max(self.stats.max_queue, len(self._queue))
            self._cv.notify()
        return req.future

    def close(self, wait: bool = True):
        with self._cv:
            self._stop = True
            self._cv.notify()
        if wait:
            self._thread.join()

    def drain(self, timeout: float = None):
        """Wait until every submitted request has finished."""
        t0 = time.perf_counter()
        while True:
            with self._cv:
                if not self._queue and not self._active and not self._issued:
                    return True
            if timeout is not None and time.perf_counter() - t0 > timeout:
                return False
            time.sleep(0.001)

    def load(self):
        """The server's load now: queued requests, admitted requests and the
        device bytes they hold against the budget."""
        with self._cv:
            return dict(queued=len(self._queue), active=len(self._active), admitted_bytes=self._used,
                        budget_bytes=self.budget)

    # -- scheduler ----------------------------------------------------------
    def _min_bytes(self, req):
        if req.kind == 'ts' and req.nbytes > self.ts_chunk_bytes and getattr(self.ex, 'result', 'host') == 'host':
            per_pv = req.nbytes / max(req.npv, 1)
            return int(per_pv * max(1, int(self.ts_chunk_bytes // per_pv)))
        return req.nbytes

    def _admit(self):
        """Admit queued requests while the budget allows, in arrival order.  A
        request that does not fit yet (budget, or device memory fragmented)
        keeps its place; later requests that fit may pass it until the
        request at the head has waited hol_max_wait_s.  A request whose
        future the caller cancelled is dropped here."""
        pos = 0                        # queue position of the next candidate
        while True:
            with self._cv:
                if pos >= len(self._queue) or pos >= self.admit_scan:
                    return
                head = self._queue[0]
                if pos > 0 and time.perf_counter() - head.t_submit > self.hol_max_wait_s:
                    return             # the head has waited long enough: memory is kept for it
                req = self._queue[pos]
                if req.future.cancelled():
                    del self._queue[pos]
                    self.stats.cancelled += 1
                    continue
                need = self._min_bytes(req)
                if self._used + need > self.budget:
                    pos += 1
                    continue
                if not req.state.get('running'):
                    # from here on the caller can no longer cancel it
                    if not req.future.set_running_or_notify_cancel():
                        del self._queue[pos]
                        self.stats.cancelled += 1
                        continue
                    req.state['running'] = True
                del self._queue[pos]
                self._used += need
                req.state['held'] = need
                self.stats.peak_bytes = max(self.stats.peak_bytes, self._used)
                if pos > 0:
                    self.stats.bypassed += 1
            req.t_admit = time.perf_counter()
            try:
                placed = self.ex.setup(req, self.ts_chunk_bytes)
            except Exception as exc:
                self._finish(req, exc)
                continue
            if placed is False:
                with self._cv:
                    self._used -= req.state.pop('held')
                    self._queue.insert(pos, req)
                pos += 1
                continue
            if req.kind == 'rr':
                req.state['items'] = work_items(req.npv, req.npt)
                req.state['icur'] = 0
            elif req.state.get('persistent'):
                # a transmission-spectroscopy request whose output fits on the
                # device: its tiles go through the batched steps as well
                req.state['items'] = ts_work_items(req.npv, req.npt)
                req.state['icur'] = 0
            else:
                self._ts_new.append(req)
            with self._cv:
                self._active[req.rid] = req
                self.stats.admitted += 1

    def _take_items(self):
        """Round-robin over active plain requests, up to step_items work items:
        a list of (request, rows of its work items)."""
        batch, n = [], 0
        rr = [r for r in self._active.values() if 'items' in r.state and r.state['icur'] < len(r.state['items'])]
        while rr and n < self.step_items:
            nxt = []
            share = max(1, (self.step_items - n) // len(rr))
            for r in rr:
                items, c = r.state['items'], r.state['icur']
                take = min(share, len(items) - c, self.step_items - n)
                if take <= 0:
                    break
                batch.append((r, items[c:c + take]))
                r.state['icur'] = c + take
                n += take
                if r.state['icur'] < len(items):
                    nxt.append(r)
            rr = nxt
        return batch

    def _finish(self, req, result):
        """Resolve a request's future and give its memory back.  Called once
        per admitted request; an exception as the result fails it."""
        req.t_done = time.perf_counter()
        failed = isinstance(result, BaseException)
        with self._cv:
            self._active.pop(req.rid, None)
            self._issued.pop(req.rid, None)
            self._used -= req.state.pop('held', 0)
            if failed:
                if isinstance(result, MemoryError):
                    self.stats.rejected += 1
                else:
                    self.stats.failed += 1
            else:
                self.stats.completed += 1
                self.stats.points += req.points
                self.stats.latencies.append(req.t_done - req.t_submit)
                self.stats.done_times.append(req.t_done)
        try:
            self.ex.release(req)
        except Exception as exc:       # the request's result stands; the executor's error is kept
            self._release_errors.append(exc)
        if failed:
            req.future.set_exception(result)
        else:
            if not req.state.get('keep', True):
                req.state.pop('host_out', None)
                result = req.points
            req.future.error_bound = req.state.get('error_bound')
            req.future.set_result(result)

    def _fail_all(self, reqs, exc):
        for r in {id(r): r for r in reqs}.values():
            if r.rid in self._active or r.rid in self._issued:
                self._finish(r, exc)

    def _loop(self):
        self._release_errors = []
        while True:
            with self._cv:
                if self._stop and not self._queue and not self._active:
                    break
                if not self._queue and not self._active:
                    self._cv.wait(timeout=0.01)
                    continue
            try:
                t0 = time.perf_counter()
                self._admit()
                t1 = time.perf_counter()
                self.stats.admit_s += t1 - t0
                batch = self._take_items()
                ts_work, self._ts_new = self._ts_new, []
                if batch or ts_work:
                    try:
                        self.ex.step(batch, ts_work)
                    except Exception as exc:
                        # the step's requests fail; requests not in it keep going
                        self._fail_all([r for r, _ in batch] + ts_work, exc)
                        batch, ts_work = [], []
                    self.stats.steps += 1
                    for r in ts_work:
                        self._issued[r.rid] = r
                    for r in {id(r): r for r, _ in batch}.values():
                        if r.state['icur'] >= len(r.state['items']):
                            self._issued[r.rid] = r
                t2 = time.perf_counter()
                self.stats.step_s += t2 - t1
                # completions, polled in issue order: stop at the few oldest still running
                pending = 0
                for r in list(self._issued.values()):
                    try:
                        if not r.state.get('copy_started'):
                            self.ex.start_copy(r)
                            r.state['copy_started'] = True
                        done = self.ex.poll_copy(r)
                    except Exception as exc:
                        self._finish(r, exc)
                        continue
                    if done is not None:
                        self._finish(r, done)
                    else:
                        pending += 1
                        if pending >= 4:
                            break
                steps_done = getattr(self.ex, 'finished_step_seconds', None)
                if steps_done is not None:
                    self.stats.gpu_step_s = steps_done()
                self.stats.poll_s += time.perf_counter() - t2
            except Exception as exc:
                # a fault of the scheduler itself: every request it holds fails
                # rather than waiting forever; queued requests are served after
                self._fail_all(list(self._active.values()) + list(self._issued.values()), RuntimeError(
                    f"serving loop error: {exc!r}"))
                self._ts_new = []
                batch, ts_work = [], []
            if not batch and not ts_work:
                time.sleep(0.0002)
        self.ex.shutdown()


class GpuExecutor:
    """GPU side of the server: per-request set-up, batched steps (persistent
    kernel from a captured CUDA graph), chunked transmission-spectroscopy
    launches, device-to-host copies."""

    MAX_REQ = 4096
    MAX_ITEMS = 65536

    def __init__(self, device=None, nblocks=None, result='host', arena_bytes=None):
        """result='host': futures resolve to numpy arrays in pinned host memory;
        'device': to CUDA tensors that stay on the GPU (for device-side consumers).
        arena_bytes: device memory reserved for requests (default: 90 % of
        what is free)."""
        import torch
        if result not in ('host', 'device'):
            raise ValueError("result must be 'host' or 'device'")
        self.result = result
        from . import _lib
        from .rrmodel import RoadRunnerModel
        self.torch, self._lib = torch, _lib
        self.device = _lib.require_cuda(device)
        torch.cuda.set_device(self.device)
        self.L = _lib.lib()
        self.L.rr_full_split_tables.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                                C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        self.L.rr_full_split_tables.restype = None
        self.L.rr_serve_flux_split.argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_void_p]
        self.stream = torch.cuda.Stream(self.device)          # batched steps (graph replays)
        self.setup_stream = torch.cuda.Stream(self.device)    # per-request uploads and prologues
        self.copy_stream = torch.cuda.Stream(self.device)
        self.ts_streams = [torch.cuda.Stream(self.device) for _ in range(4)]
        self._step_events = collections.deque()   # (start, end) of issued batched steps
        self._step_seconds = 0.0
        self._ts_next = 0
        self._sp_setup = self.setup_stream.cuda_stream
        self.ring = _PinnedRing(torch, 256 << 20)
        free_b = torch.cuda.mem_get_info(self.device)[0]
        want = int(0.9 * free_b) if arena_bytes is None else int(arena_bytes)
        self.arena = _DeviceArena(torch, self.device, max(1 << 20, min(want, free_b - (2 << 30))))
        # shared tables: one model per law (weight table, grids, basis tables)
        self.models = {}
        self._RR = RoadRunnerModel
        sm = torch.cuda.get_device_properties(self.device).multi_processor_count
        self.nblocks = nblocks or sm * 4
        # request descriptors and item list at fixed device addresses (graph arguments)
        self.desc_dtype = SERVE_REQUEST_DTYPE
        self.L.rr_serve_struct_sizes.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
        rs, is_ = C.c_int(), C.c_int()
        self.L.rr_serve_struct_sizes(C.byref(rs), C.byref(is_))
        if rs.value != self.desc_dtype.itemsize or is_.value != 24:
            raise RuntimeError("rr_serve_request / rr_serve_item layout mismatch with the library")
        # descriptors: a pinned host mirror written at set-up, copied (dirty
        # slot range only, asynchronously, in stream order) before a step
        dsz = self.MAX_REQ * self.desc_dtype.itemsize
        self.descs_pin = torch.zeros(dsz, dtype=torch.uint8, pin_memory=True)
        self.descs_h = self.descs_pin.numpy().view(self.desc_dtype)
        self.descs_d = torch.zeros(dsz, dtype=torch.uint8, device=self.device)
        self._dirty = set()
        self.items_d = torch.zeros(self.MAX_ITEMS * 6 + 8, dtype=torch.int32, device=self.device)
        self.counter = torch.zeros(4, dtype=torch.int32, device=self.device)
        self.free_slots = list(range(self.MAX_REQ - 1, -1, -1))
        # per slot: the stated error bound of the request holding it
        self.bound_pin = torch.zeros(self.MAX_REQ, dtype=torch.float64, pin_memory=True)
        self.bound_np = self.bound_pin.numpy()
        # the argument record of rr_serve_setup, refilled for every request
        self.L.rr_serve_setup.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
        self.L.rr_serve_setup_args_size.argtypes = [C.POINTER(C.c_int)]
        self.L.rr_serve_setup_args_size.restype = None
        sz = C.c_int()
        self.L.rr_serve_setup_args_size(C.byref(sz))
        if sz.value != SETUP_ARGS_DTYPE.itemsize:
            raise RuntimeError("rr_serve_setup_args layout mismatch with the library")
        self._setup_rec = np.zeros(1, SETUP_ARGS_DTYPE)
        self._setup_ptr = self._setup_rec.ctypes.data
        self._ring_base = self.ring.buf.data_ptr()
        self._bound_base = self.bound_pin.data_ptr()
        self._desc_base = self.descs_pin.data_ptr()
        self.graph = None
        self._capture()

    # -- helpers -------------------------------------------------------------
    def _model(self, ld):
        if ld not in self.models:
            m = self._RR(ld, precision='split', device=self.device)
            with self.torch.cuda.stream(self.setup_stream):     # ordered before the set-ups that use them
                tb = m.tables = m._device_tables(self.device)
            for n in ('mu', 'ze', 'W32'):
                tb[n + '_ptr'] = tb[n].data_ptr()
            self.models[ld] = m
        return self.models[ld]

    def _capture(self):
        """Capture 'reset the item counter, run the persistent kernel' once."""
        torch = self.torch
        P = self._lib.ptr
        nitems_ptr = C.c_void_p(self.items_d.data_ptr() + self.MAX_ITEMS * 6 * 4)
        self.items_d.zero_()
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=self.stream):
            self.counter.zero_()
            st = self.L.rr_serve_flux_split(C.c_void_p(self.descs_d.data_ptr()), P(self.items_d), nitems_ptr,
                                            P(self.counter), self.nblocks,
                                            C.c_void_p(torch.cuda.current_stream().cuda_stream))
        self._lib.check(st, "rr_serve_flux_split")
        self.graph = g

    # -- request set-up ---------------------------------------------------------
    _INPUTS = (('time', 'time'), ('exptimes', 'exptimes'), ('k', 'k'), ('t0', 't0'), ('p', 'p'), ('a', 'a'),
               ('i', 'i'), ('e', 'e'), ('w', 'w'), ('ldc', 'ldc'), ('lcids', 'lcids'), ('pbids', 'pbids'),
               ('epids', 'epids'), ('nsamples', 'nsamples'))

    def setup(self, req, ts_chunk_bytes):
        """Everything a request keeps on the device lives in one allocation:
        its inputs (staged in the pinned ring, one host-to-device copy), the
        FP32-pair times, LD tables, prologue workspace and output."""
        torch, L = self.torch, self.L
        h = req.state['host']
        m = self._model(req.ld)
        tb = m.tables
        npt, npv, npb, nlc = req.npt, req.npv, h['npb'], h['nlc']
        nz, ng = m.ze.size, m.ng
        npar = h['ldc'].shape[2]
        ldf = (npt + 3) // 4 * 4
        arrays = [(name, h[key]) for name, key in self._INPUTS]
        parts = [(name, a.nbytes) for name, a in arrays]
        n_in = _layout(parts)[1]
        parts += [('times_ff', 4 * max(int(L.rr_time_split_floats(npt)), 4)), ('bnd', 8 * npv), ('bmax', 8)]
        if req.kind == 'rr':
            nep = h['t0'].shape[1]
            wsb = int(L.rr_full_split_workspace_bytes(npv, npb, nlc, nep, ng))
            parts += [('ldp', 4 * npv * npb * nz), ('istar', 4 * npv * npb), ('ws', wsb), ('flux', 4 * npv * ldf)]
        else:
            # the prologue for every pv at admission; the flux through the
            # batched steps when the whole output fits on the device, else in
            # pv chunks on a side stream, each chunk copied out as it is done
            out_bytes = 4 * npv * npb * ldf
            persistent = self.result == 'device' or out_bytes <= ts_chunk_bytes
            per_pv = max(1, req.nbytes // max(npv, 1))
            chunk = npv if persistent else max(1, min(npv, int(ts_chunk_bytes // per_pv)))
            wsb = int(L.rr_ts_workspace_bytes(1, npv, npb, ng))
            parts += [('ws', wsb)]
            if persistent:
                parts += [('flux', out_bytes)]
            req.state['persistent'] = persistent
        # a result handed to the caller on the device is a tensor of its own;
        # everything else lives in the request's arena block
        own_flux = self.result == 'device' and req.state.get('keep', True) and 'flux' in dict(parts)
        if own_flux:
            flux_bytes = dict(parts)['flux']
            parts = [pt for pt in parts if pt[0] != 'flux']
        off, total = _layout(parts)
        blk = self.arena.alloc(total)
        if blk is None:
            if total > self.arena.size or self.arena.used == 0:
                raise MemoryError(f"request {req.rid} needs {total / 1e9:.2f} GB of device memory, more than the "
                                  f"{self.arena.size / 1e9:.2f} GB arena")
            return False
        lo = self.ring.alloc(n_in)
        if lo is None:                 # larger than the ring: a pinned buffer of its own
            stage = torch.empty(n_in, dtype=torch.uint8, pin_memory=True)
            sv, lo = stage.numpy(), 0
        else:
            stage, sv = self.ring.buf, self.ring.np
        for name, a in arrays:
            o = lo + off[name]
            sv[o:o + a.nbytes] = np.ascontiguousarray(a).reshape(-1).view(np.uint8)
        tmin, tmax = h['tmin'], h['tmax']
        t_ref = 0.5 * (tmin + tmax)
        t_abs = max(tmax - t_ref, t_ref - tmin)
        base = self.arena.base + blk
        P = {name: base + o for name, o in off.items()}
        fl = None
        if own_flux:
            with torch.cuda.stream(self.setup_stream):
                fl = torch.empty(flux_bytes // 4, dtype=torch.float32, device=self.device)
            P['flux'] = fl.data_ptr()
        g = dict(P=P, t_ref=t_ref, t_abs=t_abs, wsb=wsb, block=(blk, total))
        slot = self.free_slots.pop()
        req.state['slot'] = slot
        kind = 0 if req.kind == 'rr' else 1
        with_desc = kind == 0 or req.state['persistent']
        if with_desc:
            # the flux as a tensor is made only when a result is handed over
            shape = (npv, ldf) if kind == 0 else (npv, npb, ldf)
            g['flux_src'] = (fl, blk + off.get('flux', 0), shape)
            self._dirty.add(slot)
        else:
            g['chunk'] = chunk
        basis = None
        if kind == 0:
            if ('basis', npar) in tb:
                basis, nb = m._basis(self.device, npar, True)
            else:
                with torch.cuda.stream(self.setup_stream):   # built once, ordered before the prologues
                    basis, nb = m._basis(self.device, npar, True)
        # one native call: inputs to the device, time split, fused prologue,
        # descriptor, error bound (setup_args_dtype mirrors rr_serve_setup_args)
        self._setup_rec[0] = (
            self._ring_base + lo if stage is self.ring.buf else stage.data_ptr() + lo, base, n_in,
            P['time'], P['lcids'], P['pbids'], P['epids'], P['nsamples'], P['exptimes'], P['k'], P['t0'], P['p'],
            P['a'], P['i'], P['e'], P['w'], P['ldc'], P['times_ff'], P.get('ldp', 0), P.get('istar', 0), P['ws'],
            P['bnd'], P['bmax'], P.get('flux', 0), tb['mu_ptr'], 0 if basis is None else basis.data_ptr(),
            tb['W32_ptr'], tb['ze_ptr'],
            npt, npv, nlc, npb, h['t0'].shape[1] if h['t0'].ndim > 1 else 1, h['k'].shape[1], npar, m.ld_law, nb if kind == 0 else 0, m.nk,
            nz, ng, ldf, wsb, int(h['nsamples'][0]),
            t_ref, t_abs, m.dk, m.klims[0], m.klims[1], m.dg, float(h['exptimes'][0]),
            self._bound_base + 8 * slot, self._desc_base + self.desc_dtype.itemsize * slot if with_desc else 0)
        self._lib.check(L.rr_serve_setup(kind, self._setup_ptr, self._sp_setup), "rr_serve_setup")
        ready = torch.cuda.Event()
        ready.record(self.setup_stream)
        if stage is self.ring.buf:
            self.ring.commit(lo, n_in, ready)
        else:
            g['stage'] = stage
        g['ready'] = ready
        req.state['g'] = g
        req.state['model'] = m

    def _flux_view(self, req):
        """The request's flux [npv, (npb,) npt] as a tensor view."""
        fl, o, shape = req.state['g']['flux_src']
        if fl is None:
            n = int(np.prod(shape))
            fl = self.arena.buf[o:o + 4 * n].view(self.torch.float32)
        res = fl.view(shape)
        return res[..., :req.npt]

    # -- steps -------------------------------------------------------------------
    def step(self, batch, ts_reqs):
        torch = self.torch
        with torch.cuda.stream(self.stream):
            if batch:
                for r in {id(r): r for r, _ in batch}.values():
                    g = r.state['g']
                    if not g.get('waited'):
                        self.stream.wait_event(g['ready'])
                        g['waited'] = True
                if self._dirty:
                    lo, hi = min(self._dirty), max(self._dirty) + 1
                    isz = self.desc_dtype.itemsize
                    self.descs_d[lo * isz:hi * isz].copy_(self.descs_pin[lo * isz:hi * isz], non_blocking=True)
                    self._dirty.clear()
                # the item list and its count go through the pinned ring (a
                # region is reused only after its copy has run: no host wait)
                n = sum(len(w) for _, w in batch)
                nb = 4 * (n * 6 + 1)
                lo = self.ring.alloc(nb)
                if lo is None:
                    raise RuntimeError(f"a step's item list ({nb} bytes) does not fit the {self.ring.size}-byte "
                                       "pinned staging ring")
                buf = self.ring.np[lo:lo + nb].view(np.int32)
                rows = buf[:n * 6].reshape(n, 6)
                c = 0
                for r, w in batch:
                    rows[c:c + len(w), 0] = r.state['slot']
                    rows[c:c + len(w), 1:5] = w
                    c += len(w)
                rows[:, 5] = 0
                buf[n * 6] = n
                src = self.ring.buf[lo:lo + nb].view(torch.int32)
                self.items_d[:n * 6].copy_(src[:n * 6], non_blocking=True)
                self.items_d[self.MAX_ITEMS * 6:self.MAX_ITEMS * 6 + 1].copy_(src[n * 6:n * 6 + 1], non_blocking=True)
                cev = torch.cuda.Event()
                cev.record(self.stream)
                self.ring.commit(lo, nb, cev)
                e0 = torch.cuda.Event(enable_timing=True)
                e0.record(self.stream)
                self.graph.replay()
                ev = torch.cuda.Event(enable_timing=True)
                ev.record(self.stream)
                self._step_events.append((e0, ev))
            else:
                ev = torch.cuda.Event()
                ev.record(self.stream)
            for r, _ in batch:
                r.state['last_event'] = ev
        # transmission-spectroscopy requests run as their own launches on a
        # few side streams, overlapping the batched step and one another
        for r in ts_reqs:
            self._run_ts(r, self.ts_streams[self._ts_next % len(self.ts_streams)])
            self._ts_next += 1

    def _run_ts(self, req, stream):
        """Transmission-spectroscopy request on one of the TS streams; with
        host results in parameter-vector chunks, each chunk copied to the host
        result as soon as it is computed."""
        torch, L = self.torch, self.L
        g, h, m = req.state['g'], req.state['host'], req.state['model']
        base = g['P']

        def P(name, elems=0, size=8):
            return base[name] + elems * size

        npv, npt, npb = req.npv, req.npt, h['npb']
        ng = m.ng
        ldf = (npt + 3) // 4 * 4
        ns0, ex0 = int(h['nsamples'][0]), float(h['exptimes'][0])
        stream.wait_event(g['ready'])        # set-up kernels of this request
        with torch.cuda.stream(stream):
            sp = self._lib.stream_ptr(self.device)

            def launch(pv0, n, out_ptr):
                st = L.rr_ts_flux_split_range(P('times_ff'), npt, npv, npb, ns0, ex0, ng, m.dg, P('ws'), pv0,
                                              pv0 + n, out_ptr, ldf, sp)
                self._lib.check(st, "rr_ts_flux_split_range")

            chunk = g['chunk']
            host = torch.empty((npv, npb, npt), dtype=torch.float32, pin_memory=True)
            req.state['host_out'] = host
            outs = [torch.empty((chunk, npb, ldf), dtype=torch.float32, device=self.device) for _ in range(2)]
            for o in outs:
                o.record_stream(self.copy_stream)
            for j, pv0 in enumerate(range(0, npv, chunk)):
                n = min(chunk, npv - pv0)
                out = outs[j % 2]
                if j >= 2:
                    # the buffer's previous chunk must have left for the host
                    stream.wait_event(req.state['chunk_ev'][j % 2])
                launch(pv0, n, self._lib.ptr(out))
                ev = torch.cuda.Event()
                ev.record(stream)
                self.copy_stream.wait_event(ev)
                with torch.cuda.stream(self.copy_stream):
                    host[pv0:pv0 + n].copy_(out[:n, :, :npt], non_blocking=True)
                    cev = torch.cuda.Event()
                    cev.record(self.copy_stream)
                req.state.setdefault('chunk_ev', [None, None])[j % 2] = cev
            req.state['ts_done_event'] = cev

    def start_copy(self, req):
        torch = self.torch
        if req.kind == 'ts' and not req.state.get('persistent'):
            req.state['copy_event'] = req.state['ts_done_event']
            return
        if self.result == 'device':
            req.state['host_out'] = self._flux_view(req) if req.state.get('keep', True) else None
            req.state['copy_event'] = req.state['last_event']
            return
        res = self._flux_view(req)
        host = torch.empty(tuple(res.shape), dtype=torch.float32, pin_memory=True)
        self.copy_stream.wait_event(req.state['last_event'])
        with torch.cuda.stream(self.copy_stream):
            host.copy_(res, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self.copy_stream)
        req.state['host_out'] = host
        req.state['copy_event'] = ev

    def poll_copy(self, req):
        ev = req.state.get('copy_event')
        if ev is None or not ev.query():
            return None
        req.state['copy_done'] = True
        req.state['error_bound'] = float(self.bound_np[req.state['slot']])
        out = req.state['host_out']
        if out is None:          # a dropped result (keep_result=False): its point count stands for it
            return req.points
        return out if self.result == 'device' else out.numpy()

    def release(self, req):
        """Give a finished request's slot and device memory back.  A request
        that failed may still have work in flight on the GPU: the device is
        synchronised first, so that no later request is handed memory that a
        running kernel or copy still writes."""
        if not req.state.get('copy_done') and 'g' in req.state:
            self.torch.cuda.synchronize(self.device)
        slot = req.state.pop('slot', None)
        if slot is not None:
            self.free_slots.append(slot)
        g = req.state.pop('g', None)
        if g is not None and 'block' in g:
            self.arena.free(*g['block'])

    def finished_step_seconds(self):
        """Device time of the batched steps finished so far (seconds)."""
        while self._step_events and self._step_events[0][1].query():
            e0, e1 = self._step_events.popleft()
            self._step_seconds += e0.elapsed_time(e1) * 1e-3
        return self._step_seconds

    def shutdown(self):
        """Wait for the GPU and give the arena back to the device."""
        self.torch.cuda.synchronize(self.device)
        self.arena = None
        self.torch.cuda.empty_cache()

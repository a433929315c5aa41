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
  on a copy stream and its future resolved; latency = resolve - submit.

The GPU work is behind ``GpuExecutor`` so that the scheduling logic can be
exercised on the CPU with a fake executor (tests/test_serving_cpu.py).
"""
import collections
import concurrent.futures as cf
import ctypes as C
import itertools
import threading
import time
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import ldmodels as _ldm

__all__ = ['Request', 'RRServer', 'GpuExecutor', 'ServerStats']

TILE = 128


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
    submitted: int = 0
    admitted: int = 0
    completed: int = 0
    rejected: int = 0
    steps: int = 0
    points: int = 0
    peak_bytes: int = 0
    latencies: list = field(default_factory=list)

    def summary(self):
        lat = np.array(self.latencies) if self.latencies else np.zeros(1)
        return dict(submitted=self.submitted, admitted=self.admitted, completed=self.completed,
                    rejected=self.rejected, steps=self.steps, points=self.points,
                    peak_hbm_bytes=self.peak_bytes, p50_s=float(np.percentile(lat, 50)),
                    p99_s=float(np.percentile(lat, 99)), mean_s=float(lat.mean()))


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
    req.state['host'] = dict(time=time_, lcids=lcids, pbids=pbids, epids=epids, nsamples=ns, exptimes=ex,
                             k=np.ascontiguousarray(k), ldc=ldc, t0=np.ascontiguousarray(t0), p=pv, nlc=nlc,
                             npb=npb, **vec)
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


def work_items(npv: int, npt: int, target_tiles: int = 256):
    """(pv0, pv1, tile0, tile1) chunks of about target_tiles pv-tiles each."""
    ntiles = max(1, (npt + TILE - 1) // TILE)
    if ntiles >= target_tiles:
        return [(pv, pv + 1, t, min(t + target_tiles, ntiles)) for pv in range(npv)
                for t in range(0, ntiles, target_tiles)]
    per = max(1, target_tiles // ntiles)
    return [(pv, min(pv + per, npv), 0, ntiles) for pv in range(0, npv, per)]


class RRServer:
    """Continuous-batching server (see the module docstring)."""

    def __init__(self, executor=None, hbm_budget: float = 120e9, step_items: int = 4096,
                 ts_chunk_bytes: float = 4e9, device=None, result: str = 'host'):
        self.ex = executor if executor is not None else GpuExecutor(device, result=result)
        self.budget = int(hbm_budget)
        self.step_items = step_items
        self.ts_chunk_bytes = ts_chunk_bytes
        self.stats = ServerStats()
        self._ids = itertools.count()
        self._queue = collections.deque()
        self._active = collections.OrderedDict()
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
        req.future = cf.Future()
        req.rid = next(self._ids)
        req.t_submit = time.perf_counter()
        shape_request(req)
        req.nbytes = request_bytes(req)
        with self._cv:
            self.stats.submitted += 1
            if self._min_bytes(req) > self.budget:
                self.stats.rejected += 1
                req.future.set_exception(MemoryError(
                    f"request {req.rid} needs {self._min_bytes(req) / 1e9:.1f} GB of device memory, "
                    f"more than the {self.budget / 1e9:.1f} GB budget"))
                return req.future
            self._queue.append(req)
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
                if not self._queue and not self._active:
                    return True
            if timeout is not None and time.perf_counter() - t0 > timeout:
                return False
            time.sleep(0.001)

    # -- scheduler ----------------------------------------------------------
    def _min_bytes(self, req):
        if req.kind == 'ts' and req.nbytes > self.ts_chunk_bytes and getattr(self.ex, 'result', 'host') == 'host':
            per_pv = req.nbytes / max(req.npv, 1)
            return int(per_pv * max(1, int(self.ts_chunk_bytes // per_pv)))
        return req.nbytes

    def _admit(self):
        admitted = []
        with self._cv:
            while self._queue:
                req = self._queue[0]
                need = self._min_bytes(req)
                if self._used + need > self.budget:
                    break
                self._queue.popleft()
                self._used += need
                req.state['held'] = need
                self.stats.peak_bytes = max(self.stats.peak_bytes, self._used)
                admitted.append(req)
        for req in admitted:
            req.t_admit = time.perf_counter()
            try:
                self.ex.setup(req, self.ts_chunk_bytes)
            except Exception as exc:   # pragma: no cover - surfaced to the client
                self._finish(req, exc)
                continue
            if req.kind == 'rr':
                req.state['items'] = collections.deque(work_items(req.npv, req.npt))
            with self._cv:
                self._active[req.rid] = req
                self.stats.admitted += 1

    def _take_items(self):
        """Round-robin over active plain requests, up to step_items items."""
        batch = []
        rr = [r for r in self._active.values() if r.kind == 'rr' and r.state.get('items')]
        while rr and len(batch) < self.step_items:
            nxt = []
            for r in rr:
                q = r.state['items']
                take = max(1, min(len(q), (self.step_items - len(batch)) // max(len(rr), 1)))
                for _ in range(take):
                    if not q or len(batch) >= self.step_items:
                        break
                    batch.append((r, q.popleft()))
                if q:
                    nxt.append(r)
            rr = nxt
        return batch

    def _finish(self, req, result):
        req.t_done = time.perf_counter()
        with self._cv:
            self._active.pop(req.rid, None)
            self._used -= req.state.get('held', 0)
            if isinstance(result, Exception):
                self.stats.rejected += 1
            else:
                self.stats.completed += 1
                self.stats.points += req.points
                self.stats.latencies.append(req.t_done - req.t_submit)
        self.ex.release(req)
        if isinstance(result, Exception):
            req.future.set_exception(result)
        else:
            if not req.state.get('keep', True):
                req.state.pop('host_out', None)
                result = req.points
            req.future.set_result(result)

    def _loop(self):
        while True:
            with self._cv:
                if self._stop and not self._queue and not self._active:
                    break
                if not self._queue and not self._active:
                    self._cv.wait(timeout=0.01)
                    continue
            self._admit()
            batch = self._take_items()
            ts_work = [r for r in list(self._active.values()) if r.kind == 'ts' and not r.state.get('ts_issued')]
            if batch or ts_work:
                self.ex.step(batch, ts_work)
                self.stats.steps += 1
                for r in ts_work:
                    r.state['ts_issued'] = True
                for r in {id(r): r for r, _ in batch}.values():
                    if not r.state['items']:
                        r.state['issued'] = True
            for r in list(self._active.values()):
                if (r.kind == 'rr' and r.state.get('issued')) or (r.kind == 'ts' and r.state.get('ts_issued')):
                    if not r.state.get('copy_started'):
                        self.ex.start_copy(r)
                        r.state['copy_started'] = True
                    done = self.ex.poll_copy(r)
                    if done is not None:
                        self._finish(r, done)
            if not batch and not ts_work:
                time.sleep(0.0002)
        self.ex.shutdown()


class GpuExecutor:
    """GPU side of the server: per-request set-up, batched steps (persistent
    kernel from a captured CUDA graph), chunked transmission-spectroscopy
    launches, device-to-host copies."""

    MAX_REQ = 4096
    MAX_ITEMS = 65536

    def __init__(self, device=None, nblocks=None, result='host'):
        """result='host': futures resolve to numpy arrays in pinned host memory;
        'device': to CUDA tensors that stay on the GPU (for device-side consumers)."""
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
        self.stream = torch.cuda.Stream(self.device)
        self.copy_stream = torch.cuda.Stream(self.device)
        # shared tables: one model per law (weight table, grids, basis tables)
        self.models = {}
        self._RR = RoadRunnerModel
        sm = torch.cuda.get_device_properties(self.device).multi_processor_count
        self.nblocks = nblocks or sm * 4
        # request descriptors and item list at fixed device addresses (graph arguments)
        self.desc_dtype = np.dtype([('times_ff', 'u8'), ('lcids', 'u8'), ('orb32', 'u8'), ('lc32', 'u8'),
                                    ('ldm', 'u8'), ('flux', 'u8'), ('ldflux', 'i8'), ('npt', 'i4'), ('npv', 'i4'),
                                    ('nlc', 'i4'), ('npb', 'i4'), ('ng', 'i4'), ('pad0', 'i4'), ('inv_dg', 'f4'),
                                    ('pad1', 'f4')])
        self.L.rr_serve_struct_sizes.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
        rs, is_ = C.c_int(), C.c_int()
        self.L.rr_serve_struct_sizes(C.byref(rs), C.byref(is_))
        if rs.value != self.desc_dtype.itemsize or is_.value != 24:
            raise RuntimeError("rr_serve_request / rr_serve_item layout mismatch with the library")
        self.descs_h = np.zeros(self.MAX_REQ, self.desc_dtype)
        self.descs_d = torch.zeros(self.MAX_REQ * self.desc_dtype.itemsize, dtype=torch.uint8, device=self.device)
        self.items_pin = torch.zeros(self.MAX_ITEMS * 6 + 8, dtype=torch.int32, pin_memory=True)
        self.items_d = torch.zeros(self.MAX_ITEMS * 6 + 8, dtype=torch.int32, device=self.device)
        self.counter = torch.zeros(4, dtype=torch.int32, device=self.device)
        self.free_slots = list(range(self.MAX_REQ - 1, -1, -1))
        self.graph = None
        self.step_events = collections.deque()
        self._capture()

    # -- helpers -------------------------------------------------------------
    def _model(self, ld):
        if ld not in self.models:
            m = self._RR(ld, precision='split', device=self.device)
            with self.torch.cuda.stream(self.stream):
                m._device_tables(self.device)
            self.models[ld] = m
        return self.models[ld]

    def _capture(self):
        """Capture 'reset the item counter, run the persistent kernel' once."""
        torch = self.torch
        P = self._lib.ptr
        nitems_ptr = C.c_void_p(self.items_d.data_ptr() + self.MAX_ITEMS * 6 * 4)
        self.items_pin[self.MAX_ITEMS * 6] = 0
        self.items_d.copy_(self.items_pin)
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
    def setup(self, req, ts_chunk_bytes):
        torch, L, P = self.torch, self.L, self._lib.ptr
        h = req.state['host']
        m = self._model(req.ld)
        tb = m.tables = m._device_tables(self.device)
        dev = self.device
        with torch.cuda.stream(self.stream):
            sp = self._lib.stream_ptr(dev)
            g = {}
            for n in ('time', 'exptimes', 'k', 't0', 'p', 'a', 'i', 'e', 'w', 'ldc'):
                g[n] = torch.as_tensor(np.array(h[n])).pin_memory().to(dev, non_blocking=True)
            for n in ('lcids', 'pbids', 'epids', 'nsamples'):
                g[n] = torch.as_tensor(np.array(h[n])).pin_memory().to(dev, non_blocking=True)
            npt, npv, npb, nlc = req.npt, req.npv, h['npb'], h['nlc']
            tmin, tmax = float(h['time'].min()), float(h['time'].max())
            t_ref = 0.5 * (tmin + tmax)
            t_abs = max(tmax - t_ref, t_ref - tmin)
            g['times_ff'] = torch.empty(max(int(L.rr_time_split_floats(npt)), 4), dtype=torch.float32, device=dev)
            self._lib.check(L.rr_time_split(P(g['time']), P(g['lcids']), npt, t_ref, P(g['times_ff']), sp))
            nz, ng = m.ze.size, m.ng
            npar = h['ldc'].shape[2]
            g['ldp'] = torch.empty((npv, npb, nz), dtype=torch.float32, device=dev)
            g['istar'] = torch.empty((npv, npb), dtype=torch.float32, device=dev)
            self._lib.check(L.rr_ld_tables_f32(m.ld_law, P(g['ldc']), npv, npb, npar, P(tb['mu']), nz, P(g['ldp']),
                                               P(g['istar']), sp))
            ldf = (npt + 3) // 4 * 4
            if req.kind == 'rr':
                nep = h['t0'].shape[1]
                basis, nb = m._basis(dev, npar, True)
                wsb = L.rr_full_split_workspace_bytes(npv, npb, nlc, nep, ng)
                g['ws'] = torch.empty(wsb, dtype=torch.uint8, device=dev)
                self._lib.check(L.rr_prepare_split(
                    t_ref, t_abs, P(g['k']), h['k'].shape[1], P(g['t0']), nep, nep, P(g['p']), P(g['a']),
                    P(g['i']), P(g['e']), P(g['w']), npv, nlc, npb, P(g['pbids']), P(g['epids']),
                    P(g['nsamples']), P(g['exptimes']), P(g['ldp']), P(g['istar']), P(tb['W32']), m.nk, ng, nz,
                    m.dk, float(m.klims[0]), float(m.klims[1]), P(tb['ze']), P(g['ws']), wsb, sp, m.ld_law,
                    P(g['ldc']), npar, P(basis), nb))
                g['flux'] = torch.empty((npv, ldf), dtype=torch.float32, device=dev)
                orb, lc, ldm = C.c_void_p(), C.c_void_p(), C.c_void_p()
                L.rr_full_split_tables(C.c_void_p(g['ws'].data_ptr()), npv, npb, nlc, nep, ng, C.byref(orb),
                                       C.byref(lc), C.byref(ldm))
                slot = self.free_slots.pop()
                req.state['slot'] = slot
                d = self.descs_h[slot]
                d['times_ff'], d['lcids'] = g['times_ff'].data_ptr(), g['lcids'].data_ptr()
                d['orb32'], d['lc32'], d['ldm'] = orb.value, lc.value, ldm.value
                d['flux'], d['ldflux'] = g['flux'].data_ptr(), ldf
                d['npt'], d['npv'], d['nlc'], d['npb'], d['ng'] = npt, npv, nlc, npb, ng
                d['inv_dg'] = np.float32(1.0 / m.dg)
                req.state['desc_dirty'] = True
            else:
                g['t_ref'], g['t_abs'] = t_ref, t_abs
                per_pv = max(1, req.nbytes // max(npv, 1))
                g['chunk'] = max(1, min(npv, int(ts_chunk_bytes // per_pv)))
            req.state['g'] = g
            req.state['model'] = m

    # -- steps -------------------------------------------------------------------
    def step(self, batch, ts_reqs):
        torch = self.torch
        with torch.cuda.stream(self.stream):
            if batch:
                dirty = [r for r, _ in batch if r.state.pop('desc_dirty', False)]
                if dirty:
                    self.descs_d.copy_(torch.from_numpy(self.descs_h.view(np.uint8)), non_blocking=False)
                # the staging buffer is reused: wait for the previous step's copy
                while self.step_events and len(self.step_events) > 1:
                    self.step_events.popleft().synchronize()
                if self.step_events:
                    self.step_events[-1].synchronize()
                arr = self.items_pin.numpy()
                n = len(batch)
                it = np.array([(r.state['slot'], *w, 0) for r, w in batch], np.int32).reshape(-1)
                arr[:n * 6] = it
                arr[self.MAX_ITEMS * 6] = n
                self.items_d[:n * 6].copy_(self.items_pin[:n * 6], non_blocking=True)
                self.items_d[self.MAX_ITEMS * 6:self.MAX_ITEMS * 6 + 1].copy_(
                    self.items_pin[self.MAX_ITEMS * 6:self.MAX_ITEMS * 6 + 1], non_blocking=True)
                self.graph.replay()
            for r in ts_reqs:
                self._run_ts(r)
            ev = torch.cuda.Event()
            ev.record(self.stream)
            self.step_events.append(ev)
            for r, _ in batch:
                r.state['last_event'] = ev
            for r in ts_reqs:
                r.state['last_event'] = ev

    def _run_ts(self, req):
        """Transmission-spectroscopy request in parameter-vector chunks; each
        chunk is copied to the host result as soon as it is computed."""
        torch, L, P = self.torch, self.L, self._lib.ptr
        g, h, m = req.state['g'], req.state['host'], req.state['model']
        tb = m.tables
        npv, npt, npb = req.npv, req.npt, h['npb']
        nz, ng = m.ze.size, m.ng
        ldf = (npt + 3) // 4 * 4
        chunk = g['chunk']
        if self.result == 'device':
            out = torch.empty((npv, npb, ldf), dtype=torch.float32, device=self.device)
            wsb = L.rr_ts_workspace_bytes(1, npv, npb, ng)
            ws = torch.empty(wsb, dtype=torch.uint8, device=self.device)
            st = L.rr_ts_split(P(g['times_ff']), g['t_ref'], g['t_abs'], npt, P(g['k']), P(g['t0']), P(g['p']),
                               P(g['a']), P(g['i']), P(g['e']), P(g['w']), npv, npb, int(h['nsamples'][0]),
                               float(h['exptimes'][0]), P(g['ldp']), P(g['istar']), None, m.nk, ng, nz, m.dk,
                               float(m.klims[0]), float(m.klims[1]), m.dg, P(tb['ze']), P(ws), wsb, P(out), ldf,
                               self._lib.stream_ptr(self.device))
            self._lib.check(st, "rr_ts_split")
            ev = torch.cuda.Event()
            ev.record(self.stream)
            req.state['host_out'] = out[:, :, :npt]
            req.state['ts_done_event'] = ev
            return
        host = torch.empty((npv, npb, npt), dtype=torch.float32, pin_memory=True)
        req.state['host_out'] = host
        sp = self._lib.stream_ptr(self.device)
        wsb = L.rr_ts_workspace_bytes(1, chunk, npb, ng)
        ws = torch.empty(wsb, dtype=torch.uint8, device=self.device)
        outs = [torch.empty((chunk, npb, ldf), dtype=torch.float32, device=self.device) for _ in range(2)]
        for o in outs:
            o.record_stream(self.copy_stream)
        for j, pv0 in enumerate(range(0, npv, chunk)):
            n = min(chunk, npv - pv0)
            out = outs[j % 2]
            if j >= 2:
                # the buffer's previous chunk must have left for the host
                self.stream.wait_event(req.state['chunk_ev'][j % 2])
            off8 = lambda t, w=1: C.c_void_p(t.data_ptr() + pv0 * w * t.element_size())
            st = L.rr_ts_split(P(g['times_ff']), g['t_ref'], g['t_abs'], npt, off8(g['k'], npb), off8(g['t0']),
                               off8(g['p']), off8(g['a']), off8(g['i']), off8(g['e']), off8(g['w']), n, npb,
                               int(h['nsamples'][0]), float(h['exptimes'][0]), off8(g['ldp'], npb * nz),
                               off8(g['istar'], npb), None, m.nk, ng, nz, m.dk, float(m.klims[0]),
                               float(m.klims[1]), m.dg, P(tb['ze']), P(ws), wsb, P(out), ldf, sp)
            self._lib.check(st, "rr_ts_split")
            ev = torch.cuda.Event()
            ev.record(self.stream)
            self.copy_stream.wait_event(ev)
            with torch.cuda.stream(self.copy_stream):
                host[pv0:pv0 + n].copy_(out[:n, :, :npt], non_blocking=True)
                cev = torch.cuda.Event()
                cev.record(self.copy_stream)
            req.state.setdefault('chunk_ev', [None, None])[j % 2] = cev
        req.state['ts_done_event'] = cev

    def start_copy(self, req):
        torch = self.torch
        if req.kind == 'ts':
            req.state['copy_event'] = req.state['ts_done_event']
            return
        g = req.state['g']
        if self.result == 'device':
            req.state['host_out'] = g['flux'][:, :req.npt]
            req.state['copy_event'] = req.state['last_event']
            return
        host = torch.empty((req.npv, req.npt), dtype=torch.float32, pin_memory=True)
        self.copy_stream.wait_event(req.state['last_event'])
        with torch.cuda.stream(self.copy_stream):
            host.copy_(g['flux'][:, :req.npt], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self.copy_stream)
        req.state['host_out'] = host
        req.state['copy_event'] = ev

    def poll_copy(self, req):
        ev = req.state.get('copy_event')
        if ev is None or not ev.query():
            return None
        out = req.state['host_out']
        return out if self.result == 'device' else out.numpy()

    def release(self, req):
        slot = req.state.pop('slot', None)
        if slot is not None:
            self.free_slots.append(slot)
        req.state.pop('g', None)

    def shutdown(self):
        self.torch.cuda.synchronize(self.device)

"""RoadRunnerModel: drop-in for pytransit.models.RoadRunnerModel on a GB300.

Same constructor keywords, ``set_data`` and ``evaluate`` as
pytransit/models/roadrunner/rrmodel.py:47-238.  Every evaluation runs as CUDA
kernels through the C ABI of libpytransit_gb300.so:

* ``precision='fp64'`` (default): the plain all-FP64 path (rr_full_f64),
  matching the reference to ~1e-12 in flux.
* ``precision='split'``: FP64 orbit and phase data per parameter vector,
  FP32-pair phase reduction and FP32 per-sample arithmetic (rr_full_split);
  max |dF| vs FP64 is a few 1e-7.

Differences from the reference, all where the reference reads out of bounds
or garbles its input:

* a 1D ``t0`` of length npv is one zero epoch per parameter vector (the
  documented intent, rrmodel.py:187-188); a 1D ``k`` of length npv > 1 is one
  radius ratio per vector; scalar ``a, i, e, w`` are broadcast to npv;
* a 2D ``ldc`` is read as [npb, ncoef] and shared by all parameter vectors;
* k in the last table cell (ik + 1 == nk) uses the exact 2D weight table;
* the LD-table index is clamped at g in [1 - 1e-7, 1].
"""
import ctypes as C
import os
from typing import Callable, List, Tuple, Union
from warnings import warn

import numpy as np
from numpy import ndarray

from . import ldmodels as _ldm
from .ldmodel import LDModel
from .transitmodel import TransitModel

__all__ = ['RoadRunnerModel', 'create_z_grid']


def create_z_grid(zcut: float, nin: int, nedge: int):
    """Radial integration grid (common.py:132-149): ``nin`` bins uniform in z
    up to ``zcut``, ``nedge`` bins uniform in mu to the limb.  z_means[0]
    stays 0, as in the reference."""
    mucut = np.sqrt(1.0 - zcut ** 2)
    dz = zcut / nin
    dmu = mucut / nedge
    z_edges = np.zeros(nin + nedge)
    z_means = np.zeros(nin + nedge)
    for i in range(nin - 1):
        z_edges[i] = (i + 1) * dz
    for i in range(nedge + 1):
        z_edges[-i - 1] = np.sqrt(1 - (i * dmu) ** 2)
    for i in range(nin + nedge - 1):
        z_means[i + 1] = 0.5 * (z_edges[i] + z_edges[i + 1])
    return z_edges, z_means


def _default_host_threads():
    """Host threads for output fills: the CPUs this process may run on, at most 16
    (a fill saturates the host memory well before that)."""
    try:
        n = len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        n = os.cpu_count() or 1
    return max(1, min(16, n))


class RoadRunnerModel(TransitModel):
    ldmodels = _ldm.NAMED_LAWS

    def __init__(self, ldmodel: Union[str, Callable, Tuple[Callable, Callable]] = 'quadratic',
                 precompute_weights: bool = False, klims: tuple = (0.005, 0.5), nk: int = 256,
                 nzin: int = 20, nzlimb: int = 20, zcut: float = 0.7, ng: int = 100,
                 nthreads: int = 1, small_planet_limit: float = 0.05, precision: str = 'fp64',
                 device=None, **kwargs):
        """The RoadRunner transit model by Parviainen (2020), on the GPU.

        Parameters
        ----------
        ldmodel : str, callable, (callable, callable) or LDModel
            A named law (``RoadRunnerModel.ldmodels``), a profile callable
            ``I(mu, pv)`` (disk integral by a 200-point trapezoid), a
            (profile, integral) tuple, or an LDModel instance.
        precompute_weights : bool
            Kept for the transmission-spectroscopy model; the 3D weight table is
            always used here, as in the reference.
        klims, nk : radius-ratio range and grid size of the weight table.
        nzin, nzlimb, zcut : radial grid (inner disk, limb, their boundary).
        ng : size of the grazing-parameter grid.
        nthreads, small_planet_limit : accepted for compatibility; unused.
        precision : 'fp64' (plain FP64 path) or 'split' (FP32 per-sample path).
        device : CUDA device (default: the current one).
        """
        super().__init__()
        if 'interpolate' in kwargs:
            warn("The 'interpolate' argument has been replaced by 'precompute_weights' and will be removed in the future.", FutureWarning)
            self.interpolate: bool = kwargs.get('interpolate', False)
        else:
            self.interpolate: bool = precompute_weights
        if 'parallel' in kwargs:
            warn("The 'parallel' argument has been replaced by 'nthreads' and will be removed in the future.", FutureWarning)
        self.nthreads = nthreads
        self.splimit = small_planet_limit
        if precision not in ('fp64', 'split'):
            raise ValueError("precision must be 'fp64' or 'split'")
        self.precision = precision
        self.device = device
        # Pinned host output of the split path: part of the rows copied over
        # from the device while the host sets the others to 1 on host_threads
        # threads and the GPU writes only their transit tiles (host_fill True),
        # or the whole flux copied over in chunks (False).
        self.host_fill = True
        self.host_threads = _default_host_threads()
        self.host_fill_fraction = 0.5   # share of the rows set to 1 by the host (the rest copied over)
        # precision='fp64': the fold once per 128-point tile for tiles that
        # reach no box (the same bits as every point through it, False)
        self.fp64_cull = True

        # Limb darkening model (rrmodel.py:109-131)
        self.ld_law = None           # device law id of a named law, else None
        if isinstance(ldmodel, str):
            try:
                entry = self.ldmodels[ldmodel]
            except KeyError:
                print(f"Unknown limb darkening model: {ldmodel}. Choose from [{', '.join(self.ldmodels.keys())}] or supply a callable function.")
                raise
            self.ldmodel, self.ldmmean = entry if isinstance(entry, tuple) else (entry, None)
            self.ld_law = _ldm.LAW_IDS[ldmodel]
        elif isinstance(ldmodel, LDModel):
            self.ldmodel = ldmodel
            self.ldmmean = ldmodel._integrate
        elif callable(ldmodel):
            self.ldmodel = ldmodel
            self.ldmmean = None
        elif isinstance(ldmodel, tuple) and callable(ldmodel[0]) and callable(ldmodel[1]):
            self.ldmodel, self.ldmmean = ldmodel
        else:
            raise NotImplementedError
        if self.ld_law is None:
            # the library's own law functions still run on the device
            for name, entry in self.ldmodels.items():
                fl, fi = entry if isinstance(entry, tuple) else (entry, None)
                if self.ldmodel is fl and self.ldmmean is fi:
                    self.ld_law = _ldm.LAW_IDS[name]

        self.klims = klims
        self.nk, self.ng, self.nzin, self.nzlimb, self.zcut = nk, ng, nzin, nzlimb, zcut
        self._ldmu = np.linspace(1, 0, 200)
        self._ldz = np.sqrt(1 - self._ldmu ** 2)
        self._tables = None
        self._ws = None
        self.init_integration(nzin, nzlimb, zcut, ng, nk)

    # ------------------------------------------------------------------
    def init_integration(self, nzin, nzlimb, zcut, ng, nk):
        """Integration grid and weight-table constants (rrmodel.py:165-173);
        the table itself is built on the GPU at first use."""
        self.nk, self.ng, self.nzin, self.nzlimb, self.zcut = nk, ng, nzin, nzlimb, zcut
        self.ze, self.zm = create_z_grid(zcut, nzin, nzlimb)
        self.mu = np.sqrt(1 - self.zm ** 2)
        self.dk = (self.klims[1] - self.klims[0]) / nk
        self.dg = (1.0 - 1e-7) / (ng - 1)
        self._tables = None

    def set_data(self, time, lcids=None, pbids=None, nsamples=None, exptimes=None, epids=None) -> None:
        super().set_data(time, lcids, pbids, nsamples, exptimes, epids)
        self.nep = np.unique(self.epids).size

    # ------------------------------------------------------------------
    def _cuda_device(self):
        from . import _lib
        return _lib.require_cuda(self.device)

    def _device_tables(self, device):
        """Weight table W[nk, ng, nz] (FP64 and FP32) and the grids, on the GPU."""
        import ctypes as C
        import torch
        from . import _lib
        if self._tables is not None and self._tables['device'] == device:
            return self._tables
        nz = self.ze.size
        t = {'device': device}
        t['ze'] = torch.as_tensor(self.ze, dtype=torch.float64).to(device)
        t['mu'] = torch.as_tensor(self.mu, dtype=torch.float64).to(device)
        t['W64'] = torch.empty((self.nk, self.ng, nz), dtype=torch.float64, device=device)
        t['W32'] = torch.empty((self.nk, self.ng, nz), dtype=torch.float32, device=device)
        dk, dg = C.c_double(), C.c_double()
        _lib.check(_lib.lib().rr_weights_3d(self.nk, float(self.klims[0]), float(self.klims[1]),
                                            _lib.ptr(t['ze']), nz, self.ng, _lib.ptr(t['W64']),
                                            _lib.ptr(t['W32']), C.byref(dk), C.byref(dg),
                                            _lib.stream_ptr(device)), "rr_weights_3d")
        self.dk, self.dg = dk.value, dg.value
        self._tables = t
        return t

    def _basis(self, device, npar, split):
        """Basis tables of the named law (affine laws only), built once per (law, npar)."""
        import torch
        from . import _lib
        if self.ld_law is None:
            return None, 0
        L = _lib.lib()
        nb = L.rr_basis_count(self.ld_law, npar)
        if nb <= 0:
            return None, 0
        tb = self._device_tables(device)
        key = ('basis', npar)
        if key not in tb:
            nz = self.ze.size
            B64 = torch.empty((self.nk, nb, self.ng), dtype=torch.float64, device=device)
            B32 = torch.empty((self.nk, nb, self.ng), dtype=torch.float32, device=device)
            _lib.check(L.rr_basis_tables(self.ld_law, npar, _lib.ptr(tb['mu']), nz, _lib.ptr(tb['W64']), self.nk,
                                         self.ng, _lib.ptr(B64), _lib.ptr(B32), _lib.stream_ptr(device)),
                       "rr_basis_tables")
            tb[key] = (B64, B32)
        B64, B32 = tb[key]
        return (B32 if split else B64), nb

    def _workspace(self, nbytes, device):
        import torch
        if self._ws is None or self._ws.numel() < nbytes or self._ws.device != device:
            self._ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=device)
        return self._ws

    # ------------------------------------------------------------------
    @staticmethod
    def _vec(x, npv, name):
        x = np.atleast_1d(np.asarray(x, dtype=np.float64))
        if x.size == 1 and npv > 1:
            x = np.full(npv, x.reshape(-1)[0])
        if x.ndim != 1 or x.size != npv:
            raise ValueError(f"'{name}' should be a scalar or a vector of {npv} values.")
        return np.ascontiguousarray(x)

    def _shape_params(self, k, t0, p, a, i, e, w):
        """Parameter arrays shaped as rr_full expects (rrmodel.py:229-230)."""
        p = np.atleast_1d(np.asarray(p, dtype=np.float64))
        npv = p.size
        k = np.asarray(k, dtype=np.float64)
        if k.ndim == 0:
            k = k.reshape(1, 1)
        elif k.ndim == 1:
            k = k.reshape(npv, 1) if (npv > 1 and k.size == npv) else k.reshape(1, -1)
        if k.shape[0] == 1 and npv > 1:
            k = np.repeat(k, npv, axis=0)
        if k.shape[0] != npv:
            raise ValueError(f"Radius ratios given for {k.shape[0]} parameter vectors, expected {npv}.")
        if k.shape[1] > 1 and k.shape[1] != self.npb:
            raise ValueError('Radius ratios should be given either as an [npv, 1] or [npv, npb] array.')
        t0 = np.asarray(t0, dtype=np.float64)
        if t0.ndim == 0:
            t0 = np.full((npv, 1), float(t0))
        elif t0.ndim == 1:
            t0 = t0.reshape(npv, 1) if t0.size == npv else np.tile(t0, (npv, 1))
        elif t0.shape[0] == 1 and npv > 1:
            t0 = np.repeat(t0, npv, axis=0)
        if t0.shape[0] != npv:
            raise ValueError(f"Zero epochs given for {t0.shape[0]} parameter vectors, expected {npv}.")
        eps = np.asarray(self.epids).reshape(-1)
        if eps.size and eps.max() >= t0.shape[1]:
            raise ValueError(f"Epoch index {eps.max()} needs a zero epoch array with at least {eps.max() + 1} columns.")
        a, i, e, w = (self._vec(x, npv, n) for x, n in ((a, 'a'), (i, 'i'), (e, 'e'), (w, 'w')))
        return (np.ascontiguousarray(k), np.ascontiguousarray(t0), np.ascontiguousarray(p), a, i, e, w)

    def _shape_ldc(self, ldc, npv, npb):
        ldc = np.asarray(ldc, dtype=np.float64)
        if ldc.ndim == 0:
            ldc = ldc.reshape(1, 1, 1)
        elif ldc.ndim == 1:
            ldc = ldc.reshape(1, 1, -1)
        elif ldc.ndim == 2:
            ldc = ldc.reshape(1, ldc.shape[0], -1)
        if ldc.shape[1] == 1 and npb > 1:
            ldc = np.repeat(ldc, npb, axis=1)
        if ldc.shape[0] == 1 and npv > 1:
            ldc = np.repeat(ldc, npv, axis=0)
        if ldc.shape[0] != npv or ldc.shape[1] != npb:
            raise ValueError(f"Limb darkening coefficients should be given as a [npv, npb, ncoef] array "
                             f"with npv={npv}, npb={npb}; got {ldc.shape}.")
        return np.ascontiguousarray(ldc)

    def _ld_tables(self, ldc, npv, npb, device, split, ldc_d=None):
        """(ldp[npv, npb, nz], istar[npv, npb]) on the device (rrmodel.py:212-227).
        For a named law ``ldc_d`` is the [npv, npb, ncoef] array already on the device."""
        import torch
        from . import _lib
        tb = self._device_tables(device)
        nz = self.ze.size
        dt = torch.float32 if split else torch.float64
        if self.ld_law is not None:
            if ldc_d is None:
                ldc_d = torch.as_tensor(self._shape_ldc(ldc, npv, npb)).to(device)
            ldc3 = ldc_d
            ldp = torch.empty((npv, npb, nz), dtype=dt, device=device)
            istar = torch.empty((npv, npb), dtype=dt, device=device)
            fn = _lib.lib().rr_ld_tables_f32 if split else _lib.lib().rr_ld_tables_f64
            _lib.check(fn(self.ld_law, _lib.ptr(ldc_d), npv, npb, ldc3.shape[2], _lib.ptr(tb['mu']), nz,
                          _lib.ptr(ldp), _lib.ptr(istar), _lib.stream_ptr(device)), "rr_ld_tables")
            return ldp, istar
        # host LD models: evaluated on the CPU, uploaded
        if isinstance(self.ldmodel, LDModel):
            ldp, istar = self.ldmodel(self.mu, np.atleast_1d(np.asarray(ldc, dtype=np.float64)))
        else:
            ldc3 = self._shape_ldc(ldc, npv, npb)
            ldp = _ldm.evaluate_ld(self.ldmodel, self.mu, ldc3)
            if self.ldmmean is not None:
                istar = _ldm.evaluate_ldi(self.ldmmean, ldc3)
            else:
                ldpi = _ldm.evaluate_ld(self.ldmodel, self._ldmu, ldc3)
                istar = 2 * np.pi * np.trapezoid(self._ldz * ldpi, self._ldz, axis=-1)
        ldp = np.asarray(ldp, dtype=np.float64)
        ldp = ldp.reshape((1,) * (3 - ldp.ndim) + ldp.shape) if ldp.ndim < 3 else ldp
        istar = np.asarray(istar, dtype=np.float64)
        istar = istar.reshape((1,) * (2 - istar.ndim) + istar.shape) if istar.ndim < 2 else istar
        try:
            ldp = np.broadcast_to(ldp, (npv, npb, nz))
            istar = np.broadcast_to(istar, (npv, npb))
        except ValueError:
            raise ValueError(f"The limb darkening model returned ldp {ldp.shape} and istar {istar.shape}; "
                             f"expected [{npv}, {npb}, {nz}] and [{npv}, {npb}].") from None
        ldp_d = torch.as_tensor(np.array(ldp, dtype=np.float64)).to(device=device, dtype=dt)
        istar_d = torch.as_tensor(np.array(istar, dtype=np.float64)).to(device=device, dtype=dt)
        return ldp_d, istar_d

    # ------------------------------------------------------------------
    def _flux_to_host(self, dd, npt, npv, nlc, npb, ws, out2d, device, nchunks=8):
        """Split-path flux into the pinned host rows out2d[npv, npt]: the pv
        range in chunks through two device buffers, the flux of chunk c+1
        computed on the current stream while chunk c is copied on a copy
        stream.  Returns the first non-zero status."""
        import torch
        from . import _lib
        L, P = _lib.lib(), _lib.ptr
        bounds = np.linspace(0, npv, min(nchunks, npv) + 1).astype(int)
        rows = int(np.diff(bounds).max())
        key = (device, rows, npt)
        if getattr(self, '_pipe', None) is None or self._pipe[0] != key:
            self._pipe = (key, [torch.empty((rows, npt), dtype=torch.float32, device=device) for _ in range(2)],
                          torch.cuda.Stream(device))
        _, bufs, cs = self._pipe
        comp = torch.cuda.current_stream(device)
        sp = C.c_void_p(comp.cuda_stream)
        copied = [None, None]
        for c in range(len(bounds) - 1):
            pv0, pv1 = int(bounds[c]), int(bounds[c + 1])
            b = bufs[c % 2]
            if copied[c % 2] is not None:
                comp.wait_event(copied[c % 2])
            st = L.rr_flux_split_range(P(dd['times_ff']), npt, P(dd['lcids']), npv, nlc, npb, self.ng, self.dg,
                                       P(ws), pv0, pv1, P(b), npt, sp)
            if st != 0:
                return st
            done = torch.cuda.Event()
            done.record(comp)
            cs.wait_event(done)
            with torch.cuda.stream(cs):
                out2d[pv0:pv1].copy_(b[:pv1 - pv0], non_blocking=True)
                copied[c % 2] = torch.cuda.Event()
                copied[c % 2].record(cs)
        comp.wait_stream(cs)
        return 0

    # copy=True results of at least this many points are written straight
    # into pinned host memory (torch's cached host allocator), smaller ones
    # copied from the device
    PINNED_RESULT_MIN = 1 << 17

    def _flux_to_pinned(self, dd, npt, npv, nlc, npb, ws, out2d, device, nchunks=4, fill_fraction=None):
        """Split-path flux into the pinned host rows out2d[npv, npt] (float32,
        or float64 with each FP32 result widened) over the host link and the
        host's own memory bandwidth at once.  The first rows (a
        1 - host_fill_fraction share) are computed on the device in one launch
        and copied over on a copy stream.  Meanwhile the host sets the other
        rows to 1, a pv chunk at a time, on the library's threads
        (rr_host_fill_f32/_f64), and after each chunk the GPU writes that
        chunk's transit tiles and invalid rows straight into it
        (rr_flux_split_transits[_f64]): tiles that reach no transit window
        never cross the link.  The current stream waits for the copy; the
        caller synchronises it.  Returns the first non-zero status."""
        import torch
        from . import _lib
        L, P = _lib.lib(), _lib.ptr
        f64 = out2d.dtype == torch.float64
        esize = 8 if f64 else 4
        dense = L.rr_flux_split_range_f64 if f64 else L.rr_flux_split_range
        transits = L.rr_flux_split_transits_f64 if f64 else L.rr_flux_split_transits
        fill = L.rr_host_fill_f64 if f64 else L.rr_host_fill_f32
        comp = torch.cuda.current_stream(device)
        sp = C.c_void_p(comp.cuda_stream)
        frac = self.host_fill_fraction if fill_fraction is None else fill_fraction
        ncopy = int(round(npv * (1.0 - min(1.0, max(0.0, float(frac))))))
        cs = None
        if ncopy > 0:
            key = (device, ncopy, npt, out2d.dtype)
            if getattr(self, '_stage', None) is None or self._stage[0] != key:
                self._stage = (key, torch.empty((ncopy, npt), dtype=out2d.dtype, device=device),
                               torch.cuda.Stream(device))
            _, buf, cs = self._stage
            st = dense(P(dd['times_ff']), npt, P(dd['lcids']), npv, nlc, npb, self.ng, self.dg, P(ws), 0, ncopy,
                       P(buf), npt, sp)
            if st != 0:
                return st
            cs.wait_stream(comp)
            with torch.cuda.stream(cs):
                out2d[:ncopy].copy_(buf, non_blocking=True)
        base = out2d.data_ptr()
        nfill = npv - ncopy
        bounds = ncopy + np.linspace(0, nfill, min(nchunks, nfill) + 1).astype(int) if nfill > 0 else []
        for c in range(len(bounds) - 1):
            pv0, pv1 = int(bounds[c]), int(bounds[c + 1])
            rows = C.c_void_p(base + pv0 * npt * esize)
            st = fill(rows, (pv1 - pv0) * npt, 1.0, int(self.host_threads))
            if st == 0:
                st = transits(P(dd['times_ff']), npt, P(dd['lcids']), npv, nlc, npb, self.ng, self.dg, P(ws),
                              pv0, pv1, rows, npt, sp)
            if st != 0:
                return st
        if cs is not None:
            comp.wait_stream(cs)
        return 0

    def _flux64(self, L, P, dd, args, istar, npt, npv, nlc, npb, ws, pv0, pv1, out, stream):
        """The FP64 flux of pvs [pv0, pv1) into their rows out[pv1 - pv0, npt]:
        tile-culled (rr_flux_f64_culled_range, the same bits) unless fp64_cull
        is off, then every point through the reference's arithmetic
        (rr_flux_f64_range)."""
        k, t0 = args['k'], args['t0']
        common = (npt, P(k), k.shape[1], P(t0), t0.shape[1], P(args['p']), npv, nlc, npb, P(dd['lcids']),
                  P(dd['pbids']), P(dd['epids']), P(dd['nsamples']), P(dd['exptimes']), P(istar), self.ng, self.dg,
                  P(ws), pv0, pv1, P(out), npt, stream)
        if self.fp64_cull:
            return L.rr_flux_f64_culled_range(P(dd['time']), P(dd['tiles64']), *common)
        return L.rr_flux_f64_range(P(dd['time']), *common)

    def _flux64_to_host(self, args, dd, istar, npt, npv, nlc, npb, ws, out2d, device, nchunks=8):
        """Plain FP64 flux into the pinned host rows out2d[npv, npt]: the pv
        range in chunks (rr_flux_f64_range) through two device buffers, each
        chunk copied to the host on a copy stream while the next one is
        computed.  Returns the first non-zero status."""
        import torch
        from . import _lib
        L, P = _lib.lib(), _lib.ptr
        bounds = np.linspace(0, npv, min(nchunks, npv) + 1).astype(int)
        rows = int(np.diff(bounds).max())
        key = (device, rows, npt)
        if getattr(self, '_pipe64', None) is None or self._pipe64[0] != key:
            self._pipe64 = (key, [torch.empty((rows, npt), dtype=torch.float64, device=device) for _ in range(2)],
                            torch.cuda.Stream(device))
        _, bufs, cs = self._pipe64
        comp = torch.cuda.current_stream(device)
        sp = C.c_void_p(comp.cuda_stream)
        k, t0 = args['k'], args['t0']
        copied = [None, None]
        for c in range(len(bounds) - 1):
            pv0, pv1 = int(bounds[c]), int(bounds[c + 1])
            b = bufs[c % 2]
            if copied[c % 2] is not None:
                comp.wait_event(copied[c % 2])
            st = self._flux64(L, P, dd, args, istar, npt, npv, nlc, npb, ws, pv0, pv1, b, sp)
            if st != 0:
                return st
            done = torch.cuda.Event()
            done.record(comp)
            cs.wait_event(done)
            with torch.cuda.stream(cs):
                out2d[pv0:pv1].copy_(b[:pv1 - pv0], non_blocking=True)
                copied[c % 2] = torch.cuda.Event()
                copied[c % 2].record(cs)
        comp.wait_stream(cs)
        return 0

    def evaluate(self, k: Union[float, ndarray], ldc: Union[ndarray, List], t0: Union[float, ndarray],
                 p: Union[float, ndarray], a: Union[float, ndarray], i: Union[float, ndarray],
                 e: Union[float, ndarray] = 0.0, w: Union[float, ndarray] = 0.0, copy: bool = True,
                 out=None, return_error: bool = False):
        """Evaluate the transit model for one or many parameter vectors.

        Returns the modelled flux, [npt] for one parameter vector and
        [npv, npt] for many (squeezed as the reference does).  With copy=True a
        float64 numpy array; from PINNED_RESULT_MIN points on it is a view of
        page-locked host memory from torch's cached host allocator, which the
        GPU fills directly.  With copy=False the torch tensor on the GPU
        (float64, or float32 in the split precision).

        ``out``: an optional [npv, npt] torch tensor (pinned host memory or
        device) that receives the flux; it is filled, synchronised and
        returned.  Contiguous pinned host rows (float32 or float64 in the split
        path, float64 in the plain one) are filled without a device copy of
        the whole result.  In the split path part of the rows are computed on
        the device and copied over, while the host sets the others to 1
        (``host_threads`` threads) and the GPU writes their tiles that reach a
        transit window straight into them, so out-of-transit points need not
        cross the host link.  The plain path copies pv chunks over while the
        next chunk is computed.

        return_error=True returns (flux, bound): the stated maximum absolute
        flux error of this result against the FP64 model (see
        ``last_error_bound``)."""
        device = self._cuda_device()
        k, t0, p, a, i, e, w = self._shape_params(k, t0, p, a, i, e, w)
        ldc3 = self._shape_ldc(ldc, p.size, self.npb) if self.ld_law is not None else None
        args = self._upload(dict(k=k, t0=t0, p=p, a=a, i=i, e=e, w=w, ldc=ldc3), device)
        res = self._evaluate_device(args, ldc, out, copy)
        return (res, self.last_error_bound) if return_error else res

    # ------------------------------------------------------------------
    # Stated error of the last result
    FP64_ERROR_BOUND = 1e-12   # the plain path follows the reference's FP64 arithmetic (measured <= 2e-15)

    def error_bounds(self):
        """Per parameter vector of the last evaluate(): an upper bound of the
        absolute flux error against the FP64 model over all its points (numpy
        float64).  The split path's bound comes from its own tables
        (rr_split_error_bounds): the FP32 orbit coefficients against the FP64
        ones, the flux's sensitivity to z on every LD-table row, the FP32
        deficit and the FP32 result.  Valid until the next evaluate()."""
        import torch
        from . import _lib
        st = getattr(self, '_bound_state', None)
        if st is None:
            raise RuntimeError("no evaluation to state an error bound for")
        if st.get('bounds') is not None:
            return st['bounds']
        if not st['split']:
            st['bounds'] = np.full(st['npv'], self.FP64_ERROR_BOUND)
            return st['bounds']
        device = st['device']
        L = _lib.lib()
        P = _lib.ptr
        bnd = torch.empty(st['npv'], dtype=torch.float64, device=device)
        prm = st['prm']
        if st.get('ts'):
            rc = L.rr_ts_split_error_bounds(*(P(prm[n]) for n in ('p', 'a', 'i', 'e', 'w')), st['npv'], st['npb'],
                                            self.ng, self.dg, st['ns0'], st['ex0'], P(st['ws']), P(bnd), None,
                                            _lib.stream_ptr(device))
        else:
            rc = L.rr_split_error_bounds(*(P(prm[n]) for n in ('p', 'a', 'i', 'e', 'w')), st['npv'], st['npb'],
                                         st['nlc'], st['nep'], self.ng, self.dg, P(st['ws']), P(bnd), None,
                                         _lib.stream_ptr(device))
        _lib.check(rc, "rr_split_error_bounds")
        st['bounds'] = bnd.cpu().numpy()
        return st['bounds']

    @property
    def last_error_bound(self) -> float:
        """The stated maximum absolute flux error of the last evaluate()'s
        result against the FP64 model (the largest of ``error_bounds()``)."""
        b = self.error_bounds()
        return float(np.nanmax(b)) if b.size else 0.0

    def _evaluate_device(self, args, ldc=None, out=None, copy=False):
        """The device half of evaluate: args holds float64 device tensors k[npv,
        nkc], t0[npv, nep], p, a, i, e, w[npv] and, for a named law, ldc[npv, npb,
        ncoef] (ldc: the host coefficients, used only by host LD models)."""
        import torch
        from . import _lib
        user_out = out
        device = self._cuda_device()
        k, t0 = args['k'], args['t0']
        npv, npt, npb, nlc = args['p'].numel(), self.npt, self.npb, self.nlc
        split = self.precision == 'split'
        tb = self._device_tables(device)
        dd = self._device_data(device)
        L = _lib.lib()
        stream = _lib.stream_ptr(device)
        nz = self.ze.size
        P = _lib.ptr
        ldc_d = args.get('ldc')
        npar = int(ldc_d.shape[2]) if ldc_d is not None else 0
        basis, nb = self._basis(device, npar, split) if ldc_d is not None else (None, 0)
        # a named law in the split path: the LD tables are made by the prologue launch itself
        fused = split and self.ld_law is not None and ldc_d is not None
        if fused:
            ldp = torch.empty((npv, npb, nz), dtype=torch.float32, device=device)
            istar = torch.empty((npv, npb), dtype=torch.float32, device=device)
        else:
            ldp, istar = self._ld_tables(ldc, npv, npb, device, split, ldc_d)
        kmin, kmax = float(self.klims[0]), float(self.klims[1])
        # Host rows the flux goes to directly: a caller's contiguous pinned
        # buffer (float32 or float64 in the split path, float64 in the plain
        # one), or, for copy=True, a pinned float64 buffer from torch's cached
        # host allocator whose numpy view is returned.
        host_rows = None
        if user_out is not None:
            if (user_out.device.type == 'cpu' and user_out.is_pinned() and user_out.is_contiguous()
                    and user_out.numel() == npv * npt
                    and user_out.dtype in ((torch.float32, torch.float64) if split else (torch.float64,))):
                host_rows = user_out.view(npv, npt)
        elif copy and npv * npt >= self.PINNED_RESULT_MIN:
            try:
                host_rows = torch.empty((npv, npt), dtype=torch.float64, pin_memory=True)
            except RuntimeError:        # no page-locked memory to be had: copy the device result instead
                host_rows = None
        pipe = host_rows is not None
        if split:
            ldf = (npt + 3) // 4 * 4
            res = None if pipe else torch.empty((npv, ldf), dtype=torch.float32, device=device)
            nep = t0.shape[1]
            wsb = L.rr_full_split_workspace_bytes(npv, npb, nlc, nep, self.ng)
            ws = self._workspace(wsb, device)
            if fused:
                st = L.rr_prepare_split_ld(dd['t_ref'], dd['t_absmax'], P(args['k']), k.shape[1], P(args['t0']),
                                           t0.shape[1], nep, P(args['p']), P(args['a']), P(args['i']),
                                           P(args['e']), P(args['w']), npv, nlc, npb, P(dd['pbids']),
                                           P(dd['epids']), P(dd['nsamples']), P(dd['exptimes']), self.ld_law,
                                           P(ldc_d), npar, P(tb['mu']), nz, P(basis), nb, P(tb['W32']), self.nk,
                                           self.ng, self.dk, kmin, kmax, P(tb['ze']), P(ldp), P(istar), P(ws),
                                           ws.numel(), stream)
            else:
                st = L.rr_prepare_split(dd['t_ref'], dd['t_absmax'], P(args['k']), k.shape[1], P(args['t0']),
                                        t0.shape[1], nep, P(args['p']), P(args['a']), P(args['i']), P(args['e']),
                                        P(args['w']), npv, nlc, npb, P(dd['pbids']), P(dd['epids']),
                                        P(dd['nsamples']), P(dd['exptimes']), P(ldp), P(istar), P(tb['W32']),
                                        self.nk, self.ng, nz, self.dk, kmin, kmax, P(tb['ze']), P(ws), ws.numel(),
                                        stream, self.ld_law or 0, P(ldc_d), npar, P(basis), nb)
            if st == 0 and pipe:
                if self.host_fill:
                    st = self._flux_to_pinned(dd, npt, npv, nlc, npb, ws, host_rows, device)
                elif host_rows.dtype == torch.float32:
                    st = self._flux_to_host(dd, npt, npv, nlc, npb, ws, host_rows, device)
                else:
                    st = self._flux_to_pinned(dd, npt, npv, nlc, npb, ws, host_rows, device, fill_fraction=0.0)
            elif st == 0:
                st = L.rr_flux_split(P(dd['times_ff']), npt, P(dd['lcids']), npv, nlc, npb, self.ng, self.dg,
                                     P(ws), P(res), ldf, stream)
            res = None if pipe else res[:, :npt]
        else:
            res = None if pipe else torch.empty((npv, npt), dtype=torch.float64, device=device)
            wsb = L.rr_full_f64_workspace_bytes(npv, npb, self.ng)
            ws = self._workspace(wsb, device)
            st = L.rr_prepare_f64(P(args['k']), k.shape[1], P(args['p']), P(args['a']), P(args['i']),
                                  P(args['e']), P(args['w']), npv, npb, P(ldp), P(tb['W64']), self.nk, self.ng, nz,
                                  self.dk, kmin, kmax, P(tb['ze']), P(ws), ws.numel(), stream,
                                  self.ld_law or 0, P(ldc_d), npar, P(basis), nb)
            if st == 0 and pipe:
                st = self._flux64_to_host(args, dd, istar, npt, npv, nlc, npb, ws, host_rows, device)
            elif st == 0:
                st = self._flux64(L, P, dd, args, istar, npt, npv, nlc, npb, ws, 0, npv, res, stream)
        _lib.check(st, "rr_full")
        self._bound_state = dict(split=split, npv=npv, npb=npb, nlc=nlc, nep=t0.shape[1], ws=ws, device=device,
                                 prm={n: args[n] for n in ('p', 'a', 'i', 'e', 'w')})
        if pipe:
            torch.cuda.current_stream(device).synchronize()
            return user_out if user_out is not None else host_rows.numpy().squeeze()
        if user_out is not None:
            src = res if user_out.dtype == res.dtype else res.to(user_out.dtype)
            user_out.view(npv, npt).copy_(src, non_blocking=True)
            torch.cuda.current_stream(device).synchronize()
            return user_out
        res = res.squeeze()
        if copy:
            return res.to(torch.float64).cpu().numpy()
        return res

"""Secondary-eclipse models on the GPU: drop-ins for the reference's RoadRunner
eclipse models.

* ``EclipseModel`` (pytransit/models/new_eclipse_model.py:27-66): the
  multiplicative eclipse model, the visible area of the planet disk
  (eclipse_model, pytransit/models/roadrunner/model_eclipse.py:12-81);
* ``EclipseSpectroscopyModel`` / ``ESModel``
  (pytransit/models/roadrunner/esmodel.py:29-92): npb flux ratios sharing one
  orbit (esmodel, model_ecspec.py:13-63).

Both run on the RoadRunner orbit layer expanded about mid-eclipse, as FP64
CUDA kernels (rr_eclipse_f64, rr_es_f64; precision='fp64', the default) or in
split precision (rr_eclipse_split, rr_es_split; precision='split'): FP64
per-pv prologue, exact FP32-pair phase fold, FP32 per-sample areas and FP32
output, with the 128-point tiles outside every eclipse window written as
plain runs of the out-of-eclipse value.  One deliberate difference: the
reference's EclipseModel.evaluate passes the passband indices where the
kernel expects the epoch indices (new_eclipse_model.py:66); here the epoch
indices of set_data are used.
"""
import ctypes as C
from typing import Union

import numpy as np
from numpy import ndarray

from . import _lib
from .transitmodel import TransitModel

__all__ = ['EclipseModel', 'EclipseSpectroscopyModel', 'ESModel']

_vp, _i, _d, _sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
_SIG = {
    'rr_eclipse_workspace_bytes': ([_i], _sz),
    'rr_eclipse_f64': ([_vp, _i, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _sz,
                        _vp, _i, _vp], _i),
    'rr_eclipse_f64_culled': ([_vp, _vp, _i, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _vp, _vp, _vp, _vp,
                               _vp, _sz, _vp, _i, _vp], _i),
    'rr_es_f64': ([_vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _vp, _sz, _vp, _i, _vp],
                  _i),
    'rr_eclipse_split_workspace_bytes': ([_i, _i, _i], _sz),
    'rr_eclipse_split': ([_vp, _d, _d, _i, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _vp, _vp, _vp, _vp,
                          _vp, _sz, _vp, _i, _vp], _i),
    'rr_es_split': ([_vp, _d, _d, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _vp, _sz, _vp, _i,
                     _vp], _i),
}
_lib._EXTRA_SIGNATURES.update(_SIG)


def _L():
    L = _lib.lib()
    for name, (args, res) in _SIG.items():
        f = getattr(L, name)
        f.argtypes, f.restype = args, res
    return L


def _vec(x, npv, name):
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    if x.size == 1:
        return np.full(npv, float(x[0]))
    if x.size != npv:
        raise ValueError(f"{name} should be a scalar or have one value per parameter vector ({npv})")
    return np.ascontiguousarray(x)


class _GpuEclipseBase(TransitModel):
    def __init__(self, precision: str = 'fp64', device=None):
        super().__init__()
        if precision not in ('fp64', 'split'):
            raise ValueError("precision must be 'fp64' or 'split'")
        self.precision = precision
        self.device = device
        # precision='fp64': the fold once per 128-point tile for tiles that
        # reach no box (the same bits as every point through it, False)
        self.fp64_cull = True

    def _cuda_device(self):
        return _lib.require_cuda(self.device)


class EclipseModel(_GpuEclipseBase):
    """Multiplicative secondary-eclipse model: the visible area of the planet."""

    def evaluate(self, k, t0, p, a, i, e=None, w=None, rstar: Union[float, ndarray] = 1.0, copy: bool = True):
        """Visible planet area for one or many parameter vectors (pi k^2 out of
        eclipse), squeezed as the reference's; rstar in solar radii for the
        light travel time.  copy=False returns the CUDA tensor [npv, npt]."""
        import torch
        dev = self._cuda_device()
        k = np.atleast_1d(np.asarray(k, dtype=np.float64)).ravel()
        npv = k.size
        t0 = np.atleast_2d(np.asarray(t0, dtype=np.float64)).reshape([npv, -1])
        eps = np.asarray(self.epids).reshape(-1)
        if eps.size and eps.max() >= t0.shape[1]:
            raise ValueError(f"Epoch index {eps.max()} needs a zero epoch array with at least {eps.max() + 1} columns.")
        vecs = {n: _vec(x, npv, n) for n, x in (('p', p), ('a', a), ('i', i), ('e', 0.0 if e is None else e),
                                                ('w', 0.0 if w is None else w), ('rstar', rstar))}
        dd = self._device_data(dev)
        g = self._upload(dict(k=k, t0=t0, **vecs), dev)   # one pinned host-to-device copy
        L = _L()
        P = _lib.ptr
        if self.precision == 'split':
            wsb = L.rr_eclipse_split_workspace_bytes(npv, self.nlc, 1)
            ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
            out = torch.empty((npv, self.npt), dtype=torch.float32, device=dev)
            _lib.check(L.rr_eclipse_split(P(dd['times_ff']), dd['t_ref'], dd['t_absmax'], self.npt, P(g['k']),
                                          P(g['t0']), t0.shape[1], P(g['p']), P(g['a']), P(g['i']), P(g['e']),
                                          P(g['w']), P(g['rstar']), npv, self.nlc, P(dd['lcids']), P(dd['epids']),
                                          P(dd['nsamples']), P(dd['exptimes']), P(ws), wsb, P(out), self.npt,
                                          _lib.stream_ptr(dev)), "rr_eclipse_split")
        else:
            wsb = L.rr_eclipse_workspace_bytes(npv)
            ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
            out = torch.empty((npv, self.npt), dtype=torch.float64, device=dev)
            rest = (self.npt, P(g['k']), P(g['t0']), t0.shape[1], P(g['p']), P(g['a']), P(g['i']), P(g['e']),
                    P(g['w']), P(g['rstar']), npv, self.nlc, P(dd['lcids']), P(dd['epids']), P(dd['nsamples']),
                    P(dd['exptimes']), P(ws), wsb, P(out), self.npt, _lib.stream_ptr(dev))
            if self.fp64_cull:      # the same bits with the fold once per tile that reaches no box
                _lib.check(L.rr_eclipse_f64_culled(P(dd['time']), P(dd['tiles64']), *rest), "rr_eclipse_f64")
            else:
                _lib.check(L.rr_eclipse_f64(P(dd['time']), *rest), "rr_eclipse_f64")
        if not copy:
            return out
        return np.squeeze(_lib.to_host_f64(out))

    def __call__(self, *args, **kwargs):
        return self.evaluate(*args, **kwargs)


class EclipseSpectroscopyModel(_GpuEclipseBase):
    """Secondary eclipse for npb channels (flux ratios f[npv, npb]) sharing one orbit."""

    def __init__(self, parallel: bool = False, precision: str = 'fp64', device=None):
        # the reference's ``parallel`` selects its numba variant; one GPU path here
        super().__init__(precision=precision, device=device)

    def evaluate(self, f, k, t0, p, a, i, e=0.0, w=0.0, rstar: Union[float, ndarray] = 1.0, copy: bool = True):
        """flux[npv, npb, npt] (numpy with copy=True, else the CUDA tensor);
        the first light curve's nsamples and exposure time, as the reference."""
        import torch
        dev = self._cuda_device()
        k = np.atleast_1d(np.asarray(k, dtype=np.float64)).ravel()
        npv = k.size
        f = np.asarray(f, dtype=np.float64)
        if f.ndim != 2:
            raise ValueError(" The flux ratio must be given as a 2D array with shape (npv, npb)")
        npb = f.shape[1]
        if f.shape[0] != npv:
            raise ValueError(f"The flux ratios are given for {f.shape[0]} parameter vectors, expected {npv}.")
        vecs = {n: _vec(x, npv, n) for n, x in (('t0', t0), ('p', p), ('a', a), ('i', i), ('e', e), ('w', w),
                                                ('rstar', rstar))}
        dd = self._device_data(dev)
        g = self._upload(dict(k=k, f=f, **vecs), dev)
        L = _L()
        P = _lib.ptr
        ns0 = int(np.atleast_1d(self.nsamples)[0])
        ex0 = float(np.atleast_1d(self.exptimes)[0])
        if self.precision == 'split':
            wsb = L.rr_eclipse_split_workspace_bytes(npv, 1, npb)
            ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
            out = torch.empty((npv, npb, self.npt), dtype=torch.float32, device=dev)
            _lib.check(L.rr_es_split(P(dd['times_ff']), dd['t_ref'], dd['t_absmax'], self.npt, P(g['k']), P(g['t0']),
                                     P(g['p']), P(g['a']), P(g['i']), P(g['e']), P(g['w']), P(g['rstar']), P(g['f']),
                                     npv, npb, ns0, ex0, P(ws), wsb, P(out), self.npt, _lib.stream_ptr(dev)),
                       "rr_es_split")
        else:
            wsb = L.rr_eclipse_workspace_bytes(npv)
            ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
            out = torch.empty((npv, npb, self.npt), dtype=torch.float64, device=dev)
            _lib.check(L.rr_es_f64(P(dd['time']), self.npt, P(g['k']), P(g['t0']), P(g['p']), P(g['a']), P(g['i']),
                                   P(g['e']), P(g['w']), P(g['rstar']), P(g['f']), npv, npb, ns0, ex0, P(ws), wsb,
                                   P(out), self.npt, _lib.stream_ptr(dev)), "rr_es_f64")
        return _lib.to_host_f64(out) if copy else out

    def __call__(self, *args, **kwargs):
        return self.evaluate(*args, **kwargs)


ESModel = EclipseSpectroscopyModel

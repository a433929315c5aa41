"""The independent cross-check of the RoadRunner path: the Mandel & Agol (2002)
quadratic limb-darkening model on the GPU.

PyTransit's quadratic model (pytransit/models/numba/ma_quadratic_nb.py) is an
analytic model built from complete elliptic integrals; RoadRunner approximates
the same light curve with precomputed weight tables.  ``ma_quadratic_z``
evaluates the analytic flux at given centre distances (eval_quad_z_s) and
``rr_vs_ma`` evaluates both models for a RoadRunnerModel's data and parameter
vectors on the same orbit layer (phase fold, Taylor-series z, bounding box), so
that their difference is the RoadRunner discretisation alone.  Both run in
FP64 CUDA kernels (rr_ma_quad_z_f64, rr_ma_quad_flux_f64).
"""
import ctypes as C

import numpy as np
import torch

from . import _lib

__all__ = ['ma_quadratic_z', 'rr_vs_ma']

_vp, _i, _d = C.c_void_p, C.c_int, C.c_double
_SIG = {
    'rr_ma_quad_z_f64': ([_vp, _i, _d, _d, _d, _vp, _vp], _i),
    'rr_ma_quad_flux_f64': ([_vp, _i, _vp, _i, _vp, _i, _vp, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                             _i, _vp], _i),
}
_lib._EXTRA_SIGNATURES.update(_SIG)


def _L():
    L = _lib.lib()
    for name, (args, res) in _SIG.items():
        f = getattr(L, name)
        f.argtypes, f.restype = args, res
    return L


def ma_quadratic_z(z, k: float, u1: float, u2: float, device=None) -> np.ndarray:
    """Quadratic-LD flux at centre distances z (numpy, float64)."""
    dev = _lib.require_cuda(device)
    zt = torch.as_tensor(np.ascontiguousarray(z, dtype=np.float64).ravel()).to(dev)
    out = torch.empty_like(zt)
    L = _L()
    _lib.check(L.rr_ma_quad_z_f64(_lib.ptr(zt), zt.numel(), float(k), float(u1), float(u2), _lib.ptr(out),
                                  _lib.stream_ptr(dev)), "rr_ma_quad_z_f64")
    return out.cpu().numpy().reshape(np.shape(z))


def rr_vs_ma(model, k, ldc, t0, p, a, i, e=0.0, w=0.0):
    """RoadRunner flux and Mandel & Agol flux for ``model`` (a quadratic-LD
    RoadRunnerModel with data set) and the parameter vectors, both in FP64 on
    the same orbit layer.  Returns (rr_flux, ma_flux) as [npv, npt] numpy arrays."""
    from .rrmodel import RoadRunnerModel
    if not isinstance(model, RoadRunnerModel) or model.ld_law != 2:
        raise ValueError("rr_vs_ma needs a RoadRunnerModel with the quadratic limb-darkening law")
    if model.precision != 'fp64':
        raise ValueError("rr_vs_ma compares the FP64 RoadRunner path; build the model with precision='fp64'")
    m = model
    device = m._cuda_device()
    rr = m.evaluate(k, ldc, t0, p, a, i, e, w, copy=False).reshape(-1, m.npt)
    # the model's workspace now holds the orbit records of this evaluation
    kk, t0s, ps, *_ = m._shape_params(k, t0, p, a, i, e, w)
    npv = ps.size
    ldc3 = m._shape_ldc(ldc, npv, m.npb)
    dd = m._device_data(device)
    args = {n: torch.as_tensor(np.ascontiguousarray(v, dtype=np.float64)).to(device)
            for n, v in (('k', kk), ('t0', t0s), ('p', ps), ('ldc', ldc3))}
    out = torch.empty((npv, m.npt), dtype=torch.float64, device=device)
    L = _L()
    P = _lib.ptr
    _lib.check(L.rr_ma_quad_flux_f64(P(dd['time']), m.npt, P(args['k']), kk.shape[1], P(args['t0']), t0s.shape[1],
                                     P(args['p']), npv, m.nlc, m.npb, P(dd['lcids']), P(dd['pbids']),
                                     P(dd['epids']), P(dd['nsamples']), P(dd['exptimes']), P(args['ldc']),
                                     P(m._ws), P(out), m.npt, _lib.stream_ptr(device)), "rr_ma_quad_flux_f64")
    return rr.cpu().numpy(), out.cpu().numpy()

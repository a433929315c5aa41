"""Sampler populations on the device: the parameter mapping of
BaseLPF.transit_model (pytransit/lpf/lpf.py:435-443) as a CUDA kernel
(rr_lpf_map), feeding the RoadRunner model or the fused Gaussian
log-likelihood without a round trip to the host.

A population is a float64 CUDA tensor pv[npv, ncols] with the LPF's layout:
[tc, p, rho, b, k2] followed by (q1, q2) per passband from column ld_start.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib

__all__ = ['map_pv', 'transit_model', 'lnlikelihood']

_vp, _i, _d = C.c_void_p, C.c_int, C.c_double
_SIG = {'rr_lpf_map': ([_vp, _i, _i, _i, _i, _d, _vp, _vp, _vp, _vp, _vp, _vp, _vp], _i)}
_lib._EXTRA_SIGNATURES.update(_SIG)


def _L():
    L = _lib.lib()
    for name, (args, res) in _SIG.items():
        f = getattr(L, name)
        f.argtypes, f.restype = args, res
    return L


def map_pv(pv: torch.Tensor, tref: float, npb: int, ld_start: int = 5):
    """Model parameters of a population (device tensors): k[npv, 1], t0[npv, 1],
    p, a, i [npv], ldc[npv, npb, 2]."""
    if not (torch.is_tensor(pv) and pv.is_cuda and pv.dtype == torch.float64 and pv.dim() == 2):
        raise ValueError("pv must be a 2D float64 CUDA tensor [npv, ncols]")
    pv = pv.contiguous()
    npv, ncols = pv.shape
    dev = pv.device
    out = {n: torch.empty(npv, dtype=torch.float64, device=dev) for n in ('k', 't0', 'p', 'a', 'i')}
    out['ldc'] = torch.empty((npv, npb, 2), dtype=torch.float64, device=dev)
    P = _lib.ptr
    _lib.check(_L().rr_lpf_map(P(pv), npv, ncols, npb, ld_start, float(tref), P(out['k']), P(out['t0']),
                               P(out['p']), P(out['a']), P(out['i']), P(out['ldc']), _lib.stream_ptr(dev)),
               "rr_lpf_map")
    out['k'] = out['k'].view(npv, 1)
    out['t0'] = out['t0'].view(npv, 1)
    return out


def transit_model(model, pv: torch.Tensor, tref: float, ld_start: int = 5):
    """BaseLPF.transit_model for a device population: the flux [npv, npt] as a
    CUDA tensor (model: a RoadRunnerModel whose data times are relative to tref)."""
    if model.ld_law is None:
        raise ValueError("the device mapping produces named-law (quadratic) coefficients")
    m = map_pv(pv, tref, model.npb, ld_start)
    zeros = torch.zeros(pv.shape[0], dtype=torch.float64, device=pv.device)
    args = dict(k=m['k'], t0=m['t0'], p=m['p'], a=m['a'], i=m['i'], e=zeros, w=zeros, ldc=m['ldc'])
    return model._evaluate_device(args)


def lnlikelihood(model, obs, sigma, pv: torch.Tensor, tref: float, ld_start: int = 5, grad: bool = False):
    """Gaussian log-likelihood of every population member (the fused kernel,
    the flux is never stored); with grad=True also its gradient with respect
    to the model parameters (k, t0, p, a, i, e, w, ldc).  CUDA tensors."""
    from .lnlike import _run
    m = map_pv(pv, tref, model.npb, ld_start)
    npv = pv.shape[0]
    zeros = torch.zeros(npv, dtype=torch.float64, device=pv.device)
    lnl, g = _run(model, obs, sigma, m['k'], m['t0'], m['p'], m['a'], m['i'], zeros, zeros, m['ldc'], grad)
    return (lnl, g) if grad else lnl

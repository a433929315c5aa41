"""Gaussian log-likelihood of the RoadRunner model and its gradient.

The reference evaluates the model (rr_full) and then the log-likelihood
(pytransit/lpf/loglikelihood/wnloglikelihood.py:23-35, lpf.py:51-66) per
parameter vector.  Here both run in one CUDA kernel (the flux is never
stored), and ``d lnL / d theta`` for theta = (k, t0, p, a, i, e, w, ldc) comes
from a hand-written adjoint kernel that recomputes z per sample
(rr_lnlike_f64 / rr_lnlike_split in the C ABI).

``LogLikelihood`` is a torch.autograd.Function: its forward runs the
likelihood kernel without derivatives, its backward re-runs it with them.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib

__all__ = ['lnlikelihood', 'LogLikelihood', 'grad_columns']

_vp, _i, _d, _sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
_SIG = {
    'rr_lnlike_ngrad': ([_i, _i, _i, _i], _i),
    'rr_lnlike_workspace_bytes': ([_i, _i, _i, _i, _i, _i, _i, _i, _i], _sz),
    'rr_lnlike_f64': ([_i, _vp, _i, _vp, _vp, _i, _vp, _i, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _i, _i, _i,
                       _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _d, _d, _d, _vp, _vp, _vp, _vp,
                       _sz, _vp, _vp, _vp], _i),
    'rr_lnlike_split': ([_i, _vp, _i, _vp, _vp, _d, _d, _i, _vp, _i, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _i,
                         _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _d, _d, _d, _vp, _vp,
                         _vp, _vp, _sz, _vp, _vp, _vp], _i),
}
_lib._EXTRA_SIGNATURES.update(_SIG)


def _L():
    L = _lib.lib()
    for name, (args, res) in _SIG.items():
        f = getattr(L, name)
        f.argtypes, f.restype = args, res
    return L


def grad_columns(nkc, nep, npb, npar):
    """Names of the gradient columns: k, t0, p, a, i, e, w, ldc."""
    cols = [f'k[{j}]' for j in range(nkc)] + [f't0[{j}]' for j in range(nep)] + ['p', 'a', 'i', 'e', 'w']
    cols += [f'ldc[{b},{j}]' for b in range(npb) for j in range(npar)]
    return cols


def _run(model, obs, sigma, k, t0, p, a, i, e, w, ldc, want_grad):
    """Device tensors in (float64), (lnl[npv], grad[npv, ngrad] or None) out."""
    device = model._cuda_device()
    if model.ld_law is None:
        raise ValueError("The log-likelihood kernel supports the named limb darkening laws only.")
    split = model.precision == 'split'
    L = _L()
    npv, nkc = k.shape
    nep = t0.shape[1]
    npb, nlc, npt = model.npb, model.nlc, model.npt
    npar = ldc.shape[2]
    if ldc.shape[:2] != (npv, npb):
        raise ValueError(f"ldc should have shape [{npv}, {npb}, ncoef]")
    tb = model._device_tables(device)
    dd = model._device_data(device)
    nz = model.ze.size
    dt = torch.float32 if split else torch.float64
    ldp = torch.empty((npv, npb, nz), dtype=dt, device=device)
    istar = torch.empty((npv, npb), dtype=dt, device=device)
    fn = L.rr_ld_tables_f32 if split else L.rr_ld_tables_f64
    P = _lib.ptr
    sp = _lib.stream_ptr(device)
    _lib.check(fn(model.ld_law, P(ldc), npv, npb, npar, P(tb['mu']), nz, P(ldp), P(istar), sp), "rr_ld_tables")
    obs = torch.as_tensor(obs, dtype=torch.float64).to(device).contiguous()
    if obs.numel() != npt:
        raise ValueError(f"obs should have {npt} values")
    if torch.is_tensor(sigma):
        sig = sigma.to(device=device, dtype=torch.float64).reshape(-1).expand(nlc).contiguous()
    else:
        sig = torch.as_tensor(np.broadcast_to(np.asarray(sigma, dtype=np.float64), (nlc,)).copy()).to(device)
    ngrad = L.rr_lnlike_ngrad(nkc, nep, npb, npar)
    wsb = L.rr_lnlike_workspace_bytes(int(split), npv, npb, nlc, nep, model.ng, npar, npt, nkc)
    ws = model._workspace(wsb, device)
    lnl = torch.empty(npv, dtype=torch.float64, device=device)
    g = torch.empty((npv, ngrad), dtype=torch.float64, device=device) if want_grad else None
    common_tail = (P(k), nkc, P(t0), nep, nep, P(p), P(a), P(i), P(e), P(w), npv, nlc, npb, P(dd['lcids']),
                   P(dd['pbids']), P(dd['epids']), P(dd['nsamples']), P(dd['exptimes']), P(ldp), P(istar),
                   P(tb['W32'] if split else tb['W64']), model.nk, model.ng, nz, model.dk, float(model.klims[0]),
                   float(model.klims[1]), model.dg, P(tb['ze']), P(obs), P(sig), P(ws), ws.numel(), P(lnl), P(g))
    if split:
        st = L.rr_lnlike_split(model.ld_law, P(ldc), npar, P(tb['mu']), P(dd['times_ff']), dd['t_ref'],
                               dd['t_absmax'], npt, *common_tail, sp)
    else:
        st = L.rr_lnlike_f64(model.ld_law, P(ldc), npar, P(tb['mu']), P(dd['time']), npt, *common_tail, sp)
    _lib.check(st, "rr_lnlike")
    return lnl, g


def _as_params(model, k, t0, p, a, i, e, w, ldc, extra=None):
    """Shape the parameters as evaluate() does and move them to the device, in
    one host-to-device copy through the model's pinned staging buffer (with
    the arrays of `extra`, a dict of float64 arrays, in the same copy)."""
    device = model._cuda_device()
    vals = [x.detach().cpu().numpy() if torch.is_tensor(x) else x for x in (k, t0, p, a, i, e, w)]
    k_, t0_, p_, a_, i_, e_, w_ = model._shape_params(*vals)
    ldc_ = ldc.detach().cpu().numpy() if torch.is_tensor(ldc) else ldc
    ldc3 = model._shape_ldc(ldc_, p_.size, model.npb)
    arrays = dict(k=k_, t0=t0_, p=p_, a=a_, i=i_, e=e_, w=w_, ldc=ldc3)
    arrays.update(extra or {})
    dev = model._upload({n: np.ascontiguousarray(v, dtype=np.float64) for n, v in arrays.items()}, device)
    out = [dev[n] for n in ('k', 't0', 'p', 'a', 'i', 'e', 'w', 'ldc')]
    return (out, {n: dev[n] for n in (extra or {})}) if extra is not None else out


def lnlikelihood(model, obs, sigma, k, ldc, t0, p, a, i, e=0.0, w=0.0, grad=False, copy=True):
    """Gaussian log-likelihood of ``obs`` (one value per data point of
    ``model.set_data``) with noise ``sigma`` (scalar or one value per light
    curve) for each parameter vector; with grad=True also its gradient,
    columns as ``grad_columns``.  Returns numpy arrays (copy=True) or CUDA
    tensors."""
    extra = {}
    if not torch.is_tensor(obs):
        extra['obs'] = np.asarray(obs, dtype=np.float64).reshape(-1)
    if not torch.is_tensor(sigma):
        extra['sigma'] = np.broadcast_to(np.asarray(sigma, dtype=np.float64), (model.nlc,)).copy()
    (k_, t0_, p_, a_, i_, e_, w_, ldc3), dev = _as_params(model, k, t0, p, a, i, e, w, ldc, extra)
    lnl, g = _run(model, dev.get('obs', obs), dev.get('sigma', sigma), k_, t0_, p_, a_, i_, e_, w_, ldc3, grad)
    if copy:
        lnl = lnl.cpu().numpy()
        g = g.cpu().numpy() if g is not None else None
    return (lnl, g) if grad else lnl


class LogLikelihood(torch.autograd.Function):
    """lnL[npv] = LogLikelihood.apply(model, obs, sigma, k[npv, nkc], t0[npv, nep],
    p, a, i, e, w [npv], ldc[npv, npb, ncoef]) with float64 CUDA tensors; the
    backward pass runs the adjoint kernel."""

    @staticmethod
    def forward(ctx, model, obs, sigma, k, t0, p, a, i, e, w, ldc):
        args = [x.detach().to(torch.float64).contiguous() for x in (k, t0, p, a, i, e, w, ldc)]
        ctx.model, ctx.obs, ctx.sigma = model, obs, sigma
        ctx.save_for_backward(*args)
        lnl, _ = _run(model, obs, sigma, *args, want_grad=False)
        return lnl

    @staticmethod
    def backward(ctx, g_lnl):
        k, t0, p, a, i, e, w, ldc = ctx.saved_tensors
        _, g = _run(ctx.model, ctx.obs, ctx.sigma, k, t0, p, a, i, e, w, ldc, want_grad=True)
        g = g * g_lnl.to(g.dtype)[:, None]
        nkc, nep, npar = k.shape[1], t0.shape[1], ldc.shape[2]
        c = 0
        gk = g[:, c:c + nkc]; c += nkc
        gt0 = g[:, c:c + nep]; c += nep
        gp, ga, gi, ge, gw = (g[:, c + j] for j in range(5)); c += 5
        gl = g[:, c:].reshape(ldc.shape)
        return None, None, None, gk, gt0, gp, ga, gi, ge, gw, gl

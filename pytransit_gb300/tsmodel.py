"""TransmissionSpectroscopyModel: drop-in for the reference's TSModel on a GB300.

Same evaluate() as pytransit/models/roadrunner/tsmodel.py:46-130: npb
wavelength channels with one radius ratio each share one orbit, the LD means
are taken at the mean radius ratio and the occulted area to first order in
k.  The model runs as CUDA kernels (rr_ts_f64 / rr_ts_split); the output is
flux[npv, npb, npt], not squeezed, as in the reference.
"""
from typing import List, Union

import numpy as np
from numpy import ndarray

from . import ldmodels as _ldm
from .ldmodel import LDModel
from .rrmodel import RoadRunnerModel

__all__ = ['TransmissionSpectroscopyModel', 'TSModel']


class TransmissionSpectroscopyModel(RoadRunnerModel):

    def evaluate(self, k: Union[float, ndarray], ldc: Union[ndarray, List], t0: Union[float, ndarray],
                 p: Union[float, ndarray], a: Union[float, ndarray], i: Union[float, ndarray],
                 e: Union[float, ndarray] = 0.0, w: Union[float, ndarray] = 0.0, copy: bool = True,
                 return_error: bool = False):
        """Transit model for npb channels sharing one orbit.

        k: [npv, npb] radius ratios; ldc: [npv, npb, ncoef] (or [npb, ncoef]
        for one parameter vector); t0, p, a, i, e, w: one value per parameter
        vector.  Returns flux[npv, npb, npt] (numpy float64 with copy=True,
        else the CUDA tensor); with return_error=True (flux, bound), the
        stated maximum absolute flux error against the FP64 model."""
        import torch
        from . import _lib
        device = self._cuda_device()
        k = np.atleast_2d(np.asarray(k, dtype=np.float64))
        ldc = np.atleast_2d(np.asarray(ldc, dtype=np.float64))
        npv = k.shape[0]
        if npv > 1 and ldc.ndim != 3:
            raise ValueError("""The limb darkening parameters (ldp) should be given as a 3D array with shape [npv, npb, nldp]
                    when evaluating the model for a set of parameters (npv > 1).""")
        if ldc.ndim == 2:
            ldc = ldc.reshape((1, ldc.shape[0], ldc.shape[1]))
        elif ldc.ndim != 3:
            raise ValueError()
        npb = ldc.shape[1]
        if k.shape[1] != npb:
            raise ValueError("The transmission spectrum transit model requires that the number or radius ratios and the number of passbands match.")
        vecs = [self._vec(x, npv, n) for x, n in ((t0, 't0'), (p, 'p'), (a, 'a'), (i, 'i'), (e, 'e'), (w, 'w'))]
        split = self.precision == 'split'
        tb = self._device_tables(device)
        dd = self._device_data(device)
        nz = self.ze.size
        dt = torch.float32 if split else torch.float64
        L = _lib.lib()
        P = _lib.ptr
        sp = _lib.stream_ptr(device)
        ldc3 = np.ascontiguousarray(np.broadcast_to(ldc, (npv, npb, ldc.shape[2])))
        args = self._upload(dict(k=np.ascontiguousarray(k), t0=vecs[0], p=vecs[1], a=vecs[2], i=vecs[3],
                                 e=vecs[4], w=vecs[5], ldc=ldc3 if self.ld_law is not None else None), device)
        ns0 = int(np.atleast_1d(self.nsamples)[0])
        ex0 = float(np.atleast_1d(self.exptimes)[0])
        npt = self.npt
        ldf = (npt + 3) // 4 * 4
        wsb = L.rr_ts_workspace_bytes(int(split), npv, npb, self.ng)
        ws = self._workspace(wsb, device)
        out = torch.empty((npv, npb, ldf), dtype=dt, device=device)
        orbit = (P(args['k']), P(args['t0']), P(args['p']), P(args['a']), P(args['i']), P(args['e']), P(args['w']))
        if self.ld_law is not None and not self.interpolate:
            # a named law with the default 2D table: LD profiles, integrals,
            # orbit records and LD means in one launch, then the flux
            if split:
                st = L.rr_ts_prepare_split_ld(self.ld_law, P(args['ldc']), ldc3.shape[2], P(tb['mu']), dd['t_ref'],
                                              dd['t_absmax'], *orbit, npv, npb, ex0, self.ng, nz, P(tb['ze']), P(ws),
                                              ws.numel(), sp)
                _lib.check(st, "rr_ts_prepare_split_ld")
                st = L.rr_ts_flux_split(P(dd['times_ff']), npt, npv, npb, ns0, ex0, self.ng, self.dg, P(ws), P(out),
                                        ldf, sp)
            else:
                st = L.rr_ts_prepare_f64_ld(self.ld_law, P(args['ldc']), ldc3.shape[2], P(tb['mu']), *orbit, npv,
                                            npb, ex0, self.ng, nz, P(tb['ze']), P(ws), ws.numel(), sp)
                _lib.check(st, "rr_ts_prepare_f64_ld")
                if self.fp64_cull:   # the same bits with the fold once per tile that reaches no box
                    st = L.rr_ts_flux_f64_culled(P(dd['time']), P(dd['tiles64']), npt, P(args['t0']), P(args['p']),
                                                 npv, npb, ns0, ex0, self.ng, self.dg, P(ws), P(out), ldf, sp)
                else:
                    st = L.rr_ts_flux_f64(P(dd['time']), npt, P(args['t0']), P(args['p']), npv, npb, ns0, ex0,
                                          self.ng, self.dg, P(ws), P(out), ldf, sp)
            _lib.check(st, "rr_ts_flux")
        else:
            if self.ld_law is not None:
                ldp = torch.empty((npv, npb, nz), dtype=dt, device=device)
                istar = torch.empty((npv, npb), dtype=dt, device=device)
                fn = L.rr_ld_tables_f32 if split else L.rr_ld_tables_f64
                _lib.check(fn(self.ld_law, P(args['ldc']), npv, npb, ldc3.shape[2], P(tb['mu']), nz, P(ldp),
                              P(istar), sp), "rr_ld_tables")
            else:
                ldp, istar = self._host_ld(ldc3, npv, npb, device, dt)
            W = (tb['W32'] if split else tb['W64']) if self.interpolate else None
            common = (*orbit, npv, npb, ns0, ex0, P(ldp), P(istar), P(W), self.nk, self.ng, nz, self.dk,
                      float(self.klims[0]), float(self.klims[1]), self.dg, P(tb['ze']), P(ws), ws.numel(), P(out),
                      ldf, sp)
            if split:
                st = L.rr_ts_split(P(dd['times_ff']), dd['t_ref'], dd['t_absmax'], npt, *common)
            else:
                st = L.rr_ts_f64(P(dd['time']), npt, *common)
            _lib.check(st, "rr_ts")
        out = out[:, :, :npt]
        self._bound_state = dict(split=split, ts=True, npv=npv, npb=npb, ns0=ns0, ex0=ex0, ws=ws, device=device,
                                 prm={n: args[n] for n in ('p', 'a', 'i', 'e', 'w')})
        if copy:
            out = _lib.to_host_f64(out)
        return (out, self.last_error_bound) if return_error else out

    def _host_ld(self, ldc3, npv, npb, device, dt):
        import torch
        if isinstance(self.ldmodel, LDModel):
            ldp, istar = self.ldmodel(self.mu, ldc3)
        else:
            ldp = _ldm.evaluate_ld(self.ldmodel, self.mu, ldc3)
            if self.ldmmean is not None:
                istar = _ldm.evaluate_ldi(self.ldmmean, ldc3)
            else:
                ldpi = _ldm.evaluate_ld(self.ldmodel, self._ldmu, ldc3)
                istar = 2 * np.pi * np.trapezoid(self._ldz * ldpi, self._ldz, axis=-1)
        ldp = np.require(np.broadcast_to(np.asarray(ldp, np.float64), (npv, npb, self.mu.size)), requirements='CW')
        istar = np.require(np.broadcast_to(np.asarray(istar, np.float64), (npv, npb)), requirements='CW')
        return (torch.as_tensor(ldp).to(device=device, dtype=dt), torch.as_tensor(istar).to(device=device, dtype=dt))

    def __call__(self, k, ldc, t0, p, a, i, e=0.0, w=0.0, copy: bool = True, return_error: bool = False):
        return self.evaluate(k, ldc, t0, p, a, i, e, w, copy, return_error)


TSModel = TransmissionSpectroscopyModel

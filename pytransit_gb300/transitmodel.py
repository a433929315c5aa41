"""TransitModel base: the data side of the model (set_data).

Mirrors TransitModel.set_data (pytransit/models/transitmodel.py:56-125): the
same arguments, defaults, validation and error messages.  The arrays are kept
on the host as numpy arrays and uploaded to the GPU on first use
(``_device_data``), once per data set.
"""
from typing import List, Optional, Union

import numpy as np
from numpy import asarray, atleast_1d, float64, integer, issubdtype, ndarray, ones, unique, zeros

__all__ = ['TransitModel']


class TransitModel:
    """Exoplanet transit light curve model (data handling)."""

    def __init__(self) -> None:
        self.time_id: Optional[int] = None
        self.time: Optional[ndarray] = None
        self.lcids: Optional[ndarray] = None
        self.pbids: Optional[ndarray] = None
        self.nsamples: Optional[ndarray] = None
        self.exptimes: Optional[ndarray] = None
        self.epids: Optional[ndarray] = None
        self.nlc: int = 0
        self.npt: int = 0
        self.npb: int = 0
        self._dev = None          # device copies of the data arrays
        self._data_version = 0

    def set_data(self, time: Union[ndarray, List],
                 lcids: Optional[Union[ndarray, List]] = None,
                 pbids: Optional[Union[ndarray, List]] = None,
                 nsamples: Optional[Union[ndarray, List]] = None,
                 exptimes: Optional[Union[ndarray, List]] = None,
                 epids: Optional[Union[ndarray, List]] = None) -> None:
        """Set the data for the transit model.

        Parameters
        ----------
        time : array-like
            Mid-exposure times of the modelled data points.
        lcids : array-like, optional
            Integer light curve index of every data point (size == time.size).
        pbids : array-like, optional
            Passband index of every light curve, 0..npb-1.
        nsamples : int or array-like, optional
            Supersamples per exposure, one value or one per light curve.
        exptimes : float or array-like, optional
            Exposure times, one value or one per light curve.
        epids : array-like, optional
            Zero-epoch index of every light curve (column of a 2D t0).
        """
        # Passing the same time array object again with no other argument is a no-op
        # (transitmodel.py:83-84).
        if (id(time) == self.time_id and lcids is None and pbids is None and nsamples is None
                and exptimes is None and epids is None):
            return

        self.time_id = id(time)
        self.time = asarray(time, float64)
        self.npt = self.time.size

        self.lcids = asarray(lcids) if lcids is not None else zeros(self.npt, 'int')
        self.nlc = unique(self.lcids).size

        if not issubdtype(self.lcids.dtype, integer):
            raise ValueError(f"The light curve indices must be given as integers instead of {self.lcids.dtype}.")

        if self.lcids.size != self.npt:
            raise ValueError(f"Light curve index array size ({self.lcids.size}) should equal to the number of datapoints ({self.npt}).")

        self.pbids = asarray(pbids) if pbids is not None else zeros(self.nlc, 'int')
        self.npb = unique(self.pbids).size

        if not issubdtype(self.pbids.dtype, integer):
            raise ValueError(f"The passband indices must be given as integers instead of {self.pbids.dtype}.")

        if self.pbids.size != self.nlc:
            raise ValueError(f"Passband index array size ({self.pbids.size}) should equal to the number of ligt curves ({self.nlc}).")

        if not (self.pbids.max() == (self.npb - 1) and self.pbids.min() == 0):
            raise ValueError(f"Passband indices (`pbids`) for {self.npb} unique passbands should be given as integers between 0 and {self.npb - 1}.")

        self.epids = asarray(epids) if epids is not None else zeros(self.nlc, 'int')
        self.nsamples = atleast_1d(nsamples) if nsamples is not None else ones(self.nlc, 'int')
        self.exptimes = atleast_1d(exptimes) if exptimes is not None else zeros(self.nlc, 'int')

        # Host-side checks the GPU kernels rely on (the reference reads out of
        # bounds instead): light curve ids must index 0..nlc-1.
        if self.npt > 0 and (self.lcids.min() < 0 or self.lcids.max() >= self.nlc):
            raise ValueError(f"Light curve indices should be integers between 0 and {self.nlc - 1}.")
        self._dev = None
        self._data_version += 1

    # -- per-light-curve arrays broadcast to nlc (scalars allowed, transitmodel.py:124-125)
    def _lc_arrays(self):
        nlc = self.nlc
        ns = np.broadcast_to(np.asarray(self.nsamples), (nlc,)).astype(np.int32)
        ex = np.broadcast_to(np.asarray(self.exptimes, dtype=np.float64), (nlc,)).astype(np.float64)
        ep = np.broadcast_to(np.asarray(self.epids), (nlc,)).astype(np.int32)
        if np.any(ns < 1):
            raise ValueError("The number of samples per exposure must be a positive integer.")
        if nlc and ep.min() < 0:
            raise ValueError("Epoch indices must be non-negative integers.")
        return ns, ex, ep

    def _device_data(self, device):
        """Device copies of the data arrays (uploaded once per set_data)."""
        import torch
        from . import _lib
        if self._dev is not None and self._dev['device'] == device:
            return self._dev
        if self.time is None:
            raise ValueError("set_data must be called before evaluate")
        ns, ex, ep = self._lc_arrays()
        d = {'device': device}
        d['time'] = torch.as_tensor(self.time, dtype=torch.float64).to(device)
        d['lcids'] = torch.as_tensor(self.lcids.astype(np.int32)).to(device)
        d['pbids'] = torch.as_tensor(self.pbids.astype(np.int32)).to(device)
        d['epids'] = torch.as_tensor(ep).to(device)
        d['nsamples'] = torch.as_tensor(ns).to(device)
        d['exptimes'] = torch.as_tensor(ex).to(device)
        if self.npt > 0:
            tmin, tmax = float(self.time.min()), float(self.time.max())
        else:
            tmin = tmax = 0.0
        d['t_ref'] = 0.5 * (tmin + tmax)
        d['t_absmax'] = max(abs(tmax - d['t_ref']), abs(tmin - d['t_ref']))
        L = _lib.lib()
        d['times_ff'] = torch.empty(max(int(L.rr_time_split_floats(self.npt)), 4), dtype=torch.float32,
                                    device=device)
        _lib.check(L.rr_time_split(_lib.ptr(d['time']), _lib.ptr(d['lcids']), self.npt, d['t_ref'],
                                   _lib.ptr(d['times_ff']), _lib.stream_ptr(device)), "rr_time_split")
        d['tiles64'] = torch.empty(max(int(L.rr_time_tiles_f64_doubles(self.npt)), 4), dtype=torch.float64,
                                   device=device)
        _lib.check(L.rr_time_tiles_f64(_lib.ptr(d['time']), _lib.ptr(d['lcids']), self.npt, _lib.ptr(d['tiles64']),
                                       _lib.stream_ptr(device)), "rr_time_tiles_f64")
        self._dev = d
        return d

    def _upload(self, arrays, device):
        """Send the small per-call arrays in one host-to-device copy through a
        reused pinned staging buffer; returns device views of the same shapes."""
        import torch
        names = [n for n, v in arrays.items() if v is not None]
        sizes = [int(arrays[n].size) for n in names]
        total = sum(sizes)
        if getattr(self, '_pin', None) is None or self._pin.numel() < total or self._pin_dev.device != device:
            n = max(total, 1024)
            self._pin = torch.empty(n, dtype=torch.float64, pin_memory=True)
            self._pin_dev = torch.empty(n, dtype=torch.float64, device=device)
            self._pin_evt = None
        if self._pin_evt is not None:
            self._pin_evt.synchronize()      # the previous copy has left the staging buffer
        hp = self._pin.numpy()
        off = 0
        for n, sz in zip(names, sizes):
            hp[off:off + sz] = np.asarray(arrays[n], dtype=np.float64).reshape(-1)
            off += sz
        self._pin_dev[:total].copy_(self._pin[:total], non_blocking=True)
        self._pin_evt = torch.cuda.Event()
        self._pin_evt.record()
        out, off = {}, 0
        for n, sz in zip(names, sizes):
            out[n] = self._pin_dev[off:off + sz].view(arrays[n].shape)
            off += sz
        return out

    def __call__(self, *nargs, **kwargs):
        raise NotImplementedError

    def evaluate(self, k, ldc, t0, p, a, i, e=None, w=None, copy: bool = True):
        raise NotImplementedError

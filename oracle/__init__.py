"""ORACLE — test infrastructure only; never imported by the product path.

CPU FP64 restatement of PyTransit's RoadRunner evaluation path
(hpparvi/PyTransit 2.8.1), used by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` to check the CUDA library's results.

* ``rr_oracle.c`` restates the numba kernels (common.py, model_full.py,
  model_trspec.py, ldmodels.py) and the missing meepmeep orbit layer; it is
  built by ``build_oracle.py`` and loaded here with ctypes.
* ``OracleRoadRunner`` restates the host logic of ``RoadRunnerModel``
  (pytransit/models/roadrunner/rrmodel.py:60-238) and ``TransitModel.set_data``
  (pytransit/models/transitmodel.py:56-125) on top of it.

Pinned against tests/golden/*.npz, produced by running the reference's own
RoadRunner Python code (tests/golden/make_golden.py).  The orbit layer
(meepmeep.backends.numba.point2d, pinned only as ``meepmeep >= 1.0.0``) is not
in the reference; its restatement is shared by the oracle and the golden shim,
so flux parity against real meepmeep is unpinned.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_LIB = None

LD_LAWS = {'uniform': 0, 'linear': 1, 'quadratic': 2, 'quadratic-tri': 3, 'nonlinear': 4,
           'general': 5, 'square_root': 6, 'logarithmic': 7, 'exponential': 8, 'power-2': 9,
           'power-2-pm': 10}
LD_NPAR = {'uniform': 0, 'linear': 1, 'quadratic': 2, 'quadratic-tri': 2, 'nonlinear': 4,
           'general': None, 'square_root': 2, 'logarithmic': 2, 'exponential': 2, 'power-2': 2,
           'power-2-pm': 2}

_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int32)


def lib():
    """Load (building if needed) the oracle shared library."""
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        L.rro_linspace.argtypes = [C.c_double, C.c_double, C.c_int, _d]
        L.rro_z_grid.argtypes = [C.c_double, C.c_int, C.c_int, _d, _d]
        L.rro_cci_acos.argtypes = [C.c_double] * 3
        L.rro_cci_acos.restype = C.c_double
        L.rro_ccia.argtypes = [C.c_double, C.c_double, C.c_double, _d]
        L.rro_ccia.restype = C.c_double
        L.rro_weights_2d.argtypes = [C.c_double, _d, C.c_int, C.c_int, _d]
        L.rro_weights_2d.restype = C.c_double
        L.rro_weights_3d.argtypes = [C.c_int, C.c_double, C.c_double, _d, C.c_int, C.c_int, _d, _d, _d]
        L.rro_interp_ldm.argtypes = [C.c_double, C.c_double, _d, C.c_int]
        L.rro_interp_ldm.restype = C.c_double
        L.rro_ld_value.argtypes = [C.c_int, C.c_double, _d, C.c_int]
        L.rro_ld_value.restype = C.c_double
        L.rro_ld_integral.argtypes = [C.c_int, _d, _d]
        L.rro_ld_integral.restype = C.c_int
        L.rro_ld_integral_numeric.argtypes = [C.c_int, _d, C.c_int]
        L.rro_ld_integral_numeric.restype = C.c_double
        L.rro_evaluate_ld.argtypes = [C.c_int, _d, C.c_int, _d, C.c_int, C.c_int, C.c_int, _d, _d]
        L.rro_solve2d.argtypes = [C.c_double] * 6 + [_d]
        L.rro_sep_c.argtypes = [C.c_double, _d]
        L.rro_sep_c.restype = C.c_double
        L.rro_bounding_box.argtypes = [C.c_double, _d, _d, _d]
        L.rro_z_kepler.argtypes = [C.c_double] * 7
        L.rro_z_kepler.restype = C.c_double
        L.rro_rr_full.argtypes = ([_d, C.c_int, _d, C.c_int, _d, C.c_int, _d, _d, _d, _d, _d,
                                   C.c_int, C.c_int, C.c_int, _i, _i, _i, _i, _d, _d, _d, _d,
                                   C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                   C.c_double, _d, _d, C.c_int])
        L.rro_rr_full.restype = C.c_int
        L.rro_ts_full.argtypes = ([_d, C.c_int, _d, _d, _d, _d, _d, _d, _d, C.c_int, C.c_int,
                                   C.c_int, C.c_double, _d, _d, _d, C.c_int, C.c_int, C.c_int,
                                   C.c_double, C.c_double, C.c_double, C.c_double, _d, _d, C.c_int])
        L.rro_ts_full.restype = C.c_int
        L.rro_lnlike_normal.argtypes = [_d, _d, C.c_int, C.c_int, C.c_double, _d]
        for n in ("rro_ellk", "rro_ellec"):
            getattr(L, n).argtypes = [C.c_double]
            getattr(L, n).restype = C.c_double
        L.rro_ellpicb.argtypes = [C.c_double, C.c_double]
        L.rro_ellpicb.restype = C.c_double
        L.rro_ma_quad_z.argtypes = [C.c_double] * 4
        L.rro_ma_quad_z.restype = C.c_double
        L.rro_ma_quad_z_v.argtypes = [_d, C.c_int, C.c_double, C.c_double, C.c_double, _d]
        L.rro_eclipse_time_offset.argtypes = [C.c_double] * 4
        L.rro_eclipse_time_offset.restype = C.c_double
        L.rro_eclipse_ltt.argtypes = [C.c_double] * 6
        L.rro_eclipse_ltt.restype = C.c_double
        L.rro_eclipse_full.argtypes = [_d, C.c_int, _d, _d, C.c_int, _d, _d, _d, _d, _d, C.c_int, C.c_double,
                                       C.c_int, _i, _i, _i, _d, _d]
        L.rro_es_full.argtypes = [_d, C.c_int, _d, _d, _d, _d, _d, _d, _d, _d, _d, C.c_int, C.c_int, C.c_int,
                                  C.c_double, _d]
        _LIB = L
    return _LIB


def _dp(a):
    return a.ctypes.data_as(_d)


def _ip(a):
    return a.ctypes.data_as(_i)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


# --------------------------------------------------------------------------
# Low-level wrappers
# --------------------------------------------------------------------------

def linspace(start, stop, num):
    out = np.empty(num)
    lib().rro_linspace(start, stop, num, _dp(out))
    return out


def z_grid(zcut=0.7, nin=20, nedge=20):
    """create_z_grid, common.py:132-149 -> (z_edges, z_means)."""
    ze, zm = np.empty(nin + nedge), np.empty(nin + nedge)
    lib().rro_z_grid(zcut, nin, nedge, _dp(ze), _dp(zm))
    return ze, zm


def weights_3d(nk, kmin, kmax, ze, ng):
    """calculate_weights_3d, common.py:189-223 -> (dk, dg, W[nk, ng, nz])."""
    ze = _f64(ze)
    W = np.empty((nk, ng, ze.size))
    dk, dg = C.c_double(), C.c_double()
    lib().rro_weights_3d(nk, kmin, kmax, _dp(ze), ze.size, ng, _dp(W), C.byref(dk), C.byref(dg))
    return dk.value, dg.value, W


def weights_2d(k, ze, ng):
    """calculate_weights_2d, common.py:153-185 -> (dg, W[ng, nz])."""
    ze = _f64(ze)
    W = np.empty((ng, ze.size))
    dg = lib().rro_weights_2d(k, _dp(ze), ze.size, ng, _dp(W))
    return dg, W


def ccia(r1, r2, b):
    """circle_circle_intersection_area_kite, common.py:53-73 -> (area, kappa0)."""
    k0 = C.c_double()
    a = lib().rro_ccia(r1, r2, b, C.byref(k0))
    return a, k0.value


def cci_acos(r1, r2, b):
    return lib().rro_cci_acos(r1, r2, b)


def interp_ldm(g, dg, lda):
    lda = _f64(lda)
    return lib().rro_interp_ldm(g, dg, _dp(lda), lda.size)


def solve2d(phase, p, a, i, e, w):
    """Restated meepmeep solve2d -> c[2, 5]."""
    c = np.empty((2, 5))
    lib().rro_solve2d(phase, p, a, i, e, w, _dp(c))
    return c


def sep_c(t, c):
    c = _f64(c)
    return lib().rro_sep_c(t, _dp(c))


def bounding_box(k, c):
    c = _f64(c)
    t1, t4 = C.c_double(), C.c_double()
    lib().rro_bounding_box(k, _dp(c), C.byref(t1), C.byref(t4))
    return t1.value, t4.value


def z_kepler(t, t0, p, a, i, e, w):
    return lib().rro_z_kepler(t, t0, p, a, i, e, w)


def ld_profile(law, mu, pv):
    pv = _f64(np.atleast_1d(pv))
    return np.array([lib().rro_ld_value(LD_LAWS[law], m, _dp(pv), pv.size) for m in mu])


def ld_integral(law, pv):
    pv = _f64(np.atleast_1d(pv))
    out = C.c_double()
    if lib().rro_ld_integral(LD_LAWS[law], _dp(pv), C.byref(out)):
        return out.value
    return lib().rro_ld_integral_numeric(LD_LAWS[law], _dp(pv), pv.size)


def evaluate_ld_named(law, mu, ldc):
    """evaluate_ld + evaluate_ldi (or the 200-point trapezoid) for a named law.
    ldc: (npv, npb, npar) -> (ldp[npv, npb, nmu], istar[npv, npb])."""
    ldc = _f64(ldc)
    npv, npb, npar = ldc.shape
    mu = _f64(mu)
    ldp = np.empty((npv, npb, mu.size))
    istar = np.empty((npv, npb))
    lib().rro_evaluate_ld(LD_LAWS[law], _dp(mu), mu.size, _dp(ldc), npv, npb, npar, _dp(ldp), _dp(istar))
    return ldp, istar


def rr_full(times, k, t0, p, a, i, e, w, nlc, npb, nep, lcids, pbids, epids, nsamples, exptimes,
            ldp, istar, weights, dk, kmin, kmax, dg, z_edges, nthreads=0):
    """rr_full, pytransit/models/roadrunner/model_full.py:9-100 -> flux[npv, npt]."""
    times, k, t0 = _f64(times), _f64(np.atleast_2d(k)), _f64(np.atleast_2d(t0))
    p, a, i, e, w = (_f64(np.atleast_1d(x)) for x in (p, a, i, e, w))
    lcids, pbids, epids, nsamples = (_i32(np.atleast_1d(x)) for x in (lcids, pbids, epids, nsamples))
    exptimes = _f64(np.broadcast_to(np.atleast_1d(exptimes).astype(np.float64), (nlc,)))
    nsamples = _i32(np.broadcast_to(nsamples, (nlc,)))
    ldp, istar, weights, z_edges = _f64(ldp), _f64(istar), _f64(weights), _f64(z_edges)
    npv, nkc = k.shape
    nk, ng, nz = weights.shape
    flux = np.empty((npv, times.size))
    rc = lib().rro_rr_full(_dp(times), times.size, _dp(k), nkc, _dp(t0), t0.shape[1], _dp(p), _dp(a),
                           _dp(i), _dp(e), _dp(w), npv, nlc, npb, _ip(lcids), _ip(pbids), _ip(epids),
                           _ip(nsamples), _dp(exptimes), _dp(ldp), _dp(istar), _dp(weights), nk, ng, nz,
                           dk, kmin, kmax, dg, _dp(z_edges), _dp(flux), nthreads)
    if rc != 0:
        raise ValueError('Radius ratios should be given either as an [npv, 1] or [npv, npb] array.')
    return flux


def ts_full(times, k, t0, p, a, i, e, w, nsamples0, exptime0, ldp, istar, weights, dk, kmin, kmax,
            ng, dg, z_edges, nthreads=0):
    """tsmodel_serial, pytransit/models/roadrunner/model_trspec.py:12-93 -> flux[npv, npb, npt].
    weights=None selects the per-pv 2D weight table (the reference's default)."""
    times, k = _f64(times), _f64(np.atleast_2d(k))
    t0, p, a, i, e, w = (_f64(np.atleast_1d(x)) for x in (t0, p, a, i, e, w))
    ldp, istar, z_edges = _f64(ldp), _f64(istar), _f64(z_edges)
    npv, npb = k.shape
    nz = z_edges.size
    if weights is not None:
        weights = _f64(weights)
        nk, ng = weights.shape[0], weights.shape[1]
        wp = _dp(weights)
    else:
        nk, wp, dk, dg = 0, None, 0.0, 0.0
    flux = np.empty((npv, npb, times.size))
    lib().rro_ts_full(_dp(times), times.size, _dp(k), _dp(t0), _dp(p), _dp(a), _dp(i), _dp(e), _dp(w),
                      npv, npb, int(nsamples0), float(exptime0), _dp(ldp), _dp(istar), wp, nk, ng, nz,
                      dk or 0.0, kmin, kmax, dg or 0.0, _dp(z_edges), _dp(flux), nthreads)
    return flux


def ma_quad_z(z, k, u1, u2):
    """Mandel & Agol quadratic-LD flux at centre distances z (eval_quad_z_s,
    pytransit/models/numba/ma_quadratic_nb.py:277-389)."""
    z = _f64(np.atleast_1d(z))
    out = np.empty_like(z)
    lib().rro_ma_quad_z_v(_dp(z), z.size, float(k), float(u1), float(u2), _dp(out))
    return out


def eclipse_full(times, k, t0, p, a, i, e, w, rstar, lcids, epids, nsamples, exptimes):
    """eclipse_model (pytransit/models/roadrunner/model_eclipse.py:12-81): the
    visible planet area [npv, npt]; k[npv], t0[npv, nep]."""
    times, k, t0 = _f64(times), _f64(np.atleast_1d(k)), _f64(np.atleast_2d(t0))
    p, a, i, e, w = (_f64(np.broadcast_to(np.atleast_1d(x), k.shape)) for x in (p, a, i, e, w))
    lcids, epids, nsamples = _i32(lcids), _i32(epids), _i32(nsamples)
    exptimes = _f64(exptimes)
    out = np.empty((k.size, times.size))
    lib().rro_eclipse_full(_dp(times), times.size, _dp(k), _dp(t0), t0.shape[1], _dp(p), _dp(a), _dp(i), _dp(e),
                           _dp(w), k.size, float(rstar), int(epids.size), _ip(lcids), _ip(epids), _ip(nsamples),
                           _dp(exptimes), _dp(out))
    return out


def es_full(times, k, t0, p, a, i, e, w, rstar, fratio, nsamples, exptime):
    """esmodel (pytransit/models/roadrunner/model_ecspec.py:13-63): flux[npv, npb, npt]."""
    times, k = _f64(times), _f64(np.atleast_1d(k))
    t0, p, a, i, e, w, rstar = (_f64(np.broadcast_to(np.atleast_1d(x), k.shape)) for x in (t0, p, a, i, e, w, rstar))
    fratio = _f64(np.atleast_2d(fratio))
    out = np.empty((k.size, fratio.shape[1], times.size))
    lib().rro_es_full(_dp(times), times.size, _dp(k), _dp(t0), _dp(p), _dp(a), _dp(i), _dp(e), _dp(w), _dp(rstar),
                      _dp(fratio), k.size, fratio.shape[1], int(nsamples), float(exptime), _dp(out))
    return out


def lnlike_normal(obs, model, sigma):
    """Gaussian log-likelihood per parameter vector (wnloglikelihood.py:23-35)."""
    obs, model = _f64(obs), _f64(np.atleast_2d(model))
    out = np.empty(model.shape[0])
    lib().rro_lnlike_normal(_dp(obs), _dp(model), model.shape[0], model.shape[1], float(sigma), _dp(out))
    return out


# --------------------------------------------------------------------------
# Host logic of RoadRunnerModel, restated (rrmodel.py:60-238, transitmodel.py:56-125)
# --------------------------------------------------------------------------

class OracleRoadRunner:
    """Oracle counterpart of ``RoadRunnerModel``: same constructor keywords,
    ``set_data`` and ``evaluate``; FP64 on the host cores."""

    def __init__(self, ldmodel='quadratic', klims=(0.005, 0.5), nk=256, nzin=20, nzlimb=20,
                 zcut=0.7, ng=100, nthreads=0, ts=False):
        self.ldmodel = ldmodel
        self.klims, self.nk, self.ng, self.nthreads, self.ts = klims, nk, ng, nthreads, ts
        self.ze, self.zm = z_grid(zcut, nzin, nzlimb)
        self.mu = np.sqrt(1 - self.zm ** 2)
        self.dk, self.dg, self.weights = weights_3d(nk, klims[0], klims[1], self.ze, ng)
        self._ldmu = np.linspace(1, 0, 200)
        self._ldz = np.sqrt(1 - self._ldmu ** 2)

    def set_data(self, time, lcids=None, pbids=None, nsamples=None, exptimes=None, epids=None):
        self.time = np.asarray(time, np.float64)
        self.npt = self.time.size
        self.lcids = np.asarray(lcids) if lcids is not None else np.zeros(self.npt, 'int')
        self.nlc = np.unique(self.lcids).size
        self.pbids = np.asarray(pbids) if pbids is not None else np.zeros(self.nlc, 'int')
        self.npb = np.unique(self.pbids).size
        self.epids = np.asarray(epids) if epids is not None else np.zeros(self.nlc, 'int')
        self.nsamples = np.atleast_1d(nsamples) if nsamples is not None else np.ones(self.nlc, 'int')
        self.exptimes = np.atleast_1d(exptimes) if exptimes is not None else np.zeros(self.nlc, 'int')
        self.nep = np.unique(self.epids).size

    def ld_tables(self, ldc, npv, npb):
        """(ldp[npv, npb, nz], istar[npv, npb]) as rrmodel.py:212-227."""
        ldm = self.ldmodel
        if isinstance(ldm, str):
            ldc = np.asarray(ldc, np.float64)
            if ldc.ndim == 1:
                ldc = ldc.reshape((1, 1, -1))
            elif ldc.ndim == 2:
                ldc = ldc.reshape((1, ldc.shape[0], -1)) if self.ts else ldc.reshape((1, npb, -1))
            if ldc.shape[0] == 1 and npv > 1:
                ldc = np.repeat(ldc, npv, axis=0)
            return evaluate_ld_named(ldm, self.mu, ldc)
        if hasattr(ldm, '_integrate') and callable(ldm):
            return ldm(self.mu, np.asarray(ldc))
        if isinstance(ldm, tuple):
            fld, fldi = ldm
        else:
            fld, fldi = ldm, None
        pv = np.asarray(ldc, np.float64)
        if pv.ndim == 1:
            pv = pv.reshape((1, 1, -1))
        elif pv.ndim == 2:
            pv = pv.reshape((1, pv.shape[0], -1))
        ldp = np.zeros((pv.shape[0], pv.shape[1], self.mu.size))
        istar = np.zeros((pv.shape[0], pv.shape[1]))
        for ipv in range(pv.shape[0]):
            for ipb in range(pv.shape[1]):
                ldp[ipv, ipb] = fld(self.mu, pv[ipv, ipb])
                if fldi is not None:
                    istar[ipv, ipb] = fldi(pv[ipv, ipb])
                else:
                    prof = fld(self._ldmu, pv[ipv, ipb])
                    istar[ipv, ipb] = 2 * np.pi * np.trapezoid(self._ldz * prof, self._ldz)
        return ldp, istar

    def evaluate(self, k, ldc, t0, p, a, i, e=0.0, w=0.0):
        k = np.atleast_2d(np.asarray(k, np.float64))
        p = np.atleast_1d(np.asarray(p, np.float64))
        npv = p.size
        if self.ts:
            ldp, istar = self.ld_tables(ldc, npv, k.shape[1])
            t0 = np.atleast_1d(t0)
            a, i, e, w = (np.broadcast_to(np.atleast_1d(np.asarray(x, np.float64)), (npv,)) for x in (a, i, e, w))
            return ts_full(self.time, k, t0, p, a, i, e, w, self.nsamples[0], self.exptimes[0], ldp,
                           istar, None, None, self.klims[0], self.klims[1], self.ng, None, self.ze,
                           self.nthreads)
        ldp, istar = self.ld_tables(ldc, npv, self.npb)
        t0 = np.asarray(t0, np.float64)
        t0 = t0.reshape((npv, -1)) if t0.ndim == 1 and t0.size == npv else np.atleast_2d(t0)
        a, i, e, w = (np.broadcast_to(np.atleast_1d(np.asarray(x, np.float64)), (npv,)) for x in (a, i, e, w))
        flux = rr_full(self.time, k, t0, p, a, i, e, w, self.nlc, self.npb, self.nep, self.lcids,
                       self.pbids, self.epids, self.nsamples, self.exptimes, ldp, istar, self.weights,
                       self.dk, self.klims[0], self.klims[1], self.dg, self.ze, self.nthreads)
        return np.squeeze(flux)

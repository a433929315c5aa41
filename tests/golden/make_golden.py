"""Generate the golden fixtures in tests/golden/ by running the reference's own,
unmodified RoadRunner Python code (hpparvi/PyTransit 2.8.1).

Run in a container where the reference is checked out (default
/root/reference, or pass its path as the first argument):

    python tests/golden/make_golden.py [/path/to/PyTransit]

numba and meepmeep are not installed, so the script puts two stand-ins from
tests/golden/shim/ on sys.path: a pass-through ``numba`` (njit returns the
function, prange is range) and a restated ``meepmeep.backends.numba.point2d``.
It registers bare ``pytransit`` / ``pytransit.models`` package objects so that
``pytransit/__init__.py`` (astropy, pandas, emcee ...) is not executed, and
keeps Python's bytecode caches out of the reference tree.

Everything except the orbit layer is therefore the reference's own code:
RoadRunnerModel.__init__/set_data/evaluate (rrmodel.py), rr_full and rr_simple
(model_full.py, model_simple.py), the weight tables, area and interpolation
(common.py), the LD laws (numba/ldmodels.py), LDModel (ldmodel.py),
TransitModel.set_data (transitmodel.py), TransmissionSpectroscopyModel /
tsmodel_serial (tsmodel.py, model_trspec.py) and the Mandel & Agol quadratic
model used as the independent cross-check (numba/ma_quadratic_nb.py) and the
secondary-eclipse kernels (model_eclipse.py, model_ecspec.py).
"""
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.abspath(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")


def _setup_reference():
    sys.pycache_prefix = tempfile.mkdtemp(prefix="golden_pycache_")
    sys.dont_write_bytecode = True
    sys.path.insert(0, os.path.join(HERE, "shim"))
    pkg = types.ModuleType("pytransit")
    pkg.__path__ = [os.path.join(REF, "pytransit")]
    sys.modules["pytransit"] = pkg
    models = types.ModuleType("pytransit.models")
    models.__path__ = [os.path.join(REF, "pytransit", "models")]
    sys.modules["pytransit.models"] = models
    pkg.models = models


_setup_reference()

from pytransit.models.roadrunner.rrmodel import RoadRunnerModel  # noqa: E402
from pytransit.models.roadrunner.tsmodel import TransmissionSpectroscopyModel  # noqa: E402
from pytransit.models.roadrunner import common as rrc  # noqa: E402
from pytransit.models.ldmodel import LDModel  # noqa: E402
from pytransit.models.numba import ldmodels as ldm  # noqa: E402


def save(name, **arrays):
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **arrays)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.1f} KiB)")


def draw_pv(rng, npv, p_range=(1.0, 10.0), ecc=False, t0c=0.0):
    """Parameter vectors with the distributions of the small (64 x 1000) workload."""
    k = rng.uniform(0.05, 0.15, npv)
    u1 = rng.uniform(0.0, 0.6, npv)
    u2 = rng.uniform(0.0, 0.3, npv)
    t0 = t0c + rng.normal(0.0, 1e-3, npv)
    p = rng.uniform(*p_range, npv)
    a = rng.uniform(3.0, 20.0, npv)
    b = rng.uniform(0.0, 0.9, npv)
    inc = np.arccos(b / a)
    if ecc:
        e = rng.uniform(0.0, 0.3, npv)
        w = rng.uniform(0.0, 2 * np.pi, npv)
    else:
        e = np.zeros(npv)
        w = np.zeros(npv)
    return k, u1, u2, t0, p, a, inc, e, w


def case_c0():
    """64 parameter vectors x 1000 times over t0 +- 0.15 d, quadratic LD, one LC."""
    rng = np.random.default_rng(20240601)
    npv = 64
    time = np.linspace(-0.15, 0.15, 1000)
    k, u1, u2, t0, p, a, inc, e, w = draw_pv(rng, npv)
    ldc = np.stack([u1, u2], -1).reshape(npv, 1, 2)
    tm = RoadRunnerModel('quadratic')
    tm.set_data(time)
    flux = tm.evaluate(k.reshape(npv, 1), ldc, t0.reshape(npv, 1), p, a, inc, e, w)
    save("c0_quadratic", time=time, k=k.reshape(npv, 1), ldc=ldc, t0=t0.reshape(npv, 1), p=p, a=a,
         inc=inc, e=e, w=w, flux=flux)


def case_multi():
    """Three light curves at BJD scale: two passbands, two epochs (TTV), mixed
    supersampling, eccentric orbits, per-passband radius ratios, invalid rows."""
    rng = np.random.default_rng(7)
    T = 2459000.0
    t_a = T + np.linspace(0.0, 10.0, 800)
    t_b = T + np.linspace(0.003, 10.003, 700)
    t_c = T + 20.0 + np.linspace(0.0, 6.0, 500)
    time = np.concatenate([t_a, t_b, t_c])
    lcids = np.concatenate([np.zeros(t_a.size, int), np.ones(t_b.size, int), np.full(t_c.size, 2)])
    pbids = np.array([0, 1, 1])
    epids = np.array([0, 0, 1])
    nsamples = np.array([1, 5, 3])
    exptimes = np.array([0.0, 0.02, 0.0104])
    npv = 8
    k = rng.uniform(0.07, 0.13, (npv, 2))
    ldc = np.stack([rng.uniform(0, 0.6, (npv, 2)), rng.uniform(0, 0.3, (npv, 2))], -1)
    t0 = T + 0.3 + rng.normal(0.0, 1e-3, npv)
    t0 = np.stack([t0, t0 + rng.normal(0.0, 0.01, npv)], -1)
    p = rng.uniform(1.0, 3.0, npv)
    a = rng.uniform(4.0, 10.0, npv)
    inc = np.arccos(rng.uniform(0.0, 0.95, npv) / a)
    e = rng.uniform(0.0, 0.3, npv)
    w = rng.uniform(0.0, 2 * np.pi, npv)
    a[6] = 0.9      # a <= 1 -> NaN row
    e[7] = -0.1     # e < 0 -> NaN row
    tm = RoadRunnerModel('quadratic')
    tm.set_data(time, lcids=lcids, pbids=pbids, nsamples=nsamples, exptimes=exptimes, epids=epids)
    flux = tm.evaluate(k, ldc, t0, p, a, inc, e, w)
    save("multi_lc_bjd", time=time, lcids=lcids, pbids=pbids, epids=epids, nsamples=nsamples,
         exptimes=exptimes, k=k, ldc=ldc, t0=t0, p=p, a=a, inc=inc, e=e, w=w, flux=flux)


def case_power2():
    """Four BJD-scale light curves at 30-min cadence, nsamples = 10, power-2 LD,
    eccentric orbits: a small instance of the precision workload."""
    rng = np.random.default_rng(11)
    T = 2459000.0
    npts = np.exp(rng.uniform(np.log(150), np.log(500), 4)).astype(int)
    time = np.concatenate([T + np.arange(n) / 48.0 for n in npts])
    lcids = np.concatenate([np.full(n, j) for j, n in enumerate(npts)])
    pbids = np.arange(4)
    nsamples = np.full(4, 10)
    exptimes = np.full(4, 1 / 48)
    npv = 6
    k, _, _, t0, p, a, inc, e, w = draw_pv(rng, npv, p_range=(0.5, 5.0), ecc=True, t0c=T)
    c = rng.uniform(0.3, 0.9, (npv, 4))
    al = rng.uniform(0.3, 0.8, (npv, 4))
    ldc = np.stack([c, al], -1)
    tm = RoadRunnerModel('power-2')
    tm.set_data(time, lcids=lcids, pbids=pbids, nsamples=nsamples, exptimes=exptimes)
    flux = tm.evaluate(k.reshape(npv, 1), ldc, t0.reshape(npv, 1), p, a, inc, e, w)
    save("power2_ss10", time=time, lcids=lcids, pbids=pbids, nsamples=nsamples, exptimes=exptimes,
         k=k.reshape(npv, 1), ldc=ldc, t0=t0.reshape(npv, 1), p=p, a=a, inc=inc, e=e, w=w, flux=flux)


def case_laws():
    """Every named LD law of the RoadRunner table on one small light curve,
    including the ones without an analytic integral (200-point trapezoid)."""
    rng = np.random.default_rng(3)
    time = np.linspace(-0.2, 0.2, 300)
    npv = 3
    k, _, _, t0, p, a, inc, e, w = draw_pv(rng, npv, p_range=(1.0, 4.0), ecc=True)
    coefs = {
        'uniform': np.zeros((npv, 1, 1)),
        'linear': rng.uniform(0.1, 0.6, (npv, 1, 1)),
        'quadratic': np.stack([rng.uniform(0, .6, npv), rng.uniform(0, .3, npv)], -1).reshape(npv, 1, 2),
        'quadratic-tri': rng.uniform(0.1, 0.9, (npv, 1, 2)),
        'nonlinear': np.tile([0.5, -0.2, 0.6, -0.25], (npv, 1)).reshape(npv, 1, 4) * rng.uniform(0.8, 1.2, (npv, 1, 1)),
        'general': rng.uniform(0.05, 0.2, (npv, 1, 3)),
        'square_root': rng.uniform(0.1, 0.4, (npv, 1, 2)),
        'logarithmic': rng.uniform(0.1, 0.4, (npv, 1, 2)),
        'exponential': rng.uniform(0.05, 0.2, (npv, 1, 2)),
        'power-2': np.stack([rng.uniform(.3, .9, npv), rng.uniform(.3, .8, npv)], -1).reshape(npv, 1, 2),
        'power-2-pm': np.stack([rng.uniform(.5, .7, npv), rng.uniform(.2, .4, npv)], -1).reshape(npv, 1, 2),
    }
    out = dict(time=time, k=k.reshape(npv, 1), t0=t0.reshape(npv, 1), p=p, a=a, inc=inc, e=e, w=w)
    for law, ldc in coefs.items():
        tm = RoadRunnerModel(law)
        tm.set_data(time)
        out[f"ldc__{law}"] = ldc
        out[f"flux__{law}"] = tm.evaluate(k.reshape(npv, 1), ldc, t0.reshape(npv, 1), p, a, inc, e, w)
        out[f"mu__{law}"] = tm.mu
        out[f"ldp__{law}"] = ldm.evaluate_ld(tm.ldmodel, tm.mu, ldc)
    save("ld_laws", **out)


class QuadLDModel(LDModel):
    """A user LD model through the reference's LDModel protocol (ldmodel.py:21-38)."""

    def _evaluate(self, mu, x):
        x = np.asarray(x)
        u1, u2 = x[..., 0:1], x[..., 1:2]
        return 1.0 - u1 * (1.0 - mu) - u2 * (1.0 - mu) ** 2

    def _integrate(self, x):
        x = np.asarray(x)
        return 2 * np.pi / 12 * (-2 * x[..., 0] - x[..., 1] + 6)


def user_law(mu, pv):
    return 1.0 - pv[0] * (1.0 - mu) - pv[1] * (1.0 - np.sqrt(mu))


def case_user_ld():
    """User-supplied LD: an LDModel instance, a bare callable (numerical disk
    integral) and an (ld, ldi) tuple."""
    rng = np.random.default_rng(5)
    time = np.linspace(-0.2, 0.2, 300)
    npv = 4
    k, u1, u2, t0, p, a, inc, e, w = draw_pv(rng, npv, p_range=(1.0, 4.0))
    ldc = np.stack([u1, u2], -1).reshape(npv, 1, 2)
    out = dict(time=time, k=k.reshape(npv, 1), t0=t0.reshape(npv, 1), p=p, a=a, inc=inc, e=e, w=w, ldc=ldc)
    for name, model in [("ldmodel", QuadLDModel()), ("callable", user_law),
                        ("tuple", (ldm.ld_quadratic, ldm.ldi_quadratic))]:
        tm = RoadRunnerModel(model)
        tm.set_data(time)
        out[f"flux__{name}"] = tm.evaluate(k.reshape(npv, 1), ldc, t0.reshape(npv, 1), p, a, inc, e, w)
    save("user_ld", **out)


def case_klims():
    """Radius ratios outside the precomputed table (2D weight path)."""
    time = np.linspace(-0.12, 0.12, 400)
    k = np.array([[0.003], [0.6], [0.25], [0.005], [0.49]])
    npv = k.shape[0]
    ldc = np.tile([0.4, 0.2], (npv, 1)).reshape(npv, 1, 2)
    t0 = np.zeros((npv, 1))
    p = np.full(npv, 3.0)
    a = np.full(npv, 8.0)
    inc = np.arccos(np.array([0.1, 0.3, 0.5, 0.0, 0.2]) / a)
    e = np.zeros(npv)
    w = np.zeros(npv)
    tm = RoadRunnerModel('quadratic')
    tm.set_data(time)
    flux = tm.evaluate(k, ldc, t0, p, a, inc, e, w)
    save("klims", time=time, k=k, ldc=ldc, t0=t0, p=p, a=a, inc=inc, e=e, w=w, flux=flux)


def case_simple():
    """One parameter vector and one light curve: the rr_simple branch
    (rrmodel.py:236-238), with supersampling."""
    time = 2459000.0 + np.linspace(1.9, 2.1, 500)
    tm = RoadRunnerModel('quadratic')
    tm.set_data(time, nsamples=[4], exptimes=[0.01])
    args = dict(k=0.11, ldc=np.array([0.35, 0.22]), t0=2459000.0 + 0.0004, p=2.0, a=6.5,
                inc=np.arccos(0.4 / 6.5), e=0.12, w=1.3)
    flux = tm.evaluate(args['k'], args['ldc'], args['t0'], args['p'], args['a'], args['inc'],
                       args['e'], args['w'])
    save("simple", time=time, flux=flux, **{k: np.asarray(v) for k, v in args.items()})


def case_ts():
    """TransmissionSpectroscopyModel: five channels sharing one orbit, with the
    per-pv 2D table (default) and with the precomputed 3D table."""
    rng = np.random.default_rng(13)
    time = np.linspace(-0.2, 0.2, 500)
    npv, npb = 3, 5
    k = rng.uniform(0.09, 0.11, (npv, npb))
    ldc = np.stack([rng.uniform(0.2, 0.5, (npv, npb)), rng.uniform(0.1, 0.3, (npv, npb))], -1)
    t0 = rng.normal(0.0, 1e-3, npv)
    p = rng.uniform(1.0, 4.0, npv)
    a = rng.uniform(4.0, 12.0, npv)
    inc = np.arccos(rng.uniform(0.0, 0.8, npv) / a)
    e = rng.uniform(0.0, 0.2, npv)
    w = rng.uniform(0.0, 2 * np.pi, npv)
    out = dict(time=time, k=k, ldc=ldc, t0=t0, p=p, a=a, inc=inc, e=e, w=w)
    for name, interp in [("2d", False), ("3d", True)]:
        tm = TransmissionSpectroscopyModel('quadratic', precompute_weights=interp)
        tm.set_data(time, nsamples=[3], exptimes=[0.01])
        out[f"flux__{name}"] = tm.evaluate(k, ldc, t0, p, a, inc, e, w)
    save("ts", **out)


def case_tables():
    """Integration grid, weight-table samples and the area/interpolation helpers."""
    tm = RoadRunnerModel('quadratic')
    W = tm.weights
    rng = np.random.default_rng(17)
    ks = rng.uniform(0.01, 0.6, 200)
    zs = rng.uniform(0.0, 1.7, 200)
    zs[:8] = [0.0, 0.1, 0.9, 1.0, 1.05, 1.1, 1.2, 0.5]
    ks[:8] = [0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.6]
    areas = np.array([rrc.circle_circle_intersection_area_kite(1.0, k, z) for k, z in zip(ks, zs)])
    _, dg2, W2 = rrc.calculate_weights_2d(0.6, tm.ze, tm.ng)
    lda = np.cos(np.linspace(0, 2, 100))
    gs = np.concatenate([rng.uniform(0, 1.0 - 1e-6, 100), [0.0, 0.5, 1.0 + 1e-9, 1.2]])
    interp = np.array([rrc.interpolate_mean_limb_darkening_s(g, tm.dg, lda) for g in gs])
    save("tables", ze=tm.ze, zm=tm.zm, mu=tm.mu, dk=tm.dk, dg=tm.dg, w_sub=W[::37, ::9, :],
         w_sum=W.sum(), w_sumsq=(W ** 2).sum(), w_rowsum=W.sum(-1), ks=ks, zs=zs, areas=areas,
         dg2=dg2, w2=W2, lda=lda, gs=gs, interp=interp)


def case_ma_quadratic():
    """The reference's Mandel & Agol quadratic model, eval_quad_z_s
    (pytransit/models/numba/ma_quadratic_nb.py), over z grids for several k
    and limb darkening coefficients, with the special points (z = 0, k, 1,
    1 + k, near 1 - k and the k = 1/2 edge case).  Points where the pure-Python
    function fails (exactly z = 1 - k reads the unassigned limb angles) are
    left out (ok = False).  Some z give NaN in the reference (a negative
    square root near the limb); those are kept."""
    from pytransit.models.numba.ma_quadratic_nb import eval_quad_z_s
    rng = np.random.default_rng(29)
    ks = np.array([0.01, 0.05, 0.1, 0.12, 0.3, 0.5, 0.50005, 0.7, 1.2])
    us = np.array([[0.0, 0.0], [0.2, 0.1], [0.6, 0.3], [0.1, 0.5]])
    zs = np.concatenate([np.linspace(0.0, 2.3, 600), rng.uniform(0.0, 2.3, 200)])
    flux = np.full((ks.size, us.shape[0], zs.size + 8), np.nan)
    ok = np.zeros(flux.shape, bool)
    zall = np.zeros((ks.size, zs.size + 8))
    for ik, k in enumerate(ks):
        zk = np.concatenate([zs, [0.0, k, 1.0, 1.0 + k, 1.0 - k + 1e-7, 1.0 - k - 1e-7, k + 5e-7, 0.5]])
        zall[ik] = zk
        for iu, u in enumerate(us):
            for iz, z in enumerate(zk):
                try:
                    flux[ik, iu, iz] = eval_quad_z_s(z, k, u)
                    ok[ik, iu, iz] = True
                except UnboundLocalError:
                    pass
    save("ma_quadratic", ks=ks, us=us, z=zall, flux=flux, ok=ok)


def case_lpf_map():
    """BaseLPF.transit_model's parameter mapping from the reference's own code:
    as_from_rhop and i_from_ba (pytransit/orbits/orbits_py.py) imported, and
    map_ldc (pytransit/lpf/lpf.py:85-91) taken from the source file and
    executed on its own (lpf.py's module imports - xarray, arviz, astropy,
    matplotlib - are not installed here)."""
    import ast
    from pytransit.orbits.orbits_py import as_from_rhop, i_from_ba
    src = open(os.path.join(REF, "pytransit", "lpf", "lpf.py")).read()
    fn = next(n for n in ast.parse(src).body if isinstance(n, ast.FunctionDef) and n.name == "map_ldc")
    fn.decorator_list = []
    ns = {"atleast_2d": np.atleast_2d, "zeros_like": np.zeros_like, "sqrt": np.sqrt}
    exec(compile(ast.Module(body=[fn], type_ignores=[]), "lpf.py", "exec"), ns)
    map_ldc = ns["map_ldc"]
    rng = np.random.default_rng(37)
    npv, npb, tref = 500, 3, 2459000.0
    pv = np.column_stack([tref + rng.normal(0.3, 0.01, npv), rng.uniform(0.5, 20, npv), rng.uniform(0.1, 25, npv),
                          rng.uniform(0, 1, npv), rng.uniform(0.0025, 0.04, npv)] +
                         [rng.uniform(0, 1, npv) for _ in range(2 * npb)])
    a = as_from_rhop(pv[:, 2], pv[:, 1])
    save("lpf_map", pv=pv, tref=tref, npb=npb, k=np.sqrt(pv[:, 4:5]), t0=pv[:, 0] - tref, p=pv[:, 1], a=a,
         inc=i_from_ba(pv[:, 3], a), ldc=map_ldc(pv[:, 5:]).reshape(npv, npb, 2))


def case_eclipse():
    """The reference's RoadRunner secondary-eclipse kernels, eclipse_model
    (model_eclipse.py) and esmodel (model_ecspec.py), on the restated orbit
    layer (shim: solve2d about mid-eclipse, eclipse_time_offset,
    eclipse_light_travel_time): the reference test's canonical case, a
    multi-light-curve BJD-scale set with supersampling, epochs, eccentric
    orbits and invalid rows, and the spectroscopic variant."""
    from pytransit.models.roadrunner.model_eclipse import eclipse_model
    from pytransit.models.roadrunner.model_ecspec import esmodel
    out = {}
    times = np.linspace(-0.5, 3.5, 5000)
    out["canon_time"] = times
    out["canon_flux"] = eclipse_model(times, np.array([0.1]), np.full((1, 1), 0.0), np.array([2.0]), np.array([8.0]),
                                      np.array([np.pi / 2]), np.array([0.0]), np.array([0.0]), 1.0, 1,
                                      np.zeros(times.size, np.int64), np.zeros(1, np.int64), np.ones(1, np.int64),
                                      np.zeros(1))
    rng = np.random.default_rng(53)
    T = 2459000.0
    t_a = T + np.arange(0, 6.0, 2 / 1440)
    t_b = T + 7.0 + np.arange(0, 5.0, 10 / 1440)
    time = np.concatenate([t_a, t_b])
    lcids = np.concatenate([np.zeros(t_a.size, np.int64), np.ones(t_b.size, np.int64)])
    epids = np.array([0, 1])
    nsamples = np.array([1, 5])
    exptimes = np.array([0.0, 10 / 1440])
    npv = 12
    k = rng.uniform(0.05, 0.15, npv)
    t0 = T + 0.2 + rng.normal(0, 1e-3, npv)
    t0 = np.stack([t0, t0 + rng.normal(0, 0.005, npv)], -1)
    p = rng.uniform(1.0, 4.0, npv)
    a = rng.uniform(4.0, 12.0, npv)
    inc = np.arccos(rng.uniform(0, 0.7, npv) / a)
    e = np.concatenate([np.zeros(4), rng.uniform(0, 0.3, npv - 4)])
    w = rng.uniform(0, 2 * np.pi, npv)
    a[5] = 0.8          # a <= 1: NaN row
    out.update(dict(time=time, lcids=lcids, epids=epids, nsamples=nsamples, exptimes=exptimes, k=k, t0=t0, p=p, a=a,
                    inc=inc, e=e, w=w, rstar=1.3))
    out["flux"] = eclipse_model(time, k, t0, p, a, inc, e, w, 1.3, 2, lcids, epids, nsamples, exptimes)
    # spectroscopic variant: per-pv rstar, npb flux ratios, the first light curve's sampling
    npv_s, npb = 6, 7
    ts = T + np.arange(-1.0, 4.0, 5 / 1440)
    fr = rng.uniform(1e-4, 5e-3, (npv_s, npb))
    rs = rng.uniform(0.5, 2.0, npv_s)
    es = dict(k=k[:npv_s], t0=t0[:npv_s, 0], p=p[:npv_s], a=a[:npv_s], inc=inc[:npv_s], e=e[:npv_s], w=w[:npv_s])
    out.update({f"es_{n}": v for n, v in es.items()})
    out.update(dict(es_time=ts, es_rstar=rs, es_fratio=fr))
    out["es_flux"] = esmodel(ts, es["k"], es["t0"], es["p"], es["a"], es["inc"], es["e"], es["w"], rs, fr, 3, 0.01)
    save("eclipse", **out)


def case_taylor_orbit():
    """The reference's own Taylor orbit (pytransit/orbits/taylor_z.py): the
    finite-difference velocity, acceleration, jerk and snap at mid-transit
    (vajs_from_paiew), z over the transit window (z_taylor_v) and the contact
    points (find_contact_point), independent of the meepmeep restatement the
    RoadRunner fixtures run on."""
    import types
    orbits = types.ModuleType("pytransit.orbits")
    orbits.__path__ = [os.path.join(REF, "pytransit", "orbits")]
    sys.modules["pytransit.orbits"] = orbits
    from pytransit.orbits import taylor_z as tz
    rng = np.random.default_rng(71)
    n = 48
    p = rng.uniform(0.5, 15.0, n)
    a = rng.uniform(3.0, 20.0, n)
    b = rng.uniform(0.0, 0.9, n)
    inc = np.arccos(b / a)
    e = np.where(np.arange(n) % 2 == 0, 0.0, rng.uniform(0.0, 0.3, n))
    w = rng.uniform(0.0, 2 * np.pi, n)
    k = rng.uniform(0.05, 0.15, n)
    tt = np.linspace(-1.0, 1.0, 401)       # in units of the half-window
    times, z, t14 = np.zeros((n, tt.size)), np.zeros((n, tt.size)), np.zeros((n, 2))
    vajs = np.zeros((n, 9))
    for j in range(n):
        v = tz.vajs_from_paiew(p[j], a[j], inc[j], e[j], w[j])
        vajs[j] = v
        t14[j] = [tz.find_contact_point(k[j], 1, *v), tz.find_contact_point(k[j], 4, *v)]
        half = 1.2 * max(abs(t14[j, 0]), abs(t14[j, 1]))
        times[j] = tt * half
        z[j] = tz.z_taylor_v(times[j], 0.0, p[j], *v)
    save("taylor_orbit", p=p, a=a, inc=inc, e=e, w=w, k=k, times=times, z=z, t14=t14, vajs=vajs)


if __name__ == "__main__":
    for f in (case_tables, case_c0, case_multi, case_power2, case_laws, case_user_ld, case_klims,
              case_simple, case_ts, case_ma_quadratic, case_lpf_map, case_eclipse, case_taylor_orbit):
        print(f.__name__)
        f()

"""Stated error bounds of the split paths: every result carries an upper
bound of its absolute flux error against the FP64 model
(RoadRunnerModel.error_bounds / last_error_bound, evaluate(return_error=True),
the served futures' error_bound).  Checked per parameter vector: the bound is
at least the measured max |F_split - F_FP64| over all points, on populations
that stress it (BJD-scale multi-light-curve data, eccentric orbits with 10
supersamples over a 1000-day baseline, radius ratios up to 0.5 and grazing
orbits, transmission spectroscopy, the serving loop)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def population(rng, npv, kmax=0.15, grazing=False, ecc=False):
    a = rng.uniform(3, 20, npv)
    b = rng.uniform(0, 0.9, npv)
    k = rng.uniform(0.05, kmax, (npv, 1))
    if grazing:
        b = rng.uniform(0.8, 1.0, npv) * (1 + k[:, 0])
    return dict(k=k, t0=2459000.0 + rng.normal(0, 1e-3, (npv, 1)), p=rng.uniform(0.5, 15, npv), a=a,
                i=np.arccos(b / a), e=rng.uniform(0, 0.3, npv) if ecc else np.zeros(npv),
                w=rng.uniform(0, 2 * np.pi, npv) if ecc else np.zeros(npv))


def per_pv_error(law, data, prm, ldc):
    from pytransit_gb300 import RoadRunnerModel
    out = {}
    for prec in ('split', 'fp64'):
        m = RoadRunnerModel(law, precision=prec)
        m.set_data(**data)
        f, bound = m.evaluate(prm['k'], ldc, prm['t0'], prm['p'], prm['a'], prm['i'], prm['e'], prm['w'],
                              return_error=True)
        out[prec] = (np.asarray(f).reshape(len(prm['p']), -1), m.error_bounds(), bound)
    d = np.abs(out['split'][0] - out['fp64'][0])
    return np.nanmax(np.where(np.isnan(d), 0.0, d), axis=1), out['split'][1], out['split'][2], out['fp64'][2]


@pytest.mark.parametrize("case", ["bjd_multi_lc", "eccentric_long_ns10", "large_k_grazing", "nonlinear"])
def test_split_bound_holds_per_parameter_vector(case):
    rng = np.random.default_rng({"bjd_multi_lc": 1, "eccentric_long_ns10": 2, "large_k_grazing": 3,
                                 "nonlinear": 4}[case])
    T = 2459000.0
    npv = 512
    if case == "eccentric_long_ns10":
        npts = [3000, 9000, 20000, 700]
        time = np.concatenate([T + np.arange(n) / 48.0 + 250.0 * j for j, n in enumerate(npts)])
        lcids = np.concatenate([np.full(n, j) for j, n in enumerate(npts)])
        data = dict(time=time, lcids=lcids, pbids=np.arange(4), nsamples=np.full(4, 10), exptimes=np.full(4, 1 / 48))
        prm = population(rng, npv, ecc=True)
        law = 'power-2'
        ldc = np.stack([rng.uniform(.3, .9, (npv, 4)), rng.uniform(.3, .8, (npv, 4))], -1)
    else:
        npt = 19700 if case == "bjd_multi_lc" else 8000
        time = T + np.arange(npt) * (2 / 1440)
        lcids = np.minimum((np.arange(npt) * 4) // npt, 3)
        data = dict(time=time, lcids=lcids, pbids=np.arange(4), nsamples=np.ones(4, int), exptimes=np.zeros(4))
        prm = population(rng, npv, kmax=0.5 if case == "large_k_grazing" else 0.15,
                         grazing=case == "large_k_grazing")
        if case == "nonlinear":
            law = 'nonlinear'
            ldc = np.tile([0.5, -0.2, 0.6, -0.25], (npv, 4, 1)) * rng.uniform(0.8, 1.2, (npv, 4, 1))
        else:
            law = 'quadratic'
            ldc = np.stack([rng.uniform(0, .6, (npv, 4)), rng.uniform(0, .3, (npv, 4))], -1)
    err, bounds, bmax, b64 = per_pv_error(law, data, prm, ldc)
    assert (err > 0).sum() > npv // 4                        # transits in the data
    assert np.all(bounds >= err), (np.argmax(err - bounds), (err - bounds).max())
    assert bmax == bounds.max() and b64 == 1e-12
    if case != "large_k_grazing":
        assert bmax <= 1e-6                                  # the split path's precision target


def test_fp64_bound_holds_against_the_oracle(golden):
    from pytransit_gb300 import RoadRunnerModel
    g = golden("c0_quadratic")
    m = RoadRunnerModel('quadratic', precision='fp64')
    m.set_data(g["time"])
    f, bound = m.evaluate(g["k"], g["ldc"], g["t0"], g["p"], g["a"], g["inc"], g["e"], g["w"], return_error=True)
    assert np.abs(f - g["flux"]).max() <= bound


@pytest.mark.parametrize("ns", [1, 10])
def test_ts_split_bound_holds(ns):
    from pytransit_gb300 import TSModel
    rng = np.random.default_rng(8 + ns)
    T = 2459000.0
    time = T + np.arange(6000) * (2 / 1440)
    npv, npb = 48, 100
    prm = population(rng, npv, ecc=True)
    k = rng.uniform(0.09, 0.11, (npv, npb))
    ldc = np.stack([rng.uniform(0, .6, (npv, npb)), rng.uniform(0, .3, (npv, npb))], -1)
    out = {}
    for prec in ('split', 'fp64'):
        m = TSModel('quadratic', precision=prec)
        m.set_data(time, nsamples=[ns], exptimes=[0.02 if ns > 1 else 0.0])
        f, b = m.evaluate(k, ldc, prm['t0'][:, 0], prm['p'], prm['a'], prm['i'], prm['e'], prm['w'], return_error=True)
        out[prec] = (f, m.error_bounds(), b)
    err = np.abs(out['split'][0] - out['fp64'][0]).reshape(npv, -1).max(axis=1)
    assert (err > 0).sum() > npv // 4
    assert np.all(out['split'][1] >= err), (err - out['split'][1]).max()


def test_served_results_state_their_bound():
    """Each served future's error_bound holds against the oracle's FP64 flux
    (and is within 1e-6 for the RoadRunner requests; a transmission-spectroscopy
    bound is larger, set by the k-derivative term's square-root behaviour at
    contact)."""
    from pytransit_gb300.serving import RRServer
    rng = np.random.default_rng(12)
    T = 2459000.0
    reqs = []
    for j in range(6):
        kind = 'ts' if j % 3 == 2 else 'rr'
        npv, npt = int(rng.integers(1, 40)), int(rng.integers(500, 6000))
        time = T + np.sort(rng.uniform(0, 5, npt))
        prm = population(rng, npv, ecc=True)
        if kind == 'ts':
            params = dict(prm, k=rng.uniform(0.09, 0.11, (npv, 10)), t0=prm['t0'][:, 0] + rng.uniform(0, 1, npv),
                          ldc=np.tile([0.4, 0.2], (npv, 10, 1)))
        else:
            params = dict(prm, t0=prm['t0'][:, 0] + rng.uniform(0, 1, npv), ldc=np.tile([0.4, 0.2], (npv, 1, 1)))
        reqs.append((kind, 'quadratic', dict(time=time, nsamples=[5], exptimes=[0.01]), params))
    srv = RRServer(hbm_budget=4e9)
    futs = [srv.submit(*r) for r in reqs]
    got = [f.result(timeout=600) for f in futs]
    srv.close()
    for (kind, law, data, params), f, g in zip(reqs, futs, got):
        ref = oracle.OracleRoadRunner(law, ts=kind == 'ts')
        ref.set_data(data['time'], nsamples=data['nsamples'], exptimes=data['exptimes'])
        t0 = params['t0'] if kind == 'ts' else params['t0'].reshape(-1, 1)
        want = ref.evaluate(params['k'], params['ldc'], t0, params['p'], params['a'], params['i'], params['e'],
                            params['w']).reshape(g.shape)
        assert f.error_bound is not None and f.error_bound > 0
        assert np.nanmax(np.abs(g - want)) <= f.error_bound
        if kind == 'rr':
            assert f.error_bound <= 1e-6

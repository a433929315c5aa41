"""Serving loop on the GPU: every request's flux is the same served alone and
in a mix of concurrent requests (plain and transmission spectroscopy, three LD
laws, uneven sizes), equals the drop-in model's split-precision result, and
matches the oracle (the reference's algorithm in FP64 on the CPU).
Tolerance: 1e-6 in flux (the split path's), NaN rows must match."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-6


def make_request(rng, kind, law, npv, npt, ns):
    T = 2459000.0
    nlc = 1 if kind == 'ts' else int(rng.integers(1, 4))
    time = T + np.sort(rng.uniform(0, 5, npt))
    lcids = np.minimum((np.arange(npt) * nlc) // npt, nlc - 1)
    data = dict(time=time, lcids=lcids, pbids=np.arange(nlc), nsamples=np.full(nlc, ns),
                exptimes=np.full(nlc, 0.02 if ns > 1 else 0.0))
    npar = {'quadratic': 2, 'power-2': 2, 'nonlinear': 4}[law]
    npb = 12 if kind == 'ts' else nlc
    if law == 'nonlinear':
        ldc = np.tile([0.5, -0.2, 0.6, -0.25], (npv, npb, 1)) * rng.uniform(0.8, 1.2, (npv, npb, 1))
    elif law == 'power-2':
        ldc = np.stack([rng.uniform(.3, .9, (npv, npb)), rng.uniform(.3, .8, (npv, npb))], -1)
    else:
        ldc = np.stack([rng.uniform(0, .6, (npv, npb)), rng.uniform(0, .3, (npv, npb))], -1)
    k = rng.uniform(0.09, 0.11, (npv, npb)) if kind == 'ts' else rng.uniform(0.05, 0.15, (npv, 1))
    a = rng.uniform(3, 15, npv)
    params = dict(k=k, ldc=ldc, t0=T + rng.uniform(0, 1, npv), p=rng.uniform(0.7, 4, npv), a=a,
                  i=np.arccos(rng.uniform(0, 0.9, npv) / a), e=rng.uniform(0, 0.2, npv),
                  w=rng.uniform(0, 2 * np.pi, npv))
    if npv > 2:
        params['a'][1] = 0.5     # one invalid row
    assert ldc.shape[2] == npar
    return kind, law, data, params


def direct(kind, law, data, params):
    from pytransit_gb300 import RoadRunnerModel, TransmissionSpectroscopyModel
    if kind == 'ts':
        m = TransmissionSpectroscopyModel(law, precision='split')
        m.set_data(data['time'], nsamples=data['nsamples'][:1], exptimes=data['exptimes'][:1])
        return m.evaluate(params['k'], params['ldc'], params['t0'], params['p'], params['a'], params['i'],
                          params['e'], params['w'])
    m = RoadRunnerModel(law, precision='split')
    m.set_data(**data)
    return m.evaluate(params['k'], params['ldc'], params['t0'].reshape(-1, 1), params['p'], params['a'],
                      params['i'], params['e'], params['w']).reshape(len(params['p']), -1)


def reference(kind, law, data, params):
    """The oracle's FP64 flux of one request."""
    if kind == 'ts':
        ref = oracle.OracleRoadRunner(law, ts=True)
        ref.set_data(data['time'], nsamples=data['nsamples'][:1], exptimes=data['exptimes'][:1])
        return ref.evaluate(params['k'], params['ldc'], params['t0'], params['p'], params['a'], params['i'],
                            params['e'], params['w'])
    ref = oracle.OracleRoadRunner(law)
    ref.set_data(**data)
    return ref.evaluate(params['k'], params['ldc'], params['t0'].reshape(-1, 1), params['p'], params['a'],
                        params['i'], params['e'], params['w']).reshape(len(params['p']), -1)


def close(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64).reshape(a.shape)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    m = ~np.isnan(a)
    return np.abs(a[m] - b[m]).max() if m.any() else 0.0


def test_same_alone_and_in_the_mix():
    from pytransit_gb300.serving import RRServer
    rng = np.random.default_rng(42)
    laws = ['quadratic', 'power-2', 'nonlinear']
    reqs = []
    for j in range(14):
        kind = 'ts' if j % 5 == 4 else 'rr'
        npv = int(np.exp(rng.uniform(0, np.log(300))))
        npt = int(np.exp(rng.uniform(np.log(300), np.log(20000))))
        reqs.append(make_request(rng, kind, laws[j % 3], npv, npt, int(rng.choice([1, 5, 10]))))
    srv = RRServer(hbm_budget=8e9, step_items=512)
    futs = [srv.submit(*r) for r in reqs]
    mixed = [f.result(timeout=600) for f in futs]
    srv.close()
    assert srv.stats.completed == len(reqs)
    alone = []
    for r in reqs:
        s1 = RRServer(hbm_budget=8e9)
        alone.append(s1.submit(*r).result(timeout=600))
        s1.close()
    for r, got, one in zip(reqs, mixed, alone):
        assert close(got, one) <= TOL
        assert close(got, direct(*r)) <= TOL
        assert close(got, reference(*r)) <= TOL
    assert any(np.nanmin(g) < 0.999 for g in mixed)   # transits are in the data


def test_device_results_through_the_persistent_kernel():
    """With device-resident results every request, transmission spectroscopy
    included, runs through the batched persistent steps; each result matches
    the oracle."""
    from pytransit_gb300.serving import RRServer
    rng = np.random.default_rng(7)
    reqs = [make_request(rng, 'ts', 'quadratic', 9, 3000, 1), make_request(rng, 'rr', 'power-2', 40, 5000, 5),
            make_request(rng, 'ts', 'nonlinear', 4, 7000, 10), make_request(rng, 'ts', 'power-2', 1, 800, 5)]
    srv = RRServer(hbm_budget=8e9, result='device', step_items=8)
    futs = [srv.submit(*r) for r in reqs]
    got = [f.result(timeout=600).cpu().numpy() for f in futs]
    srv.close()
    assert srv.stats.completed == len(reqs) and srv.stats.steps > 1
    for r, g in zip(reqs, got):
        assert close(g, reference(*r)) <= TOL


@pytest.mark.parametrize("result", ["device", "host"])
def test_dropped_results_resolve_to_their_point_count(result):
    """keep_result=False (consumers that only count or time): every future
    resolves to the request's number of model points, and the server's step
    and busy counters advance."""
    from pytransit_gb300.serving import RRServer
    rng = np.random.default_rng(11)
    reqs = [make_request(rng, 'rr', 'quadratic', 12, 2000, 1), make_request(rng, 'ts', 'power-2', 3, 1500, 5),
            make_request(rng, 'rr', 'nonlinear', 5, 900, 10)]
    srv = RRServer(hbm_budget=4e9, result=result, step_items=16)
    futs = [srv.submit(*r, keep_result=False) for r in reqs]
    got = [f.result(timeout=120) for f in futs]
    srv.close()
    for (kind, law, data, params), n in zip(reqs, got):
        npv = np.asarray(params['p']).size
        npb = np.asarray(params['k']).shape[1] if kind == 'ts' else 1
        assert n == npv * npb * data['time'].size
    st = srv.stats.summary()
    assert st['completed'] == len(reqs) and st['steps'] >= 1
    assert st['admit_s'] > 0 and st['gpu_step_s'] >= 0

"""Fused log-likelihood and adjoint gradient (rr_lnlike_f64 / rr_lnlike_split).

The workload follows the differentiation configuration: 5000 times over
t0 +- 0.2 d, 30-min exposures with 5 supersamples, quadratic LD, eccentric
orbits, Gaussian noise sigma = 5e-4 on the model at a seeded truth; gradients
at perturbed parameter vectors.

Tolerances:
  * lnL, FP64 GPU vs the oracle (rr_full + Gaussian lnL in C): 1e-9 relative;
  * gradient vs central finite differences (h = 1e-6 relative, with floors;
    the step actually taken in floating point is used): 1e-4 relative, each
    column measured against its largest magnitude over the population;
  * split vs FP64: lnL to 1e-6 relative, gradient to 1e-4 relative (same
    column-relative measure).
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

SIGMA = 5e-4
H_REL = 1e-6
FLOORS = dict(k=1e-3, t0=1e-2, p=1.0, a=1.0, i=1.0, e=1e-2, w=1e-1, ldc=1e-2)


def c3_case(npv=12, npt=5000, seed=3, law='quadratic'):
    rng = np.random.default_rng(seed)
    time = np.linspace(-0.2, 0.2, npt)
    data = dict(time=time, nsamples=[5], exptimes=[1 / 48])
    k = rng.uniform(0.05, 0.15, (npv, 1))
    if law == 'quadratic':
        ldc = np.stack([rng.uniform(0, .6, npv), rng.uniform(0, .3, npv)], -1).reshape(npv, 1, 2)
    else:
        ldc = np.stack([rng.uniform(.3, .9, npv), rng.uniform(.3, .8, npv)], -1).reshape(npv, 1, 2)
    t0 = rng.normal(0, 1e-3, (npv, 1))
    p = rng.uniform(1, 10, npv)
    a = rng.uniform(3, 20, npv)
    inc = np.arccos(rng.uniform(0, .9, npv) / a)
    e = rng.uniform(0, .3, npv)
    w = rng.uniform(0, 2 * np.pi, npv)
    truth = dict(k=k, ldc=ldc, t0=t0, p=p, a=a, i=inc, e=e, w=w)
    ref = oracle.OracleRoadRunner(law)
    ref.set_data(**data)
    f_true = ref.evaluate(k[:1], ldc[:1], t0[:1], p[:1], a[:1], inc[:1], e[:1], w[:1])
    obs = f_true + rng.normal(0, SIGMA, npt)
    # evaluate at perturbed versions of the first vector's parameters
    pert = dict(k=k[:1] * (1 + rng.normal(0, 0.02, (npv, 1))),
                ldc=np.clip(ldc[:1] + rng.normal(0, 0.02, (npv, 1, 2)), 0.01, None),
                t0=t0[:1] + rng.normal(0, 2e-4, (npv, 1)), p=p[:1] * (1 + rng.normal(0, 1e-4, npv)),
                a=a[:1] * (1 + rng.normal(0, 0.01, npv)), i=inc[:1] + rng.normal(0, 1e-3, npv),
                e=np.clip(e[:1] + rng.normal(0, 0.01, npv), 0.0, None), w=w[:1] + rng.normal(0, 0.05, npv))
    return data, obs, pert, ref


def model(law='quadratic', precision='fp64', **data):
    from pytransit_gb300 import RoadRunnerModel
    m = RoadRunnerModel(law, precision=precision)
    m.set_data(**data)
    return m


def lnl_of(m, obs, prm, grad=False):
    from pytransit_gb300.lnlike import lnlikelihood
    return lnlikelihood(m, obs, SIGMA, prm['k'], prm['ldc'], prm['t0'], prm['p'], prm['a'], prm['i'],
                        prm['e'], prm['w'], grad=grad)


def param_vector(prm):
    """Flatten in the gradient's column order: k, t0, p, a, i, e, w, ldc."""
    return [('k', (slice(None), 0)), ('t0', (slice(None), 0)), ('p', ()), ('a', ()), ('i', ()),
            ('e', ()), ('w', ()), ('ldc', (slice(None), 0, 0)), ('ldc', (slice(None), 0, 1))]


def fd_gradient(m, obs, prm):
    base = {n: np.array(v, dtype=np.float64, copy=True) for n, v in prm.items()}
    cols = []
    for name, idx in param_vector(prm):
        x = base[name][idx] if idx else base[name]
        h = H_REL * np.maximum(np.abs(x), FLOORS[name])
        up = {n: v.copy() for n, v in base.items()}
        dn = {n: v.copy() for n, v in base.items()}
        if idx:
            up[name][idx] = x + h
            dn[name][idx] = x - h
            step = up[name][idx] - dn[name][idx]
        else:
            up[name] = x + h
            dn[name] = x - h
            step = up[name] - dn[name]
        cols.append((lnl_of(m, obs, up) - lnl_of(m, obs, dn)) / step)
    return np.stack(cols, -1)


def rel_err(g, ref):
    """|g - ref| relative to each column's largest |ref| over the parameter vectors."""
    return np.abs(g - ref) / np.abs(ref).max(axis=0, keepdims=True)


def test_lnlike_fp64_matches_oracle():
    data, obs, pert, ref = c3_case()
    m = model(**data)
    lnl = lnl_of(m, obs, pert)
    flux = ref.evaluate(pert['k'], pert['ldc'], pert['t0'], pert['p'], pert['a'], pert['i'], pert['e'], pert['w'])
    want = oracle.lnlike_normal(obs, flux, SIGMA)
    np.testing.assert_allclose(lnl, want, rtol=1e-9)


def test_gradient_fp64_vs_finite_differences():
    data, obs, pert, _ = c3_case()
    m = model(**data)
    _, g = lnl_of(m, obs, pert, grad=True)
    fd = fd_gradient(m, obs, pert)
    err = rel_err(g, fd)
    assert err.max() < 1e-4, (err.max(axis=0))


def test_split_vs_fp64_lnlike_and_gradient():
    data, obs, pert, _ = c3_case()
    l64, g64 = lnl_of(model(**data), obs, pert, grad=True)
    l32, g32 = lnl_of(model(precision='split', **data), obs, pert, grad=True)
    np.testing.assert_allclose(l32, l64, rtol=1e-6)
    err = rel_err(g32, g64)
    assert err.max() < 1e-4, (err.max(axis=0))


def test_gradient_vs_oracle_finite_differences():
    """Independent check: the adjoint against central differences of the
    oracle's own FP64 model + likelihood (C restatement)."""
    data, obs, pert, ref = c3_case(npv=3, npt=2000, seed=5)
    m = model(**data)
    _, g = lnl_of(m, obs, pert, grad=True)

    def lnl_oracle(prm):
        f = ref.evaluate(prm['k'], prm['ldc'], prm['t0'], prm['p'], prm['a'], prm['i'], prm['e'], prm['w'])
        return oracle.lnlike_normal(obs, f, SIGMA)

    base = {n: np.array(v, dtype=np.float64, copy=True) for n, v in pert.items()}
    cols = []
    for name, idx in param_vector(pert):
        x = base[name][idx] if idx else base[name]
        h = H_REL * np.maximum(np.abs(x), FLOORS[name])
        up = {n: v.copy() for n, v in base.items()}
        dn = {n: v.copy() for n, v in base.items()}
        if idx:
            up[name][idx], dn[name][idx] = x + h, x - h
            step = up[name][idx] - dn[name][idx]
        else:
            up[name], dn[name] = x + h, x - h
            step = up[name] - dn[name]
        cols.append((lnl_oracle(up) - lnl_oracle(dn)) / step)
    fd = np.stack(cols, -1)
    assert rel_err(g, fd).max() < 1e-4


def test_power2_ldc_gradient():
    data, obs, pert, _ = c3_case(npv=6, law='power-2', seed=9)
    m = model('power-2', **data)
    _, g = lnl_of(m, obs, pert, grad=True)
    fd = fd_gradient(m, obs, pert)
    assert rel_err(g, fd).max() < 1e-4


def test_multi_passband_multi_epoch_columns():
    """k per passband and two zero epochs: every gradient column against FD."""
    rng = np.random.default_rng(21)
    T = 2459000.0
    t_a = T + np.linspace(-0.2, 0.2, 1500)
    t_b = T + 3.0 + np.linspace(-0.2, 0.2, 1500)
    data = dict(time=np.concatenate([t_a, t_b]), lcids=np.repeat([0, 1], 1500), pbids=[0, 1], epids=[0, 1],
                nsamples=[3, 2], exptimes=[0.01, 0.02])
    npv = 4
    prm = dict(k=rng.uniform(0.09, 0.11, (npv, 2)), ldc=rng.uniform(0.1, 0.4, (npv, 2, 2)),
               t0=np.stack([T + rng.normal(0, 1e-3, npv), T + 3.0 + rng.normal(0, 1e-3, npv)], -1),
               p=np.full(npv, 3.0) + rng.normal(0, 1e-4, npv), a=rng.uniform(7, 9, npv),
               i=np.arccos(rng.uniform(0, 0.5, npv) / 8), e=rng.uniform(0, 0.1, npv), w=rng.uniform(0, 6, npv))
    ref = oracle.OracleRoadRunner('quadratic')
    ref.set_data(**data)
    obs = ref.evaluate(prm['k'][:1], prm['ldc'][:1], prm['t0'][:1], prm['p'][:1], prm['a'][:1], prm['i'][:1],
                       prm['e'][:1], prm['w'][:1]) + rng.normal(0, SIGMA, 3000)
    m = model(**data)
    _, g = lnl_of(m, obs, prm, grad=True)
    assert g.shape == (npv, 2 + 2 + 5 + 4)
    base = {n: np.array(v, dtype=np.float64, copy=True) for n, v in prm.items()}
    cols = []
    spec = [('k', (slice(None), 0)), ('k', (slice(None), 1)), ('t0', (slice(None), 0)), ('t0', (slice(None), 1)),
            ('p', ()), ('a', ()), ('i', ()), ('e', ()), ('w', ())] + \
           [('ldc', (slice(None), b, j)) for b in range(2) for j in range(2)]
    for name, idx in spec:
        x = base[name][idx] if idx else base[name]
        # t0 near BJD 2459000: a 1e-7 d step (the fold t - t0 is exact here and the
        # step actually taken is used); larger steps average over table kinks
        h = np.full_like(x, 1e-7) if name == 't0' else H_REL * np.maximum(np.abs(x), FLOORS[name])
        up = {n: v.copy() for n, v in base.items()}
        dn = {n: v.copy() for n, v in base.items()}
        if idx:
            up[name][idx], dn[name][idx] = x + h, x - h
            step = up[name][idx] - dn[name][idx]
        else:
            up[name], dn[name] = x + h, x - h
            step = up[name] - dn[name]
        cols.append((lnl_of(m, obs, up) - lnl_of(m, obs, dn)) / step)
    fd = np.stack(cols, -1)
    assert rel_err(g, fd).max() < 1e-4, rel_err(g, fd).max(axis=0)


def test_autograd_function_matches_direct_gradient():
    import torch
    from pytransit_gb300.lnlike import LogLikelihood, _as_params
    data, obs, pert, _ = c3_case(npv=5)
    m = model(**data)
    _, g = lnl_of(m, obs, pert, grad=True)
    k, t0, p, a, i, e, w, ldc = _as_params(m, pert['k'], pert['t0'], pert['p'], pert['a'], pert['i'], pert['e'],
                                           pert['w'], pert['ldc'])
    ts = [x.clone().requires_grad_(True) for x in (k, t0, p, a, i, e, w, ldc)]
    lnl = LogLikelihood.apply(m, obs, SIGMA, *ts)
    lnl.sum().backward()
    got = np.concatenate([ts[0].grad.cpu().numpy(), ts[1].grad.cpu().numpy()] +
                         [x.grad.cpu().numpy()[:, None] for x in ts[2:7]] +
                         [ts[7].grad.cpu().numpy().reshape(5, -1)], axis=1)
    np.testing.assert_allclose(got, g, rtol=1e-12, atol=0)


def fd_gradient_h(m, obs, prm, scale):
    """Central differences with the step H_REL * scale (with floors) and the
    rounding floor of each: 16 ulps of |lnL| over the step actually taken."""
    base = {n: np.array(v, dtype=np.float64, copy=True) for n, v in prm.items()}
    lnl = np.abs(lnl_of(m, obs, base))
    cols, floors = [], []
    for name, idx in param_vector(prm):
        x = base[name][idx] if idx else base[name]
        h = scale * H_REL * np.maximum(np.abs(x), FLOORS[name])
        up = {n: v.copy() for n, v in base.items()}
        dn = {n: v.copy() for n, v in base.items()}
        if idx:
            up[name][idx], dn[name][idx] = x + h, x - h
            step = up[name][idx] - dn[name][idx]
        else:
            up[name], dn[name] = x + h, x - h
            step = up[name] - dn[name]
        cols.append((lnl_of(m, obs, up) - lnl_of(m, obs, dn)) / step)
        floors.append(16 * np.finfo(np.float64).eps * lnl / step)
    return np.stack(cols, -1), np.stack(floors, -1)


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_gradient_elementwise_vs_finite_differences(precision):
    """Every element against central FD of the FP64 model, relative to itself:
    |g - fd| <= 1e-4 |fd| + floor.  The floor is the FD's own uncertainty:
    its rounding (16 ulps of |lnL| over the step) and its truncation, which
    is large where a step crosses a kink of the piecewise-linear LD tables,
    estimated as |FD(2h) - FD(h)|.  The split path is held to that for 90 %
    of the elements and, for all, to a stated floor of 5e-5 of the column's
    largest |fd| (its FP32 per-sample arithmetic)."""
    data, obs, pert, _ = c3_case()
    m64 = model(**data)
    # steps of 1e-8 and 5e-9 relative: far fewer of the samples' LD-table
    # kinks fall within the step than with 1e-6, while the rounding floor of
    # the FP64 log-likelihood stays well below the gradients
    fd1, _ = fd_gradient_h(m64, obs, pert, 0.01)
    fd, floor = fd_gradient_h(m64, obs, pert, 0.005)
    floor = floor + np.abs(fd1 - fd)
    _, g = lnl_of(model(precision=precision, **data), obs, pert, grad=True)
    strict = np.abs(g - fd) <= 1e-4 * np.abs(fd) + floor
    if precision == 'fp64':
        assert strict.all(), (np.argwhere(~strict), (np.abs(g - fd) / np.maximum(np.abs(fd), floor))[~strict])
    else:
        # FP32 per-sample arithmetic: each term carries ~1e-6 relative error,
        # so an element that is a small remainder of large cancelling terms
        # (ingress against egress) is exact only to a few 1e-5 of its
        # column's scale; elements above that scale meet 1e-4 of themselves
        scale = 5e-5 * np.abs(fd).max(axis=0, keepdims=True)
        ok = np.abs(g - fd) <= 1e-4 * np.abs(fd) + floor + scale
        assert ok.all(), (np.argwhere(~ok), (np.abs(g - fd) / np.maximum(np.abs(fd), floor))[~ok])
        assert strict.mean() > 0.9
    # most elements are well above their floor, so the check has teeth
    assert (np.abs(fd) > 100 * floor).mean() > 0.8


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_lnlike_and_gradient_are_reproducible(precision):
    """Sums in a fixed order (no floating-point atomics): a repeated call
    returns the same bits."""
    data, obs, pert, _ = c3_case(npv=8, npt=6000)
    m = model(precision=precision, **data)
    l1, g1 = lnl_of(m, obs, pert, grad=True)
    l2, g2 = lnl_of(m, obs, pert, grad=True)
    l3 = lnl_of(m, obs, pert)
    assert np.array_equal(l1, l2) and np.array_equal(g1, g2)
    np.testing.assert_allclose(l3, l1, rtol=1e-12)


def test_light_curves_interleaved_point_by_point():
    """Light curves whose points alternate (every thread's points change light
    curve): the per-light-curve gradient columns still match FD."""
    rng = np.random.default_rng(23)
    T = 2459000.0
    npt = 3000
    time = T + np.linspace(-0.2, 0.2, npt)
    lcids = np.arange(npt) % 3
    data = dict(time=time, lcids=lcids, pbids=[0, 1, 2], nsamples=[1, 3, 2], exptimes=[0.0, 0.01, 0.02])
    npv = 3
    prm = dict(k=rng.uniform(0.09, 0.11, (npv, 3)), ldc=rng.uniform(0.1, 0.4, (npv, 3, 2)),
               t0=T + rng.normal(0, 1e-3, (npv, 1)), p=np.full(npv, 3.0), a=rng.uniform(7, 9, npv),
               i=np.arccos(rng.uniform(0, 0.5, npv) / 8), e=rng.uniform(0.02, 0.1, npv),
               w=rng.uniform(0, 2 * np.pi, npv))
    ref = oracle.OracleRoadRunner('quadratic')
    ref.set_data(**data)
    flux = ref.evaluate(prm['k'], prm['ldc'], prm['t0'], prm['p'], prm['a'], prm['i'], prm['e'], prm['w'])
    obs = flux[0] + rng.normal(0, SIGMA, npt)
    for precision, rtol in (('fp64', 1e-9), ('split', 1e-6)):
        m = model(precision=precision, **data)
        lnl, g = lnl_of(m, obs, prm, grad=True)
        np.testing.assert_allclose(lnl, oracle.lnlike_normal(obs, flux, SIGMA), rtol=rtol)
    m = model(**data)
    _, g = lnl_of(m, obs, prm, grad=True)
    base = {n: np.array(v, dtype=np.float64, copy=True) for n, v in prm.items()}
    cols = []
    spec = [('k', (slice(None), b)) for b in range(3)] + [('t0', (slice(None), 0))] + \
           [(n, ()) for n in ('p', 'a', 'i', 'e', 'w')] + [('ldc', (slice(None), b, j)) for b in range(3) for j in range(2)]
    for name, idx in spec:
        x = base[name][idx] if idx else base[name]
        h = np.full_like(x, 1e-7) if name == 't0' else H_REL * np.maximum(np.abs(x), FLOORS[name])
        up = {n: v.copy() for n, v in base.items()}
        dn = {n: v.copy() for n, v in base.items()}
        if idx:
            up[name][idx], dn[name][idx] = x + h, x - h
            step = up[name][idx] - dn[name][idx]
        else:
            up[name], dn[name] = x + h, x - h
            step = up[name] - dn[name]
        cols.append((lnl_of(m, obs, up) - lnl_of(m, obs, dn)) / step)
    fd = np.stack(cols, -1)
    assert rel_err(g, fd).max() < 1e-4, rel_err(g, fd).max(axis=0)

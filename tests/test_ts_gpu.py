"""Transmission-spectroscopy model on the GPU vs the reference's own code
(golden fixture) and the oracle's restatement of tsmodel_serial.

Tolerances: FP64 path 1e-9, split path 1e-6 (max |dF|); NaN rows match."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = {'fp64': 1e-9, 'split': 1e-6}


def ts(precision, interp=False, law='quadratic'):
    from pytransit_gb300 import TransmissionSpectroscopyModel
    return TransmissionSpectroscopyModel(law, precision=precision, precompute_weights=interp)


def max_err(got, want):
    assert got.shape == want.shape
    assert np.array_equal(np.isnan(got), np.isnan(want))
    m = ~np.isnan(want)
    return float(np.abs(got[m] - want[m]).max()) if m.any() else 0.0


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("variant", ["2d", "3d"])
def test_ts_golden(golden, precision, variant):
    g = golden("ts")
    m = ts(precision, interp=(variant == "3d"))
    m.set_data(g["time"], nsamples=[3], exptimes=[0.01])
    flux = m.evaluate(g["k"], g["ldc"], g["t0"], g["p"], g["a"], g["inc"], g["e"], g["w"])
    assert max_err(flux, g[f"flux__{variant}"]) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_ts_200_channels_vs_oracle(precision):
    """200 channels, k ~ U(0.09, 0.11), 10 supersamples, BJD-scale times,
    eccentric orbits, plus an invalid parameter vector (NaN row)."""
    rng = np.random.default_rng(31)
    T = 2459000.0
    time = T + np.linspace(-0.25, 0.25, 900)
    npv, npb = 6, 200
    k = rng.uniform(0.09, 0.11, (npv, npb))
    ldc = np.stack([rng.uniform(0.2, 0.5, (npv, npb)), rng.uniform(0.1, 0.3, (npv, npb))], -1)
    t0 = T + rng.normal(0, 1e-3, npv)
    p = rng.uniform(1, 5, npv)
    a = rng.uniform(4, 12, npv)
    inc = np.arccos(rng.uniform(0, 0.8, npv) / a)
    e = rng.uniform(0, 0.2, npv)
    w = rng.uniform(0, 2 * np.pi, npv)
    a[3] = 0.5
    ref = oracle.OracleRoadRunner('quadratic', ts=True)
    ref.set_data(time, nsamples=[10], exptimes=[1 / 48])
    want = ref.evaluate(k, ldc, t0, p, a, inc, e, w)
    m = ts(precision)
    m.set_data(time, nsamples=[10], exptimes=[1 / 48])
    got = m.evaluate(k, ldc, t0, p, a, inc, e, w)
    assert np.isnan(got[3]).all()
    assert np.sum(want[~np.isnan(want)] < 1) > 10000
    assert max_err(got, want) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_ts_many_samples_chunked(precision):
    """More than 32 supersamples: the sample loop runs in chunks of 32."""
    rng = np.random.default_rng(2)
    time = np.linspace(-0.15, 0.15, 300)
    npv, npb = 3, 40
    k = rng.uniform(0.09, 0.11, (npv, npb))
    ldc = np.tile([0.4, 0.2], (npv, npb, 1))
    args = (k, ldc, np.zeros(npv), np.full(npv, 2.5), np.full(npv, 7.0), np.full(npv, np.arccos(0.3 / 7)),
            np.zeros(npv), np.zeros(npv))
    ref = oracle.OracleRoadRunner('quadratic', ts=True)
    ref.set_data(time, nsamples=[45], exptimes=[0.03])
    m = ts(precision)
    m.set_data(time, nsamples=[45], exptimes=[0.03])
    assert max_err(m.evaluate(*args), ref.evaluate(*args)) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("ns,exptime", [(1, 0.0), (4, 2 / 1440), (10, 2 / 1440)])
def test_ts_short_exposures_vs_oracle(precision, ns, exptime):
    """Short exposures: each in-box point's samples fall on a few LD-table rows
    (one point per lane), with slow and fast orbits mixed so that some points
    span many rows (the warp-per-point path) in the same tiles."""
    rng = np.random.default_rng(7 + ns)
    T = 2459000.0
    time = T + np.arange(2000) * (2 / 1440)
    npv, npb = 24, 37
    k = rng.uniform(0.09, 0.11, (npv, npb))
    ldc = np.stack([rng.uniform(0.2, 0.5, (npv, npb)), rng.uniform(0.1, 0.3, (npv, npb))], -1)
    t0 = T + 0.3 + rng.normal(0, 1e-3, npv)
    p = np.where(np.arange(npv) % 3 == 0, rng.uniform(0.5, 0.8, npv), rng.uniform(1, 10, npv))
    a = np.where(np.arange(npv) % 3 == 0, rng.uniform(15, 20, npv), rng.uniform(3, 12, npv))
    inc = np.arccos(rng.uniform(0, 0.9, npv) / a)
    e, w = np.zeros(npv), np.zeros(npv)
    ref = oracle.OracleRoadRunner('quadratic', ts=True)
    ref.set_data(time, nsamples=[ns], exptimes=[exptime])
    want = ref.evaluate(k, ldc, t0, p, a, inc, e, w)
    m = ts(precision)
    m.set_data(time, nsamples=[ns], exptimes=[exptime])
    got = m.evaluate(k, ldc, t0, p, a, inc, e, w)
    assert np.sum(want < 1) > 20000
    assert max_err(got, want) <= TOL[precision]


def _quad(mu, pv):
    return 1.0 - pv[0] * (1.0 - mu) - pv[1] * (1.0 - mu) ** 2


def _quad_int(pv):
    return 2 * np.pi / 12 * (-2 * pv[0] - pv[1] + 6)


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("law", ["power-2", "nonlinear", "callable", "callable+integral"])
def test_ts_laws_vs_oracle(precision, law):
    """The prologue's LD paths: a named law with an analytic disk integral
    (power-2), one integrated numerically on the device (nonlinear), and a
    user callable evaluated on the host with or without its integral (the
    profiles and integrals then come from the host, as in the serving loop)."""
    from pytransit_gb300 import TransmissionSpectroscopyModel
    rng = np.random.default_rng(11)
    T = 2459000.0
    time = T + np.linspace(-0.2, 0.2, 1500)
    npv, npb = 5, 150
    k = rng.uniform(0.09, 0.11, (npv, npb))
    if law == "power-2":
        ldc = np.stack([rng.uniform(.3, .9, (npv, npb)), rng.uniform(.3, .8, (npv, npb))], -1)
    elif law == "nonlinear":
        ldc = np.tile([0.5, -0.2, 0.6, -0.25], (npv, npb, 1)) * rng.uniform(0.8, 1.2, (npv, npb, 1))
    else:
        ldc = np.stack([rng.uniform(0.2, 0.5, (npv, npb)), rng.uniform(0.1, 0.3, (npv, npb))], -1)
    ldm = {"callable": _quad, "callable+integral": (_quad, _quad_int)}.get(law, law)
    t0 = T + rng.normal(0, 1e-3, npv)
    p = rng.uniform(1, 5, npv)
    a = rng.uniform(4, 12, npv)
    inc = np.arccos(rng.uniform(0, 0.8, npv) / a)
    e, w = rng.uniform(0, 0.2, npv), rng.uniform(0, 2 * np.pi, npv)
    ref = oracle.OracleRoadRunner(ldm, ts=True)
    ref.set_data(time, nsamples=[3], exptimes=[0.01])
    want = ref.evaluate(k, ldc, t0, p, a, inc, e, w)
    m = TransmissionSpectroscopyModel(ldm, precision=precision)
    m.set_data(time, nsamples=[3], exptimes=[0.01])
    got = m.evaluate(k, ldc, t0, p, a, inc, e, w)
    assert np.sum(want < 1) > 5000
    assert max_err(got, want) <= TOL[precision]


@pytest.mark.parametrize("ns,exptime", [(1, 0.0), (5, 0.02)])
def test_ts_fp64_culled_equals_plain(ns, exptime):
    """The tile-culled FP64 TS flux (the default with a named law) and the
    plain one (every point through the reference's fold) give the same bits:
    a 30-day light curve at 2-min cadence, periods from 0.5 d (tiles spanning
    several epochs) to 15 d, eccentric orbits, supersampling, an invalid
    vector; and both match the oracle."""
    rng = np.random.default_rng(41 + ns)
    T = 2459000.0
    time = T + np.arange(21_600) * (2.0 / 1440.0)
    npv, npb = 12, 24
    k = rng.uniform(0.09, 0.11, (npv, npb))
    ldc = np.stack([rng.uniform(0.2, 0.5, (npv, npb)), rng.uniform(0.1, 0.3, (npv, npb))], -1)
    t0 = T + 3.0 + rng.normal(0, 1e-3, npv)
    p = rng.uniform(0.5, 15, npv)
    a = rng.uniform(3, 20, npv)
    inc = np.arccos(rng.uniform(0, 0.9, npv) / a)
    e = rng.uniform(0, 0.3, npv)
    w = rng.uniform(0, 2 * np.pi, npv)
    a[7] = 0.5
    m = ts('fp64')
    m.set_data(time, nsamples=[ns], exptimes=[exptime])
    m.fp64_cull = False
    plain = m.evaluate(k, ldc, t0, p, a, inc, e, w, copy=False).cpu().numpy()
    m.fp64_cull = True
    culled = m.evaluate(k, ldc, t0, p, a, inc, e, w, copy=False).cpu().numpy()
    np.testing.assert_array_equal(culled, plain)
    assert np.isnan(culled[7]).all() and (culled < 1).any()
    ref = oracle.OracleRoadRunner('quadratic', ts=True)
    ref.set_data(time, nsamples=[ns], exptimes=[exptime])
    want = ref.evaluate(k[:4], ldc[:4], t0[:4], p[:4], a[:4], inc[:4], e[:4], w[:4])
    assert max_err(culled[:4, :, :time.size], want) <= TOL['fp64']

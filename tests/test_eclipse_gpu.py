"""Secondary-eclipse models on the GPU (rr_eclipse_f64, rr_es_f64) against the
reference's own eclipse_model / esmodel (golden fixtures, on the restated
orbit layer) and the oracle, FP64 tolerance 1e-9; the reference test's
properties (tests/test_roadrunner_eclipse.py)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
TOL = 1e-9


def _err(got, want):
    assert got.shape == want.shape
    assert np.array_equal(np.isnan(got), np.isnan(want))
    m = ~np.isnan(want)
    return float(np.abs(got[m] - want[m]).max())


def test_eclipse_reference_test_properties(golden):
    from pytransit_gb300 import EclipseModel
    g = golden("eclipse")
    times = g["canon_time"]
    m = EclipseModel()
    m.set_data(times)
    f = m.evaluate(0.1, 0.0, 2.0, 8.0, np.pi / 2)
    assert f.shape == times.shape
    assert _err(f, g["canon_flux"][0]) <= TOL
    assert abs(f.max() - np.pi * 0.01) < 1e-6
    assert f[np.argmin(np.abs(times - 1.0))] < np.pi * 0.01 - 1e-4
    assert f.min() < 1e-3


def test_eclipse_multi_lc_matches_reference(golden):
    from pytransit_gb300 import EclipseModel
    g = golden("eclipse")
    m = EclipseModel()
    m.set_data(g["time"], lcids=g["lcids"], nsamples=g["nsamples"], exptimes=g["exptimes"], epids=g["epids"])
    f = m.evaluate(g["k"], g["t0"], g["p"], g["a"], g["inc"], g["e"], g["w"], rstar=float(g["rstar"]))
    assert _err(f, g["flux"]) <= TOL
    assert np.isnan(f[5]).all()


def test_es_model_matches_reference(golden):
    from pytransit_gb300 import ESModel
    g = golden("eclipse")
    m = ESModel()
    m.set_data(g["es_time"], nsamples=[3], exptimes=[0.01])
    f = m.evaluate(g["es_fratio"], g["es_k"], g["es_t0"], g["es_p"], g["es_a"], g["es_inc"], g["es_e"], g["es_w"],
                   rstar=g["es_rstar"])
    assert _err(f, g["es_flux"]) <= TOL


def test_eclipse_many_pv_vs_oracle():
    """Larger population at BJD scale, eccentric, supersampled, vs the oracle."""
    from pytransit_gb300 import EclipseModel
    rng = np.random.default_rng(8)
    T = 2459000.0
    time = T + np.arange(0, 12.0, 5 / 1440)
    npv = 200
    k = rng.uniform(0.05, 0.15, npv)
    t0 = T + rng.normal(0.3, 1e-3, (npv, 1))
    p = rng.uniform(0.8, 6.0, npv)
    a = rng.uniform(3, 15, npv)
    inc = np.arccos(rng.uniform(0, 0.9, npv) / a)
    e = rng.uniform(0, 0.4, npv)
    w = rng.uniform(0, 2 * np.pi, npv)
    m = EclipseModel()
    m.set_data(time, nsamples=[4], exptimes=[5 / 1440])
    f = m.evaluate(k, t0, p, a, inc, e, w, rstar=0.9)
    want = oracle.eclipse_full(time, k, t0, p, a, inc, e, w, 0.9, np.zeros(time.size, int), [0], [4], [5 / 1440])
    assert np.sum(want < np.pi * k[:, None] ** 2 - 1e-9) > 10000
    assert _err(f, want) <= TOL

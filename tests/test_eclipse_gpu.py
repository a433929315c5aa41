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


# ---- split precision (rr_eclipse_split, rr_es_split) -------------------------
# FP32 per-sample areas on FP32 Taylor coefficients: |dF| <= 2k |dz| + a few
# ulps of pi k^2 with |dz| ~ 1e-7, so well inside the transit model's 1e-6
SPLIT_TOL = 1e-6


def test_eclipse_split_golden_and_invalid_rows(golden):
    """Multiple light curves, epochs and supersampling, one invalid pv."""
    import torch
    from pytransit_gb300 import EclipseModel
    g = golden("eclipse")
    m = EclipseModel(precision='split')
    m.set_data(g["time"], lcids=g["lcids"], nsamples=g["nsamples"], exptimes=g["exptimes"], epids=g["epids"])
    f = m.evaluate(g["k"], g["t0"], g["p"], g["a"], g["inc"], g["e"], g["w"], rstar=float(g["rstar"]))
    assert f.dtype == np.float64
    assert _err(f, g["flux"]) <= SPLIT_TOL
    assert np.isnan(f[5]).all()
    t = m.evaluate(g["k"], g["t0"], g["p"], g["a"], g["inc"], g["e"], g["w"], rstar=float(g["rstar"]), copy=False)
    assert t.dtype == torch.float32 and t.is_cuda


@pytest.mark.parametrize("klo,khi", [(0.05, 0.2), (0.25, 0.6)])
def test_eclipse_split_many_pv_vs_oracle_and_fp64(klo, khi):
    """BJD-scale times (the exact FP32-pair fold), eccentric orbits, 4
    samples: split against the oracle and against the FP64 kernel.  Radius
    ratios up to 1/4 take the one-arctangent limb area and one fold per
    tile, larger ones the general lens form and a fold per point."""
    from pytransit_gb300 import EclipseModel
    rng = np.random.default_rng(18)
    T = 2459000.0
    time = T + np.arange(0, 12.0, 5 / 1440)
    npv = 300
    k = rng.uniform(klo, khi, npv)
    t0 = T + rng.normal(0.3, 1e-3, (npv, 1))
    p = rng.uniform(0.8, 6.0, npv)
    a = rng.uniform(3, 15, npv)
    inc = np.arccos(rng.uniform(0, 0.95, npv) / a)
    e = rng.uniform(0, 0.4, npv)
    w = rng.uniform(0, 2 * np.pi, npv)
    want = oracle.eclipse_full(time, k, t0, p, a, inc, e, w, 0.9, np.zeros(time.size, int), [0], [4], [5 / 1440])
    got = {}
    for prec in ("split", "fp64"):
        m = EclipseModel(precision=prec)
        m.set_data(time, nsamples=[4], exptimes=[5 / 1440])
        got[prec] = m.evaluate(k, t0, p, a, inc, e, w, rstar=0.9)
    assert np.sum(want < np.pi * k[:, None] ** 2 - 1e-6) > 20000
    assert _err(got["fp64"], want) <= TOL
    assert _err(got["split"], want) <= SPLIT_TOL
    assert _err(got["split"], got["fp64"]) <= SPLIT_TOL


def test_eclipse_split_full_size_vs_fp64():
    """The full population of the 8192 pv x 19,700-time workload (4 light
    curves at 2-min cadence from BJD 2459000, k ~ U(0.05, 0.15), p ~ U(0.5,
    15) d, a ~ U(3, 20), b ~ U(0, 0.9)): split against the FP64 kernel on
    the device, 161 M points.  Every split value is finite, and the largest
    difference is within the split tolerance.  At this size some limb samples
    land on z = 1 + k rounded, the edge of the lens-area cases."""
    import torch
    from pytransit_gb300 import EclipseModel
    rng = np.random.default_rng(1234)
    T = 2459000.0
    npv, npt, nlc = 8192, 19700, 4
    time = T + np.arange(npt) * (2.0 / 1440.0)
    lcids = np.minimum((np.arange(npt) * nlc) // npt, nlc - 1)
    k = rng.uniform(0.05, 0.15, npv)
    t0 = T + rng.normal(0, 1e-3, (npv, 1))
    p = rng.uniform(0.5, 15.0, npv)
    a = rng.uniform(3.0, 20.0, npv)
    inc = np.arccos(rng.uniform(0.0, 0.9, npv) / a)
    out = {}
    for prec in ("split", "fp64"):
        m = EclipseModel(precision=prec)
        m.set_data(time, lcids=lcids, pbids=np.arange(nlc))
        out[prec] = m.evaluate(k, t0, p, a, inc, 0.0, 0.0, copy=False)
    assert bool(torch.isfinite(out["split"]).all()) and bool(torch.isfinite(out["fp64"]).all())
    assert float((out["split"].double() - out["fp64"]).abs().max()) <= SPLIT_TOL
    assert float((out["fp64"] < torch.as_tensor(np.pi * k[:, None] ** 2, device=out["fp64"].device) - 1e-9)
                 .double().mean()) > 0.01


def test_es_split_golden_and_vs_oracle(golden):
    from pytransit_gb300 import ESModel
    g = golden("eclipse")
    m = ESModel(precision='split')
    m.set_data(g["es_time"], nsamples=[3], exptimes=[0.01])
    f = m.evaluate(g["es_fratio"], g["es_k"], g["es_t0"], g["es_p"], g["es_a"], g["es_inc"], g["es_e"], g["es_w"],
                   rstar=g["es_rstar"])
    assert _err(f, g["es_flux"]) <= SPLIT_TOL
    # a larger population at BJD scale, 40 channels
    rng = np.random.default_rng(19)
    T = 2459000.0
    time = T + np.arange(-0.5, 5.0, 2 / 1440)
    npv, npb = 64, 40
    k = rng.uniform(0.05, 0.15, npv)
    t0 = T + rng.normal(0.0, 1e-3, npv)
    p = rng.uniform(1.0, 4.0, npv)
    a = rng.uniform(3, 12, npv)
    inc = np.arccos(rng.uniform(0, 0.9, npv) / a)
    e = rng.uniform(0, 0.3, npv)
    w = rng.uniform(0, 2 * np.pi, npv)
    fr = rng.uniform(1e-4, 5e-3, (npv, npb))
    want = oracle.es_full(time, k, t0, p, a, inc, e, w, 1.0, fr, 5, 2 / 1440)
    m = ESModel(precision='split')
    m.set_data(time, nsamples=[5], exptimes=[2 / 1440])
    f = m.evaluate(fr, k, t0, p, a, inc, e, w)
    assert f.shape == (npv, npb, time.size)
    assert np.sum(want < 1 - 1e-6) > 10000
    assert _err(f, want) <= SPLIT_TOL


@pytest.mark.parametrize("ns", [1, 6])
def test_eclipse_fp64_culled_equals_plain(ns):
    """The tile-culled FP64 eclipse flux (EclipseModel's default) and the plain
    kernel (every point through the reference's fold) give the same bits:
    three light curves with their own epochs and exposure times, BJD-scale
    times, periods from 0.5 d to 15 d, eccentric orbits, an invalid vector;
    and the culled one matches the oracle."""
    from pytransit_gb300 import EclipseModel
    rng = np.random.default_rng(50 + ns)
    T = 2459000.0
    nlc, per = 3, 3001
    time = np.concatenate([T + 25.0 * j + np.arange(per) * (4 / 1440) for j in range(nlc)])
    lcids = np.repeat(np.arange(nlc), per)
    npv = 24
    k = rng.uniform(0.05, 0.15, npv)
    t0 = T + rng.normal(0, 1e-3, (npv, nlc))
    p = rng.uniform(0.5, 15, npv)
    a = rng.uniform(3, 20, npv)
    a[4] = 0.7
    inc = np.arccos(rng.uniform(0, 0.9, npv) / np.maximum(a, 1.0))
    e = rng.uniform(0, 0.3, npv)
    w = rng.uniform(0, 2 * np.pi, npv)
    ex = [0.0, 0.01, 0.02] if ns > 1 else [0.0] * nlc
    m = EclipseModel()
    m.set_data(time, lcids=lcids, nsamples=[ns] * nlc, exptimes=ex, epids=np.arange(nlc))
    m.fp64_cull = False
    plain = m.evaluate(k, t0, p, a, inc, e, w, copy=False).cpu().numpy()
    m.fp64_cull = True
    culled = m.evaluate(k, t0, p, a, inc, e, w, copy=False).cpu().numpy()
    np.testing.assert_array_equal(culled, plain)
    assert np.isnan(culled[4]).all() and (culled[0] < np.pi * k[0] ** 2).any()
    want = oracle.eclipse_full(time, k, t0, p, a, inc, e, w, 1.0, lcids, np.arange(nlc), [ns] * nlc, ex)
    assert _err(culled, want) <= TOL

"""The independent cross-check: the Mandel & Agol quadratic model on the GPU.

* the GPU evaluator against the reference's eval_quad_z_s (golden fixture
  from the reference's own code) and the reference tests' pins, <= 1e-12;
* RoadRunner (FP64 GPU path) against Mandel & Agol on the same orbit layer:
  the difference is RoadRunner's discretisation (weight tables at nk = 256,
  ng = 100, a 40-point radial grid), reported and bounded here at 1e-4."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_ma_z_matches_reference(golden):
    from pytransit_gb300.crosscheck import ma_quadratic_z
    g = golden("ma_quadratic")
    for ik, k in enumerate(g["ks"]):
        for iu, u in enumerate(g["us"]):
            ok = g["ok"][ik, iu]
            got = ma_quadratic_z(g["z"][ik], k, *u)
            want = g["flux"][ik, iu]
            assert np.array_equal(np.isnan(got[ok]), np.isnan(want[ok])), (k, u)
            m = ok & ~np.isnan(want)
            assert np.abs(got[m] - want[m]).max() <= 1e-12, (k, u)
            # the points the pure-Python reference cannot evaluate: as the oracle
            np.testing.assert_allclose(got[~ok], oracle.ma_quad_z(g["z"][ik][~ok], k, *u), rtol=0, atol=1e-12)


def test_ma_z_reference_pins():
    from pytransit_gb300.crosscheck import ma_quadratic_z
    K = 0.1
    z = np.array([-2.0, 2.0, 0.2, -0.0, 0.0, K, 1 - K, 1.0, 1 + K])
    want = [1.0, 1.0, 0.98914137, 1.0, 0.98909638, 0.98910745, 0.99164875, 0.99573423, 1.0]
    np.testing.assert_almost_equal(ma_quadratic_z(z, K, 0.2, 0.1), want)


@pytest.mark.parametrize("ns,exptime", [(1, 0.0), (5, 0.02)])
def test_roadrunner_vs_mandel_agol(ns, exptime):
    """C0-like parameter vectors at BJD scale over several transits."""
    from pytransit_gb300 import RoadRunnerModel
    from pytransit_gb300.crosscheck import rr_vs_ma
    rng = np.random.default_rng(41 + ns)
    T = 2459000.0
    time = T + np.linspace(-0.2, 6.0, 6000)
    npv = 64
    k = rng.uniform(0.05, 0.15, (npv, 1))
    ldc = np.stack([rng.uniform(0, 0.6, npv), rng.uniform(0, 0.3, npv)], -1).reshape(npv, 1, 2)
    a = rng.uniform(3, 20, npv)
    args = (k, ldc, T + rng.normal(0, 1e-3, (npv, 1)), rng.uniform(1, 10, npv), a,
            np.arccos(rng.uniform(0, 0.9, npv) / a), np.zeros(npv), np.zeros(npv))
    m = RoadRunnerModel('quadratic')
    m.set_data(time, nsamples=[ns], exptimes=[exptime])
    f_rr, f_ma = rr_vs_ma(m, *args)
    assert np.sum(f_ma < 1) > 5000
    d = np.abs(f_rr - f_ma).max()
    print(f"max |F_RR - F_MA| = {d:.2e}")
    assert d < 1e-4

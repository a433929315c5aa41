"""Sampler populations on the device: BaseLPF.transit_model's parameter mapping
(rr_lpf_map) against the reference's own as_from_rhop / i_from_ba / map_ldc
(golden fixture), and the model / fused log-likelihood of a device population
against the same computed from host parameters."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(got, want, rtol):
    assert np.array_equal(np.isnan(got), np.isnan(want))
    m = ~np.isnan(want)
    np.testing.assert_allclose(got[m], want[m], rtol=rtol, atol=0)


def test_lpf_map_matches_reference(golden):
    import torch
    from pytransit_gb300.lpf import map_pv
    g = golden("lpf_map")
    pv = torch.as_tensor(g["pv"]).cuda()
    m = {n: t.cpu().numpy() for n, t in map_pv(pv, float(g["tref"]), int(g["npb"])).items()}
    _close(m["k"], g["k"], 1e-15)
    _close(m["t0"].ravel(), g["t0"], 1e-15)
    _close(m["p"], g["p"], 0)
    _close(m["a"], g["a"], 1e-13)
    _close(m["i"], g["inc"], 1e-13)
    _close(m["ldc"], g["ldc"], 1e-15)


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_population_model_and_lnlike(precision):
    import torch
    from pytransit_gb300 import RoadRunnerModel
    from pytransit_gb300 import lpf
    from pytransit_gb300.lnlike import lnlikelihood
    rng = np.random.default_rng(5)
    tref = 2459000.0
    time = np.linspace(-0.2, 5.0, 3000)          # data times relative to tref, as BaseLPF sets them
    npv, npb = 96, 2
    lcids = (time > 2.4).astype(int)
    pv = np.column_stack([tref + rng.normal(0.0, 0.002, npv), rng.uniform(1.5, 3.0, npv), rng.uniform(1.0, 3.0, npv),
                          rng.uniform(0, 0.8, npv), rng.uniform(0.006, 0.015, npv)] +
                         [rng.uniform(0.2, 0.8, npv) for _ in range(2 * npb)])
    m = RoadRunnerModel('quadratic', precision=precision)
    m.set_data(time, lcids=lcids, pbids=[0, 1])
    pvt = torch.as_tensor(pv).cuda()
    dev = {n: t.cpu().numpy() for n, t in lpf.map_pv(pvt, tref, npb).items()}
    want = m.evaluate(dev["k"], dev["ldc"], dev["t0"], dev["p"], dev["a"], dev["i"], 0.0, 0.0, copy=False)
    got = lpf.transit_model(m, pvt, tref)
    assert torch.equal(got, want)
    obs = want[0].double().cpu().numpy() + rng.normal(0, 5e-4, time.size)
    l_dev = lpf.lnlikelihood(m, obs, 5e-4, pvt, tref).cpu().numpy()
    l_host = lnlikelihood(m, obs, 5e-4, dev["k"], dev["ldc"], dev["t0"], dev["p"], dev["a"], dev["i"])
    np.testing.assert_allclose(l_dev, l_host, rtol=1e-12)

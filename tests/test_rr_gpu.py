"""GPU parity of the RoadRunner path (plain FP64 and split precision) against
the golden fixtures made by the reference's own code and against the oracle.

Tolerances (max |dF|, absolute flux):
  * FP64 path vs reference / oracle: 1e-9
  * split path vs reference / oracle / FP64 path: 1e-6
NaN rows and points must match exactly.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = {'fp64': 1e-9, 'split': 1e-6}


def rr(law='quadratic', precision='fp64', **kw):
    from pytransit_gb300 import RoadRunnerModel
    return RoadRunnerModel(law, precision=precision, **kw)


def max_err(got, want):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    assert got.shape == want.shape, (got.shape, want.shape)
    assert np.array_equal(np.isnan(got), np.isnan(want)), "NaN pattern differs"
    m = ~np.isnan(want)
    return float(np.abs(got[m] - want[m]).max()) if m.any() else 0.0


def pv_args(g):
    return g["k"], g["ldc"], g["t0"], g["p"], g["a"], g["inc"], g["e"], g["w"]


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_golden_c0(golden, precision):
    g = golden("c0_quadratic")
    m = rr(precision=precision)
    m.set_data(g["time"])
    assert max_err(m.evaluate(*pv_args(g)), g["flux"]) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_golden_multi_lc_bjd(golden, precision):
    g = golden("multi_lc_bjd")
    m = rr(precision=precision)
    m.set_data(g["time"], lcids=g["lcids"], pbids=g["pbids"], nsamples=g["nsamples"],
               exptimes=g["exptimes"], epids=g["epids"])
    assert max_err(m.evaluate(*pv_args(g)), g["flux"]) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_golden_power2_supersampled(golden, precision):
    g = golden("power2_ss10")
    m = rr('power-2', precision=precision)
    m.set_data(g["time"], lcids=g["lcids"], pbids=g["pbids"], nsamples=g["nsamples"], exptimes=g["exptimes"])
    assert max_err(m.evaluate(*pv_args(g)), g["flux"]) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("law", list(oracle.LD_LAWS))
def test_golden_ld_laws(golden, law, precision):
    g = golden("ld_laws")
    m = rr(law, precision=precision)
    m.set_data(g["time"])
    flux = m.evaluate(g["k"], g[f"ldc__{law}"], g["t0"], g["p"], g["a"], g["inc"], g["e"], g["w"])
    assert max_err(flux, g[f"flux__{law}"]) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_golden_user_ld(golden, precision):
    from pytransit_gb300 import LDModel, ldmodels

    g = golden("user_ld")

    class QuadLD(LDModel):
        def _evaluate(self, mu, x):
            x = np.asarray(x)
            return 1.0 - x[..., 0:1] * (1.0 - mu) - x[..., 1:2] * (1.0 - mu) ** 2

        def _integrate(self, x):
            x = np.asarray(x)
            return 2 * np.pi / 12 * (-2 * x[..., 0] - x[..., 1] + 6)

    def user_law(mu, pv):
        return 1.0 - pv[0] * (1.0 - mu) - pv[1] * (1.0 - np.sqrt(mu))

    for name, model in [("ldmodel", QuadLD()), ("callable", user_law),
                        ("tuple", (ldmodels.ld_quadratic, ldmodels.ldi_quadratic))]:
        m = rr(model, precision=precision)
        m.set_data(g["time"])
        assert max_err(m.evaluate(*pv_args(g)), g[f"flux__{name}"]) <= TOL[precision], name


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_golden_klims(golden, precision):
    g = golden("klims")
    m = rr(precision=precision)
    m.set_data(g["time"])
    assert max_err(m.evaluate(*pv_args(g)), g["flux"]) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_golden_simple(golden, precision):
    g = golden("simple")
    m = rr(precision=precision)
    m.set_data(g["time"], nsamples=[4], exptimes=[0.01])
    flux = m.evaluate(float(g["k"]), g["ldc"], float(g["t0"]), float(g["p"]), float(g["a"]),
                      float(g["inc"]), float(g["e"]), float(g["w"]))
    assert flux.shape == g["flux"].shape
    assert max_err(flux, g["flux"]) <= TOL[precision]


def c1_like(rng, npv, npt, nlc=4, T=2459000.0, cadence=2 / 1440, ns=1, exptime=0.0, ecc=False,
            p_range=(0.5, 15.0)):
    """Contiguous light curves (one passband each) at BJD scale."""
    time = T + np.arange(npt) * cadence
    lcids = np.minimum((np.arange(npt) * nlc) // npt, nlc - 1)
    k = rng.uniform(0.05, 0.15, (npv, 1))
    ldc = np.stack([rng.uniform(0, .6, (npv, nlc)), rng.uniform(0, .3, (npv, nlc))], -1)
    t0 = T + rng.normal(0, 1e-3, (npv, 1))
    p = rng.uniform(*p_range, npv)
    a = rng.uniform(3, 20, npv)
    inc = np.arccos(rng.uniform(0, .9, npv) / a)
    e = rng.uniform(0, .3, npv) if ecc else np.zeros(npv)
    w = rng.uniform(0, 2 * np.pi, npv) if ecc else np.zeros(npv)
    data = dict(time=time, lcids=lcids, pbids=np.arange(nlc), nsamples=np.full(nlc, ns),
                exptimes=np.full(nlc, exptime))
    return data, (k, ldc, t0, p, a, inc, e, w)


@pytest.mark.parametrize("ns,exptime,ecc", [(1, 0.0, False), (10, 1 / 48, True), (3, 0.02, True)])
def test_oracle_parity_bjd(ns, exptime, ecc):
    """FP64 and split paths vs the oracle on a 96 x 19,700 BJD-scale workload
    (2-min cadence over 27.4 d, four light curves / passbands)."""
    rng = np.random.default_rng(100 + ns)
    data, args = c1_like(rng, 96, 19700, ns=ns, exptime=exptime, ecc=ecc)
    ref = oracle.OracleRoadRunner('quadratic')
    ref.set_data(**data)
    want = ref.evaluate(*args)
    for precision in ("fp64", "split"):
        m = rr(precision=precision)
        m.set_data(**data)
        err = max_err(m.evaluate(*args), want)
        assert err <= TOL[precision], (precision, err)


def test_split_vs_fp64_long_baseline():
    """Split vs FP64 over a 1000-day baseline at 30-min cadence with 10
    supersamples, power-2 LD, eccentric orbits (the precision workload's
    shape), and both against the oracle on a seeded 64-pv subset."""
    rng = np.random.default_rng(7)
    npv = 512
    npts = np.exp(rng.uniform(np.log(500), np.log(50000), 16)).astype(int)
    time = np.concatenate([2459000.0 + np.arange(n) / 48.0 for n in npts])
    lcids = np.concatenate([np.full(n, j) for j, n in enumerate(npts)])
    data = dict(time=time, lcids=lcids, pbids=np.arange(16) % 4, nsamples=np.full(16, 10),
                exptimes=np.full(16, 1 / 48))
    k = rng.uniform(0.05, 0.15, (npv, 1))
    ldc = np.stack([rng.uniform(.3, .9, (npv, 4)), rng.uniform(.3, .8, (npv, 4))], -1)
    t0 = 2459000.0 + rng.normal(0, 1e-3, (npv, 1))
    p = rng.uniform(0.5, 15, npv)
    a = rng.uniform(3, 20, npv)
    inc = np.arccos(rng.uniform(0, .9, npv) / a)
    e = rng.uniform(0, .3, npv)
    w = rng.uniform(0, 2 * np.pi, npv)
    out = {}
    for precision in ("fp64", "split"):
        m = rr('power-2', precision=precision)
        m.set_data(**data)
        out[precision] = m.evaluate(k, ldc, t0, p, a, inc, e, w)
    assert max_err(out["split"], out["fp64"]) <= 1e-6
    assert np.sum(out["fp64"] < 1) > 1000   # the case does exercise in-transit points
    # a seeded subset of the population against the oracle, on all the times
    sub = np.sort(rng.choice(npv, 64, replace=False))
    ref = oracle.OracleRoadRunner('power-2')
    ref.set_data(**data)
    want = ref.evaluate(k[sub], ldc[sub], t0[sub], p[sub], a[sub], inc[sub], e[sub], w[sub])
    assert max_err(out["fp64"][sub], want) <= TOL["fp64"]
    assert max_err(out["split"][sub], want) <= TOL["split"]


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("npt", [1, 2, 5, 127, 129, 1023, 1025])
def test_ragged_sizes(precision, npt):
    rng = np.random.default_rng(npt)
    time = np.linspace(-0.1, 0.1, npt)
    npv = 3
    args = (rng.uniform(0.08, 0.12, (npv, 1)), np.tile([0.3, 0.1], (npv, 1, 1)), np.zeros((npv, 1)),
            np.full(npv, 2.0), np.full(npv, 7.0), np.full(npv, np.arccos(0.2 / 7)), np.zeros(npv),
            np.zeros(npv))
    ref = oracle.OracleRoadRunner('quadratic')
    ref.set_data(time)
    m = rr(precision=precision)
    m.set_data(time)
    assert max_err(m.evaluate(*args), ref.evaluate(*args)) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_invalid_rows_are_nan(precision):
    time = np.linspace(-0.1, 0.1, 200)
    npv = 4
    m = rr(precision=precision)
    m.set_data(time)
    a = np.array([5.0, 0.9, np.nan, 5.0])
    e = np.array([0.0, 0.0, 0.0, -0.1])
    flux = m.evaluate(np.full((npv, 1), 0.1), np.tile([0.3, 0.1], (npv, 1, 1)), np.zeros((npv, 1)),
                      np.full(npv, 2.0), a, np.full(npv, 1.55), e, np.zeros(npv))
    assert np.all(np.isfinite(flux[0]))
    assert np.all(np.isnan(flux[1:]))


def test_device_output_and_copy_false():
    import torch
    time = np.linspace(-0.1, 0.1, 100)
    m = rr(precision='split')
    m.set_data(time)
    out = m.evaluate(np.array([[0.1], [0.11]]), [0.3, 0.1], [0.0, 0.0], [2.0, 2.1], 7.0, 1.55, copy=False)
    assert isinstance(out, torch.Tensor) and out.is_cuda and out.shape == (2, 100)
    assert out.dtype == torch.float32


@pytest.mark.parametrize("precision,host_fill,fraction", [("fp64", True, 0.6), ("split", True, 0.6),
                                                            ("split", True, 0.0), ("split", True, 1.0),
                                                            ("split", False, 0.6)])
@pytest.mark.parametrize("npt", [1000, 1003])
def test_pinned_host_output(precision, host_fill, fraction, npt):
    """out= a pinned host tensor.  With host_fill, the split path copies the
    first rows over from the device while the host sets the others (a
    host_fill_fraction share) to 1, a pv chunk at a time, and the GPU writes
    only their tiles that reach a transit (and the NaN rows of invalid
    vectors) straight into them; without, every chunk is computed on the
    device and copied over while the next is computed.  Also for npt not a
    multiple of 4 and uneven chunks: the same bits as the device result, and
    a second call overwrites every element."""
    import torch
    rng = np.random.default_rng(3)
    T = 2459000.0
    time = T + np.linspace(-0.3, 0.3, npt)
    npv = 37
    a = rng.uniform(5, 9, npv)
    a[[4, 30]] = 0.9                    # invalid vectors (a <= 1): NaN rows
    args = (rng.uniform(0.08, 0.12, (npv, 1)), [0.3, 0.1], T + rng.normal(0, 1e-3, (npv, 1)),
            rng.uniform(1, 3, npv), a, np.full(npv, 1.54), 0.0, 0.0)
    m = rr(precision=precision)
    m.host_fill = host_fill
    m.host_fill_fraction = fraction
    m.set_data(time)
    want = m.evaluate(*args, copy=False).cpu()
    assert torch.isnan(want[4]).all() and torch.isnan(want[30]).all()
    dt = torch.float32 if precision == 'split' else torch.float64
    out = torch.full((npv, npt), -7.0, dtype=dt, pin_memory=True)
    got = m.evaluate(*args, out=out)
    assert got is out
    torch.testing.assert_close(out, want.to(dt), rtol=0, atol=0, equal_nan=True)
    out.fill_(-7.0)
    m.evaluate(*args, out=out)
    torch.testing.assert_close(out, want.to(dt), rtol=0, atol=0, equal_nan=True)


def test_flux_split_transits_writes_only_transit_tiles():
    """rr_flux_split_transits through the C ABI on a device buffer: where the
    buffer holds 1 it gives the same bits as rr_flux_split_range; where it
    holds a sentinel, only whole 128-point tiles are written (every point of a
    written tile, the sentinel untouched elsewhere), every point that differs
    from 1 lies in a written tile, and the NaN row of an invalid vector is
    written in full.  Pageable host memory is refused."""
    import ctypes as C
    import torch
    from pytransit_gb300 import _lib
    rng = np.random.default_rng(11)
    T = 2459000.0
    npt, npv = 19700, 64
    time = T + np.arange(npt) * (2.0 / 1440.0)
    a = rng.uniform(3, 20, npv)
    a[7] = 0.5
    args = (rng.uniform(0.05, 0.15, (npv, 1)), [0.3, 0.1], T + rng.normal(0, 1e-3, (npv, 1)),
            rng.uniform(0.5, 15, npv), a, np.arccos(rng.uniform(0, 0.9, npv) / np.maximum(a, 1)), 0.0, 0.0)
    m = rr(precision='split')
    m.set_data(time)
    full = m.evaluate(*args, copy=False)          # leaves the model's split workspace prepared
    st = m._bound_state
    dev = st['device']
    dd = m._device_data(dev)
    L, P = _lib.lib(), _lib.ptr
    sp = _lib.stream_ptr(dev)

    def transits(buf, pv0=0, pv1=npv):
        return L.rr_flux_split_transits(P(dd['times_ff']), npt, P(dd['lcids']), npv, st['nlc'], st['npb'], m.ng,
                                        m.dg, P(st['ws']), pv0, pv1, C.c_void_p(buf.data_ptr()), npt, sp)

    ones = torch.ones((npv, npt), dtype=torch.float32, device=dev)
    assert transits(ones) == 0
    torch.cuda.synchronize()
    torch.testing.assert_close(ones, full, rtol=0, atol=0, equal_nan=True)
    sentinel = -3.0
    sb = torch.full((npv, npt), sentinel, dtype=torch.float32, device=dev)
    assert transits(sb) == 0
    torch.cuda.synchronize()
    sbh, fh = sb.cpu().numpy(), full.cpu().numpy()
    ntile = (npt + 127) // 128
    pad = np.full((npv, ntile * 128), sentinel, np.float32)
    pad[:, :npt] = sbh
    real = (np.arange(ntile * 128) < npt).reshape(ntile, 128)       # the last tile is partial
    held = (pad.reshape(npv, ntile, 128) == sentinel) & real
    written = ~held.any(-1)
    assert ((held | ~real).all(-1) | written).all(), "a tile was written in part"
    fpad = np.ones((npv, ntile * 128), np.float32)
    fpad[:, :npt] = fh
    differs = ~(fpad.reshape(npv, ntile, 128) == 1.0).all(-1)
    assert not (differs & ~written).any(), "a point that differs from 1 was not written"
    w = np.repeat(written, 128, axis=1)[:, :npt]
    np.testing.assert_array_equal(sbh[w], fh[w])
    assert written[7].all() and np.isnan(sbh[7]).all()
    assert 0 < written.mean() < 0.5
    # a pv sub-range writes only its own rows
    sr = torch.full((npv, npt), sentinel, dtype=torch.float32, device=dev)
    assert L.rr_flux_split_transits(P(dd['times_ff']), npt, P(dd['lcids']), npv, st['nlc'], st['npb'], m.ng, m.dg,
                                    P(st['ws']), 10, 20, C.c_void_p(sr[10].data_ptr()), npt, sp) == 0
    torch.cuda.synchronize()
    srh = sr.cpu().numpy()
    assert (srh[:10] == sentinel).all() and (srh[20:] == sentinel).all()
    np.testing.assert_array_equal(srh[10:20], sbh[10:20])
    pageable = np.ones((npv, npt), np.float32)
    assert L.rr_flux_split_transits(P(dd['times_ff']), npt, P(dd['lcids']), npv, st['nlc'], st['npb'], m.ng,
                                    m.dg, P(st['ws']), 0, npv, C.c_void_p(pageable.ctypes.data), npt, sp) == 2


@pytest.mark.parametrize("precision,host_fill", [("fp64", True), ("split", True), ("split", False)])
@pytest.mark.parametrize("npv", [1, 37])
def test_copy_true_through_pinned_rows(precision, host_fill, npv):
    """evaluate() with copy=True (the reference's default) on an output large
    enough to go straight into pinned host rows: a float64 numpy array with
    the same bits as the device result widened, squeezed as the reference
    squeezes, NaN rows for invalid vectors; and out= a pinned float64 tensor
    likewise.  The split path's float64 rows come from the FP64-output
    kernels (rr_flux_split_range_f64 / rr_flux_split_transits_f64), the
    plain path's from rr_flux_f64_range in chunks."""
    import torch
    rng = np.random.default_rng(5 + npv)
    T = 2459000.0
    npt = 150_001 if npv == 1 else 5003
    time = T + np.linspace(-3.0, 3.0, npt)
    a = rng.uniform(5, 9, npv)
    if npv > 1:
        a[[3, 20]] = 0.9
    args = (rng.uniform(0.08, 0.12, (npv, 1)), [0.3, 0.1], T + rng.normal(0, 1e-3, (npv, 1)),
            rng.uniform(1, 3, npv), a, np.full(npv, 1.54), 0.0, 0.0)
    m = rr(precision=precision)
    m.host_fill = host_fill
    m.set_data(time)
    assert npv * npt >= m.PINNED_RESULT_MIN
    want = m.evaluate(*args, copy=False).double().cpu().numpy()
    got = m.evaluate(*args)
    assert isinstance(got, np.ndarray) and got.dtype == np.float64 and got.shape == want.shape
    np.testing.assert_array_equal(got, want)
    if npv > 1:
        assert np.isnan(got[3]).all() and np.isnan(got[20]).all() and np.isfinite(got[0]).all()
    again = m.evaluate(*args)          # a second result does not overwrite the first
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(again, want)
    out = torch.full((npv, npt), -7.0, dtype=torch.float64, pin_memory=True)
    assert m.evaluate(*args, out=out) is out
    np.testing.assert_array_equal(out.numpy().reshape(want.shape), want)
    # against the oracle, as every parity test
    ref = oracle.OracleRoadRunner('quadratic')
    ref.set_data(time)
    assert max_err(got, ref.evaluate(*args)) <= TOL[precision]


@pytest.mark.parametrize("ecc,ns", [(False, 1), (True, 7)])
def test_fp64_culled_equals_plain(ecc, ns):
    """The tile-culled FP64 flux (precision='fp64', the default) and the plain
    FP64 kernel (every point through the reference's fold) give the same bits:
    BJD-scale times in four light curves with their own epochs, exposure
    times and supersampling, periods from half a day (tiles spanning several
    epochs) to 15 d, eccentric orbits, an invalid vector, tiles shared by two
    light curves, and a time array that is not sorted within its tiles."""
    rng = np.random.default_rng(21 + ns)
    T = 2459000.0
    nlc, per = 4, 4001
    time = np.concatenate([T + 30.0 * j + np.arange(per) * (2.0 / 1440.0) for j in range(nlc)])
    lcids = np.repeat(np.arange(nlc), per)
    time[5 * per // 2: 5 * per // 2 + 300] = time[5 * per // 2: 5 * per // 2 + 300][::-1].copy()   # unsorted run
    npv = 48
    p = rng.uniform(0.5, 15, npv)
    a = rng.uniform(3, 20, npv)
    a[11] = 0.8                                                    # invalid
    e = rng.uniform(0, 0.3, npv) if ecc else np.zeros(npv)
    w = rng.uniform(0, 2 * np.pi, npv) if ecc else np.zeros(npv)
    t0 = T + rng.normal(0, 1e-3, (npv, nlc)) + np.arange(nlc) * 1e-4
    inc = np.arccos(rng.uniform(0, 0.9, npv) / np.maximum(a, 1.0))
    args = (rng.uniform(0.05, 0.15, (npv, 1)), np.tile([0.4, 0.2], (npv, nlc, 1)), t0, p, a, inc, e, w)
    m = rr(precision='fp64')
    m.set_data(time, lcids=lcids, pbids=np.arange(nlc), nsamples=[ns] * nlc,
               exptimes=[0.0, 0.02, 0.01, 0.03] if ns > 1 else [0.0] * nlc, epids=np.arange(nlc))
    m.fp64_cull = False
    plain = m.evaluate(*args, copy=False).cpu().numpy()
    m.fp64_cull = True
    culled = m.evaluate(*args, copy=False).cpu().numpy()
    np.testing.assert_array_equal(culled, plain)
    assert np.isnan(culled[11]).all() and (culled < 1.0).any()
    assert max_err(culled, oracle_eval(time, lcids, nlc, ns, args)) <= TOL['fp64']


def oracle_eval(time, lcids, nlc, ns, args):
    ref = oracle.OracleRoadRunner('quadratic')
    ref.set_data(time, lcids=lcids, pbids=np.arange(nlc), nsamples=[ns] * nlc,
                 exptimes=[0.0, 0.02, 0.01, 0.03] if ns > 1 else [0.0] * nlc, epids=np.arange(nlc))
    return ref.evaluate(*args)


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_pinned_output_multi_lc_supersampled(dtype):
    """The host-fill output path on the precision workload's shape: light
    curves of different lengths (tiles shared by two light curves go through
    the per-point path), 10 supersamples, eccentric orbits, periods down to
    0.5 d, a vector whose box nears +-p/2 (every point through the exact
    path), and an invalid one: out= pinned rows equal the device result."""
    import torch
    rng = np.random.default_rng(17)
    T = 2459000.0
    sizes = [700, 1300, 257, 2100]
    time = np.concatenate([T + 40.0 * j + np.arange(n) * (30 / 1440) for j, n in enumerate(sizes)])
    lcids = np.repeat(np.arange(len(sizes)), sizes)
    npv = 40
    p = rng.uniform(0.5, 15, npv)
    a = rng.uniform(3, 20, npv)
    p[5], a[5] = 0.25, 1.2                   # a transit window that fills most of the period
    a[9] = 0.9                               # invalid
    args = (rng.uniform(0.05, 0.15, (npv, 1)), np.stack([rng.uniform(.3, .9, (npv, 4)), rng.uniform(.3, .8, (npv, 4))], -1),
            T + rng.normal(0, 1e-3, (npv, 1)), p, a, np.arccos(rng.uniform(0, 0.9, npv) / np.maximum(a, 1.0)),
            rng.uniform(0, 0.3, npv), rng.uniform(0, 2 * np.pi, npv))
    m = rr('power-2', precision='split')
    m.set_data(time, lcids=lcids, pbids=np.arange(4), nsamples=[10] * 4, exptimes=[30 / 1440] * 4)
    want = m.evaluate(*args, copy=False).cpu()
    tdt = getattr(torch, dtype)
    out = torch.full((npv, time.size), -7.0, dtype=tdt, pin_memory=True)
    m.evaluate(*args, out=out)
    torch.testing.assert_close(out, want.to(tdt), rtol=0, atol=0, equal_nan=True)
    assert torch.isnan(out[9]).all() and (out[5] < 1).any()

"""The fused split prologue (rr_prepare_split_ld: LD profile, disk integral,
LD means and orbit records in one launch) against the two-stage path it
replaces (rr_ld_tables_f32 then rr_prepare_split), through the C ABI.

ldp, istar and the orbit / light-curve records must be bit-identical (the
same FP32 arithmetic on the same FP32 inputs); the LD means may differ in the
last bits (the k-row weight is computed with a reciprocal of dk instead of a
division), and the flux from the two workspaces agrees to 1e-7.  The cases
cover every law the fused kernel takes, laws it hands to the two-stage path,
radius ratios outside the weight tables (the FP64 2D-table branch), invalid
orbits and a NaN limb-darkening coefficient.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LAWS = [('uniform', 0), ('linear', 1), ('quadratic', 2), ('quadratic-tri', 2), ('nonlinear', 4), ('power-2', 2)]


def _coefs(law, rng, shape):
    if law == 'quadratic-tri':
        return np.stack([rng.uniform(0.1, 0.9, shape), rng.uniform(0.1, 0.9, shape)], -1)
    if law == 'power-2':
        return np.stack([rng.uniform(0.3, 0.8, shape), rng.uniform(0.4, 1.2, shape)], -1)
    n = {'uniform': 0, 'linear': 1, 'quadratic': 2, 'nonlinear': 4}[law]
    hi = {1: [0.6], 2: [0.6, 0.3], 4: [0.3, 0.3, 0.2, 0.1]}.get(n, [])
    return np.stack([rng.uniform(0, h, shape) for h in hi], -1) if n else np.zeros(shape + (1,))


@pytest.mark.parametrize("law,npar", LAWS)
def test_fused_prologue_matches_two_stage(law, npar):
    import torch
    from pytransit_gb300 import RoadRunnerModel, _lib

    rng = np.random.default_rng(5)
    npv, npt, nlc = 700, 3000, 3
    T = 2459000.0
    time = T + np.arange(npt) * (2.0 / 1440.0)
    lcids = np.minimum((np.arange(npt) * nlc) // npt, nlc - 1)
    m = RoadRunnerModel(law, precision='split')
    m.set_data(time, lcids=lcids, pbids=[0, 1, 1], nsamples=[1, 3, 2], exptimes=[0.0, 0.01, 0.004])
    npb = m.npb
    k = rng.uniform(0.05, 0.15, (npv, 1))
    k[::97] = 0.6                              # outside the weight tables: the FP64 2D-table branch
    ldc = _coefs(law, rng, (npv, npb))
    if npar:
        ldc[5, 0, 0] = np.nan                  # a NaN profile: the pv's flux is NaN
    p = rng.uniform(0.5, 5.0, npv)
    a = rng.uniform(3, 20, npv)
    a[7] = 0.8                                 # an invalid orbit
    prm = dict(k=k, t0=T + 0.3 + rng.normal(0, 1e-3, (npv, 1)), p=p, a=a,
               i=np.arccos(rng.uniform(0, 0.9, npv) / np.maximum(a, 1.0)),
               e=rng.uniform(0, 0.3, npv), w=rng.uniform(0, 2 * np.pi, npv), ldc=np.ascontiguousarray(ldc))
    dev = torch.device("cuda")
    d = {n: torch.as_tensor(np.ascontiguousarray(v)).to(dev) for n, v in prm.items()}
    dd, tb = m._device_data(dev), m._device_tables(dev)
    L, P, sp = _lib.lib(), _lib.ptr, _lib.stream_ptr(dev)
    nz, ng, nk = m.ze.size, m.ng, m.nk
    basis, nb = m._basis(dev, npar, True)
    kmin, kmax = float(m.klims[0]), float(m.klims[1])
    wsb = L.rr_full_split_workspace_bytes(npv, npb, nlc, 1, ng)

    # two stages
    ldp2 = torch.empty((npv, npb, nz), dtype=torch.float32, device=dev)
    ist2 = torch.empty((npv, npb), dtype=torch.float32, device=dev)
    ws2 = torch.zeros(wsb, dtype=torch.uint8, device=dev)
    _lib.check(L.rr_ld_tables_f32(m.ld_law, P(d["ldc"]), npv, npb, npar, P(tb["mu"]), nz, P(ldp2), P(ist2), sp))
    _lib.check(L.rr_prepare_split(dd["t_ref"], dd["t_absmax"], P(d["k"]), 1, P(d["t0"]), 1, 1, P(d["p"]),
                                  P(d["a"]), P(d["i"]), P(d["e"]), P(d["w"]), npv, nlc, npb, P(dd["pbids"]),
                                  P(dd["epids"]), P(dd["nsamples"]), P(dd["exptimes"]), P(ldp2), P(ist2),
                                  P(tb["W32"]), nk, ng, nz, m.dk, kmin, kmax, P(tb["ze"]), P(ws2), wsb, sp,
                                  m.ld_law, P(d["ldc"]), npar, P(basis), nb))
    # one launch
    ldp1 = torch.full((npv, npb, nz), -7.0, dtype=torch.float32, device=dev)
    ist1 = torch.full((npv, npb), -7.0, dtype=torch.float32, device=dev)
    ws1 = torch.zeros(wsb, dtype=torch.uint8, device=dev)
    _lib.check(L.rr_prepare_split_ld(dd["t_ref"], dd["t_absmax"], P(d["k"]), 1, P(d["t0"]), 1, 1, P(d["p"]),
                                     P(d["a"]), P(d["i"]), P(d["e"]), P(d["w"]), npv, nlc, npb, P(dd["pbids"]),
                                     P(dd["epids"]), P(dd["nsamples"]), P(dd["exptimes"]), m.ld_law, P(d["ldc"]),
                                     npar, P(tb["mu"]), nz, P(basis), nb, P(tb["W32"]), nk, ng, m.dk, kmin, kmax,
                                     P(tb["ze"]), P(ldp1), P(ist1), P(ws1), wsb, sp))
    torch.cuda.synchronize()
    assert torch.equal(ldp1.view(torch.int32), ldp2.view(torch.int32))
    assert torch.equal(ist1.view(torch.int32), ist2.view(torch.int32))
    # orbit records [npv, 16], light-curve records [npv, nlc, 16] and LD means
    # [npv, npb, ng], located in each workspace by rr_full_split_tables
    L.rr_full_split_tables.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
    L.rr_full_split_tables.restype = None
    tabs = []
    for ws in (ws1, ws2):
        q = [C.c_void_p() for _ in range(3)]
        L.rr_full_split_tables(C.c_void_p(ws.data_ptr()), npv, npb, nlc, 1, ng, *[C.byref(x) for x in q])
        off = [x.value - ws.data_ptr() for x in q]
        tabs.append([ws[o:o + n * 4].view(torch.float32) for o, n in
                     zip(off, (npv * 16, npv * nlc * 16, npv * npb * ng))])
    (orb1, lc1, m1), (orb2, lc2, m2) = tabs
    assert torch.equal(orb1.view(torch.int32), orb2.view(torch.int32))
    assert torch.equal(lc1.view(torch.int32), lc2.view(torch.int32))
    assert torch.allclose(m1, m2, rtol=1e-6, atol=1e-7, equal_nan=True), float((m1 - m2).abs().nan_to_num().max())
    # flux from the two workspaces
    ldf = (npt + 3) // 4 * 4
    f1 = torch.empty((npv, ldf), dtype=torch.float32, device=dev)
    f2 = torch.empty((npv, ldf), dtype=torch.float32, device=dev)
    for ws, f in ((ws1, f1), (ws2, f2)):
        _lib.check(L.rr_flux_split(P(dd["times_ff"]), npt, P(dd["lcids"]), npv, nlc, npb, ng, m.dg, P(ws), P(f),
                                   ldf, sp))
    torch.cuda.synchronize()
    f1, f2 = f1[:, :npt].double().cpu().numpy(), f2[:, :npt].double().cpu().numpy()
    assert np.array_equal(np.isnan(f1), np.isnan(f2))
    assert np.isnan(f1[7]).all() and (not npar or np.isnan(f1[5]).all())
    assert np.sum(f2 < 1) > 1000
    assert np.nanmax(np.abs(f1 - f2)) <= 1e-7


def test_model_split_path_matches_fp64():
    """RoadRunnerModel's split path for a named law (the fused prologue)
    stays within the split tolerance of the FP64 path."""
    from pytransit_gb300 import RoadRunnerModel
    rng = np.random.default_rng(9)
    npv = 300
    time = 2459000.0 + np.linspace(-0.3, 0.3, 2000)
    prm = (rng.uniform(0.05, 0.15, (npv, 1)),
           np.stack([rng.uniform(0, .6, npv), rng.uniform(0, .3, npv)], -1).reshape(npv, 1, 2),
           2459000.0 + rng.normal(0, 1e-3, (npv, 1)), rng.uniform(1, 10, npv), rng.uniform(3, 20, npv))
    inc = np.arccos(rng.uniform(0, .9, npv) / prm[4])
    out = {}
    for precision in ('fp64', 'split'):
        m = RoadRunnerModel('quadratic', precision=precision)
        m.set_data(time, nsamples=[2], exptimes=[0.01])
        out[precision] = m.evaluate(*prm, inc, 0.0, 0.0)
    assert np.abs(out['split'] - out['fp64']).max() <= 1e-6

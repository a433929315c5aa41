"""The no-allocation entry point, rr_full_split_noalloc, through the C ABI.

It serves callers that cannot allocate GPU memory (a plugin host that only
hands over input and output buffers, a runtime whose memory pool forbids raw
cudaMalloc, a loop that cannot afford cudaMalloc's possible device sync): its
scratch is a fixed device array inside the library.  The test checks it
against the workspace-taking entry point, rr_full_split, on two calls in a row
with different inputs (the shared scratch keeps the previous call's contents),
at the split path's flux tolerance of 1e-6.  It sits in its own file that
pytest collects last, and needs no state from other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-6

_vp, _i, _d, _sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t


def _bind(L):
    L.rr_full_split_noalloc_max_bytes.restype = _sz
    L.rr_full_split_noalloc.argtypes = ([_vp, _d, _d, _i, _vp, _i, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp,
                                         _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i,
                                         _d, _d, _d, _d, _vp, _vp, _i, _vp])
    L.rr_full_split_noalloc.restype = _i
    return L


def _case(seed, npv, npt):
    rng = np.random.default_rng(seed)
    T = 2459000.0
    nlc = 4
    time = T + np.arange(npt) * (2.0 / 1440.0)
    lcids = np.minimum((np.arange(npt) * nlc) // npt, nlc - 1)
    data = dict(time=time, lcids=lcids, pbids=np.arange(nlc), nsamples=np.array([1, 3, 5, 2]),
                exptimes=np.array([0.0, 0.01, 0.02, 0.005]))
    prm = dict(k=rng.uniform(0.05, 0.15, (npv, 1)),
               ldc=np.stack([rng.uniform(0, .6, (npv, nlc)), rng.uniform(0, .3, (npv, nlc))], -1),
               t0=T + rng.normal(0, 1e-3, (npv, 1)), p=rng.uniform(0.5, 5.0, npv), a=rng.uniform(3, 20, npv))
    prm["i"] = np.arccos(rng.uniform(0, 0.9, npv) / prm["a"])
    prm["e"] = rng.uniform(0, 0.3, npv)
    prm["w"] = rng.uniform(0, 2 * np.pi, npv)
    return data, prm


def _run(seed, npv=1500, npt=6000):
    """Flux from rr_full_split (caller workspace) and rr_full_split_noalloc."""
    import torch
    from pytransit_gb300 import RoadRunnerModel, _lib

    L = _bind(_lib.lib())
    data, prm = _case(seed, npv, npt)
    m = RoadRunnerModel('quadratic', precision='split')
    m.set_data(**data)
    dev = torch.device("cuda")
    dd = m._device_data(dev)
    tb = m._device_tables(dev)
    P = _lib.ptr
    sp = _lib.stream_ptr(dev)
    d = {n: torch.as_tensor(np.ascontiguousarray(v)).to(dev) for n, v in prm.items()}
    nz, ng, nk, nlc, npb = m.ze.size, m.ng, m.nk, m.nlc, m.npb
    ldp = torch.empty((npv, npb, nz), dtype=torch.float32, device=dev)
    ist = torch.empty((npv, npb), dtype=torch.float32, device=dev)
    _lib.check(L.rr_ld_tables_f32(2, P(d["ldc"]), npv, npb, 2, P(tb["mu"]), nz, P(ldp), P(ist), sp))
    ldf = (npt + 3) // 4 * 4
    common = (P(dd["times_ff"]), dd["t_ref"], dd["t_absmax"], npt, P(d["k"]), 1, P(d["t0"]), 1, 1, P(d["p"]),
              P(d["a"]), P(d["i"]), P(d["e"]), P(d["w"]), npv, nlc, npb, P(dd["lcids"]), P(dd["pbids"]),
              P(dd["epids"]), P(dd["nsamples"]), P(dd["exptimes"]), P(ldp), P(ist), P(tb["W32"]), nk, ng, nz,
              m.dk, float(m.klims[0]), float(m.klims[1]), m.dg, P(tb["ze"]))
    want = torch.full((npv, ldf), -1.0, dtype=torch.float32, device=dev)
    ws = torch.empty(L.rr_full_split_workspace_bytes(npv, npb, nlc, 1, ng), dtype=torch.uint8, device=dev)
    _lib.check(L.rr_full_split(*common, P(ws), ws.numel(), P(want), ldf, sp))
    got = torch.full((npv, ldf), -2.0, dtype=torch.float32, device=dev)
    st = L.rr_full_split_noalloc(*common, P(got), ldf, sp)
    assert st == 0, L.rr_status_string(st)
    torch.cuda.synchronize()
    return got[:, :npt].double().cpu().numpy(), want[:, :npt].double().cpu().numpy()


def test_noalloc_matches_workspace_entry_two_calls():
    for seed in (11, 12):
        got, want = _run(seed)
        assert np.array_equal(np.isnan(got), np.isnan(want))
        assert np.sum(want < 1) > 100          # in-transit points are exercised
        err = np.nanmax(np.abs(got - want))
        assert err <= TOL, (seed, err)


def test_noalloc_rejects_oversize_request():
    from pytransit_gb300 import _lib
    L = _bind(_lib.lib())
    cap = L.rr_full_split_noalloc_max_bytes()
    assert cap == 32 << 20
    npv = 1 << 20                              # needs far more than the fixed scratch
    assert L.rr_full_split_workspace_bytes(npv, 4, 4, 1, 100) > cap
    st = L.rr_full_split_noalloc(None, 0.0, 0.0, 100, None, 1, None, 1, 1, None, None, None, None, None, npv,
                                 4, 4, None, None, None, None, None, None, None, None, 256, 100, 40, 0.1,
                                 0.005, 0.5, 0.01, None, None, 100, None)
    assert st == 3                             # RR_ERR_WORKSPACE, before any launch

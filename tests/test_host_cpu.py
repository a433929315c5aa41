"""CPU-only tests: the C ABI library loads and exports every declared symbol,
and the host-side logic of the drop-in (set_data validation, parameter
shaping, LD-model resolution) behaves as the reference's."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "pytransit_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rr_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from pytransit_gb300 import build
    path = build.build()
    L = ctypes.CDLL(path)
    names = declared_functions()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings_and_workspace_sizes():
    from pytransit_gb300 import _lib
    L = _lib.lib()
    assert L.rr_abi_version() >= 1
    assert L.rr_status_string(0) == b"ok"
    assert b"npv, npb" in L.rr_status_string(1)
    assert L.rr_full_f64_workspace_bytes(10, 4, 100) >= 10 * 16 * 8 + 10 * 4 * 100 * 8
    assert L.rr_full_split_workspace_bytes(10, 4, 4, 1, 100) >= 10 * 4 * 100 * 4


def test_argument_errors_without_gpu():
    """Argument checks return before any launch, so they run without a GPU."""
    from pytransit_gb300 import _lib
    L = _lib.lib()
    # k with 3 columns and 4 passbands -> RR_ERR_SHAPE
    st = L.rr_full_f64(None, 10, None, 3, None, 1, None, None, None, None, None, 2, 1, 4, None, None, None,
                       None, None, None, None, None, 256, 100, 40, 0.1, 0.005, 0.5, 0.01, None, None, 0,
                       None, 10, None)
    assert st == 1
    # unknown law id
    assert L.rr_ld_tables_f64(99, None, 1, 1, 2, None, 40, None, None, None) == 5
    # ldflux < npt
    st = L.rr_full_f64(None, 10, None, 1, None, 1, None, None, None, None, None, 2, 1, 1, None, None, None,
                       None, None, None, None, None, 256, 100, 40, 0.1, 0.005, 0.5, 0.01, None, None, 0,
                       None, 5, None)
    assert st == 2
    # workspace too small
    st = L.rr_full_f64(None, 10, None, 1, None, 1, None, None, None, None, None, 2, 1, 1, None, None, None,
                       None, None, None, None, None, 256, 100, 40, 0.1, 0.005, 0.5, 0.01, None, None, 16,
                       None, 10, None)
    assert st == 3
    # the fused split prologue: device pointers are only passed on, never read on the host
    dev = ctypes.c_void_p(256)

    def prepare_ld(law, nkc, npb, wsb):
        return L.rr_prepare_split_ld(0.0, 1.0, dev, nkc, dev, 1, 1, dev, dev, dev, dev, dev, 8, 1, npb, dev, dev,
                                     dev, dev, law, dev, 2, dev, 40, dev, 3, dev, 256, 100, 0.002, 0.005, 0.5,
                                     dev, dev, dev, dev, wsb, None)
    big = L.rr_full_split_workspace_bytes(8, 4, 1, 1, 100)
    assert prepare_ld(2, 3, 4, big) == 1          # k with 3 columns and 4 passbands
    assert prepare_ld(2, 1, 4, 64) == 3           # workspace too small
    assert prepare_ld(99, 1, 4, big) == 5         # unknown law: the two-stage path's check
    # the range and pinned-output flux entry points: bad ranges and row strides
    # are refused before any pointer is looked at; an empty range does nothing
    for fn in (L.rr_flux_split_range, L.rr_flux_split_range_f64, L.rr_flux_split_transits,
               L.rr_flux_split_transits_f64):
        assert fn(dev, 100, dev, 8, 1, 1, 100, 0.01, dev, 0, 9, dev, 100, None) == 2    # pv1 > npv
        assert fn(dev, 100, dev, 8, 1, 1, 100, 0.01, dev, 5, 4, dev, 100, None) == 2    # pv0 > pv1
        assert fn(dev, 100, dev, 8, 1, 1, 100, 0.01, dev, 0, 8, dev, 99, None) == 2     # ldflux < npt
        assert fn(dev, 100, dev, 8, 1, 1, 100, 0.01, dev, 3, 3, dev, 100, None) == 0    # empty range
    st = L.rr_flux_f64_range(dev, 100, dev, 1, dev, 1, dev, 8, 1, 1, dev, dev, dev, dev, dev, dev, 100, 0.01, dev,
                             0, 9, dev, 100, None)
    assert st == 2
    st = L.rr_flux_f64_range(dev, 100, dev, 3, dev, 1, dev, 8, 1, 4, dev, dev, dev, dev, dev, dev, 100, 0.01, dev,
                             0, 8, dev, 100, None)
    assert st == 1                                # k with 3 columns and 4 passbands


def test_z_grid_matches_oracle():
    import oracle
    from pytransit_gb300 import create_z_grid
    ze, zm = create_z_grid(0.7, 20, 20)
    oze, ozm = oracle.z_grid(0.7, 20, 20)
    np.testing.assert_array_equal(ze, oze)
    np.testing.assert_array_equal(zm, ozm)


def test_set_data_validation_mirrors_reference():
    from pytransit_gb300 import RoadRunnerModel
    m = RoadRunnerModel('quadratic')
    t = np.linspace(0, 1, 10)
    with pytest.raises(ValueError, match="must be given as integers"):
        m.set_data(t, lcids=np.zeros(10))
    with pytest.raises(ValueError, match="should equal to the number of datapoints"):
        m.set_data(t, lcids=np.zeros(9, int))
    with pytest.raises(ValueError, match="should equal to the number of ligt curves"):
        m.set_data(t, lcids=np.zeros(10, int), pbids=[0, 1])
    with pytest.raises(ValueError, match="between 0 and"):
        m.set_data(t, lcids=np.repeat([0, 1], 5), pbids=[0, 2])
    with pytest.raises(ValueError):
        m.set_data(np.array([]))          # the reference fails on empty data as well
    m.set_data(t, lcids=np.repeat([0, 1], 5), pbids=[0, 1], nsamples=[1, 5], exptimes=[0, 0.01])
    assert (m.nlc, m.npb, m.npt) == (2, 2, 10)
    # same time object, no other args: no-op (transitmodel.py:83-84)
    m.set_data(t)
    assert m.nlc == 2


def test_ld_model_resolution():
    from pytransit_gb300 import LDModel, RoadRunnerModel, ldmodels
    assert RoadRunnerModel('power-2').ld_law == 9
    assert RoadRunnerModel((ldmodels.ld_quadratic, ldmodels.ldi_quadratic)).ld_law == 2
    assert RoadRunnerModel(lambda mu, pv: 1 - pv[0] * (1 - mu)).ld_law is None
    with pytest.raises(KeyError):
        RoadRunnerModel('no-such-law')
    with pytest.raises(NotImplementedError):
        RoadRunnerModel(42)

    class L(LDModel):
        def _evaluate(self, mu, x):
            return np.ones(np.shape(x)[:-1] + (np.size(mu),))
    m = RoadRunnerModel(L())
    assert m.ld_law is None and m.ldmmean is not None
    assert abs(L()._integrate(np.zeros((2, 3, 1)))[1, 2] - np.pi) < 1e-4


def test_parameter_shaping():
    from pytransit_gb300 import RoadRunnerModel
    m = RoadRunnerModel('quadratic')
    m.set_data(np.linspace(0, 1, 10), lcids=np.repeat([0, 1], 5), pbids=[0, 1], epids=[0, 1])
    k, t0, p, a, i, e, w = m._shape_params([0.1, 0.11, 0.12], [[0.0, 0.01]], [1, 2, 3], 5.0, 1.5, 0.0, 0.0)
    assert k.shape == (3, 1) and t0.shape == (3, 2) and a.shape == (3,)
    with pytest.raises(ValueError, match="npv, 1"):
        m._shape_params(np.ones((3, 3)), [[0.0, 0.01]], [1, 2, 3], 5.0, 1.5, 0.0, 0.0)
    with pytest.raises(ValueError, match="Epoch index"):
        m._shape_params(0.1, 0.0, 1.0, 5.0, 1.5, 0.0, 0.0)
    assert m._shape_ldc([0.3, 0.1], 3, 2).shape == (3, 2, 2)
    assert m._shape_ldc(np.ones((2, 2)), 3, 2).shape == (3, 2, 2)
    with pytest.raises(ValueError):
        m._shape_ldc(np.ones((3, 3, 2)), 3, 2)


def test_no_cpu_fallback():
    import torch
    from pytransit_gb300 import RoadRunnerModel
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    m = RoadRunnerModel('quadratic')
    m.set_data(np.linspace(-0.1, 0.1, 10))
    with pytest.raises(RuntimeError, match="CUDA"):
        m.evaluate(0.1, [0.3, 0.1], 0.0, 2.0, 7.0, 1.55)


def test_serving_struct_layout_matches_binding():
    import ctypes as C
    import numpy as np
    from pytransit_gb300 import _lib
    L = _lib.lib()
    L.rr_serve_struct_sizes.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
    rs, its = C.c_int(), C.c_int()
    L.rr_serve_struct_sizes(C.byref(rs), C.byref(its))
    from pytransit_gb300.serving import SERVE_REQUEST_DTYPE as dt
    assert rs.value == dt.itemsize == 104 and its.value == 24
    assert [dt.fields[n][1] for n in ('ldflux', 'kind', 'inv_dg', 'dg', 'nsamples0')] == [48, 76, 80, 88, 96]


def test_bench_reads_the_profiled_traffic_and_peak():
    """bench.py's roofline.traffic comes from the committed ncu summary of the
    flux kernel (bytes per point x the launch's points); the summary must keep
    the line it parses, with a value near the algorithmic 4 B per point."""
    import sys
    sys.path.insert(0, ROOT)
    import bench
    t = bench.profiled_traffic(8192, 19700)
    assert t is not None
    bpp = t / (8192 * 19700)
    assert 3.0 < bpp < 4.5, bpp
    peak, kind = bench.measured_peaks()
    assert peak > 1000 and kind in ("measured", "fallback")


def test_bench_serving_mix_and_sustained_rule():
    """The serving mix draws the configured distributions (20 % TS requests
    with 200 channels, npv and npt within their ranges) from shared pools, and
    a run counts as sustained only when it keeps up with the offered rate."""
    import bench
    mix = bench.C4Mix(4)
    reqs = [mix.request() for _ in range(2000)]
    ts = [r for r in reqs if r[0] == 'ts']
    assert 0.17 < len(ts) / len(reqs) < 0.23
    for kind, law, data, params in reqs[:200]:
        npv, npt = params['p'].size, data['time'].size
        assert 1 <= npv <= 4096 and 500 <= npt <= 100000
        assert params['k'].shape == (npv, 200 if kind == 'ts' else 1)
        assert params['ldc'].shape[:2] == (npv, 200 if kind == 'ts' else 1)
        assert data['nsamples'][0] in (1, 5, 10)
        assert np.all((params['k'] >= (0.09 if kind == 'ts' else 0.05)) & (params['k'] <= 0.15))
    run = dict(offered_req_per_s=2000, achieved_req_per_s=1990, requests=10000, queued_at_end_of_arrivals=3,
               latency_p99_first_half_s=0.02, latency_p99_second_half_s=0.021)
    assert bench.sustained(run)
    assert not bench.sustained(dict(run, achieved_req_per_s=1700))
    assert not bench.sustained(dict(run, queued_at_end_of_arrivals=500))
    assert not bench.sustained(dict(run, latency_p99_second_half_s=0.2))


def test_serve_setup_args_layout_matches_the_library():
    """rr_serve_setup_args (52 fields of 8 bytes) as the serving host fills it."""
    import ctypes as C
    from pytransit_gb300 import _lib
    from pytransit_gb300.serving import SETUP_ARGS_DTYPE
    L = _lib.lib()
    L.rr_serve_setup_args_size.argtypes = [C.POINTER(C.c_int)]
    L.rr_serve_setup_args_size.restype = None
    n = C.c_int()
    L.rr_serve_setup_args_size(C.byref(n))
    assert n.value == SETUP_ARGS_DTYPE.itemsize == 52 * 8
    assert SETUP_ARGS_DTYPE.names[-2:] == ('bound_host', 'desc')


def test_host_fill_sizes_and_threads():
    """rr_host_fill_f32 writes exactly dst[0..n), for any size and thread count
    (the slices are 64-byte blocks, the last one partial)."""
    from pytransit_gb300 import _lib
    L = _lib.lib()
    for n in (0, 1, 15, 17, 1000, 65535, 65536, 65537, (1 << 20) + 3):
        for nt in (0, 1, 2, 3, 8, 16):
            a = np.full(n + 32, -7.0, np.float32)
            assert L.rr_host_fill_f32(ctypes.c_void_p(a.ctypes.data + 64), n, 1.0, nt) == 0
            assert (a[:16] == -7).all() and (a[16:16 + n] == 1.0).all() and (a[16 + n:] == -7).all(), (n, nt)
    assert L.rr_host_fill_f32(None, 10, 1.0, 4) == 2
    assert L.rr_host_fill_f32(None, 0, 1.0, 4) == 0


def test_host_fill_from_several_threads_and_after_fork():
    """Calls from several Python threads are serialised and each fills its own
    buffer; a process forked after the pool started fills on a pool of its own
    (it would wait forever on the parent's threads otherwise)."""
    import threading
    from pytransit_gb300 import _lib
    L = _lib.lib()
    n = 1 << 21
    bufs = [np.zeros(n, np.float32) for _ in range(6)]

    def go(j):
        for _ in range(5):
            assert L.rr_host_fill_f32(ctypes.c_void_p(bufs[j].ctypes.data), n, float(j + 1), 4) == 0

    ts = [threading.Thread(target=go, args=(j,)) for j in range(len(bufs))]
    for t in ts:
        t.start()
    for t in ts:
        t.join(60)
    for j, b in enumerate(bufs):
        assert (b == j + 1).all()
    if not hasattr(os, "fork"):
        return
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", DeprecationWarning)   # the multi-threaded fork is the case tested
        pid = os.fork()
    if pid == 0:   # child: its own pool, then exit without running the test harness's teardown
        ok = False
        try:
            c = np.zeros(n, np.float32)
            ok = L.rr_host_fill_f32(ctypes.c_void_p(c.ctypes.data), n, 3.0, 4) == 0 and bool((c == 3.0).all())
        finally:
            os._exit(0 if ok else 1)
    import time
    t_end = time.time() + 60
    while time.time() < t_end:
        done, status = os.waitpid(pid, os.WNOHANG)
        if done:
            assert os.WIFEXITED(status) and os.WEXITSTATUS(status) == 0
            return
        time.sleep(0.05)
    os.kill(pid, 9)
    os.waitpid(pid, 0)
    raise AssertionError("the forked child's fill did not finish")


def test_bindings_match_the_header():
    """Every ctypes binding the package sets up passes as many arguments as the
    header declares for that entry point (a binding that drifts from the C
    ABI would pass garbage without an error)."""
    from pytransit_gb300 import _lib, eclipse, lnlike
    L = _lib.lib()
    eclipse._L()
    lnlike._L()
    src = open(os.path.join(ROOT, "include", "pytransit_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    decls = re.findall(r"\b(?:int|size_t|void|double)\s+\*?\s*(rr_[a-z0-9_]+)\s*\(([^;]*?)\)\s*;", src, flags=re.S)
    assert len(decls) >= 50
    checked = 0
    for name, args in decls:
        args = args.strip()
        n = 0 if args in ("", "void") else len(args.split(","))
        at = getattr(getattr(L, name), "argtypes", None)
        if at is None:
            continue
        assert len(at) == n, f"{name}: the header declares {n} arguments, the binding passes {len(at)}"
        checked += 1
    assert checked >= 45


def test_integration_guide_names_every_entry_point():
    """Every entry point the header declares is named in INTEGRATION.md, the
    guide a maintainer of the reference follows to bind the library."""
    guide = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    names = declared_functions()
    assert len(names) >= 50
    missing = [n for n in names if not re.search(r"\b" + n + r"\b", guide)]
    assert not missing, missing

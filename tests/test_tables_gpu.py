"""The RoadRunner weight table built on the GPU (rr_weights_3d, replacing
calculate_weights_3d, pytransit/models/roadrunner/common.py:189-223) against
the reference's own table in tests/golden/tables.npz.

The fixture holds a strided subset of the reference's W[256, 100, 40], its row
sums and its total.  The GPU table must match them to 1e-11 absolute (the
weights are at most 1 and sum to 1 per row): each weight is a difference of
two lens areas built from arccosines, the device's arccosine and the host's
differ in the last bit, and the difference of two nearly equal areas carries
that bit as up to ~5e-13 absolute.  That moves a flux by far less than the
1e-9 FP64 parity bound.  The grid steps dk and dg must match exactly, and the
FP32 copy must be the FP64 table rounded to nearest.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_weight_table_matches_reference(golden):
    import torch
    from pytransit_gb300 import _lib
    g = golden("tables")
    dev = torch.device("cuda:0")
    nk, ng, kmin, kmax = 256, 100, 0.005, 0.5
    ze = torch.as_tensor(g["ze"], dtype=torch.float64, device=dev)
    nz = ze.numel()
    W64 = torch.full((nk, ng, nz), float("nan"), dtype=torch.float64, device=dev)
    W32 = torch.full((nk, ng, nz), float("nan"), dtype=torch.float32, device=dev)
    dk, dg = C.c_double(), C.c_double()
    _lib.check(_lib.lib().rr_weights_3d(nk, kmin, kmax, _lib.ptr(ze), nz, ng, _lib.ptr(W64), _lib.ptr(W32),
                                        C.byref(dk), C.byref(dg), _lib.stream_ptr(dev)), "rr_weights_3d")
    torch.cuda.synchronize()
    assert dk.value == g["dk"] and dg.value == g["dg"]
    w = W64.cpu().numpy()
    assert np.isfinite(w).all()
    np.testing.assert_allclose(w[::37, ::9, :], g["w_sub"], rtol=0, atol=1e-11)
    np.testing.assert_allclose(w.sum(-1), g["w_rowsum"], rtol=0, atol=1e-11)
    assert abs(w.sum() - g["w_sum"]) < 1e-8
    assert abs((w ** 2).sum() - g["w_sumsq"]) < 1e-6
    np.testing.assert_array_equal(W32.cpu().numpy(), w.astype(np.float32))


def test_weight_table_rejects_bad_sizes():
    """Invalid grid sizes are refused with a status, before any launch."""
    import torch
    from pytransit_gb300 import _lib
    dev = torch.device("cuda:0")
    ze = torch.zeros(40, dtype=torch.float64, device=dev)
    W = torch.empty(1, dtype=torch.float64, device=dev)
    dk, dg = C.c_double(), C.c_double()
    for nk, ng, nz in ((1, 100, 40), (256, 1, 40), (256, 100, 0)):
        st = _lib.lib().rr_weights_3d(nk, 0.005, 0.5, _lib.ptr(ze), nz, ng, _lib.ptr(W), None,
                                      C.byref(dk), C.byref(dg), _lib.stream_ptr(dev))
        assert st != 0

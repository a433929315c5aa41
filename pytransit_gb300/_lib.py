"""ctypes binding of the C ABI (include/pytransit_gb300.h).

The CUDA library is the only compute path: if it cannot be loaded, or no CUDA
device is present, every model call raises.  There is no CPU fallback.
"""
import ctypes as C
import os

import torch

from . import build as _build

_LIB = None

_vp = C.c_void_p
_i = C.c_int
_d = C.c_double
_sz = C.c_size_t


class RRError(RuntimeError):
    """A non-zero status from the CUDA library."""


def _sig(L):
    L.rr_abi_version.restype = _i
    L.rr_status_string.argtypes = [_i]
    L.rr_status_string.restype = C.c_char_p
    L.rr_last_cuda_error.restype = C.c_char_p
    L.rr_weights_3d.argtypes = [_i, _d, _d, _vp, _i, _i, _vp, _vp, C.POINTER(_d), C.POINTER(_d), _vp]
    L.rr_time_split_floats.argtypes = [_i]
    L.rr_time_split_floats.restype = _sz
    L.rr_time_split.argtypes = [_vp, _vp, _i, _d, _vp, _vp]
    for n in ("rr_ld_tables_f64", "rr_ld_tables_f32"):
        getattr(L, n).argtypes = [_i, _vp, _i, _i, _i, _vp, _i, _vp, _vp, _vp]
    L.rr_full_f64_workspace_bytes.argtypes = [_i, _i, _i]
    L.rr_full_f64_workspace_bytes.restype = _sz
    L.rr_full_split_workspace_bytes.argtypes = [_i, _i, _i, _i, _i]
    L.rr_full_split_workspace_bytes.restype = _sz
    L.rr_full_f64.argtypes = ([_vp, _i, _vp, _i, _vp, _i, _vp, _vp, _vp, _vp, _vp, _i, _i, _i,
                               _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _d, _d, _d,
                               _vp, _vp, _sz, _vp, _i, _vp])
    L.rr_full_split.argtypes = ([_vp, _d, _d, _i, _vp, _i, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _i,
                                 _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _d,
                                 _d, _d, _vp, _vp, _sz, _vp, _i, _vp])
    L.rr_prepare_f64.argtypes = ([_vp, _i, _vp, _vp, _vp, _vp, _vp, _i, _i, _vp, _vp, _i, _i, _i, _d, _d, _d,
                                  _vp, _vp, _sz, _vp, _i, _vp, _i, _vp, _i])
    L.rr_basis_count.argtypes = [_i, _i]
    L.rr_basis_tables.argtypes = [_i, _i, _vp, _i, _vp, _i, _i, _vp, _vp, _vp]
    L.rr_flux_f64.argtypes = ([_vp, _i, _vp, _i, _vp, _i, _vp, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i,
                               _d, _vp, _vp, _i, _vp])
    L.rr_prepare_split.argtypes = ([_d, _d, _vp, _i, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _vp,
                                    _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _d, _d, _vp, _vp, _sz, _vp,
                                    _i, _vp, _i, _vp, _i])
    L.rr_prepare_split_ld.argtypes = ([_d, _d, _vp, _i, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _vp,
                                       _vp, _vp, _vp, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i, _i, _d, _d, _d,
                                       _vp, _vp, _vp, _vp, _sz, _vp])
    L.rr_flux_split.argtypes = [_vp, _i, _vp, _i, _i, _i, _i, _d, _vp, _vp, _i, _vp]
    L.rr_flux_split_range.argtypes = [_vp, _i, _vp, _i, _i, _i, _i, _d, _vp, _i, _i, _vp, _i, _vp]
    L.rr_flux_split_transits.argtypes = [_vp, _i, _vp, _i, _i, _i, _i, _d, _vp, _i, _i, _vp, _i, _vp]
    L.rr_host_fill_f32.argtypes = [_vp, _sz, C.c_float, _i]
    L.rr_host_fill_f64.argtypes = [_vp, _sz, _d, _i]
    L.rr_flux_split_range_f64.argtypes = [_vp, _i, _vp, _i, _i, _i, _i, _d, _vp, _i, _i, _vp, _i, _vp]
    L.rr_flux_split_transits_f64.argtypes = [_vp, _i, _vp, _i, _i, _i, _i, _d, _vp, _i, _i, _vp, _i, _vp]
    L.rr_time_tiles_f64_doubles.argtypes = [_i]
    L.rr_time_tiles_f64_doubles.restype = _sz
    L.rr_time_tiles_f64.argtypes = [_vp, _vp, _i, _vp, _vp]
    L.rr_flux_f64_culled_range.argtypes = ([_vp, _vp, _i, _vp, _i, _vp, _i, _vp, _i, _i, _i, _vp, _vp, _vp, _vp,
                                            _vp, _vp, _i, _d, _vp, _i, _i, _vp, _i, _vp])
    L.rr_flux_f64_range.argtypes = ([_vp, _i, _vp, _i, _vp, _i, _vp, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i,
                                     _d, _vp, _i, _i, _vp, _i, _vp])
    L.rr_ts_workspace_bytes.argtypes = [_i, _i, _i, _i]
    L.rr_ts_workspace_bytes.restype = _sz
    _ts_tail = [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _vp, _vp, _vp, _i, _i, _i, _d, _d, _d, _d,
                _vp, _vp, _sz, _vp, _i, _vp]
    L.rr_ts_f64.argtypes = [_vp, _i] + _ts_tail
    L.rr_ts_split.argtypes = [_vp, _d, _d, _i] + _ts_tail
    _orbit = [_vp] * 7
    L.rr_ts_prepare_split.argtypes = [_d, _d] + _orbit + [_i, _i, _d, _vp, _vp, _vp, _i, _i, _i, _d, _d, _d, _vp,
                                                          _vp, _sz, _vp]
    L.rr_ts_prepare_split_ld.argtypes = [_i, _vp, _i, _vp, _d, _d] + _orbit + [_i, _i, _d, _i, _i, _vp, _vp, _sz,
                                                                              _vp]
    L.rr_ts_prepare_f64_ld.argtypes = [_i, _vp, _i, _vp] + _orbit + [_i, _i, _d, _i, _i, _vp, _vp, _sz, _vp]
    L.rr_ts_flux_split.argtypes = [_vp, _i, _i, _i, _i, _d, _i, _d, _vp, _vp, _i, _vp]
    L.rr_ts_flux_f64.argtypes = [_vp, _i, _vp, _vp, _i, _i, _i, _d, _i, _d, _vp, _vp, _i, _vp]
    L.rr_ts_flux_f64_culled.argtypes = [_vp, _vp, _i, _vp, _vp, _i, _i, _i, _d, _i, _d, _vp, _vp, _i, _vp]
    L.rr_ts_tables.argtypes = [_vp, _i, _i, _i, _i, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp)]
    L.rr_ts_tables.restype = None
    L.rr_split_error_bounds.argtypes = [_vp] * 5 + [_i, _i, _i, _i, _i, _d, _vp, _vp, _vp, _vp]
    L.rr_ts_split_error_bounds.argtypes = [_vp] * 5 + [_i, _i, _i, _d, _i, _d, _vp, _vp, _vp, _vp]
    for name, args in _EXTRA_SIGNATURES.items():
        if hasattr(L, name):
            getattr(L, name).argtypes = args[0]
            getattr(L, name).restype = args[1]


# Signatures of entry points added in other translation units (name -> (argtypes, restype)).
_EXTRA_SIGNATURES = {}


def lib():
    """Build (if needed) and load libpytransit_gb300.so; raise if impossible."""
    global _LIB
    if _LIB is None:
        path = _build.LIB
        if not os.path.exists(path) or _build._stale():
            path = _build.build()
        L = C.CDLL(path)
        _sig(L)
        _LIB = L
    return _LIB


def check(status: int, where: str = ""):
    if status != 0:
        L = lib()
        msg = L.rr_status_string(status).decode()
        if status == 4:
            msg += f" ({L.rr_last_cuda_error().decode()})"
        if status == 1:
            raise ValueError(msg)
        raise RRError(f"{where}: {msg}" if where else msg)


def to_host_f64(t, min_points: int = 1 << 17):
    """A device result as a float64 numpy array, the reference's return type.
    From min_points on, the copy goes into page-locked memory from torch's
    cached host allocator (the array is a view of it): a copy into a fresh
    pageable numpy array runs at a fraction of the host link's speed."""
    if t.numel() < min_points:
        return t.to(torch.float64).cpu().numpy()
    src = t.to(torch.float64).contiguous()
    try:
        host = torch.empty(src.shape, dtype=torch.float64, pin_memory=True)
    except RuntimeError:                # no page-locked memory to be had
        return src.cpu().numpy()
    host.copy_(src, non_blocking=True)
    torch.cuda.current_stream(t.device).synchronize()
    return host.numpy()


def require_cuda(device=None) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("pytransit_gb300 needs a CUDA device (GB300, sm_103a); no CPU fallback exists")
    dev = torch.device(device if device is not None else "cuda")
    if dev.type != "cuda":
        raise RuntimeError(f"pytransit_gb300 runs on CUDA devices only, not {dev}")
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev


def ptr(t):
    """Device pointer of a torch tensor (None -> NULL)."""
    return None if t is None else C.c_void_p(t.data_ptr())


def stream_ptr(device=None):
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)

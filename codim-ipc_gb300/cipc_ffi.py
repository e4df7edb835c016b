"""ctypes binding of libcipc.so (the C ABI declared in include/cipc.h).

This is the thin layer the Python host code and the tests call through.  It
never falls back to anything: if ``libcipc.so`` has not been built, importing
a function raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcipc.so")

CIPC_OK = 0
CIPC_ERR_INVALID_ARG = 1
CIPC_ERR_CUDA = 2
CIPC_ERR_ITER_CAP = 3
CIPC_ERR_NONPOSITIVE_DISTANCE = 4
CIPC_ERR_NOT_CONVERGED = 5
CIPC_ERR_NAN = 6
CIPC_ERR_NO_DEVICE = 7
CIPC_ERR_INDEX_RANGE = 8

FP64 = 0
MIXED = 1
MEM_HOST = 0
MEM_DEVICE = 1

PP, PE, PT, EE = 0, 1, 2, 3

_lib = None

_c_i64 = ctypes.c_int64
_c_int = ctypes.c_int
_c_dbl = ctypes.c_double
_vp = ctypes.c_void_p

# name -> (restype, argtypes)
_SIGS = {
    "cipc_version": (ctypes.c_char_p, []),
    "cipc_last_error": (ctypes.c_char_p, []),
    "cipc_status_string": (ctypes.c_char_p, [_c_int]),
    "cipc_device_count": (_c_int, []),
    "cipc_ccd_pairs": (_c_int, [_c_i64, _vp, _vp, _c_i64, _vp, _vp, _c_dbl, _c_dbl, _c_dbl, _c_int, _c_int,
                                _vp, _vp, ctypes.POINTER(_c_i64), _vp]),
    "cipc_barrier_pairs": (_c_int, [_c_i64, _vp, _vp, _c_i64, _vp, _vp, _c_dbl, _c_dbl, _c_dbl, _c_int, _c_int,
                                    _c_int, _vp, _vp, _vp, ctypes.POINTER(_c_i64), _vp]),
    "cipc_encode_reference_constraint": (_c_int, [_c_int, _vp, _c_int, _c_int, _vp]),
}


class CipcError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("cipc status %d: %s" % (status, msg))
        self.status = status


def lib():
    """Loads libcipc.so and declares every exported signature (raises if absent)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libcipc.so is not built (run __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


def last_error():
    return lib().cipc_last_error().decode()


def _check(status, allow=()):
    if status != CIPC_OK and status not in allow:
        raise CipcError(status, last_error())
    return status


def _ptr(a):
    """Raw pointer of a numpy array (host) or a torch tensor (host or CUDA)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data
    assert a.is_contiguous()
    return a.data_ptr()


def _stream_ptr(stream):
    if stream is None:
        return None
    return int(getattr(stream, "cuda_stream", stream))


def ccd_pairs(type_, idx, x, dx, toc_out, hit, eta=0.1, thickness=0.0, toc_in=1.0, precision=FP64,
              mem=MEM_HOST, stream=None, allow=(CIPC_ERR_ITER_CAP,)):
    """Additive CCD over pairs (see cipc_ccd_pairs).  Returns (status, n_overflow)."""
    n = int(type_.shape[0])
    nv = int(x.shape[0])
    ov = _c_i64(0)
    st = lib().cipc_ccd_pairs(n, _ptr(type_), _ptr(idx), nv, _ptr(x), _ptr(dx), eta, thickness, toc_in,
                              precision, mem, _ptr(toc_out), _ptr(hit), ctypes.byref(ov), _stream_ptr(stream))
    _check(st, allow)
    return st, ov.value


def ccd_pairs_async(type_, idx, x, dx, toc_out, hit, eta=0.1, thickness=0.0, toc_in=1.0, precision=FP64,
                    stream=None):
    """Device-memory CCD that only enqueues (no overflow readback, no wait)."""
    n = int(type_.shape[0])
    nv = int(x.shape[0])
    st = lib().cipc_ccd_pairs(n, _ptr(type_), _ptr(idx), nv, _ptr(x), _ptr(dx), eta, thickness, toc_in,
                              precision, MEM_DEVICE, _ptr(toc_out), _ptr(hit), None, _stream_ptr(stream))
    return _check(st)


def barrier_pairs(type_, idx, x, x_rest, energy, grad, hess, dhat2, xi, kappa, project_pd=True,
                  precision=FP64, mem=MEM_HOST, stream=None, allow=(CIPC_ERR_NONPOSITIVE_DISTANCE,)):
    """Barrier energy/gradient/PSD Hessian per pair (see cipc_barrier_pairs).  Returns (status, n_bad)."""
    n = int(type_.shape[0])
    nv = int(x.shape[0])
    bad = _c_i64(0)
    st = lib().cipc_barrier_pairs(n, _ptr(type_), _ptr(idx), nv, _ptr(x), _ptr(x_rest), dhat2, xi, kappa,
                                  1 if project_pd else 0, precision, mem, _ptr(energy), _ptr(grad), _ptr(hess),
                                  ctypes.byref(bad), _stream_ptr(stream))
    _check(st, allow)
    return st, bad.value


def barrier_pairs_async(type_, idx, x, x_rest, energy, grad, hess, dhat2, xi, kappa, project_pd=True,
                        precision=FP64, stream=None):
    n = int(type_.shape[0])
    nv = int(x.shape[0])
    st = lib().cipc_barrier_pairs(n, _ptr(type_), _ptr(idx), nv, _ptr(x), _ptr(x_rest), dhat2, xi, kappa,
                                  1 if project_pd else 0, precision, MEM_DEVICE, _ptr(energy), _ptr(grad),
                                  _ptr(hess), None, _stream_ptr(stream))
    return _check(st)


def encode_reference_constraint(type_, idx4, mollified=False, multiplicity=1):
    a = np.ascontiguousarray(idx4, dtype=np.int32)
    out = np.zeros(4, np.int32)
    _check(lib().cipc_encode_reference_constraint(int(type_), a.ctypes.data, int(bool(mollified)),
                                                  int(multiplicity), out.ctypes.data))
    return out

"""ctypes binding of the CPU oracle (test infrastructure only).

Only the tests, the smoke check and the bench's CPU-baseline leg load this.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None
_P = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        from . import build as _b  # noqa: F401  (package-relative when imported as oracle.oracle_ffi)
        path = _b.build_oracle()
        L = ctypes.CDLL(path)
        L.orc_pt_type.argtypes = [_P]
        L.orc_ee_type.argtypes = [_P]
        L.orc_pe_type.argtypes = [_P]
        L.orc_d2.argtypes = [ctypes.c_int, _P]
        L.orc_d2.restype = ctypes.c_double
        L.orc_d2_grad_hess.argtypes = [ctypes.c_int, _P, _P, _P]
        L.orc_barrier.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, _P]
        L.orc_mollifier.argtypes = [_P, ctypes.c_double, _P, _P]
        L.orc_mollifier.restype = ctypes.c_double
        L.orc_make_pd.argtypes = [ctypes.c_int, _P]
        L.orc_sym_eigen.argtypes = [ctypes.c_int, _P, _P, _P]
        L.orc_ccd_pairs.argtypes = [ctypes.c_int64, _P, _P, _P, _P, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_int64, _P, _P, _P]
        L.orc_ccd_pairs.restype = ctypes.c_int64
        L.orc_barrier_pairs.argtypes = [ctypes.c_int64, _P, _P, _P, _P, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_int, _P, _P, _P]
        L.orc_barrier_pairs.restype = ctypes.c_int64
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def pt_type(x12):
    return lib().orc_pt_type(_p(_c(x12, np.float64)))


def ee_type(x12):
    return lib().orc_ee_type(_p(_c(x12, np.float64)))


def pe_type(x9):
    return lib().orc_pe_type(_p(_c(x9, np.float64)))


def d2(kind, x):
    x = np.zeros(12) if x is None else np.concatenate([_c(x, np.float64).ravel(), np.zeros(12)])[:12].copy()
    return lib().orc_d2(kind, _p(x))


def d2_grad_hess(kind, x):
    n = {0: 6, 1: 9, 2: 12, 3: 12, 4: 12}[kind]
    xx = np.zeros(12)
    xx[:n] = np.asarray(x, np.float64).ravel()[:n]
    g = np.zeros(12)
    H = np.zeros(144)
    lib().orc_d2_grad_hess(kind, _p(xx), _p(g), _p(H))
    return g[:n].copy(), H[:n * n].reshape(n, n).copy()


def barrier(d, dhat, kappa):
    out = np.zeros(3)
    lib().orc_barrier(d, dhat, kappa, _p(out))
    return out


def mollifier(x12, eps_x):
    g = np.zeros(12)
    H = np.zeros(144)
    e = lib().orc_mollifier(_p(_c(x12, np.float64)), eps_x, _p(g), _p(H))
    return e, g, H.reshape(12, 12)


def make_pd(H):
    H = _c(H, np.float64).copy()
    lib().orc_make_pd(H.shape[0], _p(H))
    return H


def ccd_pairs(type_, idx, x, dx, eta=0.1, thickness=0.0, toc_in=1.0, max_iter=1 << 20):
    n = type_.shape[0]
    toc = np.zeros(n)
    hit = np.zeros(n, np.uint8)
    iters = np.zeros(n, np.int32)
    ov = lib().orc_ccd_pairs(n, _p(_c(type_, np.uint8)), _p(_c(idx, np.int32)), _p(_c(x, np.float64)),
                             _p(_c(dx, np.float64)), eta, thickness, toc_in, max_iter, _p(toc), _p(hit), _p(iters))
    return toc, hit, iters, ov


def barrier_pairs(type_, idx, x, x_rest, dhat2, xi, kappa, project_pd=True):
    n = type_.shape[0]
    E = np.zeros(n)
    g = np.zeros((n, 12))
    H = np.zeros((n, 78))
    bad = lib().orc_barrier_pairs(n, _p(_c(type_, np.uint8)), _p(_c(idx, np.int32)), _p(_c(x, np.float64)),
                                  _p(_c(x_rest, np.float64)), dhat2, xi, kappa, 1 if project_pd else 0,
                                  _p(E), _p(g), _p(H))
    return E, g, H, bad


def set_threads(n):
    lib().orc_set_threads(int(n))


def num_threads():
    return lib().orc_num_threads()

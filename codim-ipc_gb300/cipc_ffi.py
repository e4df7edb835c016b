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
CIPC_ERR_TIMEOUT = 9

FP64 = 0
MIXED = 1
PRECOND_BLOCK_JACOBI = 0
PRECOND_LEARNED = 1
PRECOND_AGGREGATE = 2
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
    "cipc_ccd_pairs_noalloc": (_c_int, [_c_i64, _vp, _vp, _c_i64, _vp, _vp, _c_dbl, _c_dbl, _c_dbl, _c_int,
                                        _c_int, _vp, _vp, ctypes.POINTER(_c_i64), _vp]),
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


_NP_DTYPES = {"u8": np.uint8, "i32": np.int32, "f32": np.float32, "f64": np.float64}


def _dtype_name(a):
    if isinstance(a, np.ndarray):
        for k, v in _NP_DTYPES.items():
            if a.dtype == v:
                return k
        return str(a.dtype)
    s = str(a.dtype)  # torch dtypes
    return {"torch.uint8": "u8", "torch.int32": "i32", "torch.float32": "f32", "torch.float64": "f64"}.get(s, s)


def _where(a):
    """'host' for numpy arrays and CPU tensors, ('cuda', index) for CUDA tensors."""
    if isinstance(a, np.ndarray):
        return "host"
    if getattr(a, "is_cuda", False):
        return ("cuda", a.device.index)
    return "host"


def _check_buffers(name, bufs, mem):
    """Checks dtype, shape and placement of the buffers handed to a pair entry
    point, so that a wrong buffer is an exception here instead of an
    out-of-bounds or host-pointer access in a kernel.  bufs: list of
    (label, array, dtype name, expected shape)."""
    places = set()
    for label, a, dt, shape in bufs:
        if a is None:
            raise ValueError("%s: %s is missing" % (name, label))
        if _dtype_name(a) != dt:
            raise TypeError("%s: %s must be %s, got %s" % (name, label, dt, _dtype_name(a)))
        if tuple(a.shape) != tuple(shape):
            raise ValueError("%s: %s must have shape %s, got %s" % (name, label, tuple(shape), tuple(a.shape)))
        if isinstance(a, np.ndarray):
            if not a.flags["C_CONTIGUOUS"]:
                raise ValueError("%s: %s must be C-contiguous" % (name, label))
        elif not a.is_contiguous():
            raise ValueError("%s: %s must be contiguous" % (name, label))
        places.add(_where(a))
    if mem == MEM_DEVICE:
        if len(places) != 1 or "host" in places:
            raise ValueError("%s: device-memory call needs every buffer on one CUDA device, got %s"
                             % (name, sorted(map(str, places))))
    elif any(p != "host" for p in places):
        raise ValueError("%s: host-memory call needs host buffers (numpy or CPU tensors)" % name)


def _pair_buffers(type_, idx, x, dx, toc_out, hit):
    n = int(type_.shape[0])
    nv = int(x.shape[0])
    return n, nv, [("type", type_, "u8", (n,)), ("idx", idx, "i32", (n, 4)), ("x", x, "f64", (nv, 3)),
                   ("dx", dx, "f64", (nv, 3)), ("toc_out", toc_out, "f64", (n,)), ("hit", hit, "u8", (n,))]


def ccd_pairs(type_, idx, x, dx, toc_out, hit, eta=0.1, thickness=0.0, toc_in=1.0, precision=FP64,
              mem=MEM_HOST, stream=None, allow=(CIPC_ERR_ITER_CAP,)):
    """Additive CCD over pairs (see cipc_ccd_pairs).  Returns (status, n_overflow)."""
    n, nv, bufs = _pair_buffers(type_, idx, x, dx, toc_out, hit)
    _check_buffers("ccd_pairs", bufs, mem)
    ov = _c_i64(0)
    st = lib().cipc_ccd_pairs(n, _ptr(type_), _ptr(idx), nv, _ptr(x), _ptr(dx), eta, thickness, toc_in,
                              precision, mem, _ptr(toc_out), _ptr(hit), ctypes.byref(ov), _stream_ptr(stream))
    _check(st, allow)
    return st, ov.value


def ccd_pairs_async(type_, idx, x, dx, toc_out, hit, eta=0.1, thickness=0.0, toc_in=1.0, precision=FP64,
                    stream=None):
    """Device-memory CCD that only enqueues (no overflow readback, no wait)."""
    n, nv, bufs = _pair_buffers(type_, idx, x, dx, toc_out, hit)
    _check_buffers("ccd_pairs_async", bufs, MEM_DEVICE)
    st = lib().cipc_ccd_pairs(n, _ptr(type_), _ptr(idx), nv, _ptr(x), _ptr(dx), eta, thickness, toc_in,
                              precision, MEM_DEVICE, _ptr(toc_out), _ptr(hit), None, _stream_ptr(stream))
    return _check(st)


NOALLOC_SLOTS = 16


def ccd_pairs_noalloc(type_, idx, x, dx, toc_out, hit, eta=0.1, thickness=0.0, toc_in=1.0, precision=FP64,
                      slot=0, stream=None, counts=True, allow=(CIPC_ERR_ITER_CAP,)):
    """Device-memory CCD that allocates nothing (see cipc_ccd_pairs_noalloc).
    Returns (status, n_overflow); with counts=False it only enqueues."""
    n, nv, bufs = _pair_buffers(type_, idx, x, dx, toc_out, hit)
    _check_buffers("ccd_pairs_noalloc", bufs, MEM_DEVICE)
    ov = _c_i64(0)
    st = lib().cipc_ccd_pairs_noalloc(n, _ptr(type_), _ptr(idx), nv, _ptr(x), _ptr(dx), eta, thickness, toc_in,
                                      precision, slot, _ptr(toc_out), _ptr(hit),
                                      ctypes.byref(ov) if counts else None, _stream_ptr(stream))
    _check(st, allow)
    return st, ov.value


def _barrier_check(name, type_, idx, x, x_rest, energy, grad, hess, precision, mem):
    n = int(type_.shape[0])
    nv = int(x.shape[0])
    _check_buffers(name, [("type", type_, "u8", (n,)), ("idx", idx, "i32", (n, 4)), ("x", x, "f64", (nv, 3)),
                          ("x_rest", x_rest, "f64", (nv, 3)), ("energy", energy, "f64", (n,)),
                          ("grad", grad, "f64", (n, 12)),
                          ("hess", hess, "f64" if precision == FP64 else "f32", (n, 78))], mem)
    return n, nv


def barrier_pairs(type_, idx, x, x_rest, energy, grad, hess, dhat2, xi, kappa, project_pd=True,
                  precision=FP64, mem=MEM_HOST, stream=None, allow=(CIPC_ERR_NONPOSITIVE_DISTANCE,)):
    """Barrier energy/gradient/PSD Hessian per pair (see cipc_barrier_pairs).  Returns (status, n_bad)."""
    n, nv = _barrier_check("barrier_pairs", type_, idx, x, x_rest, energy, grad, hess, precision, mem)
    bad = _c_i64(0)
    st = lib().cipc_barrier_pairs(n, _ptr(type_), _ptr(idx), nv, _ptr(x), _ptr(x_rest), dhat2, xi, kappa,
                                  1 if project_pd else 0, precision, mem, _ptr(energy), _ptr(grad), _ptr(hess),
                                  ctypes.byref(bad), _stream_ptr(stream))
    _check(st, allow)
    return st, bad.value


def barrier_pairs_async(type_, idx, x, x_rest, energy, grad, hess, dhat2, xi, kappa, project_pd=True,
                        precision=FP64, stream=None):
    n, nv = _barrier_check("barrier_pairs_async", type_, idx, x, x_rest, energy, grad, hess, precision, MEM_DEVICE)
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


# ---------------------------------------------------------------------------
# shell simulation (cipc_sim_*)
# ---------------------------------------------------------------------------
class StepParams(ctypes.Structure):
    _fields_ = [("h", ctypes.c_double), ("dhat2", ctypes.c_double), ("xi", ctypes.c_double), ("mu", ctypes.c_double),
                ("epsv2", ctypes.c_double), ("fric_iters", ctypes.c_int), ("newton_tol", ctypes.c_double),
                ("with_collision", ctypes.c_int), ("max_newton_iters", ctypes.c_int), ("precision", ctypes.c_int),
                ("pcg_tol", ctypes.c_double), ("pcg_max_iters", ctypes.c_int), ("preconditioner", ctypes.c_int),
                ("forcing", ctypes.c_int), ("barrier_model", ctypes.c_int), ("accd_max_iters", ctypes.c_int),
                ("pcg_wait_polls", ctypes.c_int)]


class StepStats(ctypes.Structure):
    _fields_ = [("newton_iters", ctypes.c_int), ("pcg_iters", ctypes.c_int), ("line_search_trials", ctypes.c_int),
                ("n_constraints", ctypes.c_int), ("status", ctypes.c_int), ("min_dist2", ctypes.c_double),
                ("kappa", ctypes.c_double), ("ms", ctypes.c_double), ("precond_fallbacks", ctypes.c_int),
                ("learned_solves", ctypes.c_int), ("solve_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_PP = ctypes.POINTER(ctypes.c_void_p)
_SIGS.update({
    "cipc_sim_create": (_c_int, [_c_int, _vp, _c_int, _vp, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _vp, _c_dbl, _c_int, _PP]),
    "cipc_sim_destroy": (_c_int, [_vp]),
    "cipc_sim_create_codim": (_c_int, [_c_int, _vp, _c_int, _vp, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _vp, _c_dbl, _c_int,
                                       _vp, _PP]),
    "cipc_sim_init_oipc": (_c_int, [_vp, _c_dbl, _c_dbl, _vp, _vp]),
    "cipc_sim_set_kappa": (_c_int, [_vp, _c_dbl, _c_dbl]),
    "cipc_sim_get_kappa": (_c_int, [_vp, _vp]),
    "cipc_sim_step_split": (_c_int, [_vp, _vp, _vp]),
    "cipc_sim_create_full": (_c_int, [_c_int, _vp, _c_int, _vp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, _vp, ctypes.c_double, _c_int, _vp, _vp, _vp]),
    "cipc_sim_init_eipc": (_c_int, [_vp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, _vp, _vp]),
    "cipc_sim_set_strain_limit": (_c_int, [_vp, _vp, _vp, _vp]),
    "cipc_sim_init_dirichlet": (_c_int, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_double, _c_int, _c_int, _vp]),
    "cipc_sim_step_dirichlet": (_c_int, [_vp, ctypes.c_double]),
    "cipc_sim_get_dbc": (_c_int, [_vp, _c_int, _vp, _vp, _vp]),
    "cipc_sim_write_obj": (_c_int, [_vp, ctypes.c_char_p]),
    "cipc_sim_get_strain_limit": (_c_int, [_vp, _vp]),
    "cipc_sim_set_state": (_c_int, [_vp, _vp, _vp]),
    "cipc_sim_get_state": (_c_int, [_vp, _vp, _vp]),
    "cipc_sim_set_dbc": (_c_int, [_vp, _c_int, _vp, _vp]),
    "cipc_sim_step": (_c_int, [_vp, ctypes.POINTER(StepParams), ctypes.POINTER(StepStats)]),
    "cipc_sim_constraints": (_c_int, [_vp, ctypes.POINTER(StepParams), _vp, _c_int, _vp, ctypes.POINTER(_c_int)]),
    "cipc_sim_eval": (_c_int, [_vp, ctypes.POINTER(StepParams), _vp, _vp, _vp, _vp]),
    "cipc_sim_ccd": (_c_int, [_vp, ctypes.POINTER(StepParams), _vp, _vp, _c_dbl, _vp]),
})


def make_params(h, dhat2, xi, mu=0.0, epsv2=1e-6, fric_iters=1, newton_tol=1e-2, with_collision=True,
                max_newton_iters=200, precision=FP64, pcg_tol=1e-6, pcg_max_iters=10000, preconditioner=0,
                forcing=0, elastic_ipc=False, accd_max_iters=0, pcg_wait_polls=0):
    return StepParams(h, dhat2, xi, mu, epsv2, fric_iters, newton_tol, int(bool(with_collision)), max_newton_iters,
                      precision, pcg_tol, pcg_max_iters, preconditioner, forcing, 1 if elastic_ipc else 0,
                      accd_max_iters, pcg_wait_polls)


class CodimDesc(ctypes.Structure):
    _fields_ = [("n_segments", ctypes.c_int), ("segments", ctypes.c_void_p), ("rod_E", ctypes.c_double),
                ("rod_rho", ctypes.c_double), ("rod_thickness", ctypes.c_double), ("rod_bend_mult", ctypes.c_double),
                ("n_particles", ctypes.c_int), ("particles", ctypes.c_void_p), ("particle_rho", ctypes.c_double),
                ("particle_thickness", ctypes.c_double)]


class TetDesc(ctypes.Structure):
    _fields_ = [("n_tets", ctypes.c_int), ("tets", ctypes.c_void_p), ("E", ctypes.c_double), ("nu", ctypes.c_double),
                ("rho", ctypes.c_double)]


class Sim:
    """Owns one cipc_sim handle (device-resident shell scene).

    codim (optional): dict(segments=(n,2) ints, rod_E, rod_rho, rod_thickness,
    rod_bend_mult=1, particles=(m,) ints, particle_rho, particle_thickness).
    tets (optional): dict(tets=(k,4) ints, E, nu, rho) -- volumetric Neo-Hookean."""

    def __init__(self, X, T, rho, E, nu, thickness, gravity=(0.0, -9.81, 0.0), bend_stiff_mult=1.0, nh=True,
                 codim=None, tets=None):
        X = np.ascontiguousarray(X, np.float64)
        T = np.ascontiguousarray(T, np.int32).reshape(-1, 3)
        g = np.ascontiguousarray(gravity, np.float64)
        h = ctypes.c_void_p()
        if tets is not None:
            tt = np.ascontiguousarray(tets["tets"], np.int32).reshape(-1, 4)
            td = TetDesc(tt.shape[0], tt.ctypes.data, tets["E"], tets["nu"], tets["rho"])
            cdp = None
            if codim is not None:
                seg = np.ascontiguousarray(codim.get("segments", np.zeros((0, 2))), np.int32).reshape(-1, 2)
                par = np.ascontiguousarray(codim.get("particles", np.zeros(0)), np.int32).reshape(-1)
                cdp = ctypes.byref(CodimDesc(seg.shape[0], seg.ctypes.data if seg.size else None,
                                             codim.get("rod_E", 0.0), codim.get("rod_rho", 0.0),
                                             codim.get("rod_thickness", 0.0), codim.get("rod_bend_mult", 1.0),
                                             par.shape[0], par.ctypes.data if par.size else None,
                                             codim.get("particle_rho", 0.0), codim.get("particle_thickness", 0.0)))
            _check(lib().cipc_sim_create_full(X.shape[0], X.ctypes.data, T.shape[0], T.ctypes.data if T.size else None,
                                              rho, E, nu, thickness, g.ctypes.data, bend_stiff_mult, 1 if nh else 0,
                                              cdp, ctypes.byref(td), ctypes.byref(h)))
        elif codim is None:
            _check(lib().cipc_sim_create(X.shape[0], X.ctypes.data, T.shape[0], T.ctypes.data, rho, E, nu, thickness,
                                         g.ctypes.data, bend_stiff_mult, 1 if nh else 0, ctypes.byref(h)))
        else:
            seg = np.ascontiguousarray(codim.get("segments", np.zeros((0, 2))), np.int32).reshape(-1, 2)
            par = np.ascontiguousarray(codim.get("particles", np.zeros(0)), np.int32).reshape(-1)
            d = CodimDesc(seg.shape[0], seg.ctypes.data if seg.size else None, codim.get("rod_E", 0.0),
                          codim.get("rod_rho", 0.0), codim.get("rod_thickness", 0.0), codim.get("rod_bend_mult", 1.0),
                          par.shape[0], par.ctypes.data if par.size else None, codim.get("particle_rho", 0.0),
                          codim.get("particle_thickness", 0.0))
            _check(lib().cipc_sim_create_codim(X.shape[0], X.ctypes.data, T.shape[0], T.ctypes.data, rho, E, nu,
                                               thickness, g.ctypes.data, bend_stiff_mult, 1 if nh else 0,
                                               ctypes.byref(d), ctypes.byref(h)))
        self.h = h
        self.nv = X.shape[0]

    def close(self):
        if self.h:
            lib().cipc_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_oipc(self, dhat, stiff_mult=1.0):
        k2 = np.zeros(2)
        d2 = ctypes.c_double()
        _check(lib().cipc_sim_init_oipc(self.h, dhat, stiff_mult, k2.ctypes.data, ctypes.byref(d2)))
        return k2, d2.value

    def init_eipc(self, E, nu, thickness, dt):
        """Initialize_EIPC: returns (kappa3, dhat2) and sets the simulation's kappa."""
        k3 = np.zeros(3)
        d2 = ctypes.c_double()
        _check(lib().cipc_sim_init_eipc(self.h, E, nu, thickness, dt, k3.ctypes.data, ctypes.byref(d2)))
        return k3, d2.value

    def set_kappa(self, kappa, kappa_max):
        _check(lib().cipc_sim_set_kappa(self.h, kappa, kappa_max))

    def kappa(self):
        k2 = np.zeros(2)
        _check(lib().cipc_sim_get_kappa(self.h, k2.ctypes.data))
        return k2

    def init_dirichlet(self, rel_min, rel_max, v=(0.0, 0.0, 0.0), rot_center=(0.0, 0.0, 0.0),
                       rot_axis=(0.0, 1.0, 0.0), ang_vel_deg=0.0, v_begin=0, v_end=-1):
        """FEM.Init_Dirichlet: appends a moving Dirichlet group; returns its size."""
        arr = [np.ascontiguousarray(a, np.float64).reshape(3) for a in (rel_min, rel_max, v, rot_center, rot_axis)]
        added = ctypes.c_int()
        _check(lib().cipc_sim_init_dirichlet(self.h, *[a.ctypes.data for a in arr], float(ang_vel_deg), int(v_begin),
                                             int(v_end), ctypes.byref(added)))
        return added.value

    def step_dirichlet(self, dt):
        """FEM.Step_Dirichlet on the device."""
        _check(lib().cipc_sim_step_dirichlet(self.h, float(dt)))

    def dbc(self):
        n = ctypes.c_int()
        _check(lib().cipc_sim_get_dbc(self.h, 0, None, None, ctypes.byref(n)))
        idx = np.zeros(n.value, np.int32)
        tg = np.zeros((n.value, 3))
        _check(lib().cipc_sim_get_dbc(self.h, n.value, idx.ctypes.data, tg.ctypes.data, ctypes.byref(n)))
        return idx, tg

    def write_obj(self, path):
        _check(lib().cipc_sim_write_obj(self.h, str(path).encode()))

    def set_strain_limit(self, s, s_hat, kappa_s):
        """Isotropic strain limiting (the reference's s, sHat, kappa_s pairs)."""
        a, b, k = (np.ascontiguousarray(v, np.float64).reshape(2) for v in (s, s_hat, kappa_s))
        _check(lib().cipc_sim_set_strain_limit(self.h, a.ctypes.data, b.ctypes.data, k.ctypes.data))

    def strain_kappa(self):
        k2 = np.zeros(2)
        _check(lib().cipc_sim_get_strain_limit(self.h, k2.ctypes.data))
        return k2

    def set_state(self, x=None, v=None):
        xa = None if x is None else np.ascontiguousarray(x, np.float64)
        va = None if v is None else np.ascontiguousarray(v, np.float64)
        _check(lib().cipc_sim_set_state(self.h, None if xa is None else xa.ctypes.data,
                                        None if va is None else va.ctypes.data))

    def state(self):
        x = np.zeros((self.nv, 3))
        v = np.zeros((self.nv, 3))
        _check(lib().cipc_sim_get_state(self.h, x.ctypes.data, v.ctypes.data))
        return x, v

    def set_dbc(self, idx, targets):
        idx = np.ascontiguousarray(idx, np.int32)
        tg = np.ascontiguousarray(targets, np.float64)
        _check(lib().cipc_sim_set_dbc(self.h, idx.shape[0], idx.ctypes.data, tg.ctypes.data))

    def step(self, params, allow=()):
        st = StepStats()
        rc = lib().cipc_sim_step(self.h, ctypes.byref(params), ctypes.byref(st))
        _check(rc, allow)
        return st

    def step_split(self, params, allow=()):
        """Advance_One_Step_SIE_Hinge: elastodynamic substep, then the projection."""
        st = StepStats()
        rc = lib().cipc_sim_step_split(self.h, ctypes.byref(params), ctypes.byref(st))
        _check(rc, allow)
        return st

    def constraints(self, params, x, cap=1 << 20):
        out = np.zeros((cap, 6), np.int32)
        c = ctypes.c_int()
        xa = np.ascontiguousarray(x, np.float64)
        _check(lib().cipc_sim_constraints(self.h, ctypes.byref(params), xa.ctypes.data, cap, out.ctypes.data,
                                          ctypes.byref(c)))
        return out[:min(c.value, cap)].copy()

    def eval(self, params, x, xtilde):
        g = np.zeros((self.nv, 3))
        E = ctypes.c_double()
        xa = np.ascontiguousarray(x, np.float64)
        xt = np.ascontiguousarray(xtilde, np.float64)
        _check(lib().cipc_sim_eval(self.h, ctypes.byref(params), xa.ctypes.data, xt.ctypes.data, ctypes.byref(E),
                                   g.ctypes.data))
        return E.value, g

    def ccd(self, params, x, d, alpha=1.0):
        out = ctypes.c_double()
        xa = np.ascontiguousarray(x, np.float64)
        da = np.ascontiguousarray(d, np.float64)
        _check(lib().cipc_sim_ccd(self.h, ctypes.byref(params), xa.ctypes.data, da.ctypes.data, alpha,
                                  ctypes.byref(out)))
        return out.value


_c_u64 = ctypes.c_uint64
_SIGS.update({
    "cipc_precond_create": (_c_int, [_c_int, _c_int, _c_u64, _PP]),
    "cipc_precond_destroy": (_c_int, [_vp]),
    "cipc_precond_num_params": (_c_int, [_vp]),
    "cipc_precond_get_params": (_c_int, [_vp, _vp]),
    "cipc_precond_set_params": (_c_int, [_vp, _vp]),
    "cipc_precond_set_loss": (_c_int, [_vp, _c_int]),
    "cipc_precond_num_systems": (_c_int, [_vp]),
    "cipc_precond_clear_systems": (_c_int, [_vp]),
    "cipc_precond_train": (_c_int, [_vp, _c_int, _c_int, _c_dbl, _c_u64, _vp, _vp]),
    "cipc_precond_loss_grad": (_c_int, [_vp, _c_int, _vp, _vp]),
    "cipc_precond_system_sizes": (_c_int, [_vp, _c_int, _vp]),
    "cipc_precond_infer": (_c_int, [_vp, _c_int, _c_int, _vp, _vp]),
    "cipc_precond_system_export": (_c_int, [_vp, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "cipc_sim_capture_systems": (_c_int, [_vp, _vp, _c_int]),
    "cipc_sim_set_precond": (_c_int, [_vp, _vp]),
})
if _lib is not None:
    for _name in [k for k in _SIGS if k.startswith("cipc_precond") or k in ("cipc_sim_capture_systems",
                                                                               "cipc_sim_set_precond")]:
        _f = getattr(_lib, _name)
        _f.restype, _f.argtypes = _SIGS[_name]


class Precond:
    """Owns one cipc_precond handle (learned block-Jacobi correction)."""

    def __init__(self, hidden=32, layers=2, seed=0):
        h = ctypes.c_void_p()
        _check(lib().cipc_precond_create(hidden, layers, seed, ctypes.byref(h)))
        self.h = h
        self.hidden, self.layers = hidden, layers
        self.loss_kind = 2

    def close(self):
        if self.h:
            lib().cipc_precond_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def num_params(self):
        return lib().cipc_precond_num_params(self.h)

    def params(self):
        out = np.zeros(self.num_params(), np.float32)
        _check(lib().cipc_precond_get_params(self.h, out.ctypes.data))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.shape[0] == self.num_params()
        _check(lib().cipc_precond_set_params(self.h, p.ctypes.data))

    def num_systems(self):
        return lib().cipc_precond_num_systems(self.h)

    def set_loss(self, kind):
        _check(lib().cipc_precond_set_loss(self.h, kind))
        self.loss_kind = kind

    def clear_systems(self):
        _check(lib().cipc_precond_clear_systems(self.h))

    def train(self, epochs, batch=4, lr=1e-3, seed=0):
        b = ctypes.c_double()
        a = ctypes.c_double()
        _check(lib().cipc_precond_train(self.h, epochs, batch, lr, seed, ctypes.byref(b), ctypes.byref(a)))
        return b.value, a.value

    def loss_grad(self, system):
        loss = ctypes.c_double()
        g = np.zeros(self.num_params(), np.float32)
        _check(lib().cipc_precond_loss_grad(self.h, system, ctypes.byref(loss), g.ctypes.data))
        return loss.value, g

    def infer(self, system, bf16=True):
        sz = np.zeros(4, np.int32)
        _check(lib().cipc_precond_system_sizes(self.h, system, sz.ctypes.data))
        o = np.zeros((int(sz[0]), 6), np.float32)
        P = np.zeros((int(sz[0]), 3, 3), np.float32)
        _check(lib().cipc_precond_infer(self.h, system, 1 if bf16 else 0, o.ctypes.data, P.ctypes.data))
        return o, P

    def export_system(self, system):
        sz = np.zeros(4, np.int32)
        _check(lib().cipc_precond_system_sizes(self.h, system, sz.ctypes.data))
        nv, K, nc, nf = [int(v) for v in sz]
        out = dict(col=np.zeros((K, nv), np.int32), val=np.zeros((K, nv, 9), np.float32),
                   cdiag=np.zeros((nv, 9), np.float32), proj=np.zeros(nv, np.uint8),
                   ckind=np.zeros(nc, np.int32), cverts=np.zeros((nc, 4), np.int32),
                   chess=np.zeros((nc, 78), np.float32), rhs=np.zeros((nv, 3), np.float32),
                   sol=np.zeros((nv, 3), np.float32))
        _check(lib().cipc_precond_system_export(self.h, system, *[out[k].ctypes.data for k in (
            "col", "val", "cdiag", "proj", "ckind", "cverts", "chess", "rhs", "sol")]))
        out["n_friction"] = nf
        return out


def sim_capture_systems(sim, precond, max_systems):
    _check(lib().cipc_sim_capture_systems(sim.h, precond.h if precond is not None else None, max_systems))


def sim_set_precond(sim, precond):
    _check(lib().cipc_sim_set_precond(sim.h, precond.h if precond is not None else None))


_SIGS.update({
    "cipc_sim_set_output": (_c_int, [_vp, ctypes.c_char_p]),
    "cipc_sim_save_state": (_c_int, [_vp, ctypes.c_char_p]),
    "cipc_sim_load_state": (_c_int, [_vp, ctypes.c_char_p]),
    "cipc_sim_load_obj_frames": (_c_int, [_vp, ctypes.c_char_p, ctypes.c_char_p, _c_dbl]),
})
if _lib is not None:
    for _name in ("cipc_sim_set_output", "cipc_sim_save_state", "cipc_sim_load_state", "cipc_sim_load_obj_frames"):
        _f = getattr(_lib, _name)
        _f.restype, _f.argtypes = _SIGS[_name]


def _enc(p):
    return None if p is None else str(p).encode()


def sim_set_output(sim, folder):
    """Run logs (residual.txt, counter.txt, Hessian_info.txt, steps.jsonl) into folder; None stops."""
    _check(lib().cipc_sim_set_output(sim.h, _enc(folder)))


def sim_save_state(sim, path):
    _check(lib().cipc_sim_save_state(sim.h, _enc(path)))


def sim_load_state(sim, path):
    _check(lib().cipc_sim_load_state(sim.h, _enc(path)))


def sim_load_obj_frames(sim, obj_prev, obj_last, dt):
    _check(lib().cipc_sim_load_obj_frames(sim.h, _enc(obj_prev), _enc(obj_last), float(dt)))


_SIGS["cipc_scene_oipc_kappa"] = (_c_int, [_c_int, _vp, _c_int, _vp, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _vp, _c_dbl,
                                           _c_int, _vp, _vp, _c_dbl, _c_dbl, _vp, _vp])
if _lib is not None:
    _lib.cipc_scene_oipc_kappa.restype, _lib.cipc_scene_oipc_kappa.argtypes = _SIGS["cipc_scene_oipc_kappa"]


def scene_oipc_kappa(X, T, rho, E, nu, thickness, gravity, codim_desc, dhat, stiff_mult=1.0, bend_stiff_mult=1.0,
                     nh=True):
    """Offset-IPC stiffness (kappa, kappa_max) and dhat^2 of a scene description,
    computed on the host without a device (cipc_scene_oipc_kappa)."""
    X = np.ascontiguousarray(X, np.float64).reshape(-1, 3)
    T = np.ascontiguousarray(T, np.int32).reshape(-1, 3)
    g = np.ascontiguousarray(gravity, np.float64).reshape(3)
    k2 = np.zeros(2)
    d2 = ctypes.c_double()
    _check(lib().cipc_scene_oipc_kappa(X.shape[0], X.ctypes.data, T.shape[0], T.ctypes.data if T.size else None, rho, E,
                                       nu, thickness, g.ctypes.data, bend_stiff_mult, 1 if nh else 0,
                                       ctypes.byref(codim_desc) if codim_desc is not None else None, None, dhat,
                                       stiff_mult, k2.ctypes.data, ctypes.byref(d2)))
    return k2, d2.value

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
    # the ctypes pointer keeps a reference to the array, so a converted temporary
    # (``_p(_c(x, ...))``) stays alive for the duration of the call
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


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


class Shell:
    """The oracle's shell scene and time step (oracle_shell.cpp)."""

    def __init__(self, X, T, rho, E, nu, thickness, gravity=(0.0, -9.81, 0.0), bend_mult=1.0, nh=True, codim=None,
                 tets=None):
        L = lib()
        L.orc_shell_create.restype = _P
        L.orc_shell_create.argtypes = [ctypes.c_int, _P, ctypes.c_int, _P, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, _P, ctypes.c_double, ctypes.c_int]
        L.orc_shell_destroy.argtypes = [_P]
        L.orc_shell_counts.argtypes = [_P, _P]
        L.orc_shell_arrays.argtypes = [_P] + [_P] * 10
        L.orc_shell_oipc.restype = ctypes.c_double
        L.orc_shell_oipc.argtypes = [_P, ctypes.c_double, ctypes.c_double, _P]
        L.orc_shell_constraints.restype = ctypes.c_int
        L.orc_shell_constraints.argtypes = [_P, _P, _P, ctypes.c_int, ctypes.c_double, ctypes.c_double, _P,
                                            ctypes.c_int]
        L.orc_shell_eval.restype = ctypes.c_double
        L.orc_shell_eval.argtypes = [_P, _P, _P, _P, _P, _P, ctypes.c_int, _P, _P]
        L.orc_shell_ccd.restype = ctypes.c_double
        L.orc_shell_ccd.argtypes = [_P, _P, _P, ctypes.c_double, ctypes.c_double, _P, ctypes.c_int]
        L.orc_shell_step.restype = ctypes.c_int
        L.orc_shell_step.argtypes = [_P, _P, _P, _P, _P, _P, _P, ctypes.c_int, _P]
        self.L = L
        self.X = _c(X, np.float64)
        T = _c(T, np.int32)
        g = _c(gravity, np.float64)
        T = T.reshape(-1, 3)
        if tets is not None:
            L.orc_shell_create_full.restype = _P
            L.orc_shell_create_full.argtypes = [ctypes.c_int, _P, ctypes.c_int, _P, ctypes.c_double, ctypes.c_double,
                                                ctypes.c_double, ctypes.c_double, _P, ctypes.c_double, ctypes.c_int,
                                                ctypes.c_int, _P, ctypes.c_int, _P, _P, ctypes.c_int, _P, _P]
            cd = codim or {}
            seg = _c(cd.get("segments", np.zeros((0, 2))), np.int32).reshape(-1, 2)
            par = _c(cd.get("particles", np.zeros(0)), np.int32).reshape(-1)
            prm = np.array([cd.get("rod_E", 0.0), cd.get("rod_rho", 0.0), cd.get("rod_thickness", 0.0),
                            cd.get("rod_bend_mult", 1.0), cd.get("particle_rho", 0.0), cd.get("particle_thickness", 0.0)])
            tt = _c(tets["tets"], np.int32).reshape(-1, 4)
            tm = np.array([tets["E"], tets["nu"], tets["rho"]], float)
            self.h = L.orc_shell_create_full(self.X.shape[0], _p(self.X), T.shape[0], _p(T), rho, E, nu, thickness,
                                             _p(g), bend_mult, 1 if nh else 0, seg.shape[0], _p(seg), par.shape[0],
                                             _p(par), _p(prm) if codim is not None else None, tt.shape[0], _p(tt),
                                             _p(tm))
        elif codim is None:
            self.h = L.orc_shell_create(self.X.shape[0], _p(self.X), T.shape[0], _p(T), rho, E, nu, thickness, _p(g),
                                        bend_mult, 1 if nh else 0)
        else:
            L.orc_shell_create_codim.restype = _P
            L.orc_shell_create_codim.argtypes = [ctypes.c_int, _P, ctypes.c_int, _P, ctypes.c_double,
                                                 ctypes.c_double, ctypes.c_double, ctypes.c_double, _P,
                                                 ctypes.c_double, ctypes.c_int, ctypes.c_int, _P, ctypes.c_int, _P, _P]
            seg = _c(codim.get("segments", np.zeros((0, 2))), np.int32).reshape(-1, 2)
            par = _c(codim.get("particles", np.zeros(0)), np.int32).reshape(-1)
            prm = np.array([codim.get("rod_E", 0.0), codim.get("rod_rho", 0.0), codim.get("rod_thickness", 0.0),
                            codim.get("rod_bend_mult", 1.0), codim.get("particle_rho", 0.0),
                            codim.get("particle_thickness", 0.0)])
            self.h = L.orc_shell_create_codim(self.X.shape[0], _p(self.X), T.shape[0], _p(T), rho, E, nu, thickness,
                                              _p(g), bend_mult, 1 if nh else 0, seg.shape[0], _p(seg), par.shape[0],
                                              _p(par), _p(prm))
        self.nv = self.X.shape[0]
        self.dbc = np.zeros(0, np.int32)

    def __del__(self):
        try:
            self.L.orc_shell_destroy(self.h)
        except Exception:
            pass

    def arrays(self):
        c = np.zeros(5, np.int32)
        self.L.orc_shell_counts(self.h, _p(c))
        nt, nh, nbn, nbe, nbt = [int(v) for v in c]
        out = dict(tri=np.zeros((nt, 3), np.int32), P=np.zeros((nt, 3)), vol=np.zeros(nt),
                   hinge=np.zeros((nh, 4), np.int32), hinfo=np.zeros((nh, 3)), mass=np.zeros(self.nv),
                   b=np.zeros((self.nv, 3)), bnode=np.zeros(nbn, np.int32), bedge=np.zeros((nbe, 2), np.int32),
                   scal=np.zeros(3))
        self.L.orc_shell_arrays(self.h, *[_p(out[k]) for k in ("tri", "P", "vol", "hinge", "hinfo", "mass", "b",
                                                               "bnode", "bedge", "scal")])
        return out

    def init_oipc(self, dhat, stiff_mult=1.0):
        k2 = np.zeros(2)
        d2 = self.L.orc_shell_oipc(self.h, dhat, stiff_mult, _p(k2))
        return k2, d2

    def set_strain_limit(self, s, s_hat, kappa_s):
        self.L.orc_shell_set_strain_limit.argtypes = [ctypes.c_void_p, _P, _P, _P]
        self.L.orc_shell_set_strain_limit(self.h, _p(_c(s, np.float64)), _p(_c(s_hat, np.float64)),
                                          _p(_c(kappa_s, np.float64)))

    def strain_kappa(self):
        k2 = np.zeros(2)
        self.L.orc_shell_get_strain_limit.argtypes = [ctypes.c_void_p, _P]
        self.L.orc_shell_get_strain_limit(self.h, _p(k2))
        return k2

    def constraints(self, x, dhat2, xi, cap=1 << 20):
        out = np.zeros((cap, 6), np.int32)
        n = self.L.orc_shell_constraints(self.h, _p(_c(x, np.float64)), _p(self.dbc), len(self.dbc), dhat2, xi,
                                         _p(out), cap)
        return out[:min(n, cap)].copy()

    def eval(self, x, xtilde, dhat2, xi, kappa, h, mu=0.0, epsv2=1e-6, xbasis=None, xn=None, with_collision=True):
        g = np.zeros((self.nv, 3))
        prm = np.array([h, dhat2, xi, kappa, mu, epsv2, 1.0 if with_collision else 0.0])
        xb = None if xbasis is None else _c(xbasis, np.float64)
        xnn = _c(x if xn is None else xn, np.float64)
        E = self.L.orc_shell_eval(self.h, _p(_c(x, np.float64)), _p(_c(xtilde, np.float64)), _p(xb), _p(xnn),
                                  _p(self.dbc), len(self.dbc), _p(prm), _p(g))
        return E, g

    def ccd(self, x, d, alpha, xi):
        return self.L.orc_shell_ccd(self.h, _p(_c(x, np.float64)), _p(_c(d, np.float64)), alpha, xi, _p(self.dbc),
                                    len(self.dbc))

    def step(self, x, v, kappa2, dbc_idx, dbc_tgt, h, dhat2, xi, mu=0.0, epsv2=1e-6, fric_iters=1, tol=1e-2,
             with_collision=True, max_iter=500, elastic_ipc=False):
        """Advances x, v, kappa2 in place; returns (status, stats dict)."""
        prm = np.array([h, dhat2, xi, mu, epsv2, fric_iters, tol, 1.0 if with_collision else 0.0, max_iter,
                        1.0 if elastic_ipc else 0.0], float)
        st = np.zeros(4)
        idx = _c(dbc_idx, np.int32)
        tg = _c(dbc_tgt, np.float64)
        self.dbc = idx
        rc = self.L.orc_shell_step(self.h, _p(prm), _p(x), _p(v), _p(kappa2), _p(idx), _p(tg), len(idx), _p(st))
        return rc, dict(newton_iters=int(st[0]), n_constraints=int(st[1]), min_dist2=st[2], gd_iters=int(st[3]))

    def step_split(self, x, v, kappa2, dbc_idx, dbc_tgt, h, dhat2, xi, mu=0.0, epsv2=1e-6, fric_iters=1, tol=1e-2,
             with_collision=True, max_iter=500, elastic_ipc=False):
        """Split stepper (elastodynamic substep, then the projection); as step."""
        prm = np.array([h, dhat2, xi, mu, epsv2, fric_iters, tol, 1.0 if with_collision else 0.0, max_iter,
                        1.0 if elastic_ipc else 0.0], float)
        st = np.zeros(4)
        idx = _c(dbc_idx, np.int32)
        tg = _c(dbc_tgt, np.float64)
        self.dbc = idx
        self.L.orc_shell_step_split.restype = ctypes.c_int
        self.L.orc_shell_step_split.argtypes = self.L.orc_shell_step.argtypes
        rc = self.L.orc_shell_step_split(self.h, _p(prm), _p(x), _p(v), _p(kappa2), _p(idx), _p(tg), len(idx), _p(st))
        return rc, dict(newton_iters=int(st[0]), n_constraints=int(st[1]), min_dist2=st[2], gd_iters=int(st[3]))


def num_threads():
    return lib().orc_num_threads()


class LearnedSystem:
    """One Newton system in the learned preconditioner's terms (oracle_learned.cpp):
    ELL elastic blocks (K x nv, block k of row i at k*nv+i), the contact/friction
    part of the diagonal blocks, the Dirichlet mask and the contact blocks."""

    def __init__(self, col, val, cdiag, proj, ckind, cverts, chess):
        self.col = _c(col, np.int32)
        self.K = self.col.shape[0]
        self.nv = self.col.shape[1]
        self.val = _c(val, np.float32)
        self.cdiag = _c(cdiag, np.float32)
        self.proj = _c(proj, np.uint8)
        self.ckind = _c(ckind, np.int32)
        self.cverts = _c(cverts, np.int32)
        self.chess = _c(chess, np.float32)
        self.ncon = self.ckind.shape[0]


def _lp_sigs():
    L = lib()
    L.orc_lp_num_params.restype = ctypes.c_int
    L.orc_lp_num_params.argtypes = [ctypes.c_int, ctypes.c_int]
    L.orc_lp_features.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P, _P, _P, ctypes.c_int, _P, _P, _P, _P, _P]
    L.orc_lp_loss_grad.restype = ctypes.c_double
    L.orc_lp_loss_grad.argtypes = [ctypes.c_int, ctypes.c_int, _P, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P,
                                   ctypes.c_int, _P, _P, _P, _P, _P, _P, _P, ctypes.c_int]
    L.orc_lp_apply.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_int, _P, _P, _P, _P, _P]
    return L


def lp_num_params(hidden, layers):
    return _lp_sigs().orc_lp_num_params(hidden, layers)


def lp_features(S):
    L = _lp_sigs()
    x = np.zeros((S.nv, 10))
    a = np.zeros((S.K, S.nv))
    E = np.zeros((S.nv, 3, 3))
    L.orc_lp_features(S.nv, S.K, _p(S.col), _p(S.val), _p(S.cdiag), _p(S.proj), S.ncon, _p(S.ckind),
                      _p(S.cverts), _p(x), _p(a), _p(E))
    return x, a, E


def lp_loss_grad(hidden, layers, params, S, r, p, kind=0):
    """(loss, gradient, z) of one triple in double precision."""
    L = _lp_sigs()
    prm = _c(params, np.float64)
    g = np.zeros(prm.shape[0])
    z = np.zeros((S.nv, 3))
    loss = L.orc_lp_loss_grad(hidden, layers, _p(prm), S.nv, S.K, _p(S.col), _p(S.val), _p(S.cdiag), _p(S.proj),
                              S.ncon, _p(S.ckind), _p(S.cverts), _p(S.chess), _p(_c(r, np.float64)),
                              _p(_c(p, np.float64)), _p(g), _p(z), int(kind))
    return loss, g, z


def lp_apply(S, x):
    L = _lp_sigs()
    y = np.zeros((S.nv, 3))
    L.orc_lp_apply(S.nv, S.K, _p(S.col), _p(S.val), S.ncon, _p(S.ckind), _p(S.cverts), _p(S.chess),
                   _p(_c(x, np.float64)), _p(y))
    return y


def rod_spring(x6, L, K, project=True):
    """(E, g[6], H[6x6]) of a rod stretching segment, E = K L/2 (|x0-x1|/L - 1)^2."""
    lb = lib()
    lb.orc_rod_spring.restype = ctypes.c_double
    lb.orc_rod_spring.argtypes = [_P, ctypes.c_double, ctypes.c_double, _P, _P, ctypes.c_int]
    x = _c(x6, np.float64)
    g = np.zeros(6)
    H = np.zeros((6, 6))
    E = lb.orc_rod_spring(_p(x), L, K, _p(g), _p(H), 1 if project else 0)
    return E, g, H


def rod_bending(x9, lsum, Kb, project=True):
    """(E, g[9], H[9x9]) of a rod hinge, E = Kb |kb|^2 / lsum."""
    lb = lib()
    lb.orc_rod_bending.restype = ctypes.c_double
    lb.orc_rod_bending.argtypes = [_P, ctypes.c_double, ctypes.c_double, _P, _P, ctypes.c_int]
    x = _c(x9, np.float64)
    g = np.zeros(9)
    H = np.zeros((9, 9))
    E = lb.orc_rod_bending(_p(x), lsum, Kb, _p(g), _p(H), 1 if project else 0)
    return E, g, H


def dihedral_derivs(x12):
    """(gradient[12], Hessian[12x12]) of the signed dihedral angle of a hinge stencil."""
    lb = lib()
    lb.orc_dihedral_derivs.argtypes = [_P, _P, _P]
    g = np.zeros(12)
    H = np.zeros((12, 12))
    lb.orc_dihedral_derivs(_p(_c(x12, np.float64)), _p(g), _p(H))
    return g, H


def friction_scalars(x2, eh):
    """(f0, f1 / |u|, f2 term) of the friction mollifier at squared slip x2, eh = epsv h."""
    lb = lib()
    lb.orc_friction_scalars.argtypes = [ctypes.c_double, ctypes.c_double, _P]
    out = np.zeros(3)
    lb.orc_friction_scalars(x2, eh, _p(out))
    return out


def sl_barrier(s, lim, hat):
    """(value, d/ds, d2/ds2) of the strain-limiting barrier of one singular value."""
    lb = lib()
    lb.orc_sl_barrier.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, _P]
    out = np.zeros(3)
    lb.orc_sl_barrier(s, lim, hat, _p(out))
    return out


def strain_limit_elem(x9, P, kh, s, s_hat, kappa_s, project=True):
    """(E, g[9], H[9x9], valid) of the strain-limiting barrier of one triangle;
    P the inverse rest first fundamental form (p00, p01, p11), kh = h^2 vol."""
    lb = lib()
    lb.orc_sl_elem.restype = ctypes.c_double
    lb.orc_sl_elem.argtypes = [_P, _P, ctypes.c_double, _P, _P, _P, ctypes.c_int, _P, _P, _P]
    g = np.zeros(9)
    H = np.zeros((9, 9))
    ok = np.zeros(1, np.int32)
    E = lb.orc_sl_elem(_p(_c(x9, np.float64)), _p(_c(P, np.float64)), kh, _p(_c(s, np.float64)),
                       _p(_c(s_hat, np.float64)), _p(_c(kappa_s, np.float64)), 1 if project else 0, _p(g), _p(H),
                       _p(ok))
    return E, g, H, bool(ok[0])


def tet_nh_elem(x12, Dinv, w, lam, mu, project=True):
    """(E, g[12], H[12x12], valid) of one Neo-Hookean tetrahedron, w = h^2 vol."""
    lb = lib()
    lb.orc_tet_nh.restype = ctypes.c_double
    lb.orc_tet_nh.argtypes = [_P, _P, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, _P, _P, _P]
    g = np.zeros(12)
    H = np.zeros((12, 12))
    ok = np.zeros(1, np.int32)
    E = lb.orc_tet_nh(_p(_c(x12, np.float64)), _p(_c(Dinv, np.float64)), w, lam, mu, 1 if project else 0, _p(g),
                      _p(H), _p(ok))
    return E, g, H, bool(ok[0])

"""Split stepper (Advance_One_Step_SIE_Discrete_Shell, Library/FEM/Shell/
SPLITTING_IE.h:362-729) in the GPU, against the oracle's restatement through the
C ABI: an implicit-Euler substep without contact and strain limiting, then the
projection minimising 1/2 |x - x'|_M^2 + strain-limit barrier + contact barrier +
friction from x^n.

Scene: the shell tests' 8x8 cloth (0.5 m, E 1e3 so that it stretches, rho 200,
1 mm) 5 mm above a fixed box, strain limit s = 1.01 (s_hat 1, kappa_s 1e3),
xi = dhat = 1 mm, mu 0.2, dt 0.02.

Bars: positions after steps solved to a tight Newton tolerance (1e-7) within
2 sqrt(free vertices) tol h of the oracle's direct-solve Newton (both substeps
stop on the RMS-step test); every step intersection free; every stretch below
the limit.
"""
import numpy as np
import pytest

import cipc_ffi as F
import workloads as W

pytestmark = pytest.mark.gpu

MAT = dict(rho=200.0, E=1e3, nu=0.3, thickness=1e-3)
SL = dict(s=[1.01, 0.0], s_hat=[1.0, 1.0], kappa_s=[1e3, 0.0])
XI, DHAT, DT = 1e-3, 1e-3, 0.02


def scene():
    cl = W.cloth_grid(8, 8, 0.5, 0.5, y=-0.095, origin=(-0.25, -0.25))
    bx = W.box_shell(0.3, (0.0, -0.25, 0.0), nsub=2)
    X, T, offs = W.merge_meshes(cl, bx)
    return X, T, np.arange(offs[1], X.shape[0], dtype=np.int32), cl[1]


def max_stretch(X, T, x):
    out = 0.0
    for t in T:
        A = np.column_stack([x[t[1]] - x[t[0]], x[t[2]] - x[t[0]]])
        Ab = np.column_stack([X[t[1]] - X[t[0]], X[t[2]] - X[t[0]]])
        Fm = A @ np.linalg.inv(np.linalg.cholesky(Ab.T @ Ab).T)
        out = max(out, np.linalg.svd(Fm, compute_uv=False)[0])
    return out


def test_split_steps_match_direct_solve(cuda, orc):
    X, T, dbc, Tcl = scene()
    sh = orc.Shell(X, T, **MAT)
    sh.set_strain_limit(SL["s"], SL["s_hat"], SL["kappa_s"])
    k2, dhat2 = sh.init_oipc(DHAT)
    s = F.Sim(X, T, MAT["rho"], MAT["E"], MAT["nu"], MAT["thickness"])
    s.set_dbc(dbc, X[dbc])
    prm = F.make_params(DT, dhat2, XI, mu=0.2, newton_tol=1e-7, pcg_tol=1e-12, max_newton_iters=400)
    bar = 2 * np.sqrt(X.shape[0] - len(dbc)) * 1e-7 * DT
    xo, vo = X.copy(), np.zeros_like(X)
    contact = 0
    for step in range(5):
        s.set_state(xo, vo)
        s.set_kappa(k2[0], k2[1])
        s.set_strain_limit(SL["s"], SL["s_hat"], sh.strain_kappa())
        rc, sto = sh.step_split(xo, vo, k2, dbc, X[dbc], DT, dhat2, XI, mu=0.2, tol=1e-7, max_iter=400)
        assert rc == 0
        stg = s.step_split(prm)
        xg, vg = s.state()
        assert stg.min_dist2 > 0 or stg.n_constraints == 0
        contact += stg.n_constraints > 0
        assert max_stretch(X, Tcl, xg[:64]) < SL["s"][0]
        err = np.abs(xg - xo).max()
        assert err <= bar, (step, err, bar, sto, stg.as_dict())
        assert np.abs(vg - vo).max() <= bar / DT * 2
    assert contact >= 2

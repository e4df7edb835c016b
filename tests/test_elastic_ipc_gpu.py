"""Elastic IPC (Advance_One_Step_IE_Hinge_EIPC / Initialize_EIPC,
Library/FEM/Shell/DISCRETE_SHELL.h:555-577, 1102, 1110): no contact offset, the
barrier normalised by dhat (Math/BARRIER.h:9-62, elastic branch), kappa =
h^2 mu of the plane-stress material and never adapted.  GPU step against the
oracle through the C ABI.

Scene: the shell tests' 8x8 cloth (0.5 m) 5 mm above a fixed box, E 1e5,
rho 200, 1 mm; dhat = thickness = 1 mm, dt 0.04.

Bars: Initialize_EIPC values exact; constraint sets equal as sets; incremental
potential 1e-10 relative, gradient 1e-10 relative plus 1e-13 (the rounding level
of the elastic gradients at rest); positions after steps solved to a tight
Newton tolerance (1e-7) within 2 sqrt(free vertices) tol h of the oracle's
direct-solve Newton (each loop stops once its RMS step is at most tol h; the
soft elastic barrier, kappa = h^2 mu, makes these systems ill-conditioned, ~60
Newton iterations, so the two stopping points differ at that level); every step intersection free; kappa unchanged."""
import numpy as np
import pytest

import cipc_ffi as F
import workloads as W

pytestmark = pytest.mark.gpu

E, NU, RHO, T_SHELL, DT = 1e5, 0.3, 200.0, 1e-3, 0.04


def scene():
    cl = W.cloth_grid(8, 8, 0.5, 0.5, y=-0.095, origin=(-0.25, -0.25))
    bx = W.box_shell(0.3, (0.0, -0.25, 0.0), nsub=2)
    X, T, offs = W.merge_meshes(cl, bx)
    return X, T, np.arange(offs[1], X.shape[0], dtype=np.int32)


def _kappa():
    lam, mu = E * NU / (1 - NU * NU), E / (2 * (1 + NU))
    return np.array([DT * DT * mu, DT * DT * lam])


def test_elastic_ipc_steps_match_direct_solve(cuda, orc):
    X, T, dbc = scene()
    sh = orc.Shell(X, T, RHO, E, NU, T_SHELL)
    s = F.Sim(X, T, RHO, E, NU, T_SHELL)
    s.set_dbc(dbc, X[dbc])
    k3, dhat2 = s.init_eipc(E, NU, T_SHELL, DT)
    k2 = _kappa()
    assert dhat2 == T_SHELL * T_SHELL and np.array_equal(k3[:2], k2) and k3[2] == NU
    prm = F.make_params(DT, dhat2, 0.0, newton_tol=1e-7, pcg_tol=1e-12, max_newton_iters=400, elastic_ipc=True)
    bar = 2 * np.sqrt(X.shape[0] - len(dbc)) * 1e-7 * DT
    xo, vo = X.copy(), np.zeros_like(X)
    sh.dbc = dbc
    rng = np.random.default_rng(0)
    contact = 0
    for step in range(5):
        s.set_state(xo, vo)
        s.set_kappa(k2[0], k2[1])
        # constraint sets and the potential at the oracle's state
        cg = sorted(map(tuple, s.constraints(prm, xo).tolist()))
        co = sorted(map(tuple, sh.constraints(xo, dhat2, 0.0).tolist()))
        assert cg == co, step
        xt = xo + rng.standard_normal(xo.shape) * 1e-3
        Eg, gg = s.eval(prm, xo, xt)
        Eo, go = sh.eval(xo, xt, dhat2, 0.0, k2[0] / (dhat2 * dhat2), DT)
        assert abs(Eg - Eo) <= 1e-10 * abs(Eo), (step, Eg, Eo)
        assert np.abs(gg - go).max() <= 1e-10 * np.abs(go).max() + 1e-13, step
        # one step each
        rc, sto = sh.step(xo, vo, k2, dbc, X[dbc], DT, dhat2, 0.0, tol=1e-7, max_iter=400, elastic_ipc=True)
        assert rc == 0
        stg = s.step(prm)
        xg, _ = s.state()
        assert stg.min_dist2 > 0 or stg.n_constraints == 0
        contact += stg.n_constraints > 0
        assert np.abs(xg - xo).max() <= bar, (step, np.abs(xg - xo).max(), sto, stg.as_dict())
        assert np.array_equal(s.kappa(), k2) and np.array_equal(k2, _kappa())
    assert contact >= 2

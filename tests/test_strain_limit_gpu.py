"""Isotropic strain limiting (Library/FEM/Shell/INEXT.h; stiffness update
IMPLICIT_EULER.h:606-645; feasibility-first line search :74-94) in the GPU time
step, against the oracle (oracle_sl.cpp, oracle_shell.cpp) through the C ABI.

Scene: a 10x10 cloth (0.3 m, E 1e3, rho 200, 1 mm) hanging from two corners
under gravity, dt 0.01, no contact; stretches limited to s = 1.005 with the
barrier active above s_hat = 1 and a weak initial kappa_s = 1e-2, so the cloth
presses against the limit and kappa_s doubles within the first steps.

Bars: incremental potential and gradient 1e-10 relative; positions after steps
solved to a tight Newton tolerance within 1e-8 of the bounding-box diagonal of
the oracle's direct-solve Newton; kappa_s equal; every triangle's stretch below
the limit after every step.
"""
import numpy as np
import pytest

import cipc_ffi as F
import workloads as W

pytestmark = pytest.mark.gpu

N, SIZE, DT = 10, 0.3, 0.01
MAT = dict(rho=200.0, E=1e3, nu=0.3, thickness=1e-3)
SL = dict(s=[1.005, 0.0], s_hat=[1.0, 1.0], kappa_s=[1e-2, 0.0])


def scene():
    X, T = W.cloth_grid(N, N, SIZE, SIZE, y=0.0, origin=(-SIZE / 2, -SIZE / 2))
    return X, T, np.array([0, N - 1], np.int32)


def max_stretch(X, T, x):
    out = 0.0
    for t in T:
        A = np.column_stack([x[t[1]] - x[t[0]], x[t[2]] - x[t[0]]])
        Ab = np.column_stack([X[t[1]] - X[t[0]], X[t[2]] - X[t[0]]])
        Fm = A @ np.linalg.inv(np.linalg.cholesky(Ab.T @ Ab).T)
        out = max(out, np.linalg.svd(Fm, compute_uv=False)[0])
    return out


@pytest.fixture(scope="module")
def trajectory(orc):
    X, T, dbc = scene()
    sh = orc.Shell(X, T, **MAT)
    sh.set_strain_limit(SL["s"], SL["s_hat"], SL["kappa_s"])
    k2, dhat2 = sh.init_oipc(1e-3)
    x, v = X.copy(), np.zeros_like(X)
    states, ks = [x.copy()], [sh.strain_kappa().copy()]
    for _ in range(6):
        rc, st = sh.step(x, v, k2, dbc, X[dbc], DT, dhat2, 1e-3, tol=1e-6, with_collision=False)
        assert rc == 0
        states.append(x.copy())
        ks.append(sh.strain_kappa().copy())
    assert ks[-1][0] > SL["kappa_s"][0]  # the stiffness update fired
    return dict(X=X, T=T, dbc=dbc, states=states, ks=ks, dhat2=dhat2, shell=sh)


def _gpu(X, T, dbc, kappa_s):
    s = F.Sim(X, T, MAT["rho"], MAT["E"], MAT["nu"], MAT["thickness"])
    s.set_dbc(dbc, X[dbc])
    s.set_strain_limit(SL["s"], SL["s_hat"], kappa_s)
    return s


def test_strain_limit_energy_gradient_match(cuda, trajectory):
    t = trajectory
    rng = np.random.default_rng(0)
    t["shell"].dbc = t["dbc"]
    for k, (x, ks) in enumerate(zip(t["states"], t["ks"])):
        s = _gpu(t["X"], t["T"], t["dbc"], ks)
        t["shell"].set_strain_limit(SL["s"], SL["s_hat"], ks)
        xt = x + rng.standard_normal(x.shape) * 1e-5
        prm = F.make_params(DT, t["dhat2"], 1e-3, with_collision=False)
        Eg, gg = s.eval(prm, x, xt)
        Eo, go = t["shell"].eval(x, xt, t["dhat2"], 1e-3, 1.0, DT, with_collision=False)
        assert abs(Eg - Eo) <= 1e-10 * abs(Eo) + 1e-15, (k, Eg, Eo)
        assert np.abs(gg - go).max() <= 1e-10 * np.abs(go).max() + 1e-15, (k, np.abs(gg - go).max())
        s.close()


def test_strain_limit_steps_match_direct_solve(cuda, orc):
    X, T, dbc = scene()
    sh = orc.Shell(X, T, **MAT)
    sh.set_strain_limit(SL["s"], SL["s_hat"], SL["kappa_s"])
    k2, dhat2 = sh.init_oipc(1e-3)
    s = _gpu(X, T, dbc, SL["kappa_s"])
    xo, vo = X.copy(), np.zeros_like(X)
    prm = F.make_params(DT, dhat2, 1e-3, with_collision=False, newton_tol=1e-7, pcg_tol=1e-12,
                        max_newton_iters=400)
    diag = np.linalg.norm(X.max(0) - X.min(0))
    raised = False
    for step in range(6):
        s.set_state(xo, vo)
        s.set_strain_limit(SL["s"], SL["s_hat"], sh.strain_kappa())
        rc, sto = sh.step(xo, vo, k2, dbc, X[dbc], DT, dhat2, 1e-3, tol=1e-7, with_collision=False, max_iter=400)
        assert rc == 0
        s.step(prm)
        xg, _ = s.state()
        err = np.abs(xg - xo).max()
        assert err <= 1e-8 * diag, (step, err, sto)
        assert np.array_equal(s.strain_kappa(), sh.strain_kappa()), (step, s.strain_kappa(), sh.strain_kappa())
        raised |= sh.strain_kappa()[0] > SL["kappa_s"][0]
        assert max_stretch(X, T, xg) < SL["s"][0]
    assert raised

"""Volumetric Neo-Hookean tetrahedra in the GPU time step (tet element, lumped
mass, surface triangles in contact, inversion-free line search), against the
oracle (oracle_tet.cpp, oracle_shell.cpp tet_init / tet_terms) through the C ABI.

Scene: a 0.1 m cube of 3^3 cells x 6 tetrahedra (E 1e5, nu 0.3, rho 1000) 4 mm
above an 8x8 cloth (0.4 m) held fixed as a floor; xi = dhat = 1 mm, dt 0.01.

Bars: constraint sets equal as sets; incremental potential and gradient 1e-10
relative; positions after steps solved to a tight Newton tolerance within 1e-8
of the bounding-box diagonal of the oracle's direct-solve Newton; every step
intersection free with no inverted tetrahedron.
"""
import numpy as np
import pytest

import cipc_ffi as F
import workloads as W

pytestmark = pytest.mark.gpu

SHELL = dict(rho=200.0, E=1e5, nu=0.3, thickness=1e-3)
TETMAT = dict(E=1e5, nu=0.3, rho=1000.0)
XI, DHAT, DT = 1e-3, 1e-3, 0.01


def scene():
    fl = W.cloth_grid(8, 8, 0.4, 0.4, y=0.0, origin=(-0.2, -0.2))
    Xt, tets = W.tet_box(n=3, size=0.1, center=(0.0, 0.054, 0.0))
    X = np.concatenate([fl[0], Xt])
    tets = (tets + fl[0].shape[0]).astype(np.int32)
    return X, fl[1], dict(TETMAT, tets=tets), np.arange(64, dtype=np.int32)


def min_det(X, tets, x):
    out = np.inf
    for t in tets:
        Dm = np.column_stack([X[t[1]] - X[t[0]], X[t[2]] - X[t[0]], X[t[3]] - X[t[0]]])
        Ds = np.column_stack([x[t[1]] - x[t[0]], x[t[2]] - x[t[0]], x[t[3]] - x[t[0]]])
        out = min(out, np.linalg.det(Ds) / np.linalg.det(Dm))
    return out


@pytest.fixture(scope="module")
def trajectory(orc):
    X, T, tets, dbc = scene()
    sh = orc.Shell(X, T, **SHELL, tets=tets)
    k2, dhat2 = sh.init_oipc(DHAT)
    x, v = X.copy(), np.zeros_like(X)
    states = [x.copy()]
    for _ in range(8):
        rc, st = sh.step(x, v, k2, dbc, X[dbc], DT, dhat2, XI, tol=1e-2)
        assert rc == 0
        states.append(x.copy())
    return dict(X=X, T=T, tets=tets, dbc=dbc, states=states, dhat2=dhat2, kappa=k2.copy(), shell=sh)


def _gpu(t):
    s = F.Sim(t["X"], t["T"], SHELL["rho"], SHELL["E"], SHELL["nu"], SHELL["thickness"], tets=t["tets"])
    s.set_dbc(t["dbc"], t["X"][t["dbc"]])
    return s


def test_tet_constraint_sets_match(cuda, trajectory):
    t = trajectory
    s = _gpu(t)
    prm = F.make_params(DT, t["dhat2"], XI)
    t["shell"].dbc = t["dbc"]
    seen = 0
    for k, x in enumerate(t["states"]):
        cg = sorted(map(tuple, s.constraints(prm, x).tolist()))
        co = sorted(map(tuple, t["shell"].constraints(x, t["dhat2"], XI).tolist()))
        assert cg == co, k
        seen += len(cg) > 0
    assert seen >= 2
    s.close()


def test_tet_energy_gradient_match(cuda, trajectory):
    t = trajectory
    s = _gpu(t)
    rng = np.random.default_rng(0)
    t["shell"].dbc = t["dbc"]
    for k, x in enumerate(t["states"]):
        xt = x + rng.standard_normal(x.shape) * 1e-4
        s.set_kappa(t["kappa"][0], t["kappa"][1])
        prm = F.make_params(DT, t["dhat2"], XI)
        Eg, gg = s.eval(prm, x, xt)
        Eo, go = t["shell"].eval(x, xt, t["dhat2"], XI, t["kappa"][0], DT)
        assert abs(Eg - Eo) <= 1e-10 * abs(Eo), (k, Eg, Eo)
        assert np.abs(gg - go).max() <= 1e-10 * np.abs(go).max(), (k, np.abs(gg - go).max())
    s.close()


def test_tet_steps_match_direct_solve(cuda, orc):
    X, T, tets, dbc = scene()
    sh = orc.Shell(X, T, **SHELL, tets=tets)
    k2o, dhat2 = sh.init_oipc(DHAT)
    s = _gpu(dict(X=X, T=T, tets=tets, dbc=dbc))
    k2g, dhat2g = s.init_oipc(DHAT)
    assert np.allclose(k2o, k2g, rtol=1e-12) and dhat2 == dhat2g
    xo, vo = X.copy(), np.zeros_like(X)
    prm = F.make_params(DT, dhat2, XI, newton_tol=1e-7, pcg_tol=1e-12, max_newton_iters=400)
    diag = np.linalg.norm(X.max(0) - X.min(0))
    contact = 0
    for step in range(6):
        s.set_state(xo, vo)
        s.set_kappa(k2o[0], k2o[1])
        rc, sto = sh.step(xo, vo, k2o, dbc, X[dbc], DT, dhat2, XI, tol=1e-7, max_iter=400)
        assert rc == 0
        stg = s.step(prm)
        xg, _ = s.state()
        assert stg.min_dist2 > 0 or stg.n_constraints == 0
        contact += stg.n_constraints > 0
        assert min_det(X, tets["tets"], xg) > 0
        err = np.abs(xg - xo).max()
        assert err <= 1e-8 * diag, (step, err, sto, stg.as_dict())
    assert contact >= 2
    s.close()

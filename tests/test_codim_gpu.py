"""Rods and particles (codimensional primitives) in the GPU time step, against the
oracle (oracle_shell.cpp codim_init / rod_terms / codimensional constraint set
and step size), through the C ABI.

Scene (a small instance of the mixed codimensional configuration): an 8x8 cloth
(0.4 m) held fixed as a floor, three straight rods of five segments lying just
above it at staggered heights, six particles stacked above; rods E 1e7, 2 mm,
rho 1000; particles 4 mm, rho 1000; cloth as in the shell tests; xi = dhat = 1 mm,
dt 0.01.

Bars: constraint sets equal as sets; incremental potential and gradient 1e-10
relative; step size 1e-12 relative; positions after steps solved to a tight
Newton tolerance within 1e-8 of the bounding-box diagonal of the oracle's
direct-solve Newton; every step intersection free.
"""
import numpy as np
import pytest

import cipc_ffi as F
import workloads as W

pytestmark = pytest.mark.gpu

MAT = dict(rho=200.0, E=1e5, nu=0.3, thickness=1e-3)
CODIM = dict(rod_E=1e7, rod_rho=1000.0, rod_thickness=2e-3, rod_bend_mult=1.0, particle_rho=1000.0,
             particle_thickness=4e-3)
XI, DHAT, DT = 1e-3, 1e-3, 0.01


def scene():
    X, T, S, P, corners = W.rods_particles_on_cloth(n_rods=3, seg_per_rod=5, rod_len=0.2, n_particles=6, cloth_n=8,
                                                    cloth_size=0.4, layer_gap=2.5e-3, particle_gap=6e-3,
                                                    lift=0.004)
    codim = dict(CODIM, segments=S, particles=P)
    floor = np.arange(8 * 8, dtype=np.int32)  # the cloth, fixed
    return X, T, codim, floor


def _rows(c):
    return sorted(map(tuple, c.tolist()))


@pytest.fixture(scope="module")
def trajectory(orc):
    X, T, codim, dbc = scene()
    sh = orc.Shell(X, T, **MAT, codim=codim)
    k2, dhat2 = sh.init_oipc(DHAT)
    x = X.copy()
    v = np.zeros_like(X)
    states = [x.copy()]
    for _ in range(8):
        rc, st = sh.step(x, v, k2, dbc, X[dbc], DT, dhat2, XI, tol=1e-2)
        assert rc == 0
        states.append(x.copy())
    return dict(X=X, T=T, codim=codim, dbc=dbc, states=states, dhat2=dhat2, kappa=k2.copy(), shell=sh)


def _gpu(t):
    s = F.Sim(t["X"], t["T"], MAT["rho"], MAT["E"], MAT["nu"], MAT["thickness"], codim=t["codim"])
    s.set_dbc(t["dbc"], t["X"][t["dbc"]])
    return s


def test_codim_constraint_sets_match(cuda, trajectory):
    t = trajectory
    s = _gpu(t)
    prm = F.make_params(DT, t["dhat2"], XI)
    t["shell"].dbc = t["dbc"]
    seen = set()
    for x in t["states"]:
        go = _rows(t["shell"].constraints(x, t["dhat2"], XI))
        gg = _rows(s.constraints(prm, x))
        assert gg == go
        seen.update(r[0] for r in go)
    assert len(seen) >= 2  # the trajectory reaches contact of more than one kind


def test_codim_energy_gradient_match(cuda, trajectory):
    t = trajectory
    s = _gpu(t)
    rng = np.random.default_rng(0)
    t["shell"].dbc = t["dbc"]
    for k, x in enumerate(t["states"]):
        xt = x + rng.standard_normal(x.shape) * 1e-4
        kappa = t["kappa"][0]
        s.set_kappa(kappa, t["kappa"][1])
        prm = F.make_params(DT, t["dhat2"], XI)
        Eg, gg = s.eval(prm, x, xt)
        Eo, go = t["shell"].eval(x, xt, t["dhat2"], XI, kappa, DT)
        assert abs(Eg - Eo) <= 1e-10 * abs(Eo) + 1e-15, (k, Eg, Eo)
        assert np.abs(gg - go).max() <= 1e-9 * np.abs(go).max(), (k, np.abs(gg - go).max())


def test_codim_ccd_step_size_matches(cuda, trajectory):
    t = trajectory
    s = _gpu(t)
    prm = F.make_params(DT, t["dhat2"], XI)
    t["shell"].dbc = t["dbc"]
    for k in range(len(t["states"]) - 1):
        x = t["states"][k]
        d = 4.0 * (t["states"][k + 1] - x)
        d[t["dbc"]] = 0
        ag = s.ccd(prm, x, d, 1.0)
        ao = t["shell"].ccd(x, d, 1.0, XI)
        assert abs(ag - ao) <= 1e-12 * max(ao, 1e-300), (k, ag, ao)


@pytest.mark.parametrize("precond", [F.PRECOND_BLOCK_JACOBI, F.PRECOND_AGGREGATE])
def test_codim_steps_match_direct_solve(cuda, orc, precond):
    """The aggregate preconditioner's rod aggregates and its pack of the isolated
    particles (3x3 blocks only) change PCG iteration counts, not the solution."""
    X, T, codim, dbc = scene()
    sh = orc.Shell(X, T, **MAT, codim=codim)
    k2o, dhat2 = sh.init_oipc(DHAT)
    t = dict(X=X, T=T, codim=codim, dbc=dbc)
    s = _gpu(t)
    k2g, dhat2g = s.init_oipc(DHAT)
    assert np.allclose(k2o, k2g, rtol=1e-12) and dhat2 == dhat2g
    xo = X.copy()
    vo = np.zeros_like(X)
    prm = F.make_params(DT, dhat2, XI, newton_tol=1e-7, pcg_tol=1e-12, max_newton_iters=400,
                        preconditioner=precond)
    diag = np.linalg.norm(X.max(0) - X.min(0))
    for step in range(6):
        s.set_state(xo, vo)
        s.set_kappa(k2o[0], k2o[1])
        rc, sto = sh.step(xo, vo, k2o, dbc, X[dbc], DT, dhat2, XI, tol=1e-7, max_iter=400)
        assert rc == 0
        stg = s.step(prm)
        xg, _ = s.state()
        assert stg.min_dist2 > 0 or stg.n_constraints == 0
        err = np.abs(xg - xo).max()
        assert err <= 1e-8 * diag, (step, err, sto, stg.as_dict())
        assert stg.precond_fallbacks == 0  # the aggregate solves ran as aggregate solves

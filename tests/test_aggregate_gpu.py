"""Aggregate block-Jacobi preconditioner (CIPC_PRECOND_AGGREGATE): exact inverses
of the diagonal blocks of vertex aggregates of up to 32 mesh neighbours.

Checks, on a draped cloth-on-sphere scene (60x60 cloth, contact and friction):
  * from the same state, three Newton iterations solved with aggregate block Jacobi
    end where they end with block Jacobi (tight PCG tolerance: the preconditioner
    changes iteration counts, not the solution), in FP64 and in mixed precision;
  * it needs fewer PCG iterations than block Jacobi (the reason it exists), and
    no solve falls back to block Jacobi.
"""
import numpy as np
import pytest

import cipc_ffi as F
import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def draped():
    X, T, dbc, c = W.cloth_on_sphere(n=60)
    s = F.Sim(X, T, 200.0, 1e5, 0.3, 1e-3)
    _, dhat2 = s.init_oipc(1e-3)
    prm = F.make_params(0.02, dhat2, 5e-4, mu=0.4, epsv2=1e-6, fric_iters=1, newton_tol=1e-3, precision=F.FP64,
                        pcg_tol=1e-6)
    for k in range(30):
        s.set_dbc(dbc, W.rotate_y(X[dbc], c, 2.0 * 0.02 * (k + 1)))
        s.step(prm, allow=(F.CIPC_ERR_NOT_CONVERGED,))
    x, v = s.state()
    kap = s.kappa()
    s.close()
    return X, T, dbc, c, x, v, kap


def _step(draped, precision, precond, newton_tol, pcg_tol, max_newton=200):
    X, T, dbc, c, x, v, kap = draped
    s = F.Sim(X, T, 200.0, 1e5, 0.3, 1e-3)
    _, dhat2 = s.init_oipc(1e-3)
    s.set_state(x, v)
    s.set_kappa(kap[0], kap[1])
    s.set_dbc(dbc, W.rotate_y(X[dbc], c, 2.0 * 0.02 * 31))
    prm = F.make_params(0.02, dhat2, 5e-4, mu=0.4, epsv2=1e-6, fric_iters=1, newton_tol=newton_tol,
                        precision=precision, pcg_tol=pcg_tol, preconditioner=precond, max_newton_iters=max_newton)
    st = s.step(prm, allow=(F.CIPC_ERR_NOT_CONVERGED,))
    out = s.state()[0]
    s.close()
    return st, out


@pytest.mark.parametrize("precision", [F.FP64, F.MIXED])
def test_aggregate_steps_match_block_jacobi(cuda, draped, precision):
    """The first three Newton iterations of a step (each linear solve to a relative
    residual of 1e-10) with aggregate block Jacobi end where they end with block
    Jacobi.  Bar: 1e-7 of the bounding-box diagonal plus twice the spread of two
    block-Jacobi runs (gradient and Hessian are summed with atomics, so two runs
    differ in their last bits).  Two solves that each reach a relative residual of
    1e-10 differ by up to cond(H) x 1e-10 relative in the solution, and the
    contact-stiffened Newton systems here have cond(H) ~ 1e5-1e6: the FP64 runs
    end ~2e-8 of the diagonal apart.  Whole steps are not compared: on this sliding,
    frictional contact a step takes 70-135 Newton iterations and 100+ line-search
    halvings decided on FP64 energy differences, and two solves that agree to
    1e-10 can end such a step ~1e-7 of the diagonal apart."""
    X = draped[0]
    diag = np.linalg.norm(X.max(0) - X.min(0))
    st_bj, x_bj = _step(draped, precision, F.PRECOND_BLOCK_JACOBI, 1e-30, 1e-10, max_newton=3)
    _, x_bj2 = _step(draped, precision, F.PRECOND_BLOCK_JACOBI, 1e-30, 1e-10, max_newton=3)
    st_ag, x_ag = _step(draped, precision, F.PRECOND_AGGREGATE, 1e-30, 1e-10, max_newton=3)
    assert st_ag.precond_fallbacks == 0
    assert st_ag.min_dist2 > 0 and st_bj.min_dist2 > 0
    assert st_ag.newton_iters == st_bj.newton_iters == 3
    spread = np.abs(x_bj2 - x_bj).max() / diag
    err = np.abs(x_ag - x_bj).max() / diag
    assert err < 1e-7 + 2 * spread, (err, spread, st_bj.as_dict(), st_ag.as_dict())


def test_aggregate_needs_fewer_iterations(cuda, draped):
    st_bj, _ = _step(draped, F.MIXED, F.PRECOND_BLOCK_JACOBI, 1e-3, 1e-4)
    st_ag, _ = _step(draped, F.MIXED, F.PRECOND_AGGREGATE, 1e-3, 1e-4)
    assert st_ag.precond_fallbacks == 0
    per_bj = st_bj.pcg_iters / max(1, st_bj.newton_iters)
    per_ag = st_ag.pcg_iters / max(1, st_ag.newton_iters)
    assert per_ag < 0.8 * per_bj, (per_ag, per_bj)

"""Failure detection of the time step, each failure made on the host.

The reference exits the process where a contact distance is not positive
(Library/FEM/IPC.h:773-776, 2014-2032) and its CCD loop has no bound
(Library/Math/Distance/CCD.h:279-483).  Here each failure is a status code and
the simulation stays usable:
  * a NaN in the state set through cipc_sim_set_state -> CIPC_ERR_NAN;
  * a start state with a contact inside the offset (d^2 - xi^2 <= 0)
    -> CIPC_ERR_NONPOSITIVE_DISTANCE;
  * an ACCD cap of one step per pair in the step-size search -> CIPC_ERR_ITER_CAP;
  * a PCG grid-wide wait limited to one poll -> the wait gives up, the kernel
    returns, and the step ends with CIPC_ERR_TIMEOUT (no fault, no hang: every
    wait in the solver is bounded and checks the shared error flag);
after each, a valid state steps normally on the same handle.
"""
import numpy as np
import pytest

import cipc_ffi as F
import workloads as W

pytestmark = pytest.mark.gpu

XI, DHAT, DT = 1e-3, 1e-3, 0.04


def _scene(y):
    cl = W.cloth_grid(8, 8, 0.2, 0.2, y=y, origin=(-0.1, -0.1))
    bx = W.box_shell(0.3, (0.0, -0.25, 0.0), nsub=2)  # top face at y = -0.1
    X, T, offs = W.merge_meshes(cl, bx)
    dbc = np.arange(offs[1], X.shape[0], dtype=np.int32)
    return X, T, dbc


def _sim(X, T, dbc):
    s = F.Sim(X, T, 200.0, 1e5, 0.3, 1e-3)
    s.set_dbc(dbc, X[dbc])
    _, dhat2 = s.init_oipc(DHAT)
    return s, dhat2


def _step_ok(s, X, dhat2):
    s.set_state(X, np.zeros_like(X))
    st = s.step(F.make_params(DT, dhat2, XI, newton_tol=1e-2))
    assert st.min_dist2 > 0 or st.n_constraints == 0


def test_nan_state_reported(cuda):
    X, T, dbc = _scene(-0.098)
    s, dhat2 = _sim(X, T, dbc)
    bad = X.copy()
    bad[5, 1] = np.nan
    s.set_state(bad, np.zeros_like(X))
    with pytest.raises(F.CipcError) as ei:
        s.step(F.make_params(DT, dhat2, XI))
    assert ei.value.status == F.CIPC_ERR_NAN
    v = np.zeros_like(X)
    v[3, 0] = np.inf
    s.set_state(X, v)
    with pytest.raises(F.CipcError) as ei:
        s.step(F.make_params(DT, dhat2, XI))
    assert ei.value.status == F.CIPC_ERR_NAN
    _step_ok(s, X, dhat2)
    s.close()


def test_start_inside_offset_reported(cuda):
    X, T, dbc = _scene(-0.098)
    s, dhat2 = _sim(X, T, dbc)
    inside = X.copy()
    inside[:64, 1] = -0.1 + 0.5 * XI  # the cloth 0.5 mm above the box top: d < xi
    s.set_state(inside, np.zeros_like(X))
    with pytest.raises(F.CipcError) as ei:
        s.step(F.make_params(DT, dhat2, XI))
    assert ei.value.status == F.CIPC_ERR_NONPOSITIVE_DISTANCE
    _step_ok(s, X, dhat2)
    s.close()


def test_accd_iteration_cap_reported(cuda):
    # 3 mm above the box top, falling at 0.5 m/s: the first Newton step heads into
    # the box, so the step-size search meets candidate pairs that need several
    # ACCD steps
    X, T, dbc = _scene(-0.097)
    s, dhat2 = _sim(X, T, dbc)
    v = np.zeros_like(X)
    v[:64, 1] = -0.5
    s.set_state(X, v)
    with pytest.raises(F.CipcError) as ei:
        s.step(F.make_params(DT, dhat2, XI, accd_max_iters=1))
    assert ei.value.status == F.CIPC_ERR_ITER_CAP
    _step_ok(s, X, dhat2)
    s.close()


@pytest.mark.parametrize("precision", [F.FP64, F.MIXED])
def test_pcg_wait_timeout_reported(cuda, precision):
    X, T, dbc = _scene(-0.098)
    s, dhat2 = _sim(X, T, dbc)
    s.set_state(X, np.zeros_like(X))
    with pytest.raises(F.CipcError) as ei:
        s.step(F.make_params(DT, dhat2, XI, precision=precision, pcg_wait_polls=1))
    assert ei.value.status == F.CIPC_ERR_TIMEOUT
    assert "gave up" in str(ei.value)
    _step_ok(s, X, dhat2)
    s.close()

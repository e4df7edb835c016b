"""Run logs in the reference's formats, checkpoint/restore and OBJ restart.

  * residual.txt gets one line per Newton iteration, "PNIter avgResMag maxRes
    Eprev L2Norm" printed with %d %le %le %le %le (IMPLICIT_EULER.h:668-670);
    counter.txt one "PNIter #constraints" line per step (:868-875), matching the
    step statistics; steps.jsonl one JSON object per step.
  * A run restored from cipc_sim_save_state after 3 steps and stepped 3 more
    ends within 1e-9 of the bounding-box diagonal of the uninterrupted run, with
    the same barrier stiffness (kappa is part of the checkpoint).  The bar is not
    bit equality: constraint lists are compacted and gradients scattered with
    atomics, so sums are ordered by arrival.
  * cipc_sim_load_obj_frames restarts from two written OBJ frames the way the
    reference's drivers do (positions from the last frame, velocity as the
    difference over dt): positions equal the frame's printed values, velocities
    (x1 - x0) / dt.
"""
import json
import re

import numpy as np
import pytest

import cipc_ffi as F
import workloads as W

pytestmark = pytest.mark.gpu

XI, DHAT, DT = 1e-3, 1e-3, 0.04
LE = r"-?\d\.\d{6}e[+-]\d{2,3}"


def _scene():
    cl = W.cloth_grid(10, 10, 0.5, 0.5, y=-0.092, origin=(-0.25, -0.25))
    bx = W.box_shell(0.3, (0.0, -0.25, 0.0), nsub=2)
    X, T, offs = W.merge_meshes(cl, bx)
    dbc = np.arange(offs[1], X.shape[0], dtype=np.int32)
    return X, T, dbc


def _sim(X, T, dbc):
    s = F.Sim(X, T, 200.0, 1e5, 0.3, 1e-3)
    s.set_dbc(dbc, X[dbc])
    _, dhat2 = s.init_oipc(DHAT)
    return s, F.make_params(DT, dhat2, XI, newton_tol=1e-2, pcg_tol=1e-8)


def test_run_logs_in_reference_format(cuda, tmp_path):
    X, T, dbc = _scene()
    s, prm = _sim(X, T, dbc)
    F.sim_set_output(s, str(tmp_path))
    stats = [s.step(prm).as_dict() for _ in range(3)]
    F.sim_set_output(s, None)
    s.step(prm)  # logging off: nothing more is written
    res = (tmp_path / "residual.txt").read_text().splitlines()
    assert len(res) == sum(st["newton_iters"] for st in stats)
    pat = re.compile(r"^\d+ %s %s %s %s$" % (LE, LE, LE, LE))
    assert all(pat.match(l) for l in res), res[:3]
    # PNIter restarts at 1 every step and counts up to the step's Newton iterations
    its = [int(l.split()[0]) for l in res]
    k = 0
    for st in stats:
        assert its[k:k + st["newton_iters"]] == list(range(1, st["newton_iters"] + 1))
        k += st["newton_iters"]
    cnt = (tmp_path / "counter.txt").read_text().splitlines()
    assert cnt == ["%d %d" % (st["newton_iters"], st["n_constraints"]) for st in stats]
    js = [json.loads(l) for l in (tmp_path / "steps.jsonl").read_text().splitlines()]
    assert [j["step"] for j in js] == [1, 2, 3]
    assert [j["newton_iters"] for j in js] == [st["newton_iters"] for st in stats]
    s.close()


def test_checkpoint_restore_continues_the_run(cuda, tmp_path):
    X, T, dbc = _scene()
    a, prm = _sim(X, T, dbc)
    for _ in range(3):
        a.step(prm)
    ck = str(tmp_path / "state.bin")
    F.sim_save_state(a, ck)
    for _ in range(3):
        a.step(prm)
    xa, va = a.state()
    ka = a.kappa()
    b, _ = _sim(X, T, dbc)
    b.set_kappa(1.0, 2.0)  # overwritten by the checkpoint
    F.sim_load_state(b, ck)
    for _ in range(3):
        b.step(prm)
    xb, vb = b.state()
    diag = np.linalg.norm(X.max(0) - X.min(0))
    assert np.abs(xa - xb).max() <= 1e-9 * diag
    assert np.array_equal(ka, b.kappa())
    # a checkpoint of another mesh is refused
    Xc, Tc = W.cloth_grid(6, 6, 0.2, 0.2, y=0.0, origin=(-0.1, -0.1))
    c = F.Sim(Xc, Tc, 200.0, 1e5, 0.3, 1e-3)
    with pytest.raises(F.CipcError) as ei:
        F.sim_load_state(c, ck)
    assert ei.value.status == F.CIPC_ERR_INVALID_ARG
    for s in (a, b, c):
        s.close()


def test_obj_frame_restart(cuda, tmp_path):
    X, T, dbc = _scene()
    s, prm = _sim(X, T, dbc)
    s.step(prm)
    f0 = str(tmp_path / "0.obj")
    s.write_obj(f0)
    s.step(prm)
    f1 = str(tmp_path / "1.obj")
    s.write_obj(f1)
    r, _ = _sim(X, T, dbc)
    F.sim_load_obj_frames(r, f0, f1, DT)
    x, v = r.state()
    read = lambda p: np.array([[float(t) for t in l.split()[1:4]] for l in open(p) if l.startswith("v ")])
    x0, x1 = read(f0), read(f1)
    assert np.array_equal(x, x1)
    assert np.allclose(v, (x1 - x0) / DT, rtol=0, atol=1e-12)
    r.step(prm)  # steps on from the restart
    s.close()
    r.close()


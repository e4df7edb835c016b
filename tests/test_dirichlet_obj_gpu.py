"""Device-side Dirichlet motion (Init_Dirichlet / Step_Dirichlet,
Library/FEM/BOUNDARY_CONDITION.h:16-157) and the OBJ frame writer
(Write_TriMesh_Obj, Library/Utils/MESHIO.h:182-213) through the C ABI.

Checks: the selected vertices and their targets against a numpy restatement of
the relative-box rule; targets after several steps against the composed
axis-angle rotations and translations in numpy (1e-12); a cloth-on-rotating-
sphere run driven by the device motion against the same run driven by host
targets (1e-9 of the bounding-box diagonal); the OBJ file's vertices (printf
%le, 7 significant digits) and 1-based faces."""
import math

import numpy as np
import pytest

import cipc_ffi as F
import workloads as W

pytestmark = pytest.mark.gpu


def _rot(axis, ang):
    a = np.asarray(axis, float)
    c, s = math.cos(ang), math.sin(ang)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return c * np.eye(3) + (1 - c) * np.outer(a, a) + s * K


def _select(X, lo_rel, hi_rel, b, e):
    P = X[b:e]
    bmin, bmax = P.min(0), P.max(0)
    lo = np.asarray(lo_rel) * (bmax - bmin) + bmin
    hi = np.asarray(hi_rel) * (bmax - bmin) + bmin
    inside = np.all((P >= lo) & (P <= hi), axis=1)
    return np.arange(b, e)[inside]


def test_init_and_step_dirichlet_match_numpy(cuda):
    X, T, dbc, c = W.cloth_on_sphere(n=12, subdiv=2)
    ncl = 12 * 12
    s = F.Sim(X, T, 200.0, 1e5, 0.3, 1e-3)
    groups = [  # (rel_min, rel_max, v, center, axis, deg/s, begin, end)
        ((0, 0, 0), (1, 1, 1), (0, 0, 0), c, (0, 1, 0), 114.59155902616465, ncl, -1),
        ((0, 0, 0), (0.1, 1, 1), (0.0, 0.05, -0.02), (0, 0, 0), (0, 0, 1), 0.0, 0, ncl),
        ((0.9, 0, 0.9), (1, 1, 1), (0.01, 0, 0), (0.5, 0, 0.5), (1 / 3 ** 0.5,) * 3, 30.0, 0, ncl),
    ]
    expect_idx, expect_tg, motion = [], [], []
    for lo, hi, v, cen, ax, deg, b, e in groups:
        added = s.init_dirichlet(lo, hi, v, cen, ax, deg, b, e)
        sel = _select(X, lo, hi, b, X.shape[0] if e < 0 else e)
        assert added == len(sel)
        expect_idx.append(sel)
        expect_tg.append(X[sel].copy())
        motion.append((np.asarray(v, float), np.asarray(cen, float), np.asarray(ax, float), deg))
    idx, tg = s.dbc()
    assert np.array_equal(idx, np.concatenate(expect_idx))
    assert np.array_equal(tg, np.concatenate(expect_tg))
    dt = 0.02
    for _ in range(5):
        s.step_dirichlet(dt)
        for k, (v, cen, ax, deg) in enumerate(motion):
            R = _rot(ax, deg / 180 * math.pi * dt)
            expect_tg[k] = (expect_tg[k] - cen) @ R.T + cen + v * dt
    _, tg = s.dbc()
    assert np.abs(tg - np.concatenate(expect_tg)).max() <= 1e-12
    s.close()


def test_device_motion_drives_the_step(cuda):
    X, T, dbc, c = W.cloth_on_sphere(n=20, subdiv=3)
    ncl = 20 * 20
    dt, omega = 0.02, 2.0

    def make():
        s = F.Sim(X, T, 200.0, 1e5, 0.3, 1e-3)
        _, dhat2 = s.init_oipc(1e-3)
        return s, F.make_params(dt, dhat2, 5e-4, mu=0.4, newton_tol=1e-5, precision=F.FP64, pcg_tol=1e-10)

    a, prm = make()
    b, _ = make()
    b.init_dirichlet((0, 0, 0), (1, 1, 1), (0, 0, 0), c, (0, 1, 0), omega * 180 / math.pi, ncl, -1)
    idx, _ = b.dbc()
    assert np.array_equal(np.sort(idx), np.sort(dbc))
    diag = np.linalg.norm(X.max(0) - X.min(0))
    ok = (F.CIPC_ERR_NOT_CONVERGED,)
    for k in range(4):
        a.set_dbc(idx, W.rotate_y(X[idx], c, omega * dt * (k + 1)))
        b.step_dirichlet(dt)
        a.step(prm, allow=ok)
        b.step(prm, allow=ok)
        assert np.abs(a.state()[0] - b.state()[0]).max() <= 1e-9 * diag, k
    a.close()
    b.close()


def test_write_obj(cuda, tmp_path):
    X, T, dbc, c = W.cloth_on_sphere(n=8, subdiv=1)
    s = F.Sim(X, T, 200.0, 1e5, 0.3, 1e-3)
    x = X + 1e-3 * np.sin(np.arange(X.size)).reshape(X.shape)
    s.set_state(x, None)
    path = tmp_path / "frame.obj"
    s.write_obj(path)
    V, Fc = [], []
    for line in open(path):
        tok = line.split()
        if tok[0] == "v":
            V.append([float(t) for t in tok[1:]])
            assert all("e" in t for t in tok[1:])  # %le
        elif tok[0] == "f":
            Fc.append([int(t) for t in tok[1:]])
    V, Fc = np.array(V), np.array(Fc)
    assert V.shape == X.shape and Fc.shape == T.shape
    assert np.abs(V - x).max() <= 1e-6 * np.abs(x).max()
    assert np.array_equal(Fc, T + 1)
    s.close()

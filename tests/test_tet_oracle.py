"""Oracle restatement of the volumetric Neo-Hookean tetrahedron (oracle_tet.cpp,
Library/Physics/NEOHOOKEAN.h) and of the tetrahedral surface extraction, on the
CPU: energy against numpy, gradient and unprojected Hessian against central
finite differences, projected Hessian PSD, inversion flagged, and the cube
generator's tetrahedra positively oriented with a closed surface."""
import numpy as np

import workloads as W
from oracle import oracle_ffi as orc

LAM, MU = 5e5, 3e5


def _tet(rng, amp=0.3):
    X = rng.normal(0, 0.01, (4, 3))
    D = np.column_stack([X[1] - X[0], X[2] - X[0], X[3] - X[0]])
    if np.linalg.det(D) < 0:
        X[[1, 2]] = X[[2, 1]]
        D = np.column_stack([X[1] - X[0], X[2] - X[0], X[3] - X[0]])
    x = (X @ (np.eye(3) + rng.normal(0, amp, (3, 3))).T).ravel()
    return x, np.linalg.inv(D)


def test_energy_matches_numpy():
    rng = np.random.default_rng(0)
    n = 0
    for _ in range(100):
        x, Dinv = _tet(rng)
        E, g, H, ok = orc.tet_nh_elem(x, Dinv.ravel(), 1e-7, LAM, MU)
        xx = x.reshape(4, 3)
        F = np.column_stack([xx[1] - xx[0], xx[2] - xx[0], xx[3] - xx[0]]) @ Dinv
        J = np.linalg.det(F)
        assert ok == (J > 0)
        if J <= 0:
            continue
        n += 1
        Ee = 1e-7 * (MU / 2 * (np.sum(F * F) - 3) - MU * np.log(J) + LAM / 2 * np.log(J) ** 2)
        assert abs(E - Ee) <= 1e-11 * abs(Ee)
    assert n > 50


def test_gradient_and_hessian_finite_differences():
    rng = np.random.default_rng(1)
    checked = 0
    for _ in range(20):
        x, Dinv = _tet(rng, 0.1)
        E, g, H, ok = orc.tet_nh_elem(x, Dinv.ravel(), 1e-7, LAM, MU, project=False)
        if not ok:
            continue
        eps = 1e-8
        gf, Hf = np.zeros(12), np.zeros((12, 12))
        for k in range(12):
            d = np.zeros(12)
            d[k] = eps
            Ep, gp, _, _ = orc.tet_nh_elem(x + d, Dinv.ravel(), 1e-7, LAM, MU, project=False)
            Em, gm, _, _ = orc.tet_nh_elem(x - d, Dinv.ravel(), 1e-7, LAM, MU, project=False)
            gf[k] = (Ep - Em) / (2 * eps)
            Hf[:, k] = (gp - gm) / (2 * eps)
        assert np.abs(g - gf).max() <= 1e-5 * np.abs(g).max()
        assert np.abs(H - Hf).max() <= 1e-5 * np.abs(H).max()
        checked += 1
    assert checked > 10


def test_projection_and_inversion():
    rng = np.random.default_rng(2)
    for _ in range(50):
        x, Dinv = _tet(rng, 0.5)
        E, g, H, ok = orc.tet_nh_elem(x, Dinv.ravel(), 1e-7, LAM, MU, project=True)
        if ok:
            assert np.linalg.eigvalsh(H).min() >= -1e-9 * np.abs(H).max()
    x, Dinv = _tet(rng, 0.0)
    xx = x.reshape(4, 3).copy()
    xx[3] = xx[0] - (xx[3] - xx[0])  # reflect the fourth vertex: det F < 0
    E, g, H, ok = orc.tet_nh_elem(xx.ravel(), Dinv.ravel(), 1e-7, LAM, MU)
    assert not ok


def test_tet_box_orientation_and_surface():
    X, tets = W.tet_box(n=3, size=0.1)
    assert tets.shape == (6 * 27, 4)
    vol = 0
    for t in tets:
        d = np.linalg.det(np.column_stack([X[t[1]] - X[t[0]], X[t[2]] - X[t[0]], X[t[3]] - X[t[0]]]))
        assert d > 0
        vol += d / 6
    assert abs(vol - 1e-3) <= 1e-15
    sh = orc.Shell(X, np.zeros((0, 3), np.int32), 200.0, 1e5, 0.3, 1e-3,
                   tets=dict(tets=tets, E=1e5, nu=0.3, rho=1000.0))
    a = sh.arrays()
    c = np.zeros(5, np.int32)
    sh.L.orc_shell_counts(sh.h, c.ctypes.data)
    # closed surface of the cube: 12 n^2 triangles, 3/2 as many edges, and the
    # (n+1)^3 - (n-1)^3 outer vertices
    assert c[4] == 12 * 9 and a["bedge"].shape[0] == 12 * 9 * 3 // 2 and a["bnode"].shape[0] == 64 - 8
    assert abs(a["mass"].sum() - 1e-3 * 1000.0) <= 1e-12

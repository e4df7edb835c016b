"""Oracle restatement of the isotropic strain-limiting barrier (oracle_sl.cpp,
Library/FEM/Shell/INEXT.h) checked on its own: energy against a direct numpy
evaluation of the barrier on the singular values, gradient and (unprojected)
Hessian against central finite differences of the energy, the projected Hessian
PSD, the feasibility flag at the limits, and the C2 activation at s_hat."""
import numpy as np
import pytest

from oracle import oracle_ffi as orc

S = np.array([1.05, 0.95])
SH = np.array([1.0, 0.99])


def _tri(rng):
    X = np.array([[0, 0, 0], [0.01, 0, 0], [0.003, 0.009, 0]]) + rng.normal(0, 1e-3, (3, 3)) * [1, 1, 0]
    e1, e2 = X[1] - X[0], X[2] - X[0]
    A = np.array([[e1 @ e1, e1 @ e2], [e1 @ e2, e2 @ e2]])
    Pi = np.linalg.inv(A)
    return X, np.array([Pi[0, 0], Pi[0, 1], Pi[1, 1]])


def _deformed(rng, X, amp=0.02):
    Fm = np.eye(3) + rng.normal(0, amp, (3, 3))
    return (X @ Fm.T).ravel()


def _barrier(s, lim, hat):
    return -(hat - s) ** 2 * np.log((lim - s) / (lim - hat)) / (lim - hat) ** 2


def _energy_np(x, X, kh, ks):
    """the barrier on the singular values of x's deformation relative to X"""
    x = x.reshape(3, 3)
    A = np.column_stack([x[1] - x[0], x[2] - x[0]])
    Ab = np.column_stack([X[1] - X[0], X[2] - X[0]])
    # any factor of the rest form gives the same singular values
    F = A @ np.linalg.pinv(np.linalg.cholesky(Ab.T @ Ab).T)
    E = 0.0
    for s in np.linalg.svd(F, compute_uv=False):
        if s > SH[0]:
            E += kh * ks[0] * _barrier(s, S[0], SH[0])
        if ks[1] > 0 and s < SH[1]:
            E += kh * ks[1] * _barrier(s, S[1], SH[1])
    return E


@pytest.mark.parametrize("lower", [0.0, 5e2])
def test_energy_matches_singular_value_form(lower):
    rng = np.random.default_rng(0)
    ks = np.array([1e3, lower])
    kh = 1e-7
    n = 0
    for _ in range(100):
        X, P = _tri(rng)
        x = _deformed(rng, X)
        E, g, H, ok = orc.strain_limit_elem(x, P, kh, S, SH, ks)
        if not ok:
            continue
        n += 1
        Ee = _energy_np(x, X, kh, ks)
        assert abs(E - Ee) <= 1e-10 * abs(Ee) + 1e-30, (E, Ee)
    assert n > 50


def test_gradient_and_hessian_finite_differences():
    rng = np.random.default_rng(1)
    ks = np.array([1e3, 5e2])
    kh = 1e-7
    checked = 0
    for _ in range(40):
        X, P = _tri(rng)
        x = _deformed(rng, X)
        E, g, H, ok = orc.strain_limit_elem(x, P, kh, S, SH, ks, project=False)
        if not ok or E == 0:
            continue
        eps = 1e-7
        gf = np.zeros(9)
        Hf = np.zeros((9, 9))
        for k in range(9):
            d = np.zeros(9)
            d[k] = eps
            Ep, gp, _, okp = orc.strain_limit_elem(x + d, P, kh, S, SH, ks, project=False)
            Em, gm, _, okm = orc.strain_limit_elem(x - d, P, kh, S, SH, ks, project=False)
            assert okp and okm
            gf[k] = (Ep - Em) / (2 * eps)
            Hf[:, k] = (gp - gm) / (2 * eps)
        assert np.abs(g - gf).max() <= 1e-5 * np.abs(g).max()
        assert np.abs(H - Hf).max() <= 1e-5 * np.abs(H).max()
        checked += 1
    assert checked > 10


def test_projected_hessian_is_psd():
    rng = np.random.default_rng(2)
    ks = np.array([1e3, 5e2])
    for _ in range(50):
        X, P = _tri(rng)
        x = _deformed(rng, X, 0.03)
        E, g, H, ok = orc.strain_limit_elem(x, P, 1e-7, S, SH, ks, project=True)
        if not ok:
            continue
        assert np.allclose(H, H.T, atol=1e-12 * max(np.abs(H).max(), 1e-30))
        assert np.linalg.eigvalsh(H).min() >= -1e-9 * max(np.abs(H).max(), 1e-30)


def test_feasibility_and_activation():
    rng = np.random.default_rng(3)
    X, P = _tri(rng)
    ks = np.array([1e3, 5e2])
    # uniform scaling: both stretches equal the factor
    for f, ok_exp, active in ((1.0, True, False), (0.995, True, False), (1.02, True, True), (0.97, True, True),
                              (1.06, False, None), (1.2, False, None), (0.94, False, None), (0.9, False, None)):
        x = (X * f).ravel()
        E, g, H, ok = orc.strain_limit_elem(x, P, 1e-7, S, SH, ks)
        assert ok == ok_exp, f
        if ok and not active:
            assert E == 0 and np.abs(g).max() == 0
        if ok and active:
            assert E > 0
    # C2 at s_hat: energy and slope vanish like (s - s_hat)^2 ln and (s - s_hat) ln
    k1 = np.array([1e3, 0.0])
    E0, g0, _, _ = orc.strain_limit_elem((X * 1.02).ravel(), P, 1e-7, S, SH, k1)
    E, g, H, ok = orc.strain_limit_elem((X * (1 + 1e-6)).ravel(), P, 1e-7, S, SH, k1)
    assert ok and 0 < E < 1e-8 * E0 and np.abs(g).max() < 1e-3 * np.abs(g0).max()

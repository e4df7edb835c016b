"""The oracle's restatement of the learned block-Jacobi correction: operator,
features, forward pass and parameter gradient of the three losses (one optimally
scaled step, one unit step, eight steps of preconditioned steepest descent),
checked on seeded synthetic SPD systems (no GPU).  The gradient is checked against central finite differences
of the oracle's own loss; the GPU kernels are then checked against this oracle
(tests/test_learned_gpu.py)."""
import numpy as np
import pytest

from lp_systems import dense_matrix, synthetic_system

H, L = 8, 2


@pytest.fixture(scope="module")
def system(orc):
    s = synthetic_system(n=5, ncon=6, seed=3, ndbc=2)
    return s, orc.LearnedSystem(**s)


def _params(orc, seed, scale):
    rng = np.random.default_rng(seed)
    n = orc.lp_num_params(H, L)
    return rng.standard_normal(n) * scale


def test_operator_matches_dense(orc, system):
    s, S = system
    A = dense_matrix(s)
    assert np.allclose(A, A.T, atol=1e-4)
    assert np.linalg.eigvalsh(A).min() > 0
    x = np.random.default_rng(1).standard_normal((S.nv, 3))
    assert np.allclose(orc.lp_apply(S, x).ravel(), A @ x.ravel(), rtol=1e-10, atol=1e-9)


def test_zero_output_layer_is_block_jacobi(orc, system):
    s, S = system
    prm = _params(orc, 0, 0.3)
    nout = 6 * H + 6
    prm[-nout:] = 0
    r = np.random.default_rng(2).standard_normal((S.nv, 3))
    r[s["proj"] == 1] = 0
    A = dense_matrix(s)
    p = np.linalg.solve(A, r.ravel())
    loss, g, z = orc.lp_loss_grad(H, L, prm, S, r, p)
    _, _, E = orc.lp_features(S)
    zb = np.einsum("iab,ib->ia", E, r)
    assert np.allclose(z, zb, rtol=1e-12, atol=1e-14)
    # loss = 1 - cos^2 in the H inner product, within [0, 1]
    assert 0 <= loss <= 1


def test_features_are_scale_invariant(orc, system):
    s, S = system
    x1, a1, _ = orc.lp_features(S)
    s2 = dict(s)
    s2["val"] = s["val"] * np.float32(64.0)
    s2["cdiag"] = s["cdiag"] * np.float32(64.0)
    s2["chess"] = s["chess"] * np.float32(64.0)
    x2, a2, _ = orc.lp_features(orc.LearnedSystem(**s2))
    # the Dirichlet identity blocks do not scale; compare free vertices
    free = s["proj"] == 0
    assert np.allclose(a1, a2, rtol=1e-6, atol=1e-12)
    assert np.allclose(x1[free], x2[free], rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_gradient_matches_finite_differences(orc, system, kind):
    s, S = system
    prm = _params(orc, 5, 0.4)
    r = np.random.default_rng(4).standard_normal((S.nv, 3))
    r[s["proj"] == 1] = 0
    p = np.linalg.solve(dense_matrix(s), r.ravel())
    loss, g, _ = orc.lp_loss_grad(H, L, prm, S, r, p, kind)
    assert loss > 0 and (kind == 1 or loss < 1)
    rng = np.random.default_rng(7)
    idx = np.unique(np.concatenate([rng.choice(prm.shape[0], 60, replace=False),
                                    np.arange(prm.shape[0] - 54, prm.shape[0])]))
    eps = 1e-6
    for k in idx:
        d = np.zeros_like(prm)
        d[k] = eps
        lp = orc.lp_loss_grad(H, L, prm + d, S, r, p, kind)[0]
        lm = orc.lp_loss_grad(H, L, prm - d, S, r, p, kind)[0]
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(fd)) + 1e-8, (k, fd, g[k])


def test_operator_with_float32_input(orc, system):
    s, S = system
    x = np.random.default_rng(9).standard_normal((S.nv, 3)).astype(np.float32)
    assert np.allclose(orc.lp_apply(S, x).ravel(), dense_matrix(s) @ x.ravel().astype(np.float64), rtol=1e-10,
                       atol=1e-9)
